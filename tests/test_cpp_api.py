"""The C++ drop-in headers (include/gpusort/): they compile against the C
ABI here, and on the GPU the test program's every check passes."""
import subprocess
from pathlib import Path

import pytest

CPP = Path(__file__).resolve().parent / "cpp"


def _build():
    r = subprocess.run(["make", "-s", "-B", "-C", str(CPP), "api_test"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return CPP / "api_test"


def test_headers_compile_and_link(built_lib):
    assert _build().exists()


@pytest.mark.gpu
def test_cpp_entry_points_on_gpu(built_lib):
    exe = _build()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
