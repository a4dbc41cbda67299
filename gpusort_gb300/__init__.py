"""gpusort_gb300: a GB300-native sorting engine with the entry points of
monotone-RK/gpusort (HykSort, SampleSort, HyperQuickSort).

The compute path is the in-tree CUDA library (``_lib/libgpusort_gb300.so``,
built for sm_103a by ``gpusort_gb300._build``) behind the C ABI in
``include/gpusort_gb300.h``. This Python package is a thin host mirror over
that ABI for tests and benchmarks; the C++ drop-in headers live in
``include/gpusort/``.
"""
from .capi import Context, GsError, Server, load  # noqa: F401

__all__ = ["Context", "GsError", "Server", "load"]
