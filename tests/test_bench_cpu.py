"""Host-side logic of bench.py that its records rest on: the equal-p99
comparison of the serving sweep and the whole-job throughput."""
import pytest

import bench


def _pt(load, offered, plain, served):
    return {"load": load, "offered_gkeys_s": offered,
            "plain": {"gkeys_s": plain[0], "p99_ms": plain[1]},
            "served": {"gkeys_s": served[0], "p99_ms": served[1]}}


def test_equal_p99_takes_the_plain_arm_before_saturation():
    sweep = [
        _pt(0.5, 10.0, (10.0, 2.0), (10.0, 1.5)),
        _pt(1.0, 20.0, (19.5, 4.0), (20.0, 2.0)),   # plain still delivers (>= 95%)
        _pt(1.5, 30.0, (21.0, 30.0), (29.0, 3.9)),  # plain saturated
        _pt(2.0, 40.0, (21.0, 60.0), (36.0, 9.0)),  # served above the bound
    ]
    rec = bench.equal_p99(sweep)
    assert rec["bound_p99_ms"] == 4.0 and rec["plain_load"] == 1.0
    assert rec["served_load"] == 1.5 and rec["served_gkeys_s"] == 29.0
    assert rec["throughput_ratio"] == pytest.approx(29.0 / 19.5)


def test_equal_p99_stops_at_the_first_load_the_plain_arm_misses():
    sweep = [
        _pt(0.5, 10.0, (10.0, 2.0), (10.0, 2.0)),
        _pt(1.0, 20.0, (15.0, 9.0), (20.0, 2.0)),   # missed: later points do not count
        _pt(1.5, 30.0, (29.0, 1.0), (30.0, 1.0)),
    ]
    rec = bench.equal_p99(sweep)
    assert rec["plain_load"] == 0.5 and rec["bound_p99_ms"] == 2.0
    assert rec["served_gkeys_s"] == 30.0  # any served point within the bound


def test_equal_p99_without_a_delivered_plain_point():
    sweep = [_pt(1.0, 20.0, (10.0, 50.0), (20.0, 2.0))]
    assert bench.equal_p99(sweep) == {"bound_p99_ms": None}


def test_equal_p99_when_no_served_point_meets_the_bound():
    sweep = [_pt(1.0, 20.0, (20.0, 1.0), (20.0, 5.0))]
    rec = bench.equal_p99(sweep)
    assert rec["bound_p99_ms"] == 1.0 and "throughput_ratio" not in rec


def test_whole_job_throughput_counts_every_rank():
    # 2^30 keys per rank, 4 ranks, 13.6 ms (the slowest rank's time)
    assert bench.whole_job_gkeys(1 << 30, 4, 13.6) == pytest.approx(4 * (1 << 30) / 13.6e-3 / 1e9)
