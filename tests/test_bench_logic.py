"""Host logic of bench.py that decides what a line reports (no GPU): the serving knee,
the canonical flop count and the e2e step's fraction of the device-to-host link."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def level(offered, achieved, p50, p99, n=1000, done=None, secs=1.5):
    return {"offered_req_per_s": offered, "achieved_req_per_s": achieved, "requests": n,
            "completed": n if done is None else done, "p50_ms": p50, "p99_ms": p99,
            "probabilities_per_s": achieved * 1e6, "seconds": secs}


def test_knee_is_the_highest_load_served_without_queueing():
    import bench
    n = lambda rate: int(rate * 1.5)  # noqa: E731
    levels = [level(r, a, p50, p99, n=n(r)) for r, a, p50, p99 in (
        (9000, 8970, 0.146, 0.30), (27000, 27180, 0.20, 0.40), (54000, 54470, 0.26, 1.49),
        (63000, 63480, 1.40, 6.70),     # keeps up, but the median is queueing
        (72000, 64150, 92.0, 177.0))]   # falls behind
    knee = bench.serve_knee(levels, 1.5)
    assert knee["offered_req_per_s"] == 54000
    summary = bench.serve_summary(45000.0, knee, [], levels)
    assert summary["p99_ms"] == 1.49
    assert summary["highest_throughput"]["achieved_req_per_s"] == 64150


def test_serving_summary_reports_the_load_meeting_the_latency_target():
    import bench
    n = lambda rate: int(rate * 1.5)  # noqa: E731
    levels = []
    for r, a, p50, p99, p99_500 in ((9000, 8970, 0.15, 0.30, 0.28), (54000, 54470, 0.26, 1.49, 0.40),
                                    (63000, 63480, 0.30, 5.0, 4.9), (72000, 64150, 92.0, 177.0, 177.0)):
        lv = level(r, a, p50, p99, n=n(r))
        lv["atm500x500"] = {"n": 100, "p50_ms": p50, "p99_ms": p99_500}
        levels.append(lv)
    knee = bench.serve_knee(levels, 1.5)
    assert knee["offered_req_per_s"] == 63000  # keeps up, median within 2x of the lightest
    target = bench.serve_summary(1.0, knee, [], levels)["highest_load_meeting_p99_target_500x500"]
    assert target["offered_req_per_s"] == 54000 and target["atm500x500"]["p99_ms"] == 0.40
    assert target["fraction_of_highest_throughput"] == round(54470 / 64150, 3)


def test_knee_needs_every_request_completed():
    import bench
    levels = [level(1000, 1000, 0.1, 0.2, n=1500),
              level(2000, 2000, 0.1, 0.2, n=3000, done=2999)]
    assert bench.serve_knee(levels, 1.5)["offered_req_per_s"] == 1000
    assert bench.serve_knee([], 1.5) is None


def test_canonical_flops_per_bin():
    import bench
    assert bench.f_bin(0) == 257
    assert bench.f_bin(4) == 27 + 230 * 5 + 216 * 7
    np.testing.assert_array_equal(bench.f_bin(np.array([0, 1])), [257, 27 + 460 + 216])


def test_link_summary_is_the_e2e_bytes_over_the_measured_link():
    import bench
    s = bench.link_summary(288e6, 1.5, 192.0)
    assert s["d2h_gbs_achieved"] == 192.0
    assert s["frac_of_link"] == 1.0
    assert bench.link_summary(144e6, 1.5, 192.0)["frac_of_link"] == 0.5
