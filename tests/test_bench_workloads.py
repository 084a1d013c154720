"""The benchmark's workload definitions (bench.py, no GPU): the serving
trace with refinement is the single-level trace with 0-2 levels drawn per
request (same arrivals, separations and walls; base grid N / 2^levels, at
least the minimum base; the finest level at the single-level resolution),
the batched ensemble is seeded and within its size set, and both are
reproducible."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_serving_trace_with_refinement_is_the_same_trace():
    a = bench.serve_requests(128)
    b = bench.serve_requests(128, amr=True)
    assert len(a) == len(b) == bench.SERVE["nreq"]
    assert all(r["max_level"] == 0 for r in a)
    assert {r["max_level"] for r in b} <= set(bench.SERVE["levels"])
    for x, y in zip(a, b):
        assert x["arrival"] == y["arrival"] and x["d"] == y["d"] and x["gamma"] == y["gamma"]
        assert np.array_equal(x["centres"], y["centres"])
        m = y["max_level"]
        assert y["N"] == x["N"] >> m and y["N"] >= bench.SERVE["min_base"]
        assert abs(y["dx"] - x["dx"] * 2 ** m) <= 1e-12 * x["dx"] * 2 ** m
        assert y["t_end"] == x["t_end"]
        if m:
            assert y["regrid_dt"] > 0 and all(t > 0 for t in y["te_crit"])
    # arrivals are increasing (a Poisson trace) and reproducible
    arr = [r["arrival"] for r in a]
    assert arr == sorted(arr)
    assert [r["arrival"] for r in bench.serve_requests(128)] == arr


def test_batched_ensemble_spec_is_seeded():
    Ns, lam = bench.ensemble_spec()
    Ns2, lam2 = bench.ensemble_spec()
    assert Ns == Ns2 and np.array_equal(lam, lam2)
    assert len(Ns) == bench.ENSEMBLE["nreal"]
    assert set(Ns) <= set(bench.ENSEMBLE["sizes"])
    lo, hi = bench.ENSEMBLE["lam"]
    assert np.all((lam >= lo) & (lam <= hi))
