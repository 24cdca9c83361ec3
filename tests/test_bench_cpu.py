"""bench.py's host-side bookkeeping, without a GPU: the roofline record of
every arithmetic mode and dominant kernel, the default arguments, and the
replica aggregation without a process group."""
import math
import sys
import os

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

# per-kernel milliseconds of one step (the shape of Query.pipeline's kernel_ms)
KS = {"roadmap": 0.78, "rn_bracket": 0.019, "bvp_pairs": 0.643, "rn_edges": 0.093,
      "discretize": 0.044, "sample_free": 0.010, "free_edges": 0.111, "hsmc": 0.203}
N, E, M, W, H, P = 4000, 799800, 77174, 9, 5, 1024


@pytest.mark.parametrize("mode", ["precision", "parity", "parity_gpu"])
def test_roofline_record_every_mode(mode):
    ks = dict(KS)
    if mode != "precision":
        ks["bvp_pairs"] = 6.1 if mode == "parity" else 8.4
    r = bench.roofline("bvp_pairs", ks, N, E, M, W, H, P, mode, 1.06, 2070.0)
    assert r["kernel"] == "bvp_pairs" and r["bound"] == "issue"
    assert math.isfinite(r["frac"]) and 0.0 < r["frac"] < 1.5
    assert r["unit"] == "G warp-instructions/s"
    assert "bvp_pairs_fp64" in r["all"] and "rn_edges" in r["all"]


@pytest.mark.parametrize("dom", ["hsmc", "free_edges", "discretize"])
def test_roofline_memory_bound_kernels(dom):
    r = bench.roofline(dom, KS, N, E, M, W, H, P, "precision", 1.06, 2070.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert math.isfinite(r["achieved"]) and r["achieved"] > 0 and r["peak"] > 0


def test_defaults_and_aggregate():
    saved = sys.argv
    try:
        sys.argv = ["bench.py"]
        a = bench.parse()
    finally:
        sys.argv = saved
    assert (a.gpus, a.mode, a.num, a.particles, a.impl) == (1, "precision", 4000, 1024, "ours")
    assert a.warmup >= 3 and a.steps >= 1
    units, times = bench.aggregate(None, 123, [1.5, 2.5])
    assert units == 123 and times == [1.5, 2.5]
    assert bench.GROUPS[0] > 1 and bench.GROUPS[1] >= 0
