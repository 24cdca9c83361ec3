"""The C oracle against the reference's own outputs (CPU only).

The golden fixtures are outputs of the reference program itself, built for
the CPU (tests/golden/make_golden.py): its Halton samples, every pair's
optimal time and cost, the waypoints, edge and sample masks, half-spaces, the
exploration wavefront of every iteration and the returned path.  The oracle
must reproduce each bit for bit; it then serves as the checker of the GPU
kernels.
"""
import hashlib

import numpy as np
import pytest


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


CASES = ["ref_N64_input", "ref_N1000_input", "ref_N1000_boxes10_noise1e-3",
         "ref_N1000_boxes10_noise0.3", "ref_N4000_indoor_P1024"]


def problem(g):
    return (int(g["N"]), g["prob_obstacles"], g["prob_init"], g["prob_goal"], g["prob_lo"],
            g["prob_hi"], np.float32(g["prob_offset_mult"]))


@pytest.fixture(scope="module")
def roadmaps(oracle, goldens):
    """Oracle roadmap per distinct sample set, shared across cases."""
    cache = {}

    def get(name):
        g = goldens[name]
        N, obs, init, goal, lo, hi, om = problem(g)
        key = (N, tuple(init), tuple(goal), tuple(lo), tuple(hi))
        if key not in cache:
            s = oracle.halton_samples(N, init, goal, lo, hi)
            c, t = oracle.bvp_pairs(s)
            k = int((N - 1) * N * np.float32(0.05))
            rn = oracle.lib().orc_select_kth(c.size, c, k)
            src, dst, ce, te = oracle.build_edges(c, t, N, rn)
            disc = oracle.discretize_edges(src, dst, s, 8)
            cache[key] = dict(samples=s, copts=c, topts=t, k=k, rn=rn, src=src, dst=dst, disc=disc)
        return cache[key]
    return get


@pytest.mark.parametrize("name", CASES)
def test_samples_and_pair_bvps(name, goldens, roadmaps):
    g, r = goldens[name], roadmaps(name)
    assert np.array_equal(r["samples"].view(np.uint32), g["samples"].view(np.uint32))
    assert sha(r["copts"]) == str(g["copts_sha"])
    assert sha(r["topts"]) == str(g["topts_sha"])
    assert r["k"] == int(g["rn_idx"])
    assert float("%g" % r["rn"]) == pytest.approx(float(g["rn_printed"]), rel=1e-5)


@pytest.mark.parametrize("name", CASES)
def test_waypoints_masks_halfspaces(name, oracle, goldens, roadmaps):
    g, r = goldens[name], roadmaps(name)
    N, obs, *_rest, om = problem(g)
    E = r["src"].size
    nref = int(g["free_edges_n"])
    # the reference sizes its edge arrays at rnIdx (>= E); rows past E are unused
    disc_ref_prefix = r["disc"].reshape(-1)
    assert E <= nref
    stride = int(g["stride"]) if "stride" in g else 97
    if E == nref:
        assert sha(r["disc"]) == str(g["disc_sha"])
    elif "disc_sub" in g:
        sub = disc_ref_prefix[::stride]
        assert np.array_equal(sub[: g["disc_sub"].size], g["disc_sub"][: sub.size])
    fe = oracle.free_edges(r["disc"], obs)
    ref_fe = np.unpackbits(g["free_edges_bits"])[:nref]
    assert np.array_equal(fe, ref_fe[:E])
    fs = oracle.sample_free(r["samples"], obs)
    assert np.array_equal(fs, g["free_samples"])
    maxHS = min(obs.shape[0], 5)
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    a, b, _ = oracle.cache_halfspaces(r["disc"], fe, obs, maxHS, maxd2)
    if E == nref:
        assert sha(a) == str(g["as_sha"]) and sha(b) == str(g["bs_sha"])
    sub_a = g["as_sub"]
    stride = 1 if sub_a.size == a.size else stride
    n = min(sub_a.size, a[::stride].size)
    assert np.array_equal(a[::stride][:n].view(np.uint32), sub_a[:n].view(np.uint32))


def ctrl_text(rows):
    return "".join("".join("%g, " % v for v in row) + "\n" for row in np.asarray(rows, np.float64))


@pytest.mark.parametrize("name", CASES)
def test_whole_query(name, oracle, goldens):
    """Exploration trace, stored paths and the returned path (PUMP.cu:3-607)."""
    g = goldens[name]
    N, obs, init, goal, lo, hi, om = problem(g)
    P = int(g["hsmc_particles"]) if "hsmc_particles" in g else 128
    r = oracle.plan(N, obs, init, goal, lo, hi, om, float(g["cp_target"]), float(g["cp_factor"]),
                    P=P, T_table=400, trace_cap=4_000_000)
    sizes = r["wavefront_sizes"]
    if sizes.size and sizes[-1] == 0:  # last iteration found nothing to expand: no launch
        sizes = sizes[:-1]
    assert np.array_equal(sizes, g["wavefront_sizes"])
    assert np.array_equal(r["wf_trace"], g["wavefront_trace"])
    assert r["numPaths"] == int(g["num_paths"])
    assert r["numConsidered"] == int(g["num_considered"])
    assert r["goalPathCount"] == int(g["goal_paths"])
    assert r["success"] == int(g["success"])
    if r["success"]:
        assert r["solnPathIdx"] == int(g["soln_idx"])
        assert np.array_equal(r["nodes"], g["soln_nodes"])
        assert "%g" % r["solnCP"] == "%g" % float(g["soln_cp_printed"])
        assert "%g" % r["solnCost"] == "%g" % float(g["soln_cost_printed"])
        # path.txt as the reference prints it (printArray: "%g " per value)
        text = "".join("".join("%g " % v for v in row) + "\n" for row in r["path"].astype(np.float64))
        assert text == str(g["path_txt"])
    # discretizedPath.txt (PUMP.cu:553-579: "%g, " per value, 6 per line)
    assert ctrl_text(r["ctrl_path"]) == str(g["ctrl_txt"])


@pytest.mark.parametrize("name", ["refgpu_N1000_boxes10_noise1e-3", "refgpu_N1000_boxes10_noise0.3",
                                  "refgpu_N4000_indoor_P1024"])
def test_gpu_bvp_goldens_ran_on_the_reference_gpu_pairs(name, goldens, roadmaps):
    """The whole-query fixtures of the reference GPU's arithmetic were made on
    exactly the pair arrays its fillCoptsTopts wrote on the GB300 (the SHA-256
    of refgpu_bvp_N*.npz), on the same samples; those arrays differ from the
    parity arithmetic's (which the oracle and the CPU build compute)."""
    g = goldens[name]
    ref = goldens["refgpu_bvp_N%d" % int(g["N"])]
    assert str(g["copts_sha"]) == str(ref["copts_sha"]) and str(g["topts_sha"]) == str(ref["topts_sha"])
    r = roadmaps(name)
    assert np.array_equal(r["samples"].view(np.uint32), g["samples"].view(np.uint32))
    assert sha(r["copts"]) != str(g["copts_sha"])
