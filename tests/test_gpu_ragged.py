"""Waypoints per edge by edge length (the batched configuration's 4-32
waypoints per edge): the ragged waypoint layout through the offsets, the
waypoints, the edge check, HSMC and whole queries, each against the oracle's
restatement over the same layout.  The reference fixes numDisc per problem
(mainPUMP.cu:57), so there is no reference output to compare; with every
edge at num_disc the layout is the reference's and the uniform tests hold.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import bits_to_bytes, dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu

DISC_LEN, DISC_MIN, DISC_MAX = 0.025, 3, 31


@pytest.fixture(scope="module")
def ragged(gpu, pumplib, oracle, goldens):
    """The N = 1000 parity roadmap of the 10-box problem with the ragged
    layout, on the device and as the oracle computes it."""
    torch, ctx = gpu
    L = pumplib.load()
    g = goldens["ref_N1000_boxes10_noise0.3"]
    N = int(g["N"])
    obs = g["prob_obstacles"].astype(np.float32)
    s = oracle.halton_samples(N, g["prob_init"], g["prob_goal"], g["prob_lo"], g["prob_hi"])
    c, t = oracle.bvp_pairs(s)
    k = int((N - 1) * N * np.float32(0.05))
    rn = oracle.lib().orc_select_kth(c.size, c, k)
    src, dst, _ce, te = oracle.build_edges(c, t, N, rn)
    E = src.size
    d_s, d_src, d_dst, d_te = dev(torch, s), dev(torch, src), dev(torch, dst), dev(torch, te)
    d_off = empty(torch, E + 1, torch.int64)
    total = C.c_longlong(0)
    pumplib.check(L.pump_disc_offsets(ptr(d_s), ptr(d_src), ptr(d_dst), E, DISC_LEN, DISC_MIN, DISC_MAX,
                                      ptr(d_off), C.byref(total), stream(torch)))
    off = oracle.disc_offsets(src, dst, s, DISC_LEN, DISC_MIN, DISC_MAX)
    return dict(torch=torch, ctx=ctx, L=L, g=g, N=N, obs=obs, s=s, src=src, dst=dst, te=te, E=E,
                d_s=d_s, d_src=d_src, d_dst=d_dst, d_te=d_te, d_off=d_off, total=int(total.value), off=off)


def test_disc_offsets(ragged):
    r = ragged
    assert r["total"] == int(r["off"][-1])
    assert np.array_equal(host(r["d_off"], r["E"] + 1), r["off"])
    w = np.diff(r["off"])
    assert w.min() >= DISC_MIN + 1 and w.max() <= DISC_MAX + 1 and len(np.unique(w)) > 10


@pytest.mark.parametrize("mode", [0, 1])
def test_ragged_waypoints_and_edge_check(mode, ragged, pumplib, oracle):
    """Waypoints bit for bit with the oracle in the parity arithmetic (within
    the precision mode's stated bound in binary32), and the edge check of
    each edge's own segments equal to the oracle's on the same waypoints."""
    r, torch, L = ragged, ragged["torch"], ragged["L"]
    d_disc = empty(torch, r["total"] * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges_off(ptr(r["d_s"]), ptr(r["d_src"]), ptr(r["d_dst"]), ptr(r["d_te"]),
                                              r["E"], ptr(r["d_off"]), DISC_MAX, mode, ptr(d_disc),
                                              stream(torch)))
    disc = host(d_disc).reshape(-1, 6)
    if mode == 0:
        ref = oracle.discretize_edges_off(r["src"], r["dst"], r["s"], r["off"])
        assert np.array_equal(disc.view(np.uint32), ref.view(np.uint32))
    else:
        # every interior waypoint against pathPoint in binary64 at the same t
        e = np.repeat(np.arange(r["E"]), np.diff(r["off"]))
        i = np.arange(r["total"]) - r["off"][e]
        nd = (np.diff(r["off"]) - 1)[e]
        inner = (i > 0) & (i < nd)
        dt = (r["te"][e] / nd.astype(np.float32)).astype(np.float32)
        t = (dt * i.astype(np.float32)).astype(np.float32)
        ref = oracle.path_point64(t[inner], r["te"][e][inner], r["s"][r["src"][e][inner]],
                                  r["s"][r["dst"][e][inner]])
        assert np.abs(disc[inner][:, :3] - ref[:, :3]).max() <= 1e-6
    d_fe = empty(torch, r["E"], torch.uint8)
    d_obs = dev(torch, r["obs"])
    pumplib.check(L.pump_free_edges_off(ptr(d_obs), r["obs"].shape[0], ptr(d_disc), ptr(r["d_off"]), r["E"],
                                        DISC_MAX, ptr(d_fe), stream(torch)))
    fe = oracle.free_edges_off(disc, r["off"], r["obs"])
    assert np.array_equal(host(d_fe, r["E"]), fe) and 0 < fe.mean() < 1


def test_ragged_hsmc(ragged, pumplib, oracle):
    """HSMC with half-spaces derived in the kernel over each edge's own
    waypoints against the oracle's cacheHalfspaces + propagateValidParticles
    over the same ragged layout."""
    r, torch, L = ragged, ragged["torch"], ragged["L"]
    d_disc = empty(torch, r["total"] * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges_off(ptr(r["d_s"]), ptr(r["d_src"]), ptr(r["d_dst"]), ptr(r["d_te"]),
                                              r["E"], ptr(r["d_off"]), DISC_MAX, 0, ptr(d_disc),
                                              stream(torch)))
    disc = host(d_disc).reshape(-1, 6)
    obs, om, P, Pmc, T, maxHS = r["obs"], np.float32(0.3), 128, 2048, 400, 5
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    fe = oracle.free_edges_off(disc, r["off"], obs)
    nhs = r["total"] * maxHS
    a = np.empty(nhs * 3, np.float32)
    b = np.empty(nhs, np.float32)
    cnt = np.zeros(r["total"], np.int32)
    oracle.lib().orc_cache_halfspaces_off(r["E"], r["off"].ctypes.data, disc, fe, obs.shape[0], obs.reshape(-1),
                                          maxHS, maxd2, a, b, cnt)
    tm, _ = oracle.particle_tables(0x1234, Pmc, T, pmajor=False)
    rng = np.random.default_rng(17)
    base, n_new = 40, 3000
    edges = rng.choice(np.nonzero(fe)[0], n_new).astype(np.int32)
    prev = rng.integers(0, base, n_new).astype(np.int32)
    times = np.zeros(base + n_new, np.float32)
    times[:base] = rng.uniform(0, 6, base).astype(np.float32)
    valid = np.zeros((base + n_new, P), np.uint8)
    valid[:base] = rng.random((base, P)) < 0.9
    packed = np.packbits(valid, axis=1, bitorder="little").view(np.uint32)
    cp_o = np.zeros(base + n_new, np.float32)
    oracle.lib().orc_hsmc_propagate_off(n_new, r["off"].ctypes.data, edges, prev, base, a, b, times, r["te"],
                                        0.05, maxHS, tm.reshape(-1), om, Pmc, valid, P, cp_o)
    d_valid = dev(torch, packed)
    d_cp = empty(torch, base + n_new, torch.float32)
    d_err = dev(torch, np.zeros(1, np.int32))
    keep = [dev(torch, x) for x in (edges, prev, obs, times, tm)]
    pumplib.check(L.pump_hsmc_propagate_boxes_off(
        n_new, DISC_MAX + 1, ptr(keep[0]), ptr(keep[1]), r["E"], base, ptr(keep[2]), obs.shape[0], ptr(d_disc),
        ptr(r["d_off"]), float(maxd2), maxHS, ptr(keep[3]), ptr(r["d_te"]), 0.05, ptr(keep[4]), Pmc, T, float(om),
        ptr(d_valid), P, ptr(d_cp), ptr(d_err), stream(torch)))
    torch.cuda.synchronize()
    assert int(host(d_err)[0]) == 0
    got = bits_to_bytes(host(d_valid).reshape(base + n_new, -1), P)
    assert np.array_equal(got[base:], valid[base:])
    assert np.array_equal(host(d_cp)[base:base + n_new].view(np.uint32), cp_o[base:].view(np.uint32))
    assert 0 < valid[base:].mean() < 1


def test_ragged_offsets_rejected(ragged, pumplib):
    """Offsets with an edge count outside [2, max + 1] are refused by the
    entry points that stage waypoints (nothing is written past the stage)."""
    r, torch, L = ragged, ragged["torch"], ragged["L"]
    bad = r["off"].copy()
    bad[5:] += 40  # edge 4 gets 40 more waypoints than max_disc allows
    d_bad = dev(torch, bad)
    d_disc = empty(torch, int(bad[-1]) * 6, torch.float32)
    assert L.pump_discretize_edges_off(ptr(r["d_s"]), ptr(r["d_src"]), ptr(r["d_dst"]), ptr(r["d_te"]), r["E"],
                                       ptr(d_bad), DISC_MAX, 0, ptr(d_disc),
                                       stream(torch)) == pumplib.PUMP_ERR_BAD_INPUT
    d_obs, d_fe = dev(torch, r["obs"]), empty(torch, r["E"], torch.uint8)
    assert L.pump_free_edges_off(ptr(d_obs), r["obs"].shape[0], ptr(d_disc), ptr(d_bad), r["E"], DISC_MAX,
                                 ptr(d_fe), stream(torch)) == pumplib.PUMP_ERR_BAD_INPUT


def _problem(pumplib, g, **over):
    from test_gpu_plan import make_problem
    return make_problem(pumplib, g, num_disc=DISC_MAX, disc_len=DISC_LEN, disc_min=DISC_MIN, **over)


@pytest.mark.parametrize("name", ["ref_N1000_boxes10_noise0.3", "ref_N1000_boxes10_noise1e-3"])
def test_ragged_plan_matches_oracle(name, gpu, pumplib, goldens, oracle):
    """Whole queries with waypoints by edge length: the exploration trace,
    the stored paths, the returned path and the controller's discretisation
    bit for bit with the oracle's query over the same layout; the search
    loop as one graph launch gives the same."""
    from test_gpu_plan import run_plan
    torch, ctx = gpu
    L = pumplib.load()
    g = goldens[name]
    pb, obs = _problem(pumplib, g)
    r = oracle.plan(int(g["N"]), obs, g["prob_init"], g["prob_goal"], g["prob_lo"], g["prob_hi"],
                    np.float32(g["prob_offset_mult"]), float(g["cp_target"]), float(g["cp_factor"]),
                    numDisc=DISC_MAX, trace_cap=4_000_000, discLen=DISC_LEN, discMin=DISC_MIN)
    out = []
    try:
        for level in (0, 1):
            L.pump_search_graph(level)
            st, res, path, nodes = run_plan(pumplib, ctx, pb, trace_cap=r["wf_trace"].size + 16 if level == 0 else 0)
            assert st in (pumplib.PUMP_OK, pumplib.PUMP_ERR_NO_SOLUTION), L.pump_last_error()
            if level == 0:
                assert np.array_equal(run_plan.trace, r["wf_trace"])
            assert (res.num_paths, res.num_considered, res.success) == (r["numPaths"], r["numConsidered"],
                                                                        r["success"])
            assert res.soln_path_idx == r["solnPathIdx"] and np.array_equal(nodes, r["nodes"])
            assert np.array_equal(path.view(np.uint32), r["path"].view(np.uint32))
            assert np.array_equal(run_plan.ctrl.view(np.uint32), r["ctrl_path"].view(np.uint32))
            out.append(path.tobytes())
    finally:
        L.pump_search_graph(1)
    assert out[0] == out[1]


def test_ragged_batch_equals_single_queries(gpu, pumplib):
    """Batched queries with waypoints by edge length (edges checked when the
    search reaches their nodes) give what each query gives alone."""
    from pump_gb300 import workloads
    from test_gpu_plan import fill_problem, run_plan
    torch, ctx = gpu
    L = pumplib.load()
    qs = workloads.batch_queries(9, seed=55, n_range=(300, 1500), obs_range=(5, 40))
    keep = []
    pbs = (pumplib.Problem * len(qs))(*[fill_problem(pumplib, q, keep) for q in qs])
    for k in range(len(qs)):
        pbs[k].num_disc, pbs[k].disc_len, pbs[k].disc_min = DISC_MAX, DISC_LEN, DISC_MIN
        pbs[k].bvp_mode = (0, 1, 2)[k % 3]
    res = (pumplib.PlanResult * len(qs))()
    paths = [np.zeros((400, 6), np.float32) for _ in qs]
    for k in range(len(qs)):
        res[k].path, res[k].path_cap = paths[k].ctypes.data, 400
    sts = (C.c_int * len(qs))()
    pumplib.check(L.pump_plan_batch(0, pbs, res, sts, len(qs), 3))
    for k in range(len(qs)):
        st1, r1, p1, _ = run_plan(pumplib, ctx, pbs[k])
        assert sts[k] == st1
        assert (res[k].num_paths, res[k].num_considered, res[k].soln_path_idx) == (
            r1.num_paths, r1.num_considered, r1.soln_path_idx)
        assert np.array_equal(paths[k][: res[k].path_len].view(np.uint32), p1.view(np.uint32))
