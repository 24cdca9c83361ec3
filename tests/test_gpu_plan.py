"""Whole planning queries on the GPU (pump_plan) against the reference's own
results recorded in the golden fixtures: exploration wavefront sizes, stored
and considered path counts, goal paths, the chosen solution, its node
sequence, its printed CP and cost, and path.txt and discretizedPath.txt byte
for byte."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = ["ref_N64_input", "ref_N1000_input", "ref_N1000_boxes10_noise1e-3",
         "ref_N1000_boxes10_noise0.3", "ref_N4000_indoor_P1024"]


def make_problem(L, g, **over):
    pb = L.Problem()
    L.load().pump_problem_defaults(C.byref(pb))
    obs = np.ascontiguousarray(g["prob_obstacles"], np.float32)
    pb.N = int(g["N"])
    pb.num_obstacles = obs.shape[0]
    pb.obstacles = obs.ctypes.data
    for k in range(6):
        pb.init[k], pb.goal[k] = float(g["prob_init"][k]), float(g["prob_goal"][k])
        pb.lo[k], pb.hi[k] = float(g["prob_lo"][k]), float(g["prob_hi"][k])
    pb.offset_mult = float(g["prob_offset_mult"])
    pb.cp_target, pb.cp_factor = float(g["cp_target"]), float(g["cp_factor"])
    for k, v in over.items():
        setattr(pb, k, v)
    return pb, obs


def run_plan(L, ctx, pb, rows=400, trace_cap=0):
    res = L.PlanResult()
    path = np.zeros((rows, 6), np.float32)
    nodes = np.zeros(64, np.int32)
    res.path, res.path_cap = path.ctypes.data, rows
    res.nodes, res.nodes_cap = nodes.ctypes.data, 64
    ctrl = np.zeros((4096, 6), np.float32)
    res.ctrl_path, res.ctrl_cap = ctrl.ctypes.data, 4096
    trace = np.zeros(max(trace_cap, 1), np.int32)
    if trace_cap:
        res.wf_trace, res.wf_trace_cap = trace.ctypes.data, trace_cap
    st = L.load().pump_plan(ctx.handle, C.byref(pb), C.byref(res), None)
    run_plan.ctrl = ctrl[: min(res.ctrl_len, 4096)].copy()
    run_plan.trace = trace[: res.wf_trace_len].copy() if trace_cap else None
    return st, res, path[: res.path_len].copy(), nodes[: res.num_nodes].copy()


# Whole queries of the reference program whose pair BVPs come from its own
# GPU kernel (tests/golden/make_golden.py refgpu): the library's
# PUMP_BVP_PARITY_GPU mode
GPU_CASES = ["refgpu_N1000_boxes10_noise1e-3", "refgpu_N1000_boxes10_noise0.3",
             "refgpu_N4000_indoor_P1024"]


@pytest.mark.parametrize("name", CASES + GPU_CASES)
def test_plan_matches_reference(name, gpu, pumplib, goldens):
    """The whole query, including the exploration trace: the (parent path,
    edge) of every expansion in the reference's launch order."""
    torch, ctx = gpu
    g = goldens[name]
    P = int(g["hsmc_particles"]) if "hsmc_particles" in g else 128
    mode = pumplib.PUMP_BVP_PARITY_GPU if name.startswith("refgpu_") else pumplib.PUMP_BVP_PARITY
    pb, _obs = make_problem(pumplib, g, num_hsmc=P, bvp_mode=mode)
    st, res, path, nodes = run_plan(pumplib, ctx, pb, trace_cap=g["wavefront_trace"].size + 16)
    assert st in (pumplib.PUMP_OK, pumplib.PUMP_ERR_NO_SOLUTION), pumplib.load().pump_last_error()
    sizes = np.array(res.wavefront_sizes[: res.iterations], np.int32)
    if sizes.size and sizes[-1] == 0:
        sizes = sizes[:-1]
    assert np.array_equal(sizes, g["wavefront_sizes"])
    assert np.array_equal(run_plan.trace, g["wavefront_trace"])
    assert res.num_paths == int(g["num_paths"])
    assert res.num_considered == int(g["num_considered"])
    assert res.goal_paths == int(g["goal_paths"])
    assert res.success == int(g["success"])
    if res.success:
        assert res.soln_path_idx == int(g["soln_idx"])
        assert np.array_equal(nodes, g["soln_nodes"])
        assert "%g" % res.soln_cp == "%g" % float(g["soln_cp_printed"])
        assert "%g" % res.soln_cost == "%g" % float(g["soln_cost_printed"])
        text = "".join("".join("%g " % v for v in row) + "\n" for row in path.astype(np.float64))
        assert text == str(g["path_txt"])
    ctrl = "".join("".join("%g, " % v for v in row) + "\n" for row in run_plan.ctrl.astype(np.float64))
    assert ctrl == str(g["ctrl_txt"])


def test_plan_matches_oracle_cfg0(gpu, pumplib, oracle):
    """The benchmark's small configuration (10 boxes, 10 waypoints per edge)."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    obs = workloads.random_boxes(10, 0)
    g = dict(N=np.array(1000), prob_obstacles=obs, prob_init=np.float32(workloads.INIT),
             prob_goal=np.float32(workloads.GOAL), prob_lo=np.float32(workloads.LO),
             prob_hi=np.float32(workloads.HI), prob_offset_mult=np.float32(1e-3),
             cp_target=np.float32(0.01), cp_factor=np.float32(2))
    pb, _o = make_problem(pumplib, g, num_disc=9)
    st, res, path, nodes = run_plan(pumplib, ctx, pb)
    r = oracle.plan(1000, obs, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI,
                    np.float32(1e-3), 0.01, 2.0, numDisc=9)
    assert res.num_paths == r["numPaths"] and res.num_considered == r["numConsidered"]
    assert res.success == r["success"] and res.soln_path_idx == r["solnPathIdx"]
    assert np.array_equal(nodes, r["nodes"])
    assert np.array_equal(path.view(np.uint32), r["path"].view(np.uint32))
    assert np.float32(res.soln_cp) == np.float32(r["solnCP"])
    assert np.float32(res.soln_cost) == np.float32(r["solnCost"])
    assert res.ctrl_len == len(r["ctrl_path"])
    assert np.array_equal(run_plan.ctrl.view(np.uint32), r["ctrl_path"].view(np.uint32))


def fill_problem(L, q, keep):
    pb = L.Problem()
    L.load().pump_problem_defaults(C.byref(pb))
    obs = np.ascontiguousarray(q["obstacles"], np.float32)
    keep.append(obs)
    pb.N, pb.num_obstacles, pb.obstacles = q["N"], obs.shape[0], obs.ctypes.data
    from pump_gb300 import workloads
    for k in range(6):
        pb.init[k], pb.goal[k] = q["init"][k], q["goal"][k]
        pb.lo[k], pb.hi[k] = workloads.LO[k], workloads.HI[k]
    pb.offset_mult, pb.cp_target, pb.cp_factor = float(q["offset_mult"]), q["cp"], q["eta"]
    return pb


def test_plan_batch_equals_single_queries(gpu, pumplib):
    """Concurrent queries (pump_plan_batch, 4 workers) give exactly what each
    query gives alone: Halton queries of the three BVP modes go through the
    batch's shared roadmaps, the query with explicit samples plans on its own."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    L = pumplib.load()
    qs = workloads.batch_queries(12, seed=77, n_range=(200, 1400), obs_range=(5, 30))
    keep = []
    pbs = (pumplib.Problem * len(qs))(*[fill_problem(pumplib, q, keep) for q in qs])
    for k in range(len(qs)):
        pbs[k].bvp_mode = (pumplib.PUMP_BVP_PARITY, pumplib.PUMP_BVP_PRECISION,
                           pumplib.PUMP_BVP_PARITY_GPU)[k % 3]
    rng = np.random.default_rng(5)
    own = rng.uniform(workloads.LO, workloads.HI, size=(pbs[3].N, 6)).astype(np.float32)
    own[0], own[-1] = qs[3]["init"], qs[3]["goal"]
    keep.append(own)
    pbs[3].samples = own.ctypes.data
    res = (pumplib.PlanResult * len(qs))()
    paths = [np.zeros((400, 6), np.float32) for _ in qs]
    for k in range(len(qs)):
        res[k].path, res[k].path_cap = paths[k].ctypes.data, 400
    sts = (C.c_int * len(qs))()
    pumplib.check(L.pump_plan_batch(0, pbs, res, sts, len(qs), 4))
    f32 = lambda x: np.float32(x).view(np.uint32)
    batch_error = L.pump_last_error().decode() if hasattr(L.pump_last_error(), "decode") else ""
    for k, q in enumerate(qs):
        st1, r1, p1, _ = run_plan(pumplib, ctx, pbs[k])
        assert sts[k] == st1, batch_error
        assert f32(res[k].rn) == f32(r1.rn)
        assert (res[k].num_edges, res[k].iterations, res[k].num_paths, res[k].success,
                res[k].soln_path_idx) == (r1.num_edges, r1.iterations, r1.num_paths, r1.success,
                                          r1.soln_path_idx)
        assert list(res[k].wavefront_sizes) == list(r1.wavefront_sizes)
        assert f32(res[k].soln_cp) == f32(r1.soln_cp) and f32(res[k].soln_cost) == f32(r1.soln_cost)
        assert np.array_equal(paths[k][: res[k].path_len].view(np.uint32), p1.view(np.uint32))


@pytest.mark.parametrize("name", ["ref_N1000_boxes10_noise0.3", "ref_N1000_boxes10_noise1e-3"])
def test_plan_with_refinement(name, gpu, pumplib, goldens):
    """Refinement after the search: accepted only with MC CP <= target and a
    lower cost; the search itself is unchanged."""
    torch, ctx = gpu
    g = goldens[name]
    pb, _obs = make_problem(pumplib, g, refine_iters=30, refine_lambda=10.0)
    st, res, path, nodes = run_plan(pumplib, ctx, pb)
    assert st == pumplib.PUMP_OK, pumplib.load().pump_last_error()
    assert res.success == 1 and res.soln_path_idx == int(g["soln_idx"])
    assert np.array_equal(nodes, g["soln_nodes"])
    assert np.isfinite(res.refine_cost) and res.refine_cp >= 0
    if res.refined:
        assert res.soln_cp <= float(g["cp_target"])
        assert res.soln_cost == np.float32(res.refine_cost)
        assert res.soln_cost < float(g["soln_cost_printed"]) * (1 + 1e-5)
    else:
        assert "%g" % res.soln_cost == "%g" % float(g["soln_cost_printed"])


def _fields(res):
    f32 = lambda x: int(np.float32(x).view(np.uint32))
    return (res.num_edges, res.iterations, res.num_paths, res.num_considered, res.goal_paths,
            res.success, res.soln_path_idx, f32(res.soln_cp), f32(res.soln_cost), res.path_len,
            res.ctrl_len, tuple(res.wavefront_sizes))


def test_search_graph_equals_host_loop(gpu, pumplib, goldens):
    """The search loop as one graph launch (conditional while node, counters
    kept by a control kernel) gives exactly the host-driven loop's results,
    for single queries (edges checked up front) and batches (edges checked
    when the search reaches their nodes)."""
    torch, ctx = gpu
    L = pumplib.load()
    from pump_gb300 import workloads
    try:
        for name in CASES + GPU_CASES:
            g = goldens[name]
            P = int(g["hsmc_particles"]) if "hsmc_particles" in g else 128
            mode = pumplib.PUMP_BVP_PARITY_GPU if name in GPU_CASES else pumplib.PUMP_BVP_PARITY
            pb, _obs = make_problem(pumplib, g, num_hsmc=P, bvp_mode=mode)
            out = []
            for on in (0, 1):
                L.pump_search_graph(on)
                st, res, path, nodes = run_plan(pumplib, ctx, pb)
                out.append((st, _fields(res), path.view(np.uint32).tobytes(), nodes.tobytes(),
                            run_plan.ctrl.view(np.uint32).tobytes()))
            assert out[0] == out[1], name
        qs = workloads.batch_queries(8, seed=91, n_range=(200, 1200), obs_range=(5, 60))
        keep = []
        pbs = (pumplib.Problem * len(qs))(*[fill_problem(pumplib, q, keep) for q in qs])
        for k in range(len(qs)):
            pbs[k].bvp_mode = (pumplib.PUMP_BVP_PARITY, pumplib.PUMP_BVP_PRECISION,
                               pumplib.PUMP_BVP_PARITY_GPU)[k % 3]
        got = []
        for level in (0, 2):  # batch workers host-driven, then as graphs
            L.pump_search_graph(level)
            res = (pumplib.PlanResult * len(qs))()
            paths = [np.zeros((400, 6), np.float32) for _ in qs]
            for k in range(len(qs)):
                res[k].path, res[k].path_cap = paths[k].ctypes.data, 400
            sts = (C.c_int * len(qs))()
            pumplib.check(L.pump_plan_batch(0, pbs, res, sts, len(qs), 3))
            got.append([(sts[k], _fields(res[k]), paths[k][: res[k].path_len].view(np.uint32).tobytes())
                        for k in range(len(qs))])
        assert got[0] == got[1]
    finally:
        L.pump_search_graph(1)


@pytest.mark.parametrize("groups", [(16, 5000), (3, 0)])
def test_plan_batch_groups_equal_single_queries(groups, gpu, pumplib):
    """Grouped search loops (pump_batch_groups): the queries of a group run
    in one launch of the loop graph, each with its own box count, sample
    count and waypoints by edge length; every query gives exactly what it
    gives alone.  (16 queries, 5 ms window: large groups; 3 queries, no
    window: groups of whatever is waiting.)  The three BVP modes are mixed,
    so groups also split by mode."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    L = pumplib.load()
    qs = workloads.batch_queries(20, seed=303, n_range=(200, 2500), obs_range=(5, 100))
    keep = []
    pbs = (pumplib.Problem * len(qs))(*[fill_problem(pumplib, q, keep) for q in qs])
    for k, q in enumerate(qs):
        pbs[k].num_disc, pbs[k].disc_len, pbs[k].disc_min = q["num_disc"], q["disc_len"], q["disc_min"]
        pbs[k].bvp_mode = (pumplib.PUMP_BVP_PRECISION, pumplib.PUMP_BVP_PARITY,
                           pumplib.PUMP_BVP_PRECISION, pumplib.PUMP_BVP_PARITY_GPU)[k % 4]
    res = (pumplib.PlanResult * len(qs))()
    paths = [np.zeros((400, 6), np.float32) for _ in qs]
    for k in range(len(qs)):
        res[k].path, res[k].path_cap = paths[k].ctypes.data, 400
    sts = (C.c_int * len(qs))()
    try:
        L.pump_batch_groups(*groups)
        pumplib.check(L.pump_plan_batch(0, pbs, res, sts, len(qs), 6))
    finally:
        L.pump_batch_groups(1, 100)
    for k in range(len(qs)):
        st1, r1, p1, _ = run_plan(pumplib, ctx, pbs[k])
        assert sts[k] == st1, k
        assert _fields(res[k]) == _fields(r1), k
        assert np.array_equal(paths[k][: res[k].path_len].view(np.uint32), p1.view(np.uint32)), k


def test_plan_batch_equals_single_large(gpu, pumplib):
    """Larger batch queries (N 3000-6000, 40-100 boxes), whose search
    iterations list enough nodes for the wide form of the lazy edge checks
    (256-edge chunks, per-warp pair queue): the batch still gives exactly
    what each query gives alone."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    L = pumplib.load()
    qs = workloads.batch_queries(3, seed=123, n_range=(3000, 6000), obs_range=(40, 100))
    keep = []
    pbs = (pumplib.Problem * len(qs))(*[fill_problem(pumplib, q, keep) for q in qs])
    for k in range(len(qs)):
        pbs[k].bvp_mode = pumplib.PUMP_BVP_PRECISION
    res = (pumplib.PlanResult * len(qs))()
    paths = [np.zeros((400, 6), np.float32) for _ in qs]
    for k in range(len(qs)):
        res[k].path, res[k].path_cap = paths[k].ctypes.data, 400
    sts = (C.c_int * len(qs))()
    pumplib.check(L.pump_plan_batch(0, pbs, res, sts, len(qs), 2))
    for k in range(len(qs)):
        st1, r1, p1, _ = run_plan(pumplib, ctx, pbs[k])
        assert sts[k] == st1
        assert _fields(res[k]) == _fields(r1)
        assert np.array_equal(paths[k][: res[k].path_len].view(np.uint32), p1.view(np.uint32))


def test_plan_path_state_readback(gpu, pumplib, goldens):
    """The stored paths' times and particle masks a caller can ask for
    (pump_plan_result.path_time / path_valid): path 0 is the initial node at
    time 0 with every particle valid, every time lies inside the particle
    table, every stored path passed the CP cut-off (its invalid fraction,
    as calculateCP_HSMC computes it, is at most cpTarget * cpFactor,
    PUMP.cu:12, 175-178), and the query's other results are unchanged."""
    torch, ctx = gpu
    L = pumplib.load()
    g = goldens["ref_N1000_boxes10_noise0.3"]
    pb, _obs = make_problem(pumplib, g)
    st, res, path, _n = run_plan(pumplib, ctx, pb)
    n, P = res.num_paths, pb.num_hsmc
    words = (P + 31) // 32
    ptime = np.zeros(n, np.float32)
    pvalid = np.zeros(n * words, np.uint32)
    res2 = pumplib.PlanResult()
    res2.path_time, res2.path_valid, res2.path_state_cap = ptime.ctypes.data, pvalid.ctypes.data, n
    assert L.pump_plan(ctx.handle, C.byref(pb), C.byref(res2), None) == st
    assert (res2.num_paths, res2.soln_path_idx) == (n, res.soln_path_idx)
    assert ptime[0] == 0 and np.all(pvalid[:words] == 0xFFFFFFFF)
    assert np.all(ptime[1:] > 0) and np.all(ptime < 0.05 * (pb.table_rows - 1))
    valid = np.unpackbits(pvalid.view(np.uint8).reshape(n, -1), axis=1, bitorder="little")[:, :P]
    cp = (P - valid.sum(1)).astype(np.float32) / np.float32(P)
    assert np.all(cp <= np.float32(pb.cp_target) * np.float32(pb.cp_factor))
