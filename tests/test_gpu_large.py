"""The large configuration on one GB300: N = 32000 Halton samples (1.02e9
ordered pairs, 51.2 M edges), 200 boxes with sides U[0.02, 0.1], noise
multiplier 5e-3, 4096 particles, 16 waypoints per edge, CP target 0.005,
eta 2, precision BVP.

The reference cannot run it unmodified: its sample count is a compile-time
array size (mainPUMP.cu:47-49), its particle tables hold 2048 particles
(hardCoded.cuh:12-13) and its half-space kernel stages at most 85 boxes
(mainPUMP.cu:484-487).  Each stage is checked on sampled subsets against
the oracle or a binary64 reference, and the whole query for consistency.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large(gpu, pumplib, oracle):
    from pump_gb300 import workloads
    torch, ctx = gpu
    L = pumplib.load()
    cfg = workloads.CONFIGS["cfg4"]
    N = cfg["N"]
    obs = np.ascontiguousarray(cfg["obstacles"](0), np.float32)
    pb = pumplib.Problem()
    L.pump_problem_defaults(C.byref(pb))
    pb.N, pb.num_disc, pb.num_hsmc, pb.num_mc = N, cfg["num_disc"], cfg["num_hsmc"], cfg["num_mc"]
    pb.num_obstacles, pb.obstacles = obs.shape[0], obs.ctypes.data
    for d in range(6):
        pb.init[d], pb.goal[d] = workloads.INIT[d], workloads.GOAL[d]
        pb.lo[d], pb.hi[d] = workloads.LO[d], workloads.HI[d]
    pb.offset_mult, pb.cp_target, pb.cp_factor = cfg["offset_mult"], cfg["cp"], cfg["eta"]
    pb.bvp_mode = pumplib.PUMP_BVP_PRECISION
    pb.max_paths = cfg["max_paths"]
    return dict(torch=torch, ctx=ctx, L=L, cfg=cfg, N=N, obs=obs, pb=pb)


def test_large_roadmap_stages(large, pumplib, oracle):
    large["roadmap"] = {}
    """Pair BVPs on a strided sample against the binary64 minimiser (1 ulp in
    cost), rn the exact k-th smallest of all 1.02e9 costs, the edges exactly
    the pairs below rn in (i, j) order, waypoints and edge checks on a
    sample of edges against the oracle's checks of the same waypoints."""
    from pump_gb300 import workloads
    torch, L, N, obs = large["torch"], large["L"], large["N"], large["obs"]
    nd = large["cfg"]["num_disc"]
    W = nd + 1
    f6 = lambda v: (C.c_float * 6)(*[float(x) for x in v])  # noqa: E731
    d_s = empty(torch, N * 6, torch.float32)
    pumplib.check(L.pump_halton_samples(N, f6(workloads.LO), f6(workloads.HI), f6(workloads.INIT),
                                        f6(workloads.GOAL), ptr(d_s), stream(torch)))
    s = host(d_s).reshape(N, 6)
    npairs = N * (N - 1)
    d_c, d_t = empty(torch, npairs, torch.float32), empty(torch, npairs, torch.float32)
    pumplib.check(L.pump_bvp_pairs(ptr(d_s), N, 5.0, pumplib.PUMP_BVP_PRECISION, ptr(d_c), ptr(d_t),
                                   stream(torch)))
    # strided sample of pairs against the binary64 minimiser
    idx = np.arange(0, npairs, 50_021, dtype=np.int64)
    i = idx // (N - 1)
    r = idx - i * (N - 1)
    j = r + (r >= i)
    t64, c64 = oracle.bvp_binary64(s[i], s[j])
    ci = torch.from_numpy(idx).cuda()
    c_s, t_s = d_c[ci].cpu().numpy(), d_t[ci].cpu().numpy()
    uc = np.abs(c_s.view(np.int32).astype(np.int64) - c64.astype(np.float32).view(np.int32).astype(np.int64))
    assert uc.max() <= 1 and (uc == 0).mean() >= 0.999
    assert np.all(np.abs(t_s - t64) <= 1e-4 * t64)
    # rn and the edges
    k = int(np.float32((N - 1) * N) * np.float32(0.05))
    cap = k
    d_src, d_dst = empty(torch, cap, torch.int32), empty(torch, cap, torch.int32)
    d_ce, d_te = empty(torch, cap, torch.float32), empty(torch, cap, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, Ec = C.c_float(0), C.c_longlong(0)
    pumplib.check(L.pump_roadmap_edges(large["ctx"].handle, ptr(d_c), ptr(d_t), N, k, cap, ptr(d_src),
                                       ptr(d_dst), ptr(d_ce), ptr(d_te), ptr(d_go), C.byref(rn),
                                       C.byref(Ec), stream(torch)))
    E = int(Ec.value)
    large["roadmap"] = dict(d_s=d_s, src=host(d_src, E), dst=host(d_dst, E), te=host(d_te, E))
    rnv = torch.tensor(rn.value, dtype=torch.float32, device="cuda")
    below, at_most = int((d_c < rnv).sum()), int((d_c <= rnv).sum())
    assert below <= k < at_most  # rn is element k of the sorted costs
    assert E == below
    src, dst = d_src[:E], d_dst[:E]
    key = src.long() * N + dst.long()
    assert bool((key[1:] > key[:-1]).all())  # (i asc, j asc), no repeats
    pidx = src.long() * (N - 1) + dst.long() - (src < dst).long()
    assert bool((d_c[pidx] < rnv).all()) and bool((d_c[pidx] == d_ce[:E]).all())
    assert bool((d_t[pidx] == d_te[:E]).all())
    go = host(d_go, N + 1)
    assert go[0] == 0 and go[N] == E and np.all(np.diff(go) >= 0)
    # waypoints and edge checks on a sample of edges
    d_disc = empty(torch, E * W * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges(ptr(d_s), ptr(d_src), ptr(d_dst), ptr(d_te), E, nd,
                                          pumplib.PUMP_BVP_PRECISION, ptr(d_disc), stream(torch)))
    d_fe = empty(torch, E, torch.uint8)
    d_obs = dev(torch, obs)
    pumplib.check(L.pump_free_edges(ptr(d_obs), obs.shape[0], ptr(d_disc), E, nd, ptr(d_fe), stream(torch)))
    rng = np.random.default_rng(4)
    sel = np.sort(rng.choice(E, 20_000, replace=False))
    rows = torch.from_numpy(sel).cuda()
    disc_s = d_disc.view(-1, W * 6)[:E][rows].cpu().numpy().reshape(-1, W, 6)
    fe = oracle.free_edges(disc_s, obs)
    assert np.array_equal(fe, d_fe[:E][rows].cpu().numpy())
    assert 0 < fe.mean() < 1
    src_s, dst_s, te_s = host(d_src, E)[sel], host(d_dst, E)[sel], host(d_te, E)[sel]
    assert np.array_equal(disc_s[:, 0], s[src_s]) and np.array_equal(disc_s[:, nd], s[dst_s])
    dt = (te_s / np.float32(nd)).astype(np.float32)
    for q in (1, nd // 2, nd - 1):
        ref = oracle.path_point64((dt * np.float32(q)).astype(np.float32), te_s, s[src_s], s[dst_s])
        assert np.abs(disc_s[:, q, :3] - ref[:, :3]).max() <= 1e-6


def test_large_plan(large, pumplib, oracle):
    """The whole query, with a path store of 2^24: its largest wavefront holds
    14.1 M new paths, past the reference's 2 N sqrt(N) = 11.4 M, where the
    reference ends the search (PUMP.cu:62-76); with the default store the
    query ends with PUMP_ERR_CAPACITY there.  The first HSMC launch (the
    initial path's expansions, 4096 particles, 200 boxes) gives the masks and
    CPs the oracle's cacheHalfspaces + propagateValidParticles give on the
    same waypoints, and the returned path's Monte Carlo CP, re-judged by the
    oracle with the 4096-particle table, is the reported CP and within the
    target."""
    torch, L, ctx, pb, obs, N = large["torch"], large["L"], large["ctx"], large["pb"], large["obs"], large["N"]
    nd = large["cfg"]["num_disc"]
    W = nd + 1
    store = pb.max_paths
    pb.max_paths = 0
    res = pumplib.PlanResult()
    assert L.pump_plan(ctx.handle, C.byref(pb), C.byref(res), None) == pumplib.PUMP_ERR_CAPACITY
    pb.max_paths = store
    res = pumplib.PlanResult()
    path = np.zeros((pb.table_rows, 6), np.float32)
    res.path, res.path_cap = path.ctypes.data, pb.table_rows
    trace = np.zeros(2 * 20_000_000, np.int32)
    res.wf_trace, res.wf_trace_cap = trace.ctypes.data, trace.size
    st = L.pump_plan(ctx.handle, C.byref(pb), C.byref(res), None)
    assert st == pumplib.PUMP_OK, L.pump_last_error()
    print("large plan: edges %d, iterations %d, paths %d, expansions %d, sizes %s, cp %g, %.1f ms"
          % (res.num_edges, res.iterations, res.num_paths, res.num_considered,
             list(res.wavefront_sizes)[: res.iterations], res.soln_cp, res.ms_total))
    assert res.success == 1 and res.wf_trace_len == 2 * res.num_considered
    # the first wavefront against the oracle
    m = int(res.wavefront_sizes[0])
    tr = trace[: 2 * m].reshape(m, 2)
    assert np.all(tr[:, 0] == 0)
    r = large["roadmap"]
    e = tr[:, 1].astype(np.int64)
    src, dst, te = r["src"][e], r["dst"][e], r["te"][e]
    d_src, d_dst, d_te = dev(torch, src), dev(torch, dst), dev(torch, te)
    d_disc = empty(torch, m * W * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges(ptr(r["d_s"]), ptr(d_src), ptr(d_dst), ptr(d_te), m, nd,
                                          pumplib.PUMP_BVP_PRECISION, ptr(d_disc), stream(torch)))
    disc = host(d_disc).reshape(m, W, 6)
    P, Pmc, T = int(pb.num_hsmc), int(pb.num_mc), int(pb.table_rows)
    om = np.float32(pb.offset_mult)
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    maxHS = 5
    a, b, _ = oracle.cache_halfspaces(disc, np.ones(m, np.uint8), obs, maxHS, maxd2)
    tm, _ = oracle.particle_tables(int(pb.seed), Pmc, T, pmajor=False)
    valid = np.zeros((1 + m, P), np.uint8)
    valid[0] = 1
    cp_o = np.zeros(1 + m, np.float32)
    edges_local = np.arange(m, dtype=np.int32)
    prev = np.zeros(m, np.int32)
    times = np.zeros(1, np.float32)
    oracle.lib().orc_hsmc_propagate(m, W, edges_local, prev, 1, a, b, times, te, 0.05, maxHS,
                                    tm.reshape(-1), om, Pmc, valid, P, cp_o)
    words = P // 32
    packed = np.zeros((1 + m, words), np.uint32)
    packed[0] = 0xFFFFFFFF
    d_valid = dev(torch, packed.view(np.int32))
    d_cp = empty(torch, 1 + m, torch.float32)
    d_err = dev(torch, np.zeros(1, np.int32))
    d_obs, d_e, d_p, d_t, d_tm = (dev(torch, x) for x in (obs, edges_local, prev, times, tm))
    pumplib.check(L.pump_hsmc_propagate_boxes(m, W, ptr(d_e), ptr(d_p), m, 1, ptr(d_obs), obs.shape[0],
                                              ptr(d_disc), float(maxd2), maxHS, ptr(d_t), ptr(d_te), 0.05,
                                              ptr(d_tm), Pmc, T, float(om), ptr(d_valid), P, ptr(d_cp),
                                              ptr(d_err), stream(torch)))
    got = np.unpackbits(host(d_valid).view(np.uint32).reshape(1 + m, words).view(np.uint8), axis=1,
                        bitorder="little")
    assert int(host(d_err)[0]) == 0
    assert np.array_equal(got[1:, :P], valid[1:])
    assert np.array_equal(host(d_cp)[1:].view(np.uint32), cp_o[1:].view(np.uint32))
    assert 0 < valid[1:].mean() <= 1
    # the returned path, re-judged
    T_len = res.path_len
    _, pm = oracle.particle_tables(int(pb.seed), Pmc, T, tmajor=False)
    hits, cp = oracle.mccp(path[:T_len], T_len, pm, om, obs)
    assert np.float32(cp) == np.float32(res.soln_cp) and cp <= pb.cp_target
