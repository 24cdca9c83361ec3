"""The precision mode (the benchmark's path) checked end to end against
independent binary64 references, on the two benchmark problems:

  cfg0  N = 1000, 10 random boxes, noise 1e-3, 10 waypoints per edge
  cfg1  N = 4000, indoor map (40 boxes), noise 2e-3, 9 waypoints per edge

(a) every roadmap edge's optimal time and cost against the binary64 global
    minimiser of the pair cost (oracle.pyoracle.bvp_binary64, itself pinned
    to the long-double oracle by tests/test_oracle_precision.py); at N = 1000
    also the edge set against the one the correctly rounded costs give;
(b) the binary32 waypoints of every edge against pathPoint (2pBVP.cu:117-131)
    in binary64 at the same inputs, with the error bound stated below;
(c) the returned path of a whole pump_plan query re-judged by the oracle's
    Monte Carlo CP (collisionProbability.cu:39-92, the reference's binary32
    arithmetic): the same hit count, and a CP within the target.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu

CFGS = ["cfg0", "cfg1"]

# Stated error of the precision-mode waypoints (binary32 Hermite evaluation of
# pathPoint's cubic) against pathPoint in binary64 at the same t and tau:
# positions (in [0, 1]) within WP_POS_ABS, velocities within WP_VEL_REL of
# max(1, |v|).
WP_POS_ABS = 1e-6
WP_VEL_REL = 4e-6


def ulps(a, b):
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


def roadmap(torch, L, ctx, cfg_name, oracle):
    """The precision roadmap through the C ABI: pair BVPs, rn and edges."""
    from pump_gb300 import workloads
    cfg = workloads.CONFIGS[cfg_name]
    N = cfg["N"]
    s = oracle.halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    d_s = dev(torch, s)
    npairs = N * (N - 1)
    d_c, d_t = empty(torch, npairs, torch.float32), empty(torch, npairs, torch.float32)
    lib = L.load()
    L.check(lib.pump_bvp_pairs(ptr(d_s), N, 5.0, L.PUMP_BVP_PRECISION, ptr(d_c), ptr(d_t), stream(torch)))
    k = int(np.float32((N - 1) * N) * np.float32(0.05))
    d_src, d_dst = empty(torch, k, torch.int32), empty(torch, k, torch.int32)
    d_ce, d_te = empty(torch, k, torch.float32), empty(torch, k, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, E = C.c_float(0), C.c_longlong(0)
    L.check(lib.pump_roadmap_edges(ctx.handle, ptr(d_c), ptr(d_t), N, k, k, ptr(d_src), ptr(d_dst),
                                   ptr(d_ce), ptr(d_te), ptr(d_go), C.byref(rn), C.byref(E), stream(torch)))
    E = int(E.value)
    return dict(N=N, cfg=cfg, samples=s, k=k, rn=np.float32(rn.value), E=E, d_s=d_s, d_src=d_src,
                d_dst=d_dst, d_te=d_te, copts=host(d_c, npairs), topts=host(d_t, npairs),
                src=host(d_src, E), dst=host(d_dst, E), ce=host(d_ce, E), te=host(d_te, E))


@pytest.mark.parametrize("cfg_name", CFGS)
def test_precision_roadmap_edges_vs_binary64(cfg_name, gpu, pumplib, oracle):
    """Every edge: cost within 1 binary32 ulp of the exact minimum, and the
    correctly rounded value for at least 99.9 % of the edges; optimal time
    within 1 ulp for at least 99 % (a flat minimum leaves the time
    ill-conditioned) and within 1e-4 relative for all but 0.05 %."""
    torch, ctx = gpu
    r = roadmap(torch, pumplib, ctx, cfg_name, oracle)
    s = r["samples"]
    t64, c64 = oracle.bvp_binary64(s[r["src"]], s[r["dst"]])
    uc, ut = ulps(r["ce"], c64.astype(np.float32)), ulps(r["te"], t64.astype(np.float32))
    far_t = np.abs(r["te"] - t64) > 1e-4 * t64
    stats = dict(edges=r["E"], cost_exact=int((uc == 0).sum()), cost_max_ulp=int(uc.max()),
                 time_within1=int((ut <= 1).sum()), time_far=int(far_t.sum()),
                 cost_max_rel=float((np.abs(r["ce"] - c64) / c64).max()))
    print(cfg_name, stats)
    assert r["E"] == int((r["copts"] < r["rn"]).sum()), stats
    assert stats["cost_max_ulp"] <= 1, stats
    assert stats["cost_exact"] >= 0.999 * r["E"], stats
    assert stats["time_within1"] >= 0.99 * r["E"], stats
    assert stats["time_far"] <= 0.0005 * r["E"], stats
    if r["N"] <= 1000:
        # all pairs: the edge set the correctly rounded costs give
        N = r["N"]
        i = np.repeat(np.arange(N), N - 1)
        jj = np.tile(np.arange(N - 1), N)
        j = jj + (jj >= i)
        _, call = oracle.bvp_binary64(s[i], s[j])
        c32 = call.astype(np.float32)
        rn64 = np.partition(c32, r["k"])[r["k"]]
        e64 = np.flatnonzero(c32 < rn64)
        e_gpu = np.flatnonzero(r["copts"] < r["rn"])
        diff = np.setxor1d(e64, e_gpu).size
        print(cfg_name, "rn", r["rn"], rn64, "edge set difference", diff)
        assert diff <= 2, (diff, r["rn"], rn64)


@pytest.mark.parametrize("cfg_name", CFGS)
def test_precision_waypoints_vs_binary64(cfg_name, gpu, pumplib, oracle):
    """Every waypoint of every edge (binary32 Hermite form) against pathPoint
    in binary64 at the same t = (topt / numDisc) * i and tau = topt."""
    torch, ctx = gpu
    r = roadmap(torch, pumplib, ctx, cfg_name, oracle)
    nd = r["cfg"]["num_disc"]
    W, E = nd + 1, r["E"]
    d_disc = empty(torch, E * W * 6, torch.float32)
    pumplib.check(pumplib.load().pump_discretize_edges(
        ptr(r["d_s"]), ptr(r["d_src"]), ptr(r["d_dst"]), ptr(r["d_te"]), E, nd, pumplib.PUMP_BVP_PRECISION,
        ptr(d_disc), stream(torch)))
    disc = host(d_disc, E * W * 6).reshape(E, W, 6)
    s = r["samples"]
    assert np.array_equal(disc[:, 0], s[r["src"]]) and np.array_equal(disc[:, nd], s[r["dst"]])
    te = r["te"]
    dt = (te / np.float32(nd)).astype(np.float32)
    worst_p = worst_v = 0.0
    for i in range(1, nd):
        t = (dt * np.float32(i)).astype(np.float32)
        ref = oracle.path_point64(t, te, s[r["src"]], s[r["dst"]])
        got = disc[:, i].astype(np.float64)
        worst_p = max(worst_p, float(np.abs(got[:, :3] - ref[:, :3]).max()))
        worst_v = max(worst_v, float((np.abs(got[:, 3:] - ref[:, 3:]) / np.maximum(1, np.abs(ref[:, 3:]))).max()))
    print(cfg_name, "waypoints", E * (nd - 1), "max position error", worst_p, "max velocity error", worst_v)
    assert worst_p <= WP_POS_ABS and worst_v <= WP_VEL_REL, (worst_p, worst_v)


@pytest.mark.parametrize("cfg_name", CFGS)
def test_precision_plan_cp_rejudged_by_oracle(cfg_name, gpu, pumplib, oracle):
    """A whole precision-mode query: its roadmap is the one checked above (rn
    and edge count agree), and the oracle's Monte Carlo CP of the returned
    dense path gives the hit count the planner reported, within the target."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    r = roadmap(torch, pumplib, ctx, cfg_name, oracle)
    cfg = r["cfg"]
    L = pumplib.load()
    obs = np.ascontiguousarray(cfg["obstacles"](0), np.float32)
    pb = pumplib.Problem()
    L.pump_problem_defaults(C.byref(pb))
    pb.N, pb.num_disc, pb.num_hsmc = r["N"], cfg["num_disc"], cfg["num_hsmc"]
    pb.num_obstacles, pb.obstacles = obs.shape[0], obs.ctypes.data
    for d in range(6):
        pb.init[d], pb.goal[d] = workloads.INIT[d], workloads.GOAL[d]
        pb.lo[d], pb.hi[d] = workloads.LO[d], workloads.HI[d]
    pb.offset_mult, pb.cp_target, pb.cp_factor = cfg["offset_mult"], cfg["cp"], cfg["eta"]
    pb.bvp_mode = pumplib.PUMP_BVP_PRECISION
    res = pumplib.PlanResult()
    path = np.zeros((400, 6), np.float32)
    res.path, res.path_cap = path.ctypes.data, 400
    st = L.pump_plan(ctx.handle, C.byref(pb), C.byref(res), None)
    assert st == pumplib.PUMP_OK, L.pump_last_error()
    assert np.float32(res.rn) == r["rn"] and res.num_edges == r["E"]
    assert res.success == 1
    T = res.path_len
    _, pm = oracle.particle_tables(int(pb.seed), int(pb.num_mc), int(pb.table_rows), tmajor=False)
    hits, cp = oracle.mccp(path[:T], T, pm, np.float32(pb.offset_mult), obs)
    print(cfg_name, "path states", T, "hits", hits, "cp", cp, "reported", res.soln_cp)
    assert np.float32(cp) == np.float32(res.soln_cp)
    assert cp <= cfg["cp"]
