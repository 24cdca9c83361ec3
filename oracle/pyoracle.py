"""ctypes binding of the C oracle (pump_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker or as the timed CPU baseline.  The product
(``pump_gb300``) never imports it.

``build()`` compiles the oracle with gcc (``-ffp-contract=off``: no fused
multiply-add, the arithmetic the oracle restates) into ``oracle/_build``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SRC = os.path.join(HERE, "pump_oracle.c")

_lock = threading.Lock()
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

DEFAULT_SEED = 0x9E3779B97F4A7C15


def build(force: bool = False) -> str:
    """Compile liboracle.so (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "pump_oracle.h"))
    ):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Problem(C.Structure):
    _fields_ = [
        ("N", C.c_int), ("numDisc", C.c_int), ("P", C.c_int), ("Pmc", C.c_int),
        ("T_table", C.c_int), ("numObs", C.c_int), ("obstacles", C.c_void_p),
        ("init", C.c_float * 6), ("goal", C.c_float * 6), ("lo", C.c_float * 6),
        ("hi", C.c_float * 6), ("offsetMult", C.c_float), ("cpTarget", C.c_float),
        ("cpFactor", C.c_float), ("tmajor", C.c_void_p), ("pmajor", C.c_void_p),
        ("samples", C.c_void_p), ("discLen", C.c_float), ("discMin", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("rn", C.c_float), ("numEdges", C.c_longlong), ("itrs", C.c_int),
        ("numPaths", C.c_int), ("numConsidered", C.c_int), ("goalPathCount", C.c_int),
        ("success", C.c_int), ("solnPathIdx", C.c_int), ("solnCP", C.c_float),
        ("solnCost", C.c_float), ("pathLen", C.c_int), ("path", C.c_void_p),
        ("path_cap", C.c_int), ("nodes", C.c_void_p), ("nodes_cap", C.c_int),
        ("numNodes", C.c_int), ("wavefront_sizes", C.c_void_p), ("wf_trace", C.c_void_p),
        ("wf_trace_cap", C.c_longlong), ("wf_trace_len", C.c_longlong),
        ("ctrl_path", C.c_void_p), ("ctrl_cap", C.c_int), ("ctrlLen", C.c_int),
    ]


class RefineArgs(C.Structure):
    _fields_ = [
        ("W", C.c_int), ("tmax", C.c_double), ("numObs", C.c_int), ("obstacles", C.c_void_p),
        ("offsetMult", C.c_double), ("posVar", C.c_void_p), ("T_rows", C.c_int),
        ("dt", C.c_double), ("sigmaFloor", C.c_double),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build())
            L.orc_cost.restype = C.c_float
            L.orc_cost.argtypes = [C.c_float, f32p, f32p]
            L.orc_dcost.restype = C.c_float
            L.orc_dcost.argtypes = [C.c_float, f32p, f32p]
            L.orc_topt_bisection.restype = C.c_float
            L.orc_topt_bisection.argtypes = [f32p, f32p, C.c_float, C.c_void_p]
            L.orc_path_point.argtypes = [C.c_float, C.c_float, f32p, f32p, f32p]
            L.orc_find_discretized_path.restype = C.c_float
            L.orc_find_discretized_path.argtypes = [f32p, f32p, f32p, C.c_int]
            L.orc_find_optimal_path.restype = C.c_float
            L.orc_find_optimal_path.argtypes = [C.c_float, f32p, C.c_int, f32p, C.c_int,
                                                C.POINTER(C.c_int)]
            L.orc_bvp_pairs.argtypes = [C.c_int, f32p, C.c_float, f32p, f32p]
            L.orc_halton.restype = C.c_float
            L.orc_halton.argtypes = [C.c_int, C.c_int]
            L.orc_halton_samples.argtypes = [C.c_int, f32p, f32p, f32p, f32p, f32p]
            L.orc_sample_free.argtypes = [C.c_int, f32p, C.c_int, f32p, u8p]
            L.orc_select_kth.restype = C.c_float
            L.orc_select_kth.argtypes = [C.c_longlong, f32p, C.c_longlong]
            L.orc_build_edges.restype = C.c_longlong
            L.orc_build_edges.argtypes = [C.c_int, f32p, f32p, C.c_float, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p]
            L.orc_discretize_edges.argtypes = [C.c_longlong, i32p, i32p, f32p, C.c_int, f32p]
            L.orc_heuristic.argtypes = [C.c_int, f32p, f32p, f32p]
            L.orc_is_motion_valid.restype = C.c_int
            L.orc_is_motion_valid.argtypes = [f32p, f32p, C.c_int, f32p]
            L.orc_free_edges.argtypes = [C.c_longlong, C.c_int, f32p, C.c_int, f32p, u8p]
            L.orc_cache_halfspaces.argtypes = [C.c_longlong, C.c_int, f32p, u8p, C.c_int, f32p,
                                               C.c_int, C.c_float, f32p, f32p, i32p]
            L.orc_hsmc_propagate.argtypes = [C.c_int, C.c_int, i32p, i32p, C.c_int, f32p, f32p,
                                             f32p, f32p, C.c_float, C.c_int, f32p, C.c_float,
                                             C.c_int, u8p, C.c_int, f32p]
            L.orc_mccp64.restype = C.c_int
            L.orc_mccp64.argtypes = [f32p, C.c_int, f32p, C.c_int, C.c_float, C.c_int, f32p, C.c_int]
            L.orc_mccp.restype = C.c_int
            L.orc_mccp.argtypes = [f32p, C.c_int, f32p, C.c_int, C.c_float, C.c_int, f32p,
                                   C.c_int, C.POINTER(C.c_float)]
            L.orc_frontier_compact.restype = C.c_int
            L.orc_frontier_compact.argtypes = [C.c_int, u8p, i32p]
            L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                            C.POINTER(C.c_uint32)]
            L.orc_det_log.restype = C.c_double
            L.orc_det_log.argtypes = [C.c_double]
            L.orc_det_sincos_2pi.argtypes = [C.c_double, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]
            L.orc_bvp_precise.argtypes = [f32p, f32p, C.c_float, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
            L.orc_cost_exact.restype = C.c_double
            L.orc_cost_exact.argtypes = [C.c_double, f32p, f32p]
            L.orc_particle_tables.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
            L.orc_particle_cov.argtypes = [C.c_int, f64p]
            L.orc_tau_exact.restype = C.c_double
            L.orc_tau_exact.argtypes = [f64p, f64p, C.c_double, C.POINTER(C.c_int)]
            L.orc_position_variance.restype = None
            L.orc_position_variance.argtypes = [C.c_int, f64p]
            L.orc_refine_objective.restype = C.c_double
            L.orc_refine_objective.argtypes = [C.POINTER(RefineArgs), f64p, C.c_int, C.c_double,
                                               C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.orc_refine_grad.restype = C.c_double
            L.orc_refine_grad.argtypes = [C.POINTER(RefineArgs), f64p, C.c_int, C.c_double, f64p]
            L.orc_disc_offsets.restype = C.c_longlong
            L.orc_disc_offsets.argtypes = [C.c_longlong, i32p, i32p, f32p, C.c_float, C.c_int,
                                           C.c_int, C.c_void_p]
            L.orc_discretize_edges_off.argtypes = [C.c_longlong, i32p, i32p, f32p, C.c_void_p, f32p]
            L.orc_free_edges_off.argtypes = [C.c_longlong, C.c_void_p, f32p, C.c_int, f32p, u8p]
            L.orc_cache_halfspaces_off.argtypes = [C.c_longlong, C.c_void_p, f32p, u8p, C.c_int, f32p,
                                                   C.c_int, C.c_float, f32p, f32p, i32p]
            L.orc_hsmc_propagate_off.argtypes = [C.c_int, C.c_void_p, i32p, i32p, C.c_int, f32p, f32p,
                                                 f32p, f32p, C.c_float, C.c_int, f32p, C.c_float,
                                                 C.c_int, u8p, C.c_int, f32p]
            L.orc_plan.restype = C.c_int
            L.orc_plan.argtypes = [C.POINTER(Problem), C.POINTER(Result)]
            _lib = L
    return _lib


# ---------------------------------------------------------------- wrappers
def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def particle_tables(seed=DEFAULT_SEED, P=2048, T=400, tmajor=True, pmajor=True):
    tm = np.empty((T, P, 3), np.float32) if tmajor else None
    pm = np.empty((P, T, 3), np.float32) if pmajor else None
    lib().orc_particle_tables(C.c_uint64(seed), P, T,
                              tm.ctypes.data if tm is not None else None,
                              pm.ctypes.data if pm is not None else None)
    return tm, pm


def particle_cov(T):
    out = np.empty(T * 3, np.float64)
    lib().orc_particle_cov(T, out)
    return out.reshape(T, 3)


def halton_samples(N, init, goal, lo, hi):
    s = np.empty((N, 6), np.float32)
    lib().orc_halton_samples(N, s, f32(init), f32(goal), f32(lo), f32(hi))
    return s


def bvp_pairs(samples, tmax=5.0):
    N = samples.shape[0]
    c = np.empty(N * (N - 1), np.float32)
    t = np.empty(N * (N - 1), np.float32)
    lib().orc_bvp_pairs(N, f32(samples), tmax, c, t)
    return c, t


def topt(x0, x1, tmax=5.0):
    ev = C.c_int(0)
    r = lib().orc_topt_bisection(f32(x0), f32(x1), tmax, C.byref(ev))
    return r, ev.value


def cost(tau, x0, x1):
    return lib().orc_cost(tau, f32(x0), f32(x1))


def bvp_precise(x0, x1, tmax=5.0):
    """Long-double global minimiser (topt, cost) of the pair cost."""
    t, c = C.c_double(0), C.c_double(0)
    lib().orc_bvp_precise(f32(x0), f32(x1), tmax, C.byref(t), C.byref(c))
    return t.value, c.value


def cost_exact(t, x0, x1):
    return lib().orc_cost_exact(float(t), f32(x0), f32(x1))


def build_edges(copts, topts, N, rn):
    L = lib()
    E = L.orc_build_edges(N, f32(copts), f32(topts), rn, None, None, None, None)
    src = np.empty(E, np.int32)
    dst = np.empty(E, np.int32)
    ce = np.empty(E, np.float32)
    te = np.empty(E, np.float32)
    L.orc_build_edges(N, f32(copts), f32(topts), rn, src.ctypes.data, dst.ctypes.data,
                      ce.ctypes.data, te.ctypes.data)
    return src, dst, ce, te


def discretize_edges(src, dst, samples, numDisc):
    E = src.shape[0]
    out = np.empty((E, numDisc + 1, 6), np.float32)
    lib().orc_discretize_edges(E, np.ascontiguousarray(src, np.int32),
                               np.ascontiguousarray(dst, np.int32), f32(samples), numDisc, out)
    return out


def disc_offsets(src, dst, samples, discLen, minDisc, maxDisc):
    """Per-edge waypoint counts by edge length: the first waypoint of each
    edge in the ragged layout, E + 1 entries (no reference counterpart)."""
    E = src.shape[0]
    off = np.zeros(E + 1, np.int64)
    lib().orc_disc_offsets(E, np.ascontiguousarray(src, np.int32), np.ascontiguousarray(dst, np.int32),
                           f32(samples), discLen, minDisc, maxDisc, off.ctypes.data)
    return off


def discretize_edges_off(src, dst, samples, off):
    out = np.empty((int(off[-1]), 6), np.float32)
    lib().orc_discretize_edges_off(src.shape[0], np.ascontiguousarray(src, np.int32),
                                   np.ascontiguousarray(dst, np.int32), f32(samples),
                                   np.ascontiguousarray(off, np.int64).ctypes.data, out)
    return out


def free_edges_off(disc, off, obstacles):
    E = off.size - 1
    out = np.empty(E, np.uint8)
    ob = f32(obstacles).reshape(-1)
    lib().orc_free_edges_off(E, np.ascontiguousarray(off, np.int64).ctypes.data, f32(disc), ob.size // 12,
                             ob, out)
    return out


def heuristic(samples, goal):
    N = samples.shape[0]
    h = np.empty(N, np.float32)
    lib().orc_heuristic(N, f32(samples), f32(goal), h)
    return h


def sample_free(samples, obstacles):
    N = samples.shape[0]
    out = np.empty(N, np.uint8)
    ob = f32(obstacles).reshape(-1)
    lib().orc_sample_free(N, f32(samples), ob.size // 12, ob, out)
    return out


def free_edges(disc, obstacles):
    E, W = disc.shape[0], disc.shape[1]
    out = np.empty(E, np.uint8)
    ob = f32(obstacles).reshape(-1)
    lib().orc_free_edges(E, W - 1, f32(disc), ob.size // 12, ob, out)
    return out


def cache_halfspaces(disc, isfree, obstacles, maxHS, maxd2):
    E, W = disc.shape[0], disc.shape[1]
    ob = f32(obstacles).reshape(-1)
    a = np.empty(E * W * maxHS * 3, np.float32)
    b = np.empty(E * W * maxHS, np.float32)
    cnt = np.full(E * W, -1, np.int32)
    lib().orc_cache_halfspaces(E, W, f32(disc), np.ascontiguousarray(isfree, np.uint8),
                               ob.size // 12, ob, maxHS, maxd2, a, b, cnt)
    return a, b, cnt


def mccp(path, T, pmajor, offsetMult, obstacles):
    ob = f32(obstacles).reshape(-1)
    cp = C.c_float(0)
    Pmc, Ts = pmajor.shape[0], pmajor.shape[1]
    hits = lib().orc_mccp(f32(path).reshape(-1), T, f32(pmajor).reshape(-1), Ts, offsetMult,
                          ob.size // 12, ob, Pmc, C.byref(cp))
    return hits, cp.value


def path_cp(nodes, pmajor, offsetMult, obstacles, dt=np.float32(0.05)):
    """A candidate path as the reference evaluates it (PUMP.cu:370-385,
    492-502): the dense path of findOptimalPath (tmax 5), its MC CP, and the
    cost sum with toptBisection tmax 2.  Returns (cp, cost, dense length);
    cp -1 when the dense path has more states than the particle table."""
    xs = f32(nodes).reshape(-1)
    n = xs.size // 6
    T_table = pmajor.shape[1]
    split = np.zeros(((T_table + 2) * 6,), np.float32)
    ln = C.c_int(0)
    lib().orc_find_optimal_path(dt, split, T_table, xs, n, C.byref(ln))
    c = np.float32(0)
    for i in range(n - 1):
        tau, _ = topt(xs[6 * i:6 * i + 6], xs[6 * i + 6:6 * i + 12], 2.0)
        c = np.float32(c + np.float32(cost(tau, xs[6 * i:6 * i + 6], xs[6 * i + 6:6 * i + 12])))
    if ln.value < 0 or ln.value > T_table:
        return -1.0, float(c), ln.value
    _, cp = mccp(split[: ln.value * 6], ln.value, pmajor, offsetMult, obstacles)
    return cp, float(c), ln.value


def mccp64(path, T, pmajor, offsetMult, obstacles):
    """Hits of the Monte Carlo CP with the collision tests in binary64."""
    ob = f32(obstacles).reshape(-1)
    Pmc, Ts = pmajor.shape[0], pmajor.shape[1]
    return lib().orc_mccp64(f32(path).reshape(-1), T, f32(pmajor).reshape(-1), Ts, offsetMult,
                            ob.size // 12, ob, Pmc)


def plan(N, obstacles, init, goal, lo, hi, offsetMult, cpTarget, cpFactor, numDisc=8, P=128,
         Pmc=2048, T_table=400, seed=DEFAULT_SEED, samples=None, trace_cap=0, tables=None,
         discLen=0.0, discMin=3):
    """Whole query as the reference's main() + PUMP(); returns a dict.
    discLen > 0: per-edge waypoint counts by edge length (numDisc the largest,
    discMin the smallest), see disc_offsets."""
    ob = f32(obstacles).reshape(-1)
    tm, pm = tables if tables is not None else particle_tables(seed, Pmc, T_table)
    pb = Problem()
    pb.N, pb.numDisc, pb.P, pb.Pmc, pb.T_table = N, numDisc, P, Pmc, T_table
    pb.numObs = ob.size // 12
    pb.obstacles = ob.ctypes.data
    for k in range(6):
        pb.init[k], pb.goal[k], pb.lo[k], pb.hi[k] = init[k], goal[k], lo[k], hi[k]
    pb.offsetMult, pb.cpTarget, pb.cpFactor = offsetMult, cpTarget, cpFactor
    pb.discLen, pb.discMin = discLen, discMin
    tm = f32(tm)
    pm = f32(pm)
    pb.tmajor, pb.pmajor = tm.ctypes.data, pm.ctypes.data
    sm = f32(samples) if samples is not None else None
    pb.samples = sm.ctypes.data if sm is not None else None
    res = Result()
    path = np.zeros((T_table + 2, 6), np.float32)
    nodes = np.zeros(64, np.int32)
    wfs = np.zeros(32, np.int32)
    trace = np.zeros(max(trace_cap, 1), np.int32)
    res.path, res.path_cap = path.ctypes.data, T_table + 2
    res.nodes, res.nodes_cap = nodes.ctypes.data, 64
    res.wavefront_sizes = wfs.ctypes.data
    res.wf_trace, res.wf_trace_cap = (trace.ctypes.data, trace_cap) if trace_cap else (None, 0)
    ctrl = np.zeros((4096, 6), np.float32)
    res.ctrl_path, res.ctrl_cap = ctrl.ctypes.data, ctrl.shape[0]
    lib().orc_plan(C.byref(pb), C.byref(res))
    out = {k: getattr(res, k) for k, _ in Result._fields_ if not k.endswith(("cap",)) and k not in (
        "path", "nodes", "wavefront_sizes", "wf_trace", "ctrl_path")}
    out["ctrl_path"] = ctrl[: min(res.ctrlLen, ctrl.shape[0])].copy()
    out["path"] = path[: res.pathLen].copy()
    out["nodes"] = nodes[: res.numNodes].copy()
    out["wavefront_sizes"] = wfs[: res.itrs].copy()
    out["wf_trace"] = trace[: res.wf_trace_len].copy() if trace_cap else None
    return out


def position_variance(T):
    """Per-axis position variance of the particle model per step (binary64)."""
    out = np.zeros(T, np.float64)
    lib().orc_position_variance(T, out)
    return out


def tau_exact(x0, x1, tmax):
    """Global minimiser of the 2pBVP cost on (0, tmax] in binary64 and whether it is tmax."""
    a, b = np.ascontiguousarray(x0, np.float64), np.ascontiguousarray(x1, np.float64)
    cl = C.c_int(0)
    t = lib().orc_tau_exact(a, b, tmax, C.byref(cl))
    return t, bool(cl.value)


class Refine:
    """Path refinement objective J = cost + lambda * bound and its adjoint in
    binary64 (see pump_oracle.h)."""

    def __init__(self, obstacles, offset_mult, W=8, tmax=5.0, T_rows=400, dt=0.05, sigma_floor=1e-3):
        self.obs = f32(obstacles).reshape(-1)
        self.var = position_variance(T_rows)
        self.args = RefineArgs(W, tmax, self.obs.size // 12, self.obs.ctypes.data, float(offset_mult),
                               self.var.ctypes.data, T_rows, dt, sigma_floor)

    def objective(self, nodes, lam):
        x = np.ascontiguousarray(nodes, np.float64).reshape(-1)
        c, b = C.c_double(0), C.c_double(0)
        J = lib().orc_refine_objective(C.byref(self.args), x, x.size // 6, lam, C.byref(c), C.byref(b))
        return J, c.value, b.value

    def grad(self, nodes, lam):
        x = np.ascontiguousarray(nodes, np.float64).reshape(-1)
        g = np.zeros_like(x)
        J = lib().orc_refine_grad(C.byref(self.args), x, x.size // 6, lam, g)
        return J, g.reshape(-1, 6)


# ------------------------------------------------- binary64 restatements
# Vectorised numpy forms of the precision mode's two changed quantities, used
# to check every edge of a roadmap (the long-double orc_bvp_precise takes about
# a millisecond per pair, so it checks samples only).
G32 = float(np.float32(-9.81))  # the reference's `const float g = -9.81` (2pBVP.cu:3)


def cost_coeffs64(x0, x1):
    """Coefficients of the pair cost of 2pBVP.cu:97-107 written as
    c(t) = A0/t^3 + A1/t^2 + A2/t + A3 + A4 t, in binary64, for arrays of
    states x0, x1 (n, 6).  Expanding the reference's bracket gives
    A0 = 12 |p0 - p1|^2, A1 = 12 (p0 - p1).(v0 + v1),
    A2 = 4 (|v0|^2 + |v1|^2 + v0.v1), A3 = 2 g (v0z - v1z), A4 = 1 + g^2."""
    x0 = np.asarray(x0, np.float64).reshape(-1, 6)
    x1 = np.asarray(x1, np.float64).reshape(-1, 6)
    dp = x0[:, :3] - x1[:, :3]
    v0, v1 = x0[:, 3:], x1[:, 3:]
    A0 = 12.0 * np.sum(dp * dp, 1)
    A1 = 12.0 * np.sum(dp * (v0 + v1), 1)
    A2 = 4.0 * (np.sum(v0 * v0, 1) + np.sum(v1 * v1, 1) + np.sum(v0 * v1, 1))
    A3 = 2.0 * G32 * (x0[:, 5] - x1[:, 5])
    A4 = np.full_like(A0, 1.0 + G32 * G32)
    return A0, A1, A2, A3, A4


def cost64(t, A):
    A0, A1, A2, A3, A4 = A
    return A0 / t**3 + A1 / t**2 + A2 / t + A3 + A4 * t


def bvp_binary64(x0, x1, tmax=5.0):
    """Global minimiser (topt, cost) of the pair cost on (0, tmax] in binary64
    for arrays of pairs: the real roots of the stationarity quartic
    Q(t) = A4 t^4 - A2 t^2 - 2 A1 t - 3 A0 (c'(t) = Q(t) / t^4) from the
    eigenvalues of its companion matrix, two Newton steps on Q, and the least
    cost among those in (0, tmax] and tmax itself."""
    A = cost_coeffs64(x0, x1)
    A0, A1, A2, A3, A4 = A
    n = A0.size
    comp = np.zeros((n, 4, 4))
    # monic quartic t^4 + b t^2 + c t + d with b = -A2/A4, c = -2 A1/A4, d = -3 A0/A4
    comp[:, 0, 1] = A2 / A4
    comp[:, 0, 2] = 2.0 * A1 / A4
    comp[:, 0, 3] = 3.0 * A0 / A4
    comp[:, 1, 0] = comp[:, 2, 1] = comp[:, 3, 2] = 1.0
    roots = np.linalg.eigvals(comp)
    real = np.abs(roots.imag) <= 1e-7 * np.maximum(np.abs(roots.real), 1e-30)
    r = np.where(real, roots.real, np.nan)
    with np.errstate(invalid="ignore", divide="ignore"):
        for _ in range(2):
            q = A4[:, None] * r**4 - A2[:, None] * r**2 - 2 * A1[:, None] * r - 3 * A0[:, None]
            dq = 4 * A4[:, None] * r**3 - 2 * A2[:, None] * r - 2 * A1[:, None]
            r = np.where(dq != 0, r - q / dq, r)
    r = np.where((r > 0) & (r <= tmax), r, np.nan)
    cand = np.concatenate([r, np.full((n, 1), float(tmax))], 1)
    c = cost64(cand, tuple(a[:, None] for a in A))
    c = np.where(np.isnan(c), np.inf, c)
    k = np.argmin(c, 1)
    rows = np.arange(n)
    return cand[rows, k], c[rows, k]


def path_point64(t, tau, x0, x1):
    """pathPoint (2pBVP.cu:117-131) in binary64 for arrays: t, tau (n,),
    x0, x1 (n, 6); returns (n, 6)."""
    t = np.asarray(t, np.float64)[:, None]
    u = np.asarray(tau, np.float64)[:, None]
    a = np.asarray(x0, np.float64).reshape(-1, 6)
    b = np.asarray(x1, np.float64).reshape(-1, 6)
    p0, p1, v0, v1 = a[:, :3], b[:, :3], a[:, 3:], b[:, 3:]
    pos = (t * v0 + p0 + t**3 * (2 * p0 - 2 * p1 + (v0 + v1) * u) / u**3
           - t**2 * (3 * p0 - 3 * p1 + (2 * v0 + v1) * u) / u**2)
    vel = (-(2 * t * (3 * p0 - 3 * p1 + v1 * u)) / u**2 + (3 * t**2 * (2 * p0 - 2 * p1 + v1 * u)) / u**3
           + (v0 * (3 * t**2 - 4 * t * u + u**2)) / u**2)
    return np.concatenate([pos, vel], 1)
