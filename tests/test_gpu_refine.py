"""Path refinement on the GPU (pump_refine_fwd / pump_refine_bwd /
pump_refine_paths) against the binary64 objective and adjoint of the oracle.

Tolerances (binary32 device arithmetic, binary64 optimal time): J, cost and
bound within 2e-5 relative, the gradient within 2e-4 relative (2-norm over
the path), each plus 4x the path's own conditioning: the largest change the
binary64 objective / adjoint shows when every input is perturbed by a few
binary32 roundings (relative 2^-23).  With a small noise multiplier the
bound's terms turn on within ~1e-4 of a box, and that rounding alone moves
them by more than 2e-5 relative."""
import ctypes as C

import numpy as np
import pytest

from helpers import dev, empty, host, ptr

pytestmark = pytest.mark.gpu

REL_J = 2e-5
REL_G = 2e-4


class Case:
    def __init__(self, torch, pumplib, oracle, n_paths, seed, om, W=8, tmax=5.0, T_rows=400,
                 n_range=(8, 40)):
        from pump_gb300 import workloads
        self.obs = workloads.indoor(1000 + seed).astype(np.float32)
        self.nodes, self.offs, self.cnts = workloads.perturbed_paths(n_paths, seed, self.obs,
                                                                     n_range=n_range)
        rng = np.random.default_rng(seed)
        self.lam = np.exp(rng.uniform(np.log(0.1), np.log(100.0), n_paths)).astype(np.float32)
        self.om, self.W, self.tmax, self.T_rows = om, W, tmax, T_rows
        L = pumplib.load()
        self.d_var = empty(torch, T_rows, torch.float64)
        pumplib.check(L.pump_position_variance(T_rows, ptr(self.d_var), None))
        self.keep = [dev(torch, self.nodes), dev(torch, self.offs), dev(torch, self.cnts),
                     dev(torch, self.lam), dev(torch, self.obs)]
        a = pumplib.RefineArgs()
        a.d_nodes, a.n_nodes = ptr(self.keep[0]), self.nodes.shape[0]
        a.d_node_offset, a.d_node_count, a.n_paths = ptr(self.keep[1]), ptr(self.keep[2]), n_paths
        a.d_lambda, a.W, a.tmax = ptr(self.keep[3]), W, tmax
        a.d_obstacles, a.num_obstacles, a.offset_mult = ptr(self.keep[4]), self.obs.shape[0], om
        a.d_pos_var, a.T_rows, a.dt, a.sigma_floor = ptr(self.d_var), T_rows, 0.05, 1e-3
        self.args = a
        self.R = oracle.Refine(self.obs, om, W=W, tmax=tmax, T_rows=T_rows)

    def conditioning(self, X, lam, trials=4):
        """Largest change of (J, c, b, grad) under relative 2^-23 input perturbations."""
        rng = np.random.default_rng(0)
        J0, c0, b0 = self.R.objective(X, lam)
        _, g0 = self.R.grad(X, lam)
        d = np.zeros(4)
        for _ in range(trials):
            Xp = X * (1 + rng.choice([-1.0, 1.0], X.shape) * 2.0 ** -23)
            Jp, cp, bp = self.R.objective(Xp, lam)
            _, gp = self.R.grad(Xp, lam)
            d = np.maximum(d, [abs(Jp - J0), abs(cp - c0), abs(bp - b0), np.linalg.norm(gp - g0)])
        return d

    def path(self, k, nodes=None):
        src = self.nodes if nodes is None else nodes
        return src[self.offs[k]:self.offs[k] + self.cnts[k]]


def fwd(torch, pumplib, case):
    n = case.args.n_paths
    J, c, b = (empty(torch, n, torch.float32) for _ in range(3))
    pumplib.check(pumplib.load().pump_refine_fwd(C.byref(case.args), ptr(J), ptr(c), ptr(b), None))
    torch.cuda.synchronize()
    return host(J), host(c), host(b)


def bwd(torch, pumplib, case):
    g = empty(torch, case.nodes.size, torch.float32)
    J = empty(torch, case.args.n_paths, torch.float32)
    pumplib.check(pumplib.load().pump_refine_bwd(C.byref(case.args), ptr(g), ptr(J), None))
    torch.cuda.synchronize()
    return host(g).reshape(-1, 6), host(J)


def test_position_variance_matches_oracle(gpu, pumplib, oracle):
    torch, _ = gpu
    d = empty(torch, 400, torch.float64)
    pumplib.check(pumplib.load().pump_position_variance(400, ptr(d), None))
    torch.cuda.synchronize()
    assert np.array_equal(host(d), oracle.position_variance(400))


@pytest.mark.parametrize("om,seed", [(0.3, 1), (2e-3, 2), (0.05, 3)])
def test_fwd_bwd_match_binary64(gpu, pumplib, oracle, om, seed):
    torch, _ = gpu
    case = Case(torch, pumplib, oracle, 48, seed, om)
    J, c, b = fwd(torch, pumplib, case)
    g, Jb = bwd(torch, pumplib, case)
    assert np.array_equal(J, Jb)
    for k in range(case.args.n_paths):
        X = case.path(k).astype(np.float64)
        lam = float(case.lam[k])
        J64, c64, b64 = case.R.objective(X, lam)
        _, g64 = case.R.grad(X, lam)
        cond = 4 * case.conditioning(X, lam)
        assert abs(J[k] - J64) <= REL_J * abs(J64) + cond[0]
        assert abs(c[k] - c64) <= REL_J * abs(c64) + cond[1]
        assert abs(b[k] - b64) <= REL_J * abs(b64) + cond[2] + 1e-30
        gk = case.path(k, g)
        assert np.all(gk[0] == 0) and np.all(gk[-1] == 0)
        assert np.linalg.norm(gk - g64) <= REL_G * np.linalg.norm(g64) + cond[3]


def test_clamped_segments(gpu, pumplib, oracle):
    torch, _ = gpu
    case = Case(torch, pumplib, oracle, 16, 7, 0.3, tmax=0.3, n_range=(5, 8))
    g, J = bwd(torch, pumplib, case)
    clamped = 0
    for k in range(case.args.n_paths):
        X = case.path(k).astype(np.float64)
        clamped += sum(oracle.tau_exact(X[i], X[i + 1], 0.3)[1] for i in range(len(X) - 1))
        J64, g64 = case.R.grad(X, float(case.lam[k]))
        cond = 4 * case.conditioning(X, float(case.lam[k]))
        assert abs(J[k] - J64) <= REL_J * abs(J64) + cond[0]
        assert np.linalg.norm(case.path(k, g) - g64) <= REL_G * np.linalg.norm(g64) + cond[3]
    assert clamped > 0


def test_bwd_is_deterministic(gpu, pumplib, oracle):
    torch, _ = gpu
    case = Case(torch, pumplib, oracle, 32, 4, 0.3)
    g1, J1 = bwd(torch, pumplib, case)
    g2, J2 = bwd(torch, pumplib, case)
    assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32))
    assert np.array_equal(J1.view(np.uint32), J2.view(np.uint32))


def test_bad_node_count_gives_nan(gpu, pumplib, oracle):
    torch, _ = gpu
    case = Case(torch, pumplib, oracle, 4, 5, 0.3)
    cnts = case.cnts.copy()
    cnts[2] = 300  # above PUMP_REFINE_MAX_NODES
    t = dev(torch, cnts)
    case.args.d_node_count = ptr(t)
    J, _, _ = fwd(torch, pumplib, case)
    assert np.isnan(J[2]) and np.all(np.isfinite(J[[0, 1, 3]]))


def test_refine_paths_descends(gpu, pumplib, oracle):
    """Armijo descent never raises J; the graph replays identically; J out is
    the objective of the nodes out."""
    torch, ctx = gpu
    L = pumplib.load()
    case = Case(torch, pumplib, oracle, 64, 6, 0.3)
    J0, _, _ = fwd(torch, pumplib, case)
    out = empty(torch, case.nodes.size, torch.float32)
    Jo = empty(torch, case.args.n_paths, torch.float32)
    pumplib.check(L.pump_refine_paths(ctx.handle, C.byref(case.args), 25, ptr(out), ptr(Jo), None))
    torch.cuda.synchronize()
    X1, J1 = host(out).reshape(-1, 6).copy(), host(Jo).copy()
    pumplib.check(L.pump_refine_paths(ctx.handle, C.byref(case.args), 25, ptr(out), ptr(Jo), None))
    torch.cuda.synchronize()
    assert np.array_equal(host(out).reshape(-1, 6).view(np.uint32), X1.view(np.uint32))
    assert np.array_equal(host(Jo).view(np.uint32), J1.view(np.uint32))
    assert np.all(J1 <= J0)
    assert np.mean(J1 < 0.99 * J0) > 0.5
    for k in range(case.args.n_paths):  # endpoints fixed
        Xk = case.path(k, X1)
        assert np.array_equal(Xk[0], case.path(k)[0]) and np.array_equal(Xk[-1], case.path(k)[-1])
    keep = dev(torch, X1)
    case.args.d_nodes = ptr(keep)
    Jf, _, _ = fwd(torch, pumplib, case)
    assert np.allclose(Jf, J1, rtol=1e-6, atol=0)


def test_path_cp_matches_oracle(gpu, pumplib, oracle):
    """pump_path_cp (dense path + MC CP + smoothing cost of candidate paths)
    equals the reference's per-candidate evaluation bit for bit (parity mode)."""
    torch, ctx = gpu
    from pump_gb300 import workloads
    obs = workloads.indoor(1009).astype(np.float32)
    nodes, offs, cnts = workloads.perturbed_paths(24, 9, obs, n_range=(3, 12))
    tm, pm = oracle.particle_tables(P=2048, T=400)
    d_tm, d_obs = dev(torch, tm), dev(torch, obs)
    n = len(offs)
    cp, cost, ln = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.int32)
    pumplib.check(pumplib.load().pump_path_cp(
        ctx.handle, nodes.ctypes.data, offs.ctypes.data, cnts.ctypes.data, n, pumplib.PUMP_BVP_PARITY,
        ptr(d_tm), 2048, 400, 0.3, ptr(d_obs), obs.shape[0], cp.ctypes.data, cost.ctypes.data,
        ln.ctypes.data, None))
    hit = 0
    for k in range(n):
        c64, cost64, len64 = oracle.path_cp(nodes[offs[k]:offs[k] + cnts[k]], pm, np.float32(0.3), obs)
        assert ln[k] == len64
        assert np.float32(cp[k]) == np.float32(c64)
        assert np.float32(cost[k]) == np.float32(cost64)
        hit += cp[k] > 0
    assert hit > 0
