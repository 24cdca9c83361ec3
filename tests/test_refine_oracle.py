"""The binary64 refinement objective and its adjoint (oracle side): the
adjoint against central finite differences (h = 1e-6, binary64), including
segments whose optimal time sits at the tmax bound, and the binary64 optimal
time against the long-double grid search of the precision-mode checker."""
import numpy as np
import pytest

from pump_gb300 import workloads


def fd_grad(R, X, lam, h=1e-6):
    g = np.zeros_like(X)
    for i in range(1, X.shape[0] - 1):
        for d in range(6):
            xp, xm = X.copy(), X.copy()
            xp[i, d] += h
            xm[i, d] -= h
            g[i, d] = (R.objective(xp, lam)[0] - R.objective(xm, lam)[0]) / (2 * h)
    return g


@pytest.mark.parametrize("om,lam,W", [(0.3, 10.0, 8), (0.05, 100.0, 4), (0.3, 0.1, 16)])
def test_adjoint_matches_finite_differences(oracle, om, lam, W):
    obs = workloads.indoor(1001)
    R = oracle.Refine(obs, om, W=W)
    nodes, offs, cnts = workloads.perturbed_paths(4, 11, obs, n_range=(6, 10))
    for o, n in zip(offs, cnts):
        X = nodes[o:o + n].astype(np.float64)
        J, g = R.grad(X, lam)
        J2, c, b = R.objective(X, lam)
        assert J == J2 and abs(J - (c + lam * b)) <= 1e-12 * abs(J)
        assert b > 0
        fd = fd_grad(R, X, lam)
        assert np.all(g[0] == 0) and np.all(g[-1] == 0)
        # central differences at h = 1e-6 carry ~1e-8 relative truncation and
        # cancellation error for these scales
        assert np.abs(fd - g).max() <= 1e-6 * np.abs(g).max()


def test_adjoint_with_clamped_segments(oracle):
    """tmax small enough that some segments sit at the bound: dtau/dx = 0 there."""
    obs = workloads.indoor(1001)
    R = oracle.Refine(obs, 0.3, W=8, tmax=0.3)
    nodes, offs, cnts = workloads.perturbed_paths(3, 5, obs, n_range=(5, 7))
    clamped = 0
    for o, n in zip(offs, cnts):
        X = nodes[o:o + n].astype(np.float64)
        clamped += sum(oracle.tau_exact(X[i], X[i + 1], 0.3)[1] for i in range(n - 1))
        J, g = R.grad(X, 3.0)
        fd = fd_grad(R, X, 3.0)
        assert np.abs(fd - g).max() <= 1e-6 * np.abs(g).max()
    assert clamped > 0


def test_tau_exact_matches_long_double_search(oracle):
    rng = np.random.default_rng(3)
    x = rng.uniform(workloads.LO, workloads.HI, size=(200, 6)).astype(np.float32)
    for k in range(0, 200, 2):
        t, _ = oracle.tau_exact(x[k].astype(np.float64), x[k + 1].astype(np.float64), 5.0)
        t_ld, _c = oracle.bvp_precise(x[k], x[k + 1], 5.0)
        assert abs(t - t_ld) <= 1e-9 * t
