"""The binary64 restatements that check the precision mode over whole
roadmaps (oracle.pyoracle.bvp_binary64, path_point64) against the oracle's
independent forms: the long-double grid-and-bisection minimiser of the pair
cost and the reference-arithmetic pathPoint."""
import numpy as np

from pump_gb300 import workloads


def _pairs(oracle, n, seed):
    s = oracle.halton_samples(1000, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    rng = np.random.default_rng(seed)
    i = rng.integers(0, 1000, n)
    j = (i + rng.integers(1, 1000, n)) % 1000
    x0, x1 = s[i].copy(), s[j].copy()
    # some pairs with fast velocities, whose optimum sits at the tmax bracket end
    # or close to zero
    x0[: n // 4, 3:] *= 8
    x1[n // 4: n // 2, :3] = x0[n // 4: n // 2, :3] + np.float32(1e-3)
    return x0, x1


def test_bvp_binary64_matches_long_double(oracle):
    x0, x1 = _pairs(oracle, 400, 1)
    t64, c64 = oracle.bvp_binary64(x0, x1)
    for k in range(x0.shape[0]):
        tl, cl = oracle.bvp_precise(x0[k], x1[k])
        assert abs(c64[k] - cl) <= 1e-13 * abs(cl), (k, c64[k], cl)
        # the minimiser itself is ill-conditioned only where c'' is tiny
        assert abs(t64[k] - tl) <= 1e-9 * tl, (k, t64[k], tl)


def test_cost_coeffs_match_reference_cost(oracle):
    """c(t) from the coefficients equals the reference's cost expression
    (evaluated by the oracle in the reference's arithmetic) to binary32
    rounding."""
    x0, x1 = _pairs(oracle, 200, 2)
    A = oracle.cost_coeffs64(x0, x1)
    # At small t the reference's binary32 terms of 12 |p0 - p1|^2 cancel (up to
    # 1e-4 relative for positions 1e-3 apart); an error in the expansion would
    # be of order 1.
    for t, tol in ((0.05, 1e-3), (0.3, 1e-4), (1.0, 1e-6), (2.5, 1e-6), (5.0, 1e-6)):
        c64 = oracle.cost64(np.full(x0.shape[0], t), A)
        c32 = np.array([oracle.cost(np.float32(t), x0[k], x1[k]) for k in range(x0.shape[0])])
        assert np.all(np.abs(c32 - c64) <= tol * np.abs(c64)), t


def test_path_point64_matches_reference_arithmetic(oracle):
    x0, x1 = _pairs(oracle, 200, 3)
    rng = np.random.default_rng(4)
    tau = rng.uniform(0.2, 5.0, 200).astype(np.float32)
    t = (tau * rng.uniform(0, 1, 200)).astype(np.float32)
    ref = np.zeros((200, 6), np.float32)
    for k in range(200):
        oracle.lib().orc_path_point(t[k], tau[k], oracle.f32(x0[k]), oracle.f32(x1[k]), ref[k])
    got = oracle.path_point64(t, tau, x0, x1)
    scale = np.maximum(1.0, np.abs(got))
    assert np.all(np.abs(ref - got) <= 4e-6 * scale)


def test_disc_offsets_by_edge_length(oracle):
    """Per-edge waypoint counts by edge length: ceil(L / disc_len) clamped to
    [min, max], L = sqrt((dx*dx + dy*dy) + dz*dz) in binary32, each operation
    rounded once; the offsets are their running sum plus one per edge; with
    disc_len 0 every edge gets max."""
    s = oracle.halton_samples(500, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    rng = np.random.default_rng(6)
    src = rng.integers(0, 500, 3000).astype(np.int32)
    dst = rng.integers(0, 500, 3000).astype(np.int32)
    for disc_len, lo, hi in ((0.025, 3, 31), (0.1, 1, 8), (0.0, 3, 8)):
        off = oracle.disc_offsets(src, dst, s, disc_len, lo, hi)
        d = (s[dst, :3] - s[src, :3]).astype(np.float32)
        L = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        nd = np.full(src.size, hi) if disc_len == 0 else np.clip(
            np.ceil(L / np.float32(disc_len)), lo, hi).astype(np.int64)
        assert np.array_equal(np.diff(off), nd + 1) and off[0] == 0
    # the ragged waypoint stages with uniform offsets are the uniform ones
    c, t = oracle.bvp_pairs(s[:60])
    k = int(np.float32(59 * 60) * np.float32(0.05))
    rn = oracle.lib().orc_select_kth(c.size, c, k)
    es, ed, _ce, _te = oracle.build_edges(c, t, 60, rn)
    off = oracle.disc_offsets(es, ed, s[:60], 0.0, 3, 8)
    assert np.array_equal(oracle.discretize_edges_off(es, ed, s[:60], off).reshape(-1, 9, 6),
                          oracle.discretize_edges(es, ed, s[:60], 8))
