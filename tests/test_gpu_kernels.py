"""GPU kernels through the C ABI against the oracle, bit for bit.

Each test runs one entry point of include/pump.h on cuda:0 and compares its
output with the oracle's (oracle/pump_oracle.c), which the golden fixtures
pin to the reference program's own results.  Integer, index and mask outputs
must be identical; floating-point outputs must be identical to the last bit
(parity arithmetic is the reference's, see include/pump.h).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import bits_to_bytes, dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def same_bits_or_nan(a, b):
    """Identical bits, except that a NaN matches any NaN (GPU and host
    arithmetic produce different NaN payloads)."""
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return (a.shape == b.shape and np.array_equal(na, nb)
            and np.array_equal(a.view(np.uint32)[~na], b.view(np.uint32)[~nb]))


def golden_problem(goldens, name):
    g = goldens[name]
    return (int(g["N"]), g["prob_obstacles"].astype(np.float32), g["prob_init"], g["prob_goal"],
            g["prob_lo"], g["prob_hi"], np.float32(g["prob_offset_mult"]))


@pytest.fixture(scope="module")
def roadmap1000(oracle, goldens):
    N, obs, init, goal, lo, hi, om = golden_problem(goldens, "ref_N1000_boxes10_noise0.3")
    s = oracle.halton_samples(N, init, goal, lo, hi)
    c, t = oracle.bvp_pairs(s)
    k = int((N - 1) * N * np.float32(0.05))
    rn = oracle.lib().orc_select_kth(c.size, c, k)
    src, dst, ce, te = oracle.build_edges(c, t, N, rn)
    disc = oracle.discretize_edges(src, dst, s, 8)
    fe = oracle.free_edges(disc, obs)
    return dict(N=N, obs=obs, om=om, samples=s, copts=c, topts=t, k=k, rn=rn, src=src, dst=dst,
                ce=ce, te=te, disc=disc, fe=fe, goal=goal)


def run_bvp_pairs(torch, L, s, mode=0, tmax=5.0):
    N = s.shape[0]
    d_s = dev(torch, s)
    d_c = empty(torch, N * (N - 1), torch.float32)
    d_t = empty(torch, N * (N - 1), torch.float32)
    L.check(L.load().pump_bvp_pairs(ptr(d_s), N, tmax, mode, ptr(d_c), ptr(d_t), stream(torch)))
    torch.cuda.synchronize()
    return host(d_c, N * (N - 1)), host(d_t, N * (N - 1))


@pytest.mark.parametrize("N", [2, 64, 1000])
def test_bvp_pairs_parity_halton(N, gpu, pumplib, oracle, goldens):
    torch, _ = gpu
    _, _, init, goal, lo, hi, _ = golden_problem(goldens, "ref_N1000_input")
    s = oracle.halton_samples(N, init, goal, lo, hi)
    c, t = run_bvp_pairs(torch, pumplib, s)
    rc, rt = oracle.bvp_pairs(s)
    assert same_bits(t, rt), "topt mismatches: %d" % int((t != rt).sum())
    assert same_bits(c, rc), "copt mismatches: %d" % int((c != rc).sum())


def test_bvp_pairs_parity_random(gpu, pumplib, oracle):
    torch, _ = gpu
    rng = np.random.default_rng(7)
    s = np.concatenate([rng.uniform(-1, 2, (300, 3)), rng.uniform(-3, 3, (300, 3))], 1).astype(np.float32)
    c, t = run_bvp_pairs(torch, pumplib, s)
    rc, rt = oracle.bvp_pairs(s)
    assert same_bits(t, rt) and same_bits(c, rc)


def test_bvp_batch_parity(gpu, pumplib, oracle):
    torch, _ = gpu
    L = pumplib.load()
    rng = np.random.default_rng(11)
    n = 2000
    x0 = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.uniform(-1, 1, (n, 3))], 1).astype(np.float32)
    x1 = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.uniform(-1, 1, (n, 3))], 1).astype(np.float32)
    for tmax in (2.0, 5.0):
        d0, d1 = dev(torch, x0), dev(torch, x1)
        dt, dc = empty(torch, n, torch.float32), empty(torch, n, torch.float32)
        pumplib.check(L.pump_bvp_batch(ptr(d0), ptr(d1), n, tmax, 0, ptr(dt), ptr(dc), stream(torch)))
        t, c = host(dt, n), host(dc, n)
        rt = np.array([oracle.topt(x0[k], x1[k], tmax)[0] for k in range(n)], np.float32)
        rc = np.array([oracle.cost(rt[k], x0[k], x1[k]) for k in range(n)], np.float32)
        assert same_bits(t, rt) and same_bits(c, rc)


@pytest.mark.parametrize("N", [1000, 4000])
def test_bvp_pairs_gpu_arithmetic_matches_reference_kernel(N, gpu, pumplib, oracle, goldens):
    """PUMP_BVP_PARITY_GPU against the reference's own fillCoptsTopts run on
    the GB300 (tests/golden/refgpu_bvp_N*.npz, oracle/refgpu): every pair's
    time and cost bit for bit (SHA-256 of both whole arrays), on the Halton
    samples of the benchmark problems."""
    import hashlib
    from pump_gb300 import workloads
    torch, _ = gpu
    g = goldens["refgpu_bvp_N%d" % N]
    s = oracle.halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    c, t = run_bvp_pairs(torch, pumplib, s, mode=pumplib.PUMP_BVP_PARITY_GPU)
    st = int(g["stride"])
    assert same_bits(c[::st], g["copts_strided"]) and same_bits(t[::st], g["topts_strided"])
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g["copts_sha"])
    assert hashlib.sha256(t.tobytes()).hexdigest() == str(g["topts_sha"])
    # the rn and edge count the reference's GPU arrays give
    k = int(g["k"])
    rn = np.partition(c, k)[k]
    assert np.float32(rn) == np.float32(g["rn"]) and int((c < rn).sum()) == int(g["num_edges"])


def test_bvp_batch_gpu_arithmetic_equals_pairs(gpu, pumplib, oracle):
    """The explicit-pair kernel of PUMP_BVP_PARITY_GPU gives what the pair
    kernel gives for the same pairs (the planner's shared roadmaps use both)."""
    from pump_gb300 import workloads
    torch, _ = gpu
    L = pumplib.load()
    N = 300
    s = oracle.halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    c, t = run_bvp_pairs(torch, pumplib, s, mode=pumplib.PUMP_BVP_PARITY_GPU)
    rng = np.random.default_rng(12)
    idx = rng.choice(N * (N - 1), 3000, replace=False)
    i = idx // (N - 1)
    r = idx - i * (N - 1)
    j = r + (r >= i)
    d0, d1 = dev(torch, s[i]), dev(torch, s[j])
    dt, dc = empty(torch, idx.size, torch.float32), empty(torch, idx.size, torch.float32)
    pumplib.check(L.pump_bvp_batch(ptr(d0), ptr(d1), idx.size, 5.0, pumplib.PUMP_BVP_PARITY_GPU,
                                   ptr(dt), ptr(dc), stream(torch)))
    assert same_bits(host(dt, idx.size), t[idx]) and same_bits(host(dc, idx.size), c[idx])


def kth_in_key_order(v, k):
    """The k-th smallest float32 in the order of the sign-magnitude keys:
    negative NaNs first, then -inf .. -0.0, +0.0 .. +inf, positive NaNs."""
    u = np.ascontiguousarray(v, np.float32).view(np.uint32)
    key = np.where(u & 0x80000000, ~u, u | 0x80000000).astype(np.uint32)
    kk = np.sort(key)[k]
    b = kk & 0x7FFFFFFF if kk & 0x80000000 else ~kk & 0xFFFFFFFF
    return np.array([b], np.uint32).view(np.float32)[0]


@pytest.mark.parametrize("k", [0, 10, 100_000, 1_960_000, 1_999_999])
def test_select_kth_nan(k, gpu, pumplib):
    """NaNs of both signs keep their place in the key order (positive NaNs
    above +inf, negative ones below -inf); the value comes back bit-exact."""
    torch, ctx = gpu
    v = np.arange(1, 2_000_001, dtype=np.float32)
    v[::50] = np.float32("nan")
    v.view(np.uint32)[7::97] = 0xFFC00000
    v[3::101] *= -1
    out = C.c_float(0)
    d = dev(torch, v)
    pumplib.check(pumplib.load().pump_select_kth(ctx.handle, ptr(d), v.size, k, C.byref(out),
                                                 stream(torch)))
    assert same_bits(np.float32(out.value), kth_in_key_order(v, k))


@pytest.mark.parametrize("n,k", [(1, 0), (1000, 0), (1000, 999), (100003, 5000), (5_000_000, 250_000)])
def test_select_kth(n, k, gpu, pumplib):
    torch, ctx = gpu
    rng = np.random.default_rng(n)
    v = rng.normal(0, 10, n).astype(np.float32)
    v[: n // 10] = np.float32(3.25)  # many ties
    if n > 4:
        v[1], v[2], v[3] = -0.0, 0.0, np.float32(-1e-30)
    out = C.c_float(0)
    d = dev(torch, v)
    pumplib.check(pumplib.load().pump_select_kth(ctx.handle, ptr(d), n, k, C.byref(out), stream(torch)))
    expect = np.partition(v, k)[k]
    assert out.value == expect or (out.value == 0 and expect == 0)


def test_select_rn_of_pair_costs(gpu, pumplib, roadmap1000):
    torch, ctx = gpu
    r = roadmap1000
    out = C.c_float(0)
    d = dev(torch, r["copts"])
    pumplib.check(pumplib.load().pump_select_kth(ctx.handle, ptr(d), r["copts"].size, r["k"],
                                                 C.byref(out), stream(torch)))
    assert np.float32(out.value) == np.float32(r["rn"])


def test_build_edges_and_waypoints(gpu, pumplib, roadmap1000):
    torch, ctx = gpu
    L = pumplib.load()
    r = roadmap1000
    N = r["N"]
    d_c, d_t = dev(torch, r["copts"]), dev(torch, r["topts"])
    cap = r["k"]
    d_src, d_dst = empty(torch, cap, torch.int32), empty(torch, cap, torch.int32)
    d_ce, d_te = empty(torch, cap, torch.float32), empty(torch, cap, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    E = C.c_longlong(0)
    pumplib.check(L.pump_build_edges(ctx.handle, ptr(d_c), ptr(d_t), N, float(r["rn"]), cap,
                                     ptr(d_src), ptr(d_dst), ptr(d_ce), ptr(d_te), ptr(d_go),
                                     C.byref(E), stream(torch)))
    E = E.value
    assert E == r["src"].size
    assert np.array_equal(host(d_src, E), r["src"]) and np.array_equal(host(d_dst, E), r["dst"])
    assert same_bits(host(d_ce, E), r["ce"]) and same_bits(host(d_te, E), r["te"])
    go = host(d_go, N + 1)
    assert np.array_equal(go, np.searchsorted(r["src"], np.arange(N + 1), side="left"))
    # capacity overflow reported, not written past the buffer
    E2 = C.c_longlong(0)
    st = L.pump_build_edges(ctx.handle, ptr(d_c), ptr(d_t), N, float(r["rn"]), E - 1, ptr(d_src),
                            ptr(d_dst), ptr(d_ce), ptr(d_te), ptr(d_go), C.byref(E2), stream(torch))
    assert st == pumplib.PUMP_ERR_CAPACITY and E2.value == E
    # waypoints (findDiscretizedPath)
    d_s = dev(torch, r["samples"])
    d_src2, d_dst2, d_te2 = dev(torch, r["src"]), dev(torch, r["dst"]), dev(torch, r["te"])
    d_disc = empty(torch, E * 9 * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges(ptr(d_s), ptr(d_src2), ptr(d_dst2), ptr(d_te2), E, 8, 0,
                                          ptr(d_disc), stream(torch)))
    disc = host(d_disc, E * 54).reshape(E, 9, 6)
    assert same_bits(disc, r["disc"]), "waypoint mismatches: %d" % int((disc != r["disc"]).sum())


def roadmap_edges(torch, pumplib, ctx, c, t, N, k, cap):
    """pump_roadmap_edges on host arrays: (rn, src, dst, copt, topt, go)."""
    d_c, d_t = dev(torch, c), dev(torch, t)
    d_src, d_dst = empty(torch, cap, torch.int32), empty(torch, cap, torch.int32)
    d_ce, d_te = empty(torch, cap, torch.float32), empty(torch, cap, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, E = C.c_float(0), C.c_longlong(0)
    pumplib.check(pumplib.load().pump_roadmap_edges(
        ctx.handle, ptr(d_c), ptr(d_t), N, k, cap, ptr(d_src), ptr(d_dst), ptr(d_ce), ptr(d_te),
        ptr(d_go), C.byref(rn), C.byref(E), stream(torch)))
    E = E.value
    return (np.float32(rn.value), host(d_src, E), host(d_dst, E), host(d_ce, E), host(d_te, E),
            host(d_go, N + 1))


def test_waypoints_gpu_arithmetic_mode(gpu, pumplib, roadmap1000):
    """pump_discretize_edges and pump_discretize_edges_off in the reference
    GPU kernel's mode evaluate the reference's host findDiscretizedPath: the
    parity waypoints at each edge's time in the host arithmetic (whatever
    times d_topt holds), bit for bit; the parity waypoints themselves match
    the oracle (test_build_edges_and_waypoints)."""
    torch, _ = gpu
    L = pumplib.load()
    r = roadmap1000
    s, src, dst = r["samples"], r["src"], r["dst"]
    E = src.size
    # the host-arithmetic times: pump_bvp_batch in parity mode, tmax 5
    d0, d1 = dev(torch, s[src]), dev(torch, s[dst])
    d_th, d_c = empty(torch, E, torch.float32), empty(torch, E, torch.float32)
    pumplib.check(L.pump_bvp_batch(ptr(d0), ptr(d1), E, 5.0, pumplib.PUMP_BVP_PARITY, ptr(d_th),
                                   ptr(d_c), stream(torch)))
    d_s, d_src, d_dst = dev(torch, s), dev(torch, src), dev(torch, dst)
    d_junk = dev(torch, np.full(E, 0.37, np.float32))  # GPU-kernel times are not used
    out = {}
    for mode, d_t in ((pumplib.PUMP_BVP_PARITY, d_th), (pumplib.PUMP_BVP_PARITY_GPU, d_junk)):
        d_disc = empty(torch, E * 9 * 6, torch.float32)
        pumplib.check(L.pump_discretize_edges(ptr(d_s), ptr(d_src), ptr(d_dst), ptr(d_t), E, 8, mode,
                                              ptr(d_disc), stream(torch)))
        d_off = dev(torch, np.arange(E + 1, dtype=np.int64) * 9)
        d_disc2 = empty(torch, E * 9 * 6, torch.float32)
        pumplib.check(L.pump_discretize_edges_off(ptr(d_s), ptr(d_src), ptr(d_dst), ptr(d_t), E,
                                                  ptr(d_off), 8, mode, ptr(d_disc2), stream(torch)))
        out[mode] = (host(d_disc, E * 54), host(d_disc2, E * 54))
    a, b = out[pumplib.PUMP_BVP_PARITY], out[pumplib.PUMP_BVP_PARITY_GPU]
    assert same_bits(a[0], b[0]) and same_bits(a[1], b[1]) and same_bits(a[0], a[1])


def test_roadmap_edges_one_read(gpu, pumplib, roadmap1000):
    """rn and the edges from one read of the pair costs equal pump_select_kth +
    pump_build_edges (the oracle's sort and scan) bit for bit."""
    torch, ctx = gpu
    r = roadmap1000
    N = r["N"]
    rn, src, dst, ce, te, go = roadmap_edges(torch, pumplib, ctx, r["copts"], r["topts"], N, r["k"],
                                             r["k"])
    assert rn == np.float32(r["rn"])
    assert np.array_equal(src, r["src"]) and np.array_equal(dst, r["dst"])
    assert same_bits(ce, r["ce"]) and same_bits(te, r["te"])
    assert np.array_equal(go, np.searchsorted(r["src"], np.arange(N + 1), side="left"))


@pytest.mark.parametrize("pattern", ["plain", "sample_high", "sample_low", "ties", "small"])
def test_roadmap_edges_patterns(pattern, gpu, pumplib, oracle):
    """Cost patterns that defeat the strided sample (every sampled pair far
    above or below the rest) or crowd rn with ties, and a roadmap too small
    for the one-read pass: the result is the oracle's sort and scan."""
    torch, ctx = gpu
    N = 300 if pattern == "small" else 1200
    n = N * (N - 1)
    k = int(n * np.float32(0.05))
    rng = np.random.default_rng(N)
    c = rng.exponential(10.0, n).astype(np.float32)
    t = rng.uniform(0.1, 5.0, n).astype(np.float32)
    q = np.arange(8192, dtype=np.int64)
    pos = ((2 * q + 1) * n) // (2 * 8192)
    if pattern == "sample_high":
        c[pos] = np.float32(1e6)
    elif pattern == "sample_low":
        c[pos] = np.float32(-1.0)
    elif pattern == "ties":
        v = np.partition(c, k)[k]
        c[rng.random(n) < 0.1] = v
    rn64 = oracle.lib().orc_select_kth(c.size, c, k)
    src, dst, ce, te = oracle.build_edges(c, t, N, rn64)
    rn, s2, d2, ce2, te2, go = roadmap_edges(torch, pumplib, ctx, c, t, N, k, k)
    assert rn == np.float32(rn64)
    assert np.array_equal(s2, src) and np.array_equal(d2, dst)
    assert same_bits(ce2, ce) and same_bits(te2, te)
    assert np.array_equal(go, np.searchsorted(src, np.arange(N + 1), side="left"))


def test_roadmap_edges_nan_costs(gpu, pumplib):
    """NaN costs (either sign) order as the full radix select orders them:
    the one-read result equals pump_select_kth + pump_build_edges."""
    torch, ctx = gpu
    L = pumplib.load()
    N = 1100
    n = N * (N - 1)
    k = int(n * np.float32(0.05))
    rng = np.random.default_rng(11)
    c = rng.normal(5.0, 3.0, n).astype(np.float32)
    t = rng.uniform(0.1, 5.0, n).astype(np.float32)
    c[rng.random(n) < 0.02] = np.float32("nan")
    c.view(np.uint32)[rng.random(n) < 0.02] = 0xFFC00000  # negative NaN
    rn, src, dst, ce, te, go = roadmap_edges(torch, pumplib, ctx, c, t, N, k, k)
    assert same_bits(rn, kth_in_key_order(c, k))
    out = C.c_float(0)
    d_c, d_t = dev(torch, c), dev(torch, t)
    pumplib.check(L.pump_select_kth(ctx.handle, ptr(d_c), n, k, C.byref(out), stream(torch)))
    assert same_bits(np.float32(out.value), rn)
    d_src, d_dst = empty(torch, k, torch.int32), empty(torch, k, torch.int32)
    d_ce, d_te = empty(torch, k, torch.float32), empty(torch, k, torch.float32)
    E = C.c_longlong(0)
    pumplib.check(L.pump_build_edges(ctx.handle, ptr(d_c), ptr(d_t), N, out.value, k, ptr(d_src),
                                     ptr(d_dst), ptr(d_ce), ptr(d_te), None, C.byref(E),
                                     stream(torch)))
    E = E.value
    assert E == src.size
    assert np.array_equal(host(d_src, E), src) and np.array_equal(host(d_dst, E), dst)
    assert same_bits(host(d_ce, E), ce) and same_bits(host(d_te, E), te)


def roadmap_one_call(torch, pumplib, ctx, s, k, mode, stage_ms=None):
    """pump_roadmap on host samples: (copts, topts, rn, src, dst, copt, topt, go)."""
    N = s.shape[0]
    n = N * (N - 1)
    d_s = dev(torch, s)
    d_c, d_t = empty(torch, n, torch.float32), empty(torch, n, torch.float32)
    d_src, d_dst = empty(torch, k, torch.int32), empty(torch, k, torch.int32)
    d_ce, d_te = empty(torch, k, torch.float32), empty(torch, k, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, E = C.c_float(0), C.c_longlong(0)
    pumplib.check(pumplib.load().pump_roadmap(
        ctx.handle, ptr(d_s), N, 5.0, mode, k, k, ptr(d_c), ptr(d_t), ptr(d_src), ptr(d_dst),
        ptr(d_ce), ptr(d_te), ptr(d_go), C.byref(rn), C.byref(E), stage_ms, stream(torch)))
    E = E.value
    return (host(d_c, n), host(d_t, n), np.float32(rn.value), host(d_src, E), host(d_dst, E),
            host(d_ce, E), host(d_te, E), host(d_go, N + 1))


def roadmap_sample_sets():
    from pump_gb300 import workloads
    from oracle.pyoracle import halton_samples
    lo, hi = np.asarray(workloads.LO, np.float32), np.asarray(workloads.HI, np.float32)
    rng = np.random.default_rng(5)
    uni = (lo + (hi - lo) * rng.random((2100, 6))).astype(np.float32)
    # four tight clusters: the strided sample sees rows of very uneven density
    cen = lo + (hi - lo) * rng.random((4, 6))
    clu = (cen[rng.integers(0, 4, 1800)] + rng.normal(0, 0.02, (1800, 6))).astype(np.float32)
    # four states repeated 200 times each: the pair costs take a few values,
    # so the superset under the bracket (a quarter of all pairs) overflows
    # its buffer and the pass falls back to the full select
    ties = np.repeat(uni[:4], 200, axis=0)
    return {"halton1000": halton_samples(1000, workloads.INIT, workloads.GOAL, workloads.LO,
                                         workloads.HI),
            "uniform2100": uni, "clusters1800": clu, "ties800": ties}


@pytest.mark.parametrize("case", ["halton1000", "uniform2100", "clusters1800", "ties800"])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_roadmap_one_call(case, mode, gpu, pumplib):
    """pump_roadmap (pair BVPs counting the rn superset as they store the
    costs, in the precision arithmetic) gives the bytes of pump_bvp_pairs +
    pump_roadmap_edges, in every arithmetic."""
    torch, ctx = gpu
    L = pumplib.load()
    s = roadmap_sample_sets()[case]
    if mode != 1:
        s = s[:800]  # the bisection arithmetics: 639,200 pairs, still the one-read pass
    N = s.shape[0]
    n = N * (N - 1)
    k = int(np.float32(n) * np.float32(0.05))
    c, t = run_bvp_pairs(torch, pumplib, s, mode)
    ref = (c, t) + roadmap_edges(torch, pumplib, ctx, c, t, N, k, k)
    ms = (C.c_float * 3)()
    got = roadmap_one_call(torch, pumplib, ctx, s, k, mode, ms)
    names = ["copts", "topts", "rn", "src", "dst", "copt", "topt", "go"]
    for name, a, b in zip(names, ref, got):
        assert same_bits(np.atleast_1d(a), np.atleast_1d(b)), (case, mode, name)
    assert ms[0] >= 0 and ms[1] > 0 and ms[2] > 0
    # a second call on the same context (scratch reused) gives the same bytes
    again = roadmap_one_call(torch, pumplib, ctx, s, k, mode)
    for name, a, b in zip(names, got, again):
        assert same_bits(np.atleast_1d(a), np.atleast_1d(b)), (case, mode, name)


def test_roadmap_one_call_parity_oracle(gpu, pumplib, roadmap1000):
    """In the parity arithmetic pump_roadmap's rn and edges are the oracle's."""
    torch, ctx = gpu
    r = roadmap1000
    c, t, rn, src, dst, ce, te, go = roadmap_one_call(torch, pumplib, ctx, r["samples"], r["k"], 0)
    assert same_bits(c, r["copts"]) and same_bits(t, r["topts"])
    assert rn == np.float32(r["rn"])
    assert np.array_equal(src, r["src"]) and np.array_equal(dst, r["dst"])
    assert same_bits(ce, r["ce"]) and same_bits(te, r["te"])
    assert np.array_equal(go, np.searchsorted(r["src"], np.arange(r["N"] + 1), side="left"))


def test_roadmap_one_call_capacity(gpu, pumplib, roadmap1000):
    """Fewer edge slots than edges: PUMP_ERR_CAPACITY with the true count."""
    torch, ctx = gpu
    L = pumplib.load()
    r = roadmap1000
    N, k = r["N"], r["k"]
    d_s = dev(torch, r["samples"])
    n = N * (N - 1)
    d_c, d_t = empty(torch, n, torch.float32), empty(torch, n, torch.float32)
    cap = k // 2  # about k edges qualify
    d_src, d_dst = empty(torch, cap, torch.int32), empty(torch, cap, torch.int32)
    d_ce, d_te = empty(torch, cap, torch.float32), empty(torch, cap, torch.float32)
    rn, E = C.c_float(0), C.c_longlong(0)
    st = L.pump_roadmap(ctx.handle, ptr(d_s), N, 5.0, 1, k, cap, ptr(d_c), ptr(d_t), ptr(d_src),
                        ptr(d_dst), ptr(d_ce), ptr(d_te), None, C.byref(rn), C.byref(E), None,
                        stream(torch))
    torch.cuda.synchronize()
    assert st == pumplib.PUMP_ERR_CAPACITY
    assert E.value > cap


def test_collision_checks(gpu, pumplib, oracle, roadmap1000):
    torch, _ = gpu
    L = pumplib.load()
    r = roadmap1000
    N, obs = r["N"], r["obs"]
    E = r["src"].size
    d_obs, d_s, d_disc = dev(torch, obs), dev(torch, r["samples"]), dev(torch, r["disc"])
    d_fs = empty(torch, N, torch.uint8)
    pumplib.check(L.pump_sample_free(ptr(d_obs), obs.shape[0], ptr(d_s), N, ptr(d_fs), stream(torch)))
    assert np.array_equal(host(d_fs, N), oracle.sample_free(r["samples"], obs))
    d_fe = empty(torch, E, torch.uint8)
    pumplib.check(L.pump_free_edges(ptr(d_obs), obs.shape[0], ptr(d_disc), E, 8, ptr(d_fe), stream(torch)))
    assert np.array_equal(host(d_fe, E), r["fe"])
    for om in (np.float32(0.3), np.float32(1.0)):
        maxHS = min(obs.shape[0], 5)
        maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
        d_a = empty(torch, E * 9 * maxHS * 3, torch.float32)
        d_b = empty(torch, E * 9 * maxHS, torch.float32)
        d_n = empty(torch, E * 9, torch.int32)
        pumplib.check(L.pump_cache_halfspaces(ptr(d_obs), obs.shape[0], ptr(d_disc), ptr(d_fe), E, 9,
                                              maxHS, float(maxd2), ptr(d_a), ptr(d_b), ptr(d_n),
                                              stream(torch)))
        a, b, n = oracle.cache_halfspaces(r["disc"], r["fe"], obs, maxHS, maxd2)
        assert same_bits(host(d_a, a.size), a) and same_bits(host(d_b, b.size), b)
        free_wp = np.repeat(r["fe"].astype(bool), 9)
        assert np.array_equal(host(d_n, E * 9)[free_wp], n[free_wp])
        assert np.all(host(d_n, E * 9)[~free_wp] == 0)


@pytest.mark.parametrize("mapname", ["indoor40", "boxes100", "boxes200"])
def test_halfspaces_maps_and_gates(mapname, gpu, pumplib, oracle, roadmap1000):
    """Half-spaces on other maps and distance gates, including the gate of the
    benchmark's noise multiplier (2e-3, gate radius 6e-4), a NaN waypoint on a
    free edge, and more boxes than the per-edge box filter covers (128)."""
    torch, _ = gpu
    L = pumplib.load()
    from pump_gb300 import workloads
    obs = {"indoor40": lambda: workloads.indoor(1001),
           "boxes100": lambda: workloads.random_boxes(100, 7, side=(0.02, 0.08)),
           "boxes200": lambda: workloads.random_boxes(200, 8, side=(0.02, 0.06))}[mapname]()
    obs = np.ascontiguousarray(obs, np.float32)
    r = roadmap1000
    E = r["src"].size
    disc = r["disc"].copy()
    fe = oracle.free_edges(disc, obs)
    k = int(np.nonzero(fe)[0][len(np.nonzero(fe)[0]) // 2])
    disc.reshape(E, 9, 6)[k, 4, 1] = np.nan  # one free edge with a NaN waypoint
    d_obs, d_disc, d_fe = dev(torch, obs), dev(torch, disc), dev(torch, fe)
    # the collision check on this map, NaN waypoint included
    d_fe2 = empty(torch, E, torch.uint8)
    pumplib.check(L.pump_free_edges(ptr(d_obs), obs.shape[0], ptr(d_disc), E, 8, ptr(d_fe2),
                                    stream(torch)))
    assert np.array_equal(host(d_fe2, E), oracle.free_edges(disc, obs))
    for om in (2e-3, 0.05, 0.3):
        maxHS = min(obs.shape[0], 5)
        maxd2 = np.float32(0.1 * om * om)
        d_a = empty(torch, E * 9 * maxHS * 3, torch.float32)
        d_b = empty(torch, E * 9 * maxHS, torch.float32)
        d_n = empty(torch, E * 9, torch.int32)
        pumplib.check(L.pump_cache_halfspaces(ptr(d_obs), obs.shape[0], ptr(d_disc), ptr(d_fe), E, 9,
                                              maxHS, float(maxd2), ptr(d_a), ptr(d_b), ptr(d_n),
                                              stream(torch)))
        a, b, n = oracle.cache_halfspaces(disc, fe, obs, maxHS, maxd2)
        assert np.isnan(a).any()  # the NaN waypoint reached the half-spaces
        assert same_bits_or_nan(host(d_a, a.size), a) and same_bits_or_nan(host(d_b, b.size), b)
        free_wp = np.repeat(fe.astype(bool), 9)
        assert np.array_equal(host(d_n, E * 9)[free_wp], n[free_wp])


def test_collision_checks_many_obstacles(gpu, pumplib, oracle, roadmap1000):
    """More boxes than fit one block's threads (the reference's limit is 85)."""
    torch, _ = gpu
    L = pumplib.load()
    from pump_gb300 import workloads
    obs = workloads.random_boxes(300, 5, side=(0.02, 0.08))
    r = roadmap1000
    E = r["src"].size
    d_obs, d_disc = dev(torch, obs), dev(torch, r["disc"])
    d_fe = empty(torch, E, torch.uint8)
    pumplib.check(L.pump_free_edges(ptr(d_obs), obs.shape[0], ptr(d_disc), E, 8, ptr(d_fe), stream(torch)))
    assert np.array_equal(host(d_fe, E), oracle.free_edges(r["disc"], obs))


@pytest.mark.parametrize("P,T", [(2048, 400), (100, 37)])
def test_particle_tables(P, T, gpu, pumplib, oracle):
    torch, _ = gpu
    d_t = empty(torch, P * T * 3, torch.float32)
    d_p = empty(torch, P * T * 3, torch.float32)
    seed = 0x9E3779B97F4A7C15
    pumplib.check(pumplib.load().pump_particle_tables(seed, P, T, ptr(d_t), ptr(d_p), stream(torch)))
    tm, pm = oracle.particle_tables(seed, P, T)
    assert same_bits(host(d_t, P * T * 3).reshape(T, P, 3), tm)
    assert same_bits(host(d_p, P * T * 3).reshape(P, T, 3), pm)


@pytest.mark.parametrize("P", [128, 1024, 100])
def test_hsmc_propagate(P, gpu, pumplib, oracle, roadmap1000):
    torch, _ = gpu
    L = pumplib.load()
    r = roadmap1000
    obs, E = r["obs"], r["src"].size
    om = np.float32(0.3)
    maxHS = 5
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    a, b, _ = oracle.cache_halfspaces(r["disc"], r["fe"], obs, maxHS, maxd2)
    Pmc, T = 2048, 400
    tm, _ = oracle.particle_tables(0x1234, Pmc, T, pmajor=False)
    rng = np.random.default_rng(P)
    base = 50
    n_new = 3000
    edges = rng.choice(np.nonzero(r["fe"])[0], n_new).astype(np.int32)
    prev = rng.integers(0, base, n_new).astype(np.int32)
    times = np.zeros(base + n_new, np.float32)
    times[:base] = rng.uniform(0, 6, base).astype(np.float32)
    valid_bytes = np.zeros(((base + n_new), P), np.uint8)
    valid_bytes[:base] = rng.random((base, P)) < 0.9
    words = (P + 31) // 32
    vb = np.zeros((base + n_new, words * 32), np.uint8)
    vb[:, :P] = valid_bytes
    packed = np.packbits(vb, axis=1, bitorder="little").view(np.uint32)
    assert np.array_equal(bits_to_bytes(packed, P), vb[:, :P])
    d_valid = dev(torch, packed)
    d_cp = empty(torch, base + n_new, torch.float32)
    d_err = dev(torch, np.zeros(1, np.int32))
    # every device buffer stays referenced until the kernel has finished
    d_edges, d_prev, d_a, d_b = dev(torch, edges), dev(torch, prev), dev(torch, a), dev(torch, b)
    d_times, d_te, d_tm = dev(torch, times), dev(torch, r["te"]), dev(torch, tm)
    pumplib.check(L.pump_hsmc_propagate(n_new, 9, ptr(d_edges), ptr(d_prev), E, base, ptr(d_a), ptr(d_b),
                                        maxHS, ptr(d_times), ptr(d_te), 0.05, ptr(d_tm), Pmc, T,
                                        float(om), ptr(d_valid), P, ptr(d_cp), ptr(d_err),
                                        None, stream(torch)))
    torch.cuda.synchronize()
    got = bits_to_bytes(host(d_valid).reshape(base + n_new, words), P)
    cp_o = np.zeros(base + n_new, np.float32)
    oracle.lib().orc_hsmc_propagate(n_new, 9, edges, prev, base, a, b, times, r["te"], 0.05, maxHS,
                                    tm.reshape(-1), om, Pmc, valid_bytes, P, cp_o)
    assert np.array_equal(got[base:], valid_bytes[base:])
    assert same_bits(host(d_cp)[base:base + n_new], cp_o[base:])
    assert int(host(d_err)[0]) == 0
    assert 0 < valid_bytes[base:].mean() < 1


def test_hsmc_device_checks(gpu, pumplib, oracle, roadmap1000):
    """HSMC's device-side checks: an edge index outside [0, E) and a parent
    outside [0, base) skip their paths and record PUMP_ERR_BAD_INPUT; a time
    row past the particle table records PUMP_ERR_CAPACITY (the reference
    reads both without a bound, PUMP.cu:626-647).  Every other path is
    computed as the oracle computes it."""
    torch, _ = gpu
    L = pumplib.load()
    r = roadmap1000
    obs, E = r["obs"], r["src"].size
    om, maxHS, P, Pmc = np.float32(0.3), 5, 128, 2048
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    a, b, _ = oracle.cache_halfspaces(r["disc"], r["fe"], obs, maxHS, maxd2)
    rng = np.random.default_rng(31)
    base, n_new = 40, 500
    edges = rng.choice(np.nonzero(r["fe"])[0], n_new).astype(np.int32)
    prev = rng.integers(0, base, n_new).astype(np.int32)
    times = np.zeros(base + n_new, np.float32)
    times[:base] = rng.uniform(0, 4, base).astype(np.float32)
    valid_bytes = np.zeros((base + n_new, P), np.uint8)
    valid_bytes[:base] = rng.random((base, P)) < 0.9
    packed = np.packbits(valid_bytes, axis=1, bitorder="little").view(np.uint32)
    for T, bad, want in ((400, True, pumplib.PUMP_ERR_BAD_INPUT), (60, False, pumplib.PUMP_ERR_CAPACITY)):
        tm, _ = oracle.particle_tables(0x1234, Pmc, T, pmajor=False)
        e2, p2 = edges.copy(), prev.copy()
        if bad:
            e2[3], p2[5] = E, base  # one past the end of each
        d_valid = dev(torch, packed)
        d_cp = empty(torch, base + n_new, torch.float32)
        d_err = dev(torch, np.zeros(1, np.int32))
        keep = [dev(torch, x) for x in (e2, p2, a, b, times, r["te"], tm)]
        pumplib.check(L.pump_hsmc_propagate(n_new, 9, ptr(keep[0]), ptr(keep[1]), E, base, ptr(keep[2]),
                                            ptr(keep[3]), maxHS, ptr(keep[4]), ptr(keep[5]), 0.05,
                                            ptr(keep[6]), Pmc, T, float(om), ptr(d_valid), P, ptr(d_cp),
                                            ptr(d_err), None, stream(torch)))
        torch.cuda.synchronize()
        assert int(host(d_err)[0]) == want
        if bad:
            got = bits_to_bytes(host(d_valid).reshape(base + n_new, -1), P)
            vb = valid_bytes.copy()
            cp_o = np.zeros(base + n_new, np.float32)
            oracle.lib().orc_hsmc_propagate(n_new, 9, edges, prev, base, a, b, times, r["te"], 0.05, maxHS,
                                            tm.reshape(-1), om, Pmc, vb, P, cp_o)
            ok = np.ones(n_new, bool)
            ok[[3, 5]] = False
            assert np.array_equal(got[base:][ok], vb[base:][ok])
            assert same_bits(host(d_cp)[base:base + n_new][ok], cp_o[base:][ok])


@pytest.mark.parametrize("om", [0.3, 2e-3])
def test_sparse_halfspaces_and_hsmc(om, gpu, pumplib, oracle, roadmap1000):
    """pump_cache_halfspaces_sparse writes the reference's stored half-spaces
    and their counts only (slots past a count keep what the buffers held, NaN
    here), and HSMC reading them through the counts gives the same particle
    masks and CPs as the dense layout."""
    torch, _ = gpu
    L = pumplib.load()
    r = roadmap1000
    obs, E, W = r["obs"], r["src"].size, 9
    om = np.float32(om)
    maxHS = 5
    maxd2 = np.float32(0.1 * np.float64(om) * np.float64(om))
    a, b, n = oracle.cache_halfspaces(r["disc"], r["fe"], obs, maxHS, maxd2)
    d_obs, d_disc, d_fe = dev(torch, obs), dev(torch, r["disc"]), dev(torch, r["fe"])
    d_a = torch.full((E * W * maxHS * 3,), float("nan"), dtype=torch.float32, device="cuda")
    d_b = torch.full((E * W * maxHS,), float("nan"), dtype=torch.float32, device="cuda")
    d_n = torch.full((E * W,), 255, dtype=torch.uint8, device="cuda")
    pumplib.check(L.pump_cache_halfspaces_sparse(ptr(d_obs), obs.shape[0], ptr(d_disc), ptr(d_fe), E,
                                                 W, maxHS, float(maxd2), ptr(d_a), ptr(d_b), ptr(d_n),
                                                 stream(torch)))
    torch.cuda.synchronize()
    cnt = host(d_n).astype(np.int32)
    free_wp = np.repeat(r["fe"].astype(bool), W)
    assert np.array_equal(cnt[free_wp], n[free_wp]) and np.all(cnt[~free_wp] == 0)
    slot = np.arange(maxHS)[None, :] < cnt[:, None]
    ga, gb = host(d_a).reshape(-1, maxHS, 3), host(d_b).reshape(-1, maxHS)
    assert same_bits(gb[slot], b.reshape(-1, maxHS)[slot])
    assert same_bits(ga[slot], a.reshape(-1, maxHS, 3)[slot])
    assert np.all(np.isnan(gb[~slot]))
    # HSMC through the counts vs the oracle on the dense layout
    Pmc, T, P = 2048, 400, 1024
    tm, _ = oracle.particle_tables(0x1234, Pmc, T, pmajor=False)
    rng = np.random.default_rng(11)
    base, n_new = 50, 3000
    edges = rng.choice(np.nonzero(r["fe"])[0], n_new).astype(np.int32)
    prev = rng.integers(0, base, n_new).astype(np.int32)
    times = np.zeros(base + n_new, np.float32)
    times[:base] = rng.uniform(0, 6, base).astype(np.float32)
    valid_bytes = np.zeros((base + n_new, P), np.uint8)
    valid_bytes[:base] = rng.random((base, P)) < 0.9
    packed = np.packbits(valid_bytes, axis=1, bitorder="little").view(np.uint32)
    d_valid, d_cp = dev(torch, packed), empty(torch, base + n_new, torch.float32)
    d_err = dev(torch, np.zeros(1, np.int32))
    d_edges, d_prev, d_times = dev(torch, edges), dev(torch, prev), dev(torch, times)
    d_te, d_tm = dev(torch, r["te"]), dev(torch, tm)
    pumplib.check(L.pump_hsmc_propagate(n_new, W, ptr(d_edges), ptr(d_prev), E, base, ptr(d_a), ptr(d_b),
                                        maxHS, ptr(d_times), ptr(d_te), 0.05, ptr(d_tm), Pmc, T,
                                        float(om), ptr(d_valid), P, ptr(d_cp), ptr(d_err), ptr(d_n),
                                        stream(torch)))
    torch.cuda.synchronize()
    got = bits_to_bytes(host(d_valid).reshape(base + n_new, P // 32), P)
    cp_o = np.zeros(base + n_new, np.float32)
    oracle.lib().orc_hsmc_propagate(n_new, W, edges, prev, base, a, b, times, r["te"], 0.05, maxHS,
                                    tm.reshape(-1), om, Pmc, valid_bytes, P, cp_o)
    assert np.array_equal(got[base:], valid_bytes[base:])
    assert same_bits(host(d_cp)[base:base + n_new], cp_o[base:])
    assert int(host(d_err)[0]) == 0
    # half-spaces derived in the kernel from the boxes and waypoints: same bits
    d_valid2, d_cp2 = dev(torch, packed), empty(torch, base + n_new, torch.float32)
    d_err2 = dev(torch, np.zeros(1, np.int32))
    pumplib.check(L.pump_hsmc_propagate_boxes(
        n_new, W, ptr(d_edges), ptr(d_prev), E, base, ptr(d_obs), obs.shape[0], ptr(d_disc),
        float(maxd2), maxHS, ptr(d_times), ptr(d_te), 0.05, ptr(d_tm), Pmc, T, float(om),
        ptr(d_valid2), P, ptr(d_cp2), ptr(d_err2), stream(torch)))
    torch.cuda.synchronize()
    got2 = bits_to_bytes(host(d_valid2).reshape(base + n_new, P // 32), P)
    assert np.array_equal(got2[base:], valid_bytes[base:])
    assert same_bits(host(d_cp2)[base:base + n_new], cp_o[base:])
    assert int(host(d_err2)[0]) == 0
    if om >= 0.05:  # half-spaces are active: some particles die on the new edges
        assert np.any(valid_bytes[base:] != valid_bytes[prev])


def test_mc_cp(gpu, pumplib, oracle, goldens):
    torch, _ = gpu
    L = pumplib.load()
    g = goldens["ref_N1000_boxes10_noise0.3"]
    obs = g["prob_obstacles"].astype(np.float32)
    path = np.array([[float(x) for x in line.split()] for line in str(g["path_txt"]).splitlines()],
                    np.float32)
    Pmc, T = 2048, 400
    tm, pm = oracle.particle_tables(0x9E3779B97F4A7C15, Pmc, T)
    paths = [path, path[:10], path[::2].copy(), path + np.float32(0.01)]
    lens = np.array([p.shape[0] for p in paths], np.int32)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int32)
    allp = np.concatenate(paths, 0).astype(np.float32)
    hits = empty(torch, len(paths), torch.int32)
    cps = empty(torch, len(paths), torch.float32)
    d_allp, d_offs, d_lens = dev(torch, allp), dev(torch, offs), dev(torch, lens)
    d_tm, d_obs = dev(torch, tm), dev(torch, obs)
    for om in (np.float32(0.3), np.float32(1.0)):
        pumplib.check(L.pump_mc_cp(ptr(d_allp), ptr(d_offs), ptr(d_lens), len(paths), ptr(d_tm), Pmc,
                                   T, float(om), ptr(d_obs), obs.shape[0], ptr(hits), ptr(cps), 0,
                                   stream(torch)))
        torch.cuda.synchronize()
        for k, p in enumerate(paths):
            h, cp = oracle.mccp(p, p.shape[0], pm, om, obs)
            assert int(host(hits)[k]) == h
            assert np.float32(host(cps)[k]) == np.float32(cp)


@pytest.mark.parametrize("N,density", [(0, 0.5), (1, 1.0), (4095, 0.3), (4096, 1.0), (100_000, 0.01),
                                       (1_000_000, 0.5), (777_777, 0.0)])
def test_frontier_compact(N, density, gpu, pumplib):
    torch, ctx = gpu
    rng = np.random.default_rng(N)
    flags = (rng.random(N) < density).astype(np.uint8)
    d_f = dev(torch, flags) if N else empty(torch, 1, torch.uint8)
    d_a = empty(torch, N, torch.int32)
    d_n = empty(torch, 1, torch.int32)
    pumplib.check(pumplib.load().pump_frontier_compact(ctx.handle, ptr(d_f), N, ptr(d_a), ptr(d_n),
                                                       stream(torch)))
    n = int(host(d_n)[0])
    expect = np.nonzero(flags)[0]
    assert n == expect.size
    assert np.array_equal(host(d_a, n), expect)


def test_bvp_pairs_precision_vs_long_double(gpu, pumplib, oracle, goldens):
    """Precision mode against an independent long-double grid-and-bisection
    oracle: every cost within 1 binary32 ulp of the exact minimum and at least
    99 % of them its correctly rounded value; optimal times within 1 ulp for
    at least 99 % (near-equal minima may pick a different time at equal cost,
    at most 2 beyond 1e-5 relative)."""
    torch, _ = gpu
    _, _, init, goal, lo, hi, _ = golden_problem(goldens, "ref_N1000_input")
    N = 400
    s = oracle.halton_samples(N, init, goal, lo, hi)
    rng = np.random.default_rng(3)
    s[1:-1, :3] += rng.normal(0, 0.05, (N - 2, 3)).astype(np.float32)  # break lattice symmetry
    c, t = run_bvp_pairs(torch, pumplib, s, mode=1)
    idx = rng.choice(N * (N - 1), 4000, replace=False)
    exact_c = within1_c = exact_t = within1_t = far_t = 0
    for q in idx:
        i = q // (N - 1)
        r = q - i * (N - 1)
        j = r + (r >= i)
        topt_ref, cost_ref = oracle.bvp_precise(s[i], s[j])
        cr, tr = np.float32(cost_ref), np.float32(topt_ref)
        exact_c += c[q] == cr
        within1_c += abs(int(c[q].view(np.int32)) - int(cr.view(np.int32))) <= 1
        exact_t += t[q] == tr
        within1_t += abs(int(t[q].view(np.int32)) - int(tr.view(np.int32))) <= 1
        far_t += abs(float(t[q]) - topt_ref) > 1e-5 * topt_ref
    n = len(idx)
    stats = (exact_c, within1_c, exact_t, within1_t, far_t, n)
    assert within1_c == n, stats
    assert exact_c >= 0.99 * n, stats
    assert within1_t >= 0.99 * n, stats
    assert far_t <= 2, stats


def test_mc_cp_binary32_vs_binary64(gpu, pumplib, oracle):
    """The binary32 Monte Carlo CP (collision tests as the reference's, in
    binary32) against the same estimate with every test in binary64: hit
    counts differ by at most 2 of 2048 particles on any path (a particle whose
    segment grazes a box face within binary32 rounding)."""
    torch, _ = gpu
    L = pumplib.load()
    from pump_gb300 import workloads
    obs = workloads.indoor(1003).astype(np.float32)
    nodes, offs, cnts = workloads.perturbed_paths(64, 21, obs, n_range=(8, 16))
    paths = []
    for o, n in zip(offs, cnts):
        x = nodes[o:o + n].astype(np.float64)
        s = np.linspace(0, n - 1, 6 * n)
        paths.append(np.stack([np.interp(s, np.arange(n), x[:, d]) for d in range(6)], 1).astype(np.float32))
    lens = np.array([p.shape[0] for p in paths], np.int32)
    poff = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int32)
    allp = np.concatenate(paths, 0)
    Pmc, T = 2048, 400
    tm, pm = oracle.particle_tables(0x9E3779B97F4A7C15, Pmc, T)
    d_allp, d_offs, d_lens, d_tm, d_obs = (dev(torch, a) for a in (allp, poff, lens, tm, obs))
    hits = empty(torch, len(paths), torch.int32)
    cps = empty(torch, len(paths), torch.float32)
    for om in (0.02, 0.3):
        pumplib.check(L.pump_mc_cp(ptr(d_allp), ptr(d_offs), ptr(d_lens), len(paths), ptr(d_tm), Pmc, T,
                                   om, ptr(d_obs), obs.shape[0], ptr(hits), ptr(cps), 0, stream(torch)))
        torch.cuda.synchronize()
        h32 = host(hits)
        h64 = np.array([oracle.mccp64(p, p.shape[0], pm, np.float32(om), obs) for p in paths])
        assert np.all(np.abs(h32 - h64) <= 2), (om, np.abs(h32 - h64).max())
        assert np.count_nonzero(h64) > 10


@pytest.mark.parametrize("N", [2, 1000, 4001])
def test_halton_samples(N, gpu, pumplib, oracle, goldens):
    """pump_halton_samples: the reference's Halton samples (createSamplesHalton,
    sampler.cu:20-41) bit for bit, init first and goal last; nothing written
    past the N rows."""
    torch, _ = gpu
    _, _, init, goal, lo, hi, _ = golden_problem(goldens, "ref_N1000_input")
    f6 = lambda v: (C.c_float * 6)(*[float(x) for x in v])  # noqa: E731
    d = empty(torch, N * 6 + 6, torch.float32)
    d.fill_(7.0)
    pumplib.check(pumplib.load().pump_halton_samples(N, f6(lo), f6(hi), f6(init), f6(goal), ptr(d),
                                                     stream(torch)))
    got = host(d)
    assert same_bits(got[: N * 6].reshape(N, 6), oracle.halton_samples(N, init, goal, lo, hi))
    assert np.all(got[N * 6:] == 7.0)
    if N == 1000:
        assert same_bits(got[: N * 6].reshape(N, 6), goldens["ref_N1000_input"]["samples"])
