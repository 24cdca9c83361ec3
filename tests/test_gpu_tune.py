"""The launch-shape autotuner: the shapes it picks compute exactly what the
default shapes compute, and it records one choice per shape class."""
import ctypes as C

import numpy as np
import pytest

from helpers import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu


def roadmap_outputs(torch, pumplib, ctx, N, obs):
    """Pair BVPs (precision), rn and edges, waypoints and the edge check."""
    from pump_gb300 import workloads
    from oracle.pyoracle import halton_samples
    L = pumplib.load()
    s = halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    d_s, d_obs = dev(torch, s), dev(torch, obs)
    n = N * (N - 1)
    k = int(np.float32(n) * np.float32(0.05))
    d_c, d_t = empty(torch, n, torch.float32), empty(torch, n, torch.float32)
    pumplib.check(L.pump_bvp_pairs(ptr(d_s), N, 5.0, pumplib.PUMP_BVP_PRECISION, ptr(d_c), ptr(d_t),
                                   stream(torch)))
    d_src, d_dst = empty(torch, k, torch.int32), empty(torch, k, torch.int32)
    d_ce, d_te = empty(torch, k, torch.float32), empty(torch, k, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, E = C.c_float(0), C.c_longlong(0)
    pumplib.check(L.pump_roadmap_edges(ctx.handle, ptr(d_c), ptr(d_t), N, k, k, ptr(d_src), ptr(d_dst),
                                       ptr(d_ce), ptr(d_te), ptr(d_go), C.byref(rn), C.byref(E),
                                       stream(torch)))
    E = E.value
    d_disc = empty(torch, E * 9 * 6, torch.float32)
    pumplib.check(L.pump_discretize_edges(ptr(d_s), ptr(d_src), ptr(d_dst), ptr(d_te), E, 8,
                                          pumplib.PUMP_BVP_PRECISION, ptr(d_disc), stream(torch)))
    d_fe = empty(torch, E, torch.uint8)
    pumplib.check(L.pump_free_edges(ptr(d_obs), obs.shape[0], ptr(d_disc), E, 8, ptr(d_fe),
                                    stream(torch)))
    torch.cuda.synchronize()
    return [host(d_c, n), host(d_t, n), np.float32(rn.value), host(d_src, E), host(d_dst, E),
            host(d_ce, E), host(d_te, E), host(d_go, N + 1), host(d_disc, E * 54), host(d_fe, E)]


def roadmap_one_call(torch, pumplib, ctx, N):
    """pump_roadmap (pair BVPs, rn and edges in one call): the first eight
    outputs of roadmap_outputs."""
    from pump_gb300 import workloads
    from oracle.pyoracle import halton_samples
    L = pumplib.load()
    s = halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    d_s = dev(torch, s)
    n = N * (N - 1)
    k = int(np.float32(n) * np.float32(0.05))
    d_c, d_t = empty(torch, n, torch.float32), empty(torch, n, torch.float32)
    d_src, d_dst = empty(torch, k, torch.int32), empty(torch, k, torch.int32)
    d_ce, d_te = empty(torch, k, torch.float32), empty(torch, k, torch.float32)
    d_go = empty(torch, N + 1, torch.int32)
    rn, E = C.c_float(0), C.c_longlong(0)
    pumplib.check(L.pump_roadmap(ctx.handle, ptr(d_s), N, 5.0, pumplib.PUMP_BVP_PRECISION, k, k,
                                 ptr(d_c), ptr(d_t), ptr(d_src), ptr(d_dst), ptr(d_ce), ptr(d_te),
                                 ptr(d_go), C.byref(rn), C.byref(E), None, stream(torch)))
    E = E.value
    return [host(d_c, n), host(d_t, n), np.float32(rn.value), host(d_src, E), host(d_dst, E),
            host(d_ce, E), host(d_te, E), host(d_go, N + 1)]


def test_tuned_shapes_compute_the_defaults(gpu, pumplib):
    torch, ctx = gpu
    from pump_gb300 import workloads
    L = pumplib.load()
    obs = workloads.indoor(1002).astype(np.float32)
    N = 1500
    L.pump_tune_enable(0)
    try:
        ref = roadmap_outputs(torch, pumplib, ctx, N, obs)
        ref_one = roadmap_one_call(torch, pumplib, ctx, N)
    finally:
        L.pump_tune_enable(1)
    L.pump_tune_reset()
    first = roadmap_outputs(torch, pumplib, ctx, N, obs)   # tunes every class
    again = roadmap_outputs(torch, pumplib, ctx, N, obs)   # reuses the records
    one = roadmap_one_call(torch, pumplib, ctx, N)  # the pair kernel writing the superset
    one_again = roadmap_one_call(torch, pumplib, ctx, N)
    # the separate calls (defaults, tuning, tuned) and the one call (defaults,
    # tuning, tuned) all give the same bytes
    outs = [first, again, ref_one, one, one_again]
    for q, a in enumerate(ref):
        a = np.atleast_1d(a)
        for o in outs:
            if q < len(o):
                b = np.atleast_1d(o[q])
                assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), q
    size = L.pump_tune_report(None, 0)
    buf = C.create_string_buffer(size + 1)
    L.pump_tune_report(buf, size + 1)
    text = buf.value.decode()
    # the edge lists come from one-pass compactions (no tuned grid) unless
    # the one-read rn pass falls back, which it does not here
    for name in ("bvp_pairs_precision", "discretize", "free_edges", "compact_rn"):
        assert name in text, text
    assert len(text.strip().splitlines()) == 4, text
