"""The allocation-free frontier compaction (pump_frontier_compact_noalloc).

Some callers cannot allocate device memory while they plan -- a real-time
control loop that reserved everything at start-up, or a framework that owns
the GPU memory budget -- so this entry point keeps its scratch in a fixed
array owned by the library.  It must give exactly what the allocating entry
point gives, call after call (the array keeps the previous call's contents),
and refuse inputs larger than its array.  This file is collected last so a
failure here does not hide any other test's result."""
import ctypes as C

import numpy as np
import pytest

from helpers import dev, empty, host, ptr, stream


def test_noalloc_rejects_oversize_on_host(pumplib):
    L = pumplib.load()
    st = L.pump_frontier_compact_noalloc(None, 33_554_433, None, None, None)
    # no device buffers are touched: the size check comes first
    assert st in (pumplib.PUMP_ERR_BAD_INPUT, pumplib.PUMP_ERR_CAPACITY)
    st = L.pump_frontier_compact_noalloc(C.c_void_p(16), 33_554_433, C.c_void_p(16), C.c_void_p(16), None)
    assert st == pumplib.PUMP_ERR_CAPACITY
    assert b"33554432" in L.pump_last_error()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice(gpu, pumplib):
    torch, ctx = gpu
    L = pumplib.load()
    # two different inputs in a row: the second call must not see the first's state
    for N, density, seed in [(1_000_003, 0.3, 1), (300_000, 0.9, 2), (4096 * 8192, 0.01, 3)]:
        rng = np.random.default_rng(seed)
        flags = (rng.random(N) < density).astype(np.uint8)
        d_f = dev(torch, flags)
        d_a1, d_a2 = empty(torch, N, torch.int32), empty(torch, N, torch.int32)
        d_n1, d_n2 = empty(torch, 1, torch.int32), empty(torch, 1, torch.int32)
        pumplib.check(L.pump_frontier_compact(ctx.handle, ptr(d_f), N, ptr(d_a1), ptr(d_n1), stream(torch)))
        pumplib.check(L.pump_frontier_compact_noalloc(ptr(d_f), N, ptr(d_a2), ptr(d_n2), stream(torch)))
        n1, n2 = int(host(d_n1)[0]), int(host(d_n2)[0])
        assert n1 == n2 == int(flags.sum())
        assert np.array_equal(host(d_a1, n1), host(d_a2, n2))
        # and again on the same input, with the outputs cleared so that a call
        # that wrote the count but not the indices cannot pass
        d_n2.fill_(-1)
        d_a2.fill_(-1)
        pumplib.check(L.pump_frontier_compact_noalloc(ptr(d_f), N, ptr(d_a2), ptr(d_n2), stream(torch)))
        assert int(host(d_n2)[0]) == n1 and np.array_equal(host(d_a1, n1), host(d_a2, n1))


@pytest.mark.gpu
def test_noalloc_empty_and_all_set(gpu, pumplib):
    """N = 0 writes a zero count (after a call that left a non-zero count in
    the shared array); a frontier with every flag set lists 0 .. N-1."""
    torch, ctx = gpu
    L = pumplib.load()
    N = 70_001
    d_f = dev(torch, np.ones(N, np.uint8))
    d_a, d_n = empty(torch, N, torch.int32), empty(torch, 1, torch.int32)
    d_a.fill_(-1)
    pumplib.check(L.pump_frontier_compact_noalloc(ptr(d_f), N, ptr(d_a), ptr(d_n), stream(torch)))
    assert int(host(d_n)[0]) == N
    assert np.array_equal(host(d_a, N), np.arange(N, dtype=np.int32))
    d_n.fill_(-1)
    pumplib.check(L.pump_frontier_compact_noalloc(ptr(d_f), 0, ptr(d_a), ptr(d_n), stream(torch)))
    assert int(host(d_n)[0]) == 0
