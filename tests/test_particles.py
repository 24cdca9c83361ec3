"""The particle stream that replaces the reference's missing tables
(hardCoded.cuh:12-19): deterministic series math, Philox, and the stated
closed-loop model (CPU, oracle side; the GPU test checks the kernel against
the same oracle bit for bit)."""
import ctypes as C
import math

import numpy as np
import pytest


def test_det_log_accuracy(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.random(20000), [2.0 ** -32, 0.5, 1.0, 0.7071067811865476, 1e-300]])
    for x in xs:
        if x <= 0:
            continue
        got, ref = L.orc_det_log(float(x)), math.log(float(x))
        assert abs(got - ref) <= 4 * math.ulp(ref) + 1e-300


def test_det_sincos_accuracy(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(2)
    s, c = C.c_double(), C.c_double()
    for u in np.concatenate([rng.random(20000), [0.0, 0.25, 0.5, 0.75, 1 - 2 ** -33]]):
        L.orc_det_sincos_2pi(float(u), C.byref(s), C.byref(c))
        # the reference value itself carries the rounding of 2*pi*u (up to ~1e-15)
        assert abs(s.value - math.sin(2 * math.pi * u)) < 2e-15
        assert abs(c.value - math.cos(2 * math.pi * u)) < 2e-15


def test_philox_known_answer(oracle):
    """Philox4x32-10 known-answer vectors of the Random123 distribution (kat_vectors)."""
    L = oracle.lib()
    out = (C.c_uint32 * 4)()
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, expect in cases:
        L.orc_philox4x32_10((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), out)
        assert tuple(out) == expect


def test_table_statistics_match_model_covariance(oracle):
    P, T = 2048, 200
    tm, pm = oracle.particle_tables(oracle.DEFAULT_SEED, P, T)
    assert np.array_equal(tm.transpose(1, 0, 2), pm)
    assert np.all(tm[0] == 0)
    cov = oracle.particle_cov(T)
    var_model = cov[100:, 0].mean()
    var_emp = tm[100:].astype(np.float64).var()
    assert var_emp == pytest.approx(var_model, rel=0.05)
    assert abs(tm[100:].mean()) < 0.01 * math.sqrt(var_model) * 10
    assert math.sqrt(var_model) == pytest.approx(0.0693, rel=0.01)
