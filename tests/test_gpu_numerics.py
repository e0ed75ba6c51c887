"""The mixed path's hand-made numeric primitives against the CUDA operations
they stand for, through game_gpu_numerics (include/game_gb300.h), on 2^20
sampled inputs plus the edge values of each operation.

* to_float (double -> float by integer operations) must give the same bits
  as __double2float_rn on every input: zeros, the float subnormal boundary,
  values that overflow by rounding, exact ties between two floats, NaN and
  infinities included.
* to_double (float -> double by integer operations) must give the same bits
  as (double)f for every float.
* rcp_nr<2> (two Newton steps on rcp.approx.ftz.f64) must be within one ulp
  of IEEE 1.0 / x on normal x with a normal reciprocal (the solvers' domain)
  and equal to it on all but a few in a million inputs (measured on GB300:
  the random inputs all equal; among the edge values x = 1 - 2^-53, whose
  reciprocal lies just above the midpoint of two doubles, is one ulp off);
  rcp_nr<1> must be within 2^-39 of it, relatively.
* The double-float primitives of the column eliminations: the split of a
  double into two floats and its join within 2^-47 relative, the reciprocal
  within 2^-44, product and sum within 2^-45 of the exact results (relative
  to |x y| and |x| + |y|).
"""
import ctypes

import numpy as np
import pytest

from game_archived_gb300 import native

pytestmark = pytest.mark.gpu

N = 1 << 20


def _run(op, x, out_dtype):
    lib = native.gpu()
    x = np.ascontiguousarray(x)
    n = x.size if op < 9 else x.size // 2
    out = np.empty(n, dtype=out_dtype)
    rc = lib.game_gpu_numerics(op, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p), n)
    assert rc == 0, lib.game_gpu_last_error().decode()
    return out


def _doubles(rng, n, lo_exp, hi_exp):
    """doubles with uniformly random significands and exponents in
    [lo_exp, hi_exp), random signs"""
    m = rng.uniform(1.0, 2.0, n)
    e = rng.integers(lo_exp, hi_exp, n)
    s = rng.choice([-1.0, 1.0], n)
    return s * np.ldexp(m, e)


def _float_edges():
    f32 = np.finfo(np.float32)
    vals = [0.0, -0.0, float(f32.tiny), -float(f32.tiny), float(f32.max), -float(f32.max),
            float(f32.smallest_subnormal), np.inf, -np.inf, np.nan]
    return np.array(vals, dtype=np.float64)


def test_to_float_equals_the_conversion_instruction():
    rng = np.random.default_rng(1)
    parts = [_doubles(rng, N, -160, 140), _float_edges()]
    f32 = np.finfo(np.float32)
    # around the smallest normal float and the largest float: values that
    # round up into the normal range or overflow to infinity by rounding
    for edge in (float(f32.tiny), float(f32.max)):
        ulp = np.spacing(np.float32(edge)).astype(np.float64)
        parts.append(edge + ulp * rng.uniform(-2.0, 2.0, 4096))
        parts.append(edge + ulp * np.array([-0.5, 0.5, -0.25, 0.25, 0.5 - 2 ** -30, 0.5 + 2 ** -30]))
    # exact ties between two neighbouring floats: the low 29 bits of the
    # double's fraction are 1 followed by zeros
    f = _doubles(rng, 1 << 16, -120, 120).astype(np.float32).astype(np.float64)
    tie = f + np.spacing(f.astype(np.float32)).astype(np.float64) / 2
    parts += [tie, -tie]
    x = np.concatenate(parts)
    a = _run(3, x, np.float32)
    b = _run(4, x, np.float32)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))[:10]
    # and the instruction is numpy's rounding (round to nearest even)
    with np.errstate(over="ignore"):
        assert np.array_equal(b.view(np.uint32)[~np.isnan(x)], x[~np.isnan(x)].astype(np.float32).view(np.uint32))


def test_to_double_equals_the_conversion_instruction():
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 1 << 32, N, dtype=np.uint64).astype(np.uint32)
    edges = np.array([0, 0x80000000, 1, 0x807fffff, 0x00800000, 0x7f7fffff, 0x7f800000, 0xff800000, 0x7fc00000],
                     dtype=np.uint32)
    x = np.concatenate([bits, edges]).view(np.float32)
    a = _run(5, x, np.float64)
    b = _run(6, x, np.float64)
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan)
    assert np.array_equal(a.view(np.uint64)[~nan], b.view(np.uint64)[~nan])
    assert np.array_equal(b[~nan], x[~nan].astype(np.float64))


def _rcp_domain(rng):
    x = _doubles(rng, N, -1000, 1000)
    return np.concatenate([x, [1.0, -1.0, 2.0 ** -1000, 3.0, 1.0 / 3.0, np.nextafter(1.0, 2.0),
                               np.nextafter(1.0, 0.0)]])


def test_newton_reciprocal_two_steps_within_one_ulp():
    x = _rcp_domain(np.random.default_rng(3))
    a = _run(1, x, np.float64)
    b = _run(2, x, np.float64)
    assert np.array_equal(b, 1.0 / x)
    ulps = np.abs(a.view(np.int64) - b.view(np.int64))
    bad = np.flatnonzero(ulps != 0)
    print(f"rcp_nr<2> vs 1.0 / x: {bad.size} of {x.size} differ, at most {ulps.max()} ulp; "
          f"inputs {x[bad[:5]].tolist()}")
    assert ulps.max() <= 1
    assert bad.size <= 4, (bad.size, x[bad[:5]])


def test_newton_reciprocal_one_step_bound():
    x = _rcp_domain(np.random.default_rng(4))
    a = _run(0, x, np.float64)
    rel = np.abs(a * x - 1.0)
    assert rel.max() <= 2.0 ** -39, rel.max()


def test_double_float_split_and_join():
    rng = np.random.default_rng(5)
    x = np.concatenate([_doubles(rng, N, -100, 100), [0.0, -0.0, 1.0, -1.0, 1.0 + 2.0 ** -52]])
    y = _run(7, x, np.float64)
    assert np.all(np.abs(y - x) <= 2.0 ** -47 * np.abs(x))
    assert np.array_equal(np.signbit(y[x == 0]), np.signbit(x[x == 0]))


def test_double_float_reciprocal():
    rng = np.random.default_rng(6)
    x = _doubles(rng, N, -100, 100)
    y = _run(8, x, np.float64)
    rel = np.abs(y * x - 1.0)
    assert rel.max() <= 2.0 ** -44, rel.max()


def test_double_float_product_and_sum():
    rng = np.random.default_rng(7)
    x = _doubles(rng, N, -40, 40)
    y = _doubles(rng, N, -40, 40)
    # near-cancelling sums as well
    y[: N // 8] = -x[: N // 8] * (1.0 + _doubles(rng, N // 8, -30, -10))
    xy = np.concatenate([x, y])
    p = _run(9, xy, np.float64)
    s = _run(10, xy, np.float64)
    assert np.all(np.abs(p - x * y) <= 2.0 ** -45 * np.abs(x * y))
    assert np.all(np.abs(s - (x + y)) <= 2.0 ** -45 * (np.abs(x) + np.abs(y)))
