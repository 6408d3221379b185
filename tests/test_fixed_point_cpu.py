"""The packed fixed-point terms of the mixed forms' cluster sums (up to 32
features), checked on the host against exact arithmetic.

The library's own packing function (the host copy of the device code, through
kmc_debug_pack_fixed) must represent every float value v exactly as the
integer v 2^shift when that integer fits the 30-bit exponent window, flag the
rest, and never produce a term of 2^55 or more (the sums' bound relies on it).
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest


def _lib():
    from kmeans_dpcpp_gb300 import capi

    return capi, capi.lib()


def _unpack(p):
    if p in (0, 1):
        return 0
    ms = p >> 6          # arithmetic shift of a Python int: the signed mantissa
    sh = (p >> 1) & 31
    return ms * (1 << sh)


@pytest.mark.parametrize("shift", [-60, 0, 17, 42, 61, 100])
def test_packed_terms_are_exact_or_flagged(shift):
    capi, L = _lib()
    rng = np.random.default_rng(shift + 100)
    bits = rng.integers(0, 2 ** 32, 20_000, dtype=np.uint64).astype(np.uint32)
    # plus values around the scale's resolution and its upper end
    edge = np.array([2.0 ** (23 - shift), 2.0 ** (22 - shift), 2.0 ** (53 - shift),
                     2.0 ** (54 - shift), 0.0, -0.0], dtype=np.float64)
    vals = np.concatenate([bits.view(np.float32),
                           np.clip(edge, -3e38, 3e38).astype(np.float32)])
    out = ctypes.c_int()
    for v in vals:
        capi.check(L.kmc_debug_pack_fixed(ctypes.c_float(float(v)), shift, ctypes.byref(out)))
        p = out.value
        if p == 1:
            # flagged: not a zero, and not representable in the window
            assert v != 0
            if np.isfinite(v):
                e = (int(np.float32(v).view(np.uint32)) >> 23) & 0xFF
                assert not (0 <= e - 150 + shift <= 30) or e == 0
            continue
        if v == 0:
            assert p == 0
            continue
        q = _unpack(p)
        assert Fraction(float(v)) * Fraction(2) ** shift == q
        assert abs(q) < 2 ** 55


def test_pack_rejects_shifts_outside_the_window():
    capi, L = _lib()
    out = ctypes.c_int()
    assert L.kmc_debug_pack_fixed(ctypes.c_float(1.0), 101, ctypes.byref(out)) == 1
    assert L.kmc_debug_pack_fixed(ctypes.c_float(1.0), -75, ctypes.byref(out)) == 1


def test_high_low_totals_reassemble_the_exact_sum_in_any_order():
    """The integer totals add each term q as (q >> 32) into a high word and
    (q mod 2^32) into a low word (64-bit wrapping adds, as the device's
    atomics); high 2^32 + low is the exact sum whatever the order, so the one
    rounding to float64 gives the same bits for every order."""
    capi, L = _lib()
    rng = np.random.default_rng(7)
    shift = 40
    vals = (rng.standard_normal(20_000) * 7.0).astype(np.float32)
    vals[:50] = 0.0
    out = ctypes.c_int()
    qs = []
    for v in vals:
        capi.check(L.kmc_debug_pack_fixed(ctypes.c_float(float(v)), shift, ctypes.byref(out)))
        assert out.value != 1
        qs.append(_unpack(out.value))
    exact = sum(Fraction(float(v)) for v in vals) * Fraction(2) ** shift
    assert exact == sum(qs)
    M64 = (1 << 64) - 1
    results = set()
    for perm in range(4):
        order = rng.permutation(len(qs))
        hi = lo = 0
        for i in order:
            q = qs[i]
            hi = (hi + (q >> 32)) & M64
            lo = (lo + (q & 0xFFFFFFFF)) & M64
        if hi >= 1 << 63:
            hi -= 1 << 64          # the high word is a signed 64-bit integer
        assert hi * 2 ** 32 + lo == sum(qs)
        results.add((float(hi) * 4294967296.0 + float(lo)) * 2.0 ** -shift)
    assert len(results) == 1
