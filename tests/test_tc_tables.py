"""Host-side tables of the element contraction on the tensor cores (no GPU needed).

The operator blocks of the even/odd form are written, row by row, as signed base-256 digits
(|d| <= 255, exact in bf16 and fp16) of the 56-bit truncation of each entry scaled by the row's largest
binary exponent.  These tests rebuild every entry from its digits with exact rational arithmetic.
"""
from fractions import Fraction

import numpy as np
import pytest


def tables(pkg, N):
    lib = pkg.lib()
    dims = np.zeros(4, np.int32)
    assert lib.dg_tc_operator_digits(N, dims.ctypes.data, None, None, None) == 0
    NUe, NUo, NRe, NRo = (int(x) for x in dims)
    S = np.zeros(NRe * NUe + NRo * NUo)
    fexp = np.zeros(64, np.int32)
    dig = np.zeros(2 * 7 * 32 * 32, np.int32)
    assert lib.dg_tc_operator_digits(N, dims.ctypes.data, S.ctypes.data, fexp.ctypes.data, dig.ctypes.data) == 0
    return (NUe, NUo, NRe, NRo), S, fexp.reshape(2, 32), dig.reshape(2, 7, 32, 32)


@pytest.mark.parametrize("N", [3, 4, 5])
def test_digits_rebuild_the_operator(pkg, N):
    (NUe, NUo, NRe, NRo), S, fexp, dig = tables(pkg, N)
    assert np.abs(dig).max() <= 255
    for p, (K, R, base) in enumerate([(NUe, NRe, 0), (NUo, NRo, NRe * NUe)]):
        B = S[base:base + R * K].reshape(R, K)
        assert not dig[p, :, K:, :].any() and not dig[p, :, :, R:].any()  # padding is zero
        for n in range(R):
            F = int(fexp[p, n]) - 1023
            amax = np.abs(B[n]).max()
            assert 2.0 ** F <= amax < 2.0 ** (F + 1)  # the row's largest binary exponent
            for k in range(K):
                d = [int(dig[p, s, k, n]) for s in range(7)]
                assert all(x >= 0 for x in d) or all(x <= 0 for x in d)  # one sign per entry
                m = sum(x * 256 ** (6 - s) for s, x in enumerate(d))
                exact = Fraction(float(B[n, k])) * Fraction(2) ** (55 - F)
                trunc = int(abs(exact)) * (1 if exact >= 0 else -1)  # toward zero
                assert m == trunc, (p, n, k)


@pytest.mark.parametrize("N", [3, 4, 5])
def test_level_sums_stay_exact(pkg, N):
    """Any staged values (digits up to 255) times the operator digits: every level of the
    accumulation (at most 7 digit pairs over the slots of one parity) stays below 2^24, where
    FP32 accumulation is exact."""
    (NUe, NUo, NRe, NRo), _, _, dig = tables(pkg, N)
    for p, K in enumerate([NUe, NUo]):
        worst = 7 * 255 * np.abs(dig[p, :, :K, :]).sum(axis=1).max()
        assert K <= 32 and worst < 2 ** 24


@pytest.mark.parametrize("N", [1, 2, 6])
def test_orders_without_tensor_cores(pkg, N):
    dims = np.zeros(4, np.int32)
    assert pkg.lib().dg_tc_operator_digits(N, dims.ctypes.data, None, None, None) != 0


def _exact_rne(T, sc):
    """T * 2^sc rounded to the nearest double, ties to even (Python's int and Fraction
    conversions round correctly)."""
    if sc >= 0:
        return float(T * 2 ** sc)
    return float(Fraction(T, 2 ** (-sc)))


def test_integer_rounding_matches_exact(pkg):
    """The contraction joins its seven FP32 level sums as integers (th 2^32 + tl) and rounds
    T 2^sc to a double with integer instructions only.  The library's host copy of that code
    (the device runs the same function) against exact rational rounding: random level sums
    anywhere below 2^24, sparse and cancelling ones, and exact ties."""
    import ctypes as C
    lib = pkg.lib()
    rng = np.random.default_rng(20261203)
    out = C.c_double()

    def check(th, tl, sc):
        assert lib.dg_tc_round(int(th), int(tl), int(sc), C.byref(out)) == 0
        want = _exact_rne(int(th) * 2 ** 32 + int(tl), int(sc))
        assert np.float64(out.value).tobytes() == np.float64(want).tobytes(), (th, tl, sc, out.value, want)

    for trial in range(4000):
        mode = trial % 4
        lim = [2 ** 24, 2 ** int(rng.integers(0, 25)), 256, 3][mode]
        lev = [int(x) for x in rng.integers(-lim + 1, lim, 7)]
        for k in range(int(rng.integers(0, 7)) if trial % 3 == 0 else 0):
            lev[k] = 0
        th = lev[0] * 65536 + lev[1] * 256 + lev[2]
        tl = lev[3] * 16777216 + lev[4] * 65536 + lev[5] * 256 + lev[6]
        check(th, tl, int(rng.integers(-1022, 901)))
    # ties: 53 significant bits plus exactly half an ulp, with an even and an odd last bit
    for e in range(54, 73):
        for odd in (0, 1):
            for sign in (1, -1):
                T = sign * ((1 << e) | (odd << (e - 52)) | (1 << (e - 53)))
                th, tl = T >> 32, T - ((T >> 32) << 32)
                check(th, tl, -60)
    # zero and small values
    for th, tl in ((0, 0), (0, 1), (0, -1), (1, 0), (-1, 0), (0, 2 ** 32 - 1)):
        check(th, tl, 0)
    # outside the stated range: refused
    assert lib.dg_tc_round(0, 0, 901, C.byref(out)) != 0
    assert lib.dg_tc_round(2 ** 41, 0, 0, C.byref(out)) != 0
