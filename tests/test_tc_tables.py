"""Host-side tables of the element contraction on the tensor cores (no GPU needed).

The operator blocks of the even/odd form are written, row by row, as signed base-256 digits
(|d| <= 255, exact in bf16) of the 56-bit truncation of each entry scaled by the row's largest
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
