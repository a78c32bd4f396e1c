"""Split-precision GEMM (BF16 tensor-core digit products, FP64 recombination) against the FP64 GEMM.

The bound is elementwise relative to (|A||B|)_ij, the natural scale of rounding in a dot
product: with S digit slices the truncation is about 2^(-8S+2) per term.
"""
import ctypes as C

import numpy as np
import pytest

from xtb_gb300 import interface as X

pytestmark = pytest.mark.gpu


def check(M, N, K, slices, seed=1, exp_range=0):
    lib = X.load_library()
    out = np.zeros(6)
    rc = lib.xtbgb_splitGemmCheck(M, N, K, slices, seed, exp_range, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return out


@pytest.mark.parametrize("shape", [(64, 64, 64), (100, 77, 300), (257, 129, 4097), (1000, 1000, 1000),
                                   (128, 3000, 3000)])   # the third and the last split K (few output tiles)
def test_split_gemm_accuracy(shape):
    M, N, K = shape
    out5 = check(M, N, K, 5)
    assert out5[0] < 2.0 ** -37, out5
    out7 = check(M, N, K, 7)
    assert out7[0] < 1e-14, out7


def test_split_gemm_wide_dynamic_range():
    """Entries spread over 2^0 .. 2^-24 within rows.  The digits are fixed-point per row and
    column, so an entry 2^-24 below its row's largest keeps 24 fewer bits: the error stays
    small against the largest products (normwise), while the elementwise bound loosens by the
    spread."""
    out = check(500, 400, 700, 6, exp_range=24)
    assert out[1] < 2.0 ** -40, out
    assert out[0] < 2.0 ** -40, out


def test_split_gemm_is_faster_than_fp64():
    out = check(4096, 4096, 4096, 5)
    assert out[0] < 2.0 ** -37
    assert out[4] > 3.0 * out[5], out     # TFLOP/s split vs FP64
