"""The tensor-core building blocks (tcgen05 TF32 MMA with shared-memory
operands, TMEM accumulator, mbarrier completion, TMEM loads) against a host
product: inputs exactly representable in TF32, so the FP32 result is exact."""
import ctypes as C

import numpy as np
import pytest

import macsimus_gb300 as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(64, 32), (128, 64), (16, 8), (256, 16)])
def test_tf32_product_is_exact_on_representable_inputs(n, k):
    rng = np.random.default_rng(n * 100 + k)
    A = (rng.integers(-64, 65, (128, k)) / 64.0).astype(np.float32)
    B = (rng.integers(-64, 65, (n, k)) / 64.0).astype(np.float32)
    Cm = np.zeros((128, n), np.float32)
    fp = C.POINTER(C.c_float)
    rc = M.library().mg_tc_selftest(A.ctypes.data_as(fp), B.ctypes.data_as(fp),
                                    Cm.ctypes.data_as(fp), n, k)
    assert rc == 0
    assert np.array_equal(Cm, (A.astype(np.float64) @ B.astype(np.float64).T).astype(np.float32))
