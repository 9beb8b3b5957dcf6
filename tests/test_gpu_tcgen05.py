"""Tensor-core (tcgen05 kind::tf32) building blocks: descriptors, TMEM accumulation, 3xTF32."""
import numpy as np
import pytest

import dgtd_gb300 as dg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [8, 64, 96])
def test_tc_selftest_3xtf32(torch_cuda, k):
    rng = np.random.default_rng(k)
    a = rng.standard_normal((128, k)).astype(np.float32)
    b = rng.standard_normal((48, k)).astype(np.float32)
    d, status = dg.tc_selftest(a, b)
    assert status == 0
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    err = np.abs(d - ref).max() / np.abs(ref).max()
    # 3xTF32 recovers FP32-level accuracy (plain TF32 would be ~1e-3)
    assert err < 2e-6, err
