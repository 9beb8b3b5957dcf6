"""Stage-kernel autotuner of the batched FP32 form (dgtd_op_autotune).

Bar: every candidate evaluates the same operator, so after tuning a Mult agrees with
the oracle to FP32 rounding (relative L2 <= 2e-6), whichever kernel was kept; the
choice is cached per (order, padded batch, element count).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order,B", [(3, 64), (5, 32)])
def test_autotune_keeps_a_correct_kernel(torch_cuda, order, B):
    torch = torch_cuda
    m = dg.box_mesh((3, 3, 3), outer_bc=dg.BC_PMC)
    op = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    x = np.random.default_rng(order).standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); y = op.new_work()
    op.pack(xd, w)
    r = op.autotune(w)
    assert r["choice"] in (0, 1, 2, 3)
    times = r["ms_per_launch"]
    assert len(times) == (4 if B % 64 == 0 and order <= 4 else 3)
    assert times[r["kernel"]] == min(times.values())
    assert op.uses_tensor_cores == (r["choice"] == 0)
    op.mult(w, y, 0.0)
    yd = torch.zeros_like(xd)
    op.unpack(y, yd)
    torch.cuda.synchronize()
    orc = po.Oracle.from_mesh(m, order)
    L = op.state_len // B
    xr = x.astype(np.float32).astype(np.float64)
    got = yd.cpu().numpy()
    for b in (0, B - 1):
        assert rel_l2(got[b * L:(b + 1) * L], orc.mult(xr[b * L:(b + 1) * L], 0.0)) < 2e-6
    # a second operator of the same shape reuses the cached choice without timing
    op2 = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    w2 = op2.new_work()
    r2 = op2.autotune(w2)
    assert r2["choice"] == r["choice"] and r2["ms_per_launch"] == {}
