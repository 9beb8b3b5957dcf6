"""FP64 defect correction of the batched FP32 form (dgtd_op_set_defect_correction).

The drift it removes: a field the FP64 operator keeps static has a right-hand side made of
large terms that cancel; in FP32 their rounding repeats identically every step, so the FP32
state drifts linearly in time. The test field: E = grad(g), g a Gaussian bump (width 0.3) at the
centre of the box [-1,1]^3 with first-order absorbing (SMA) walls, H = 0, stepped 1,000 times by
the FP64 form first so that everything but its static part has left through the walls (the
FP64 state then moves by about 1e-11 relative over 400 steps).

Bars: over the next 400 steps, after the correction's first refresh that finds the state unmoved
(step 100), the corrected FP32 state drifts at most half as fast as the uncorrected one, on both
contraction paths (measured: under a quarter on the tensor cores, 0.35 in FP32 SIMT); the
refresh schedule is the documented one (first step, every `every`
steps, after a change of state buffer or a new call of the setter, not after pack); Mult is
unchanged by the correction; LSERK4 and the other forms are rejected.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
B = 64


@pytest.fixture(scope="module")
def static_case(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((4, 4, 4), lo=(-1, -1, -1), hi=(1, 1, 1), outer_bc=dg.BC_SMA)
    op64 = dg.Operator(m, order=4, batch=1)
    x, y, z = op64.node_coords()
    s2 = 0.3 ** 2
    g = np.exp(-(x * x + y * y + z * z) / (2 * s2))
    zero = np.zeros_like(x)
    x0 = np.concatenate([-x / s2 * g, -y / s2 * g, -z / s2 * g, zero, zero, zero])
    dt = op64.estimate_dt(1.0)
    xs = torch.from_numpy(x0).cuda()
    op64.step(xs, 0.0, dt, 1000)
    torch.cuda.synchronize()
    start = xs.cpu().numpy()
    refs = {}
    for n in (200, 400):
        op64.step(xs, 0.0, dt, 200)
        torch.cuda.synchronize()
        refs[n] = xs.cpu().numpy()
    assert rel_l2(refs[400], start) < 1e-9          # static under the FP64 operator
    return m, start, dt, refs


def run32(torch, m, x1, dt, contraction, every, refs):
    op = dg.Operator(m, order=4, precision=dg.FP32_3XTF32, batch=B)
    op.set_contraction(contraction)
    op.set_defect_correction(every)
    w = op.new_work()
    op.pack(torch.from_numpy(np.tile(x1, B)).cuda(), w)
    out = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    errs = {}
    n = x1.size
    for k in (200, 400):
        op.step(w, 0.0, dt, 200)
        op.unpack(w, out)
        torch.cuda.synchronize()
        op.check()
        o = out.cpu().numpy()
        # every incidence carries the same state: all must agree with incidence 0 exactly
        assert np.array_equal(o[:n], o[(B - 1) * n:])
        errs[k] = rel_l2(o[:n], refs[k])
    return op, errs


@pytest.mark.parametrize("contraction", [0, 1])
def test_defect_correction_removes_static_drift(torch_cuda, static_case, contraction):
    torch = torch_cuda
    m, x1, dt, refs = static_case
    _, plain = run32(torch, m, x1, dt, contraction, 0, refs)
    op, corr = run32(torch, m, x1, dt, contraction, 100, refs)
    assert op.defect_refreshes == 4
    grow_plain = plain[400] - plain[200]
    grow_corr = corr[400] - corr[200]
    assert grow_plain > 0, plain
    assert grow_corr <= 0.5 * grow_plain, (plain, corr)
    assert corr[400] < plain[400], (plain, corr)


def test_defect_refresh_schedule(torch_cuda, static_case):
    torch = torch_cuda
    m, x1, dt, _ = static_case
    op = dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=B)
    op.set_defect_correction(3)
    w = op.new_work()
    op.pack(torch.zeros(op.state_len, dtype=torch.float64, device="cuda"), w)
    op.step(w, 0.0, dt, 1)
    assert op.defect_refreshes == 1            # first step
    op.step(w, dt, dt, 5)
    assert op.defect_refreshes == 2            # steps 1..2 on the first, a refresh at step 3
    op.step(w, 6 * dt, dt, 1)
    assert op.defect_refreshes == 3            # step 6
    op.pack(torch.zeros(op.state_len, dtype=torch.float64, device="cuda"), w)
    op.step(w, 7 * dt, dt, 1)
    assert op.defect_refreshes == 3            # pack keeps the correction
    w2 = op.new_work()
    op.step(w2, 0.0, dt, 1)
    assert op.defect_refreshes == 4            # another state buffer
    op.set_defect_correction(3)
    op.step(w2, dt, dt, 1)
    assert op.defect_refreshes == 5            # set again: refresh at the next step
    op.set_defect_correction(0)
    op.step(w2, 0.0, dt, 4)
    assert op.defect_refreshes == 5
    torch.cuda.synchronize()
    op.check()


def test_defect_correction_leaves_mult_unchanged(torch_cuda, static_case):
    torch = torch_cuda
    m, x1, dt, _ = static_case
    op = dg.Operator(m, order=4, precision=dg.FP32_3XTF32, batch=B)
    w = op.new_work()
    op.pack(torch.from_numpy(np.tile(x1, B)).cuda(), w)
    y0, y1 = op.new_work(), op.new_work()
    op.mult(w, y0, 0.0)
    op.set_defect_correction(1)
    w2 = op.new_work()
    w2.copy_(w)
    op.step(w2, 0.0, dt, 1)                    # refresh: the correction is now installed
    op.mult(w, y1, 0.0)
    torch.cuda.synchronize()
    assert torch.equal(y0, y1)


def test_defect_correction_rejected_outside_batched_form(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2), outer_bc=dg.BC_PEC)
    op = dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=64)
    op.set_defect_correction(5)
    w = op.new_work()
    with pytest.raises(dg.DgtdError, match="classical RK4"):
        op.step(w, 0.0, 1e-3, 1, dg.LSERK4)
    op.set_defect_correction(0)
    op.step(w, 0.0, 1e-3, 1, dg.LSERK4)
    torch.cuda.synchronize()
    with pytest.raises(dg.DgtdError, match="batched FP32 form"):
        dg.Operator(m, order=2).set_defect_correction(10)
    with pytest.raises(dg.DgtdError, match="batched FP32 form"):
        dg.Operator(m, order=2, precision=dg.FP32).set_defect_correction(10)
    with pytest.raises(dg.DgtdError, match=">= 0"):
        dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=64).set_defect_correction(-1)
