"""FP64 defect correction of the batched FP32 form (dgtd_op_set_defect_correction).

The drift it removes: a field the FP64 operator keeps (nearly) static has a right-hand side
made of large terms that cancel; in FP32 their rounding repeats identically every step, so
the FP32 state drifts linearly in time. The test field is E = grad(phi),
phi = sin(pi x) sin(pi y) sin(pi z), H = 0 in a PEC unit cube: curl E = 0 and E is normal to
every wall, so the continuous field is static and the FP64 discrete field moves only by its
interpolation error.

Bars: after 400 steps the corrected FP32 state is at least 4 x closer to the FP64 state than
the uncorrected one, on both contraction paths, and within 2e-7 relative L2; the refresh
schedule is the documented one (first step, every `every` steps, after a change of state
buffer or a new call of the setter, not after pack); Mult is unchanged by the correction.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
B = 64
STEPS = 400


def grad_phi_state(xyz):
    x, y, z = xyz
    pi = np.pi
    ex = pi * np.cos(pi * x) * np.sin(pi * y) * np.sin(pi * z)
    ey = pi * np.sin(pi * x) * np.cos(pi * y) * np.sin(pi * z)
    ez = pi * np.sin(pi * x) * np.sin(pi * y) * np.cos(pi * z)
    zero = np.zeros_like(x)
    return np.concatenate([ex, ey, ez, zero, zero, zero])


@pytest.fixture(scope="module")
def static_case(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((4, 4, 4), lo=(0, 0, 0), hi=(1, 1, 1), outer_bc=dg.BC_PEC)
    op64 = dg.Operator(m, order=4, batch=1)
    x1 = grad_phi_state(op64.node_coords())
    dt = op64.estimate_dt(1.0)
    x64 = torch.from_numpy(x1.copy()).cuda()
    op64.step(x64, 0.0, dt, STEPS)
    torch.cuda.synchronize()
    return m, x1, dt, x64.cpu().numpy()


def run32(torch, m, x1, dt, contraction, every, steps=STEPS, chunks=1):
    op = dg.Operator(m, order=4, precision=dg.FP32_3XTF32, batch=B)
    op.set_contraction(contraction)
    op.set_defect_correction(every)
    w = op.new_work()
    op.pack(torch.from_numpy(np.tile(x1, B)).cuda(), w)
    t = 0.0
    per = steps // chunks
    for _ in range(chunks):
        op.step(w, t, dt, per)
        t += per * dt
    out = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    op.unpack(w, out)
    torch.cuda.synchronize()
    op.check()
    o = out.cpu().numpy()
    n = x1.size
    # every incidence carries the same state: all must agree with incidence 0 exactly
    assert np.array_equal(o[:n], o[(B - 1) * n:])
    return op, o[:n]


@pytest.mark.parametrize("contraction", [0, 1])
def test_defect_correction_removes_static_drift(torch_cuda, static_case, contraction):
    torch = torch_cuda
    m, x1, dt, ref = static_case
    _, plain = run32(torch, m, x1, dt, contraction, 0)
    op, corr = run32(torch, m, x1, dt, contraction, 100)
    e_plain, e_corr = rel_l2(plain, ref), rel_l2(corr, ref)
    assert op.defect_refreshes == STEPS // 100
    assert e_corr <= 2e-7, (e_plain, e_corr)
    assert e_corr * 4 <= e_plain, (e_plain, e_corr)


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
    m = dg.box_mesh((2, 2, 2), outer_bc=dg.BC_PEC)
    with pytest.raises(dg.DgtdError, match="batched FP32 form"):
        dg.Operator(m, order=2).set_defect_correction(10)
    with pytest.raises(dg.DgtdError, match="batched FP32 form"):
        dg.Operator(m, order=2, precision=dg.FP32).set_defect_correction(10)
    with pytest.raises(dg.DgtdError, match=">= 0"):
        dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=64).set_defect_correction(-1)
