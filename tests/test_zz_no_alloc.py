"""dgtd_op_step_noalloc against dgtd_op_step, through the C ABI.

The no-allocation entry point runs the same fused stage kernels as dgtd_op_step
with its RK registers in the library's fixed device array instead of
cudaMalloc'd scratch. Bar: relative L2 <= 1e-12 against dgtd_op_step on the same
inputs (the arithmetic is the same; the tolerance only absorbs nothing but
ordering noise), on two calls in a row so that contents left in the shared
array by one call cannot leak into the next.

This file is collected last so that it also runs after every other GPU test in
the same process; it must pass alone in a fresh process as well.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12
WAVE = dict(propagation=[1.0, 0.3, -0.2], polarization=[0.1, 0.0, 1.0], spread=0.1, mean=-0.4)


def _scatterer_op(order=3, batch=1):
    m = dg.box_mesh((4, 4, 4), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1, 1, 1), (3, 3, 3)),
                    hole=((2, 2, 2), (3, 3, 3)), outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)
    op = dg.Operator(m, order=order, batch=batch)
    op.set_planewaves([dict(WAVE, batch=b) for b in range(batch)])
    return op


@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_noalloc_matches_step_two_calls(torch_cuda, integrator):
    torch = torch_cuda
    op = _scatterer_op(batch=2)
    rng = np.random.default_rng(7)
    x0 = rng.standard_normal(op.state_len) * 1e-3
    a = torch.from_numpy(x0.copy()).cuda()
    b = torch.from_numpy(x0.copy()).cuda()
    dt = op.estimate_dt(1.0)
    t = 0.0
    for _ in range(2):
        op.step(a, t, dt, 3, integrator)
        op.step_noalloc(b, t, dt, 3, integrator)
        torch.cuda.synchronize()
        t += 3 * dt
        ra, rb = a.cpu().numpy(), b.cpu().numpy()
        assert np.linalg.norm(ra) > 0
        assert rel_l2(rb, ra) <= TOL


def test_noalloc_shared_by_operators(torch_cuda):
    """Two operators of different sizes take turns on the one scratch array."""
    torch = torch_cuda
    op1 = _scatterer_op(order=2)
    op2 = _scatterer_op(order=4)
    rng = np.random.default_rng(11)
    x1 = rng.standard_normal(op1.state_len)
    x2 = rng.standard_normal(op2.state_len)
    ref1 = torch.from_numpy(x1.copy()).cuda(); got1 = torch.from_numpy(x1.copy()).cuda()
    ref2 = torch.from_numpy(x2.copy()).cuda(); got2 = torch.from_numpy(x2.copy()).cuda()
    dt1, dt2 = op1.estimate_dt(0.5), op2.estimate_dt(0.5)
    for k in range(2):
        op1.step(ref1, k * 2 * dt1, dt1, 2, dg.LSERK4)
        op2.step(ref2, k * 2 * dt2, dt2, 2, dg.RK4)
        op1.step_noalloc(got1, k * 2 * dt1, dt1, 2, dg.LSERK4)
        op2.step_noalloc(got2, k * 2 * dt2, dt2, 2, dg.RK4)
        torch.cuda.synchronize()
        assert rel_l2(got1.cpu().numpy(), ref1.cpu().numpy()) <= TOL
        assert rel_l2(got2.cpu().numpy(), ref2.cpu().numpy()) <= TOL


def test_noalloc_samples_probes_like_step(torch_cuda):
    """With probes installed, the no-allocation call samples them on the same cadence as
    dgtd_op_step: the recorded series and DFT sums agree to the parity bar, also when the
    two calls are mixed on one operator."""
    torch = torch_cuda
    pts = np.array([[0.1, -0.2, 0.3], [-0.5, 0.4, -0.6]])
    freqs = np.array([0.7, 1.9])
    ops = [_scatterer_op(), _scatterer_op(), _scatterer_op()]
    for op in ops:
        op.set_probes(points=pts, freqs=freqs, every=2, max_records=16)
    rng = np.random.default_rng(5)
    x0 = rng.standard_normal(ops[0].state_len) * 1e-3
    xs = [torch.from_numpy(x0.copy()).cuda() for _ in ops]
    dt = ops[0].estimate_dt(1.0)
    for k in range(2):
        t = 5 * k * dt
        ops[0].step(xs[0], t, dt, 5)
        ops[1].step_noalloc(xs[1], t, dt, 5)
        (ops[2].step if k == 0 else ops[2].step_noalloc)(xs[2], t, dt, 5)
    torch.cuda.synchronize()
    want = ops[0].probe_read()
    assert want["n_samples"] == 5
    for op in ops[1:]:
        got = op.probe_read()
        assert got["n_samples"] == want["n_samples"]
        assert np.array_equal(got["times"], want["times"])
        assert rel_l2(got["series"], want["series"]) <= TOL
        assert np.abs(got["points"] - want["points"]).max() <= TOL * np.abs(want["points"]).max()


def test_noalloc_rejects_oversize_state(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((8, 8, 8), outer_bc=dg.BC_PEC)
    op = dg.Operator(m, order=3, batch=18)
    assert op.state_len > dg.noalloc_max_state()
    x = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DgtdError, match="scratch limit"):
        op.step_noalloc(x, 0.0, 1e-3, 1)


def test_noalloc_rejects_batched_form(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2), outer_bc=dg.BC_PEC)
    op = dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=64)
    w = op.new_work("cuda")
    with pytest.raises(dg.DgtdError, match="FP64 form only"):
        op.step_noalloc(w, 0.0, 1e-3, 1)
