"""TF/SF skip test (reference GlobalEvolution.cpp:587-598: the source term of a stage is
skipped while the sum over the TF/SF-submesh nodes of ||0.5 pw||^2 is below 1e-16).

For one incidence driven by one unmodulated Gaussian wave the operator decides the test
on the host from bounds (nearest node to the pulse centre) and runs the device reduction
only near the threshold; with two incidences it always runs the split device reduction.
Both must give bit-identical states, through both forms that use them, and the run must
match the oracle (which evaluates the sum exactly at every stage).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _mesh():
    return dg.box_mesh((5, 5, 5), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((2,) * 3, (3,) * 3),
                       tfsf=((1,) * 3, (4,) * 3), outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)


def _wave(batch, mean=-2.0):
    k = np.array([0.3, -0.5, 0.8]); k /= np.linalg.norm(k)
    g = np.array([1.0, 0.2, -0.1]); pol = g - g.dot(k) * k
    return dict(propagation=k, polarization=pol, spread=0.12, mean=mean, batch=batch)


@pytest.mark.parametrize("precision", [dg.FP64, dg.FP32])
def test_host_decided_skip_matches_device_test(torch_cuda, precision):
    torch = torch_cuda
    m = _mesh()
    order = 3
    one = dg.Operator(m, order=order, precision=precision, batch=1)
    two = dg.Operator(m, order=order, precision=precision, batch=2)
    one.set_planewaves([_wave(0)])
    two.set_planewaves([_wave(0), _wave(1)])
    dt = one.estimate_dt(1.0)
    # 450 steps: the pulse starts far outside the TF/SF box (skipped), crosses it (applied)
    # and leaves it again (skipped), so every branch of the host bound is taken
    n = 450

    def run(op):
        w = op.new_work()
        op.step(w, 0.0, dt, n)
        out = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
        op.unpack(w, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    a = run(one)
    b = run(two)
    L = one.state_len
    assert np.linalg.norm(a) > 1e-3
    assert np.array_equal(a, b[:L])
    assert np.array_equal(a, b[L:])


def test_host_decided_skip_matches_oracle(torch_cuda):
    torch = torch_cuda
    m = _mesh()
    order = 2
    op = dg.Operator(m, order=order, batch=1)
    w = _wave(0)
    op.set_planewaves([w])
    dt = op.estimate_dt(1.0)
    n = 120
    x = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    op.step(x, 0.0, dt, n)
    torch.cuda.synchronize()
    orc = po.Oracle.from_mesh(m, order)
    orc.set_planewaves([w])
    ref = orc.step(np.zeros(op.state_len), 0.0, dt, n)
    assert np.linalg.norm(ref) > 1e-3
    assert rel_l2(x.cpu().numpy(), ref) <= 1e-12
