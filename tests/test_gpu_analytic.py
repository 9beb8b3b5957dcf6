"""Every precision form against the analytic TE110 cavity mode and against the FP64 form.

The 3D PEC cubic resonator (unit cube, 8^3 hexes x 6 tets, p = 3, dt = 1e-3, 2,000 RK4 steps to
T = 2; reference fixtures: Solver3DTest / the analytic TE110 mode, Ez = sin(pi x) sin(pi y)
cos(w t), w = pi sqrt(2)). Bars: each FP32 form (batched with 64 incidences on the tensor cores
and on SIMT, single instance on the tensor cores and on SIMT) is within 1e-5 relative L2 of the FP64 form, and its error against
the analytic mode is the FP64 form's discretisation error to within 1e-5 (so the FP32 arithmetic
adds nothing visible to it).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
W = np.pi * np.sqrt(2.0)
DT, STEPS = 1e-3, 2000


def te110(xyz, t):
    x, y = xyz[0], xyz[1]
    z = np.zeros_like(x)
    return np.concatenate([z, z, np.sin(np.pi * x) * np.sin(np.pi * y) * np.cos(W * t),
                           -(np.pi / W) * np.sin(np.pi * x) * np.cos(np.pi * y) * np.sin(W * t),
                           (np.pi / W) * np.cos(np.pi * x) * np.sin(np.pi * y) * np.sin(W * t), z])


@pytest.fixture(scope="module")
def fp64_run(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((8, 8, 8))
    op = dg.Operator(m, order=3)
    xyz = op.node_coords()
    xd = torch.from_numpy(te110(xyz, 0.0)).cuda()
    op.step(xd, 0.0, DT, STEPS)
    torch.cuda.synchronize()
    x = xd.cpu().numpy()
    return m, xyz, x, rel_l2(x, te110(xyz, STEPS * DT))


FORMS = [("batched", 0), ("batched", 1), ("single", 0), ("single", 1)]


@pytest.mark.parametrize("form,contraction", FORMS)
def test_fp32_forms_vs_analytic_mode(torch_cuda, fp64_run, form, contraction):
    torch = torch_cuda
    m, xyz, x64, err64 = fp64_run
    B = 64 if form == "batched" else 1
    op = dg.Operator(m, order=3, precision=dg.FP32_3XTF32 if form == "batched" else dg.FP32, batch=B)
    op.set_contraction(contraction)
    assert op.uses_tensor_cores == (contraction == 0)
    x0 = np.tile(te110(xyz, 0.0), B)
    ref = torch.from_numpy(x0).cuda()
    w = op.new_work()
    op.pack(ref, w)
    op.step(w, 0.0, DT, STEPS)
    op.unpack(w, ref)
    torch.cuda.synchronize()
    op.check()
    got = ref.cpu().numpy()
    L = got.size // B
    exact = te110(xyz, STEPS * DT)
    for b in (0, B - 1):
        xb = got[b * L:(b + 1) * L]
        assert rel_l2(xb, x64) <= 1e-5
        assert abs(rel_l2(xb, exact) - err64) <= 1e-5
