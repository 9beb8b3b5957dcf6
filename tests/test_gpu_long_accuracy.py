"""The batched FP32 form over the full length of the batched scattering configuration.

The configuration is 4,000 RK4 steps at dt = 2.4835e-3 (the reference 3D estimator at cfl = 1
on its 24^3-hex mesh), T = 9.93. This test runs the same steps, dt, order (p = 4), boundaries
(first-order SMA outside, PEC scatterer), TF/SF box and 64 Gaussian plane waves on the 12^3-hex
sub-mesh, through the stage kernel the benchmark times (tensor cores, 3xTF32) with the FP64
defect correction at the benchmark's refresh period, against the plain FP64 form for the first
four incidences.

Bar: relative L2 <= 1e-5 per compared incidence at every checkpoint (250, 1,000, 2,000 and
4,000 steps).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg

pytestmark = pytest.mark.gpu
DT = 2.483457175495148e-3
CHECKPOINTS = (250, 1000, 2000, 4000)
DEFECT_EVERY = 100
B, B64 = 64, 4


def waves(n, seed=20261203, spread=0.1, mean=-0.5):
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n):
        k = rng.standard_normal(3); k /= np.linalg.norm(k)
        g = rng.standard_normal(3); pol = g - g.dot(k) * k; pol /= np.linalg.norm(pol)
        out.append(dict(propagation=k, polarization=pol, spread=spread, mean=mean, batch=b))
    return out


def test_tensor_core_form_with_defect_correction_4000_steps(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((12, 12, 12), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((5, 5, 5), (7, 7, 7)),
                    tfsf=((2, 2, 2), (10, 10, 10)), outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)
    op64 = dg.Operator(m, order=4, batch=B64)
    op64.set_planewaves(waves(B64))
    op32 = dg.Operator(m, order=4, precision=dg.FP32_3XTF32, batch=B)
    op32.set_planewaves(waves(B))
    op32.set_contraction(0)
    assert op32.uses_tensor_cores
    op32.set_defect_correction(DEFECT_EVERY)
    x64 = torch.zeros(op64.state_len, dtype=torch.float64, device="cuda")
    x32 = torch.zeros(op32.state_len, dtype=torch.float64, device="cuda")
    w = op32.new_work()
    op32.pack(x32, w)
    L = op64.state_len // B64
    n, t = 0, 0.0
    errs = {}
    for c in CHECKPOINTS:
        op64.step(x64, t, DT, c - n)
        op32.step(w, t, DT, c - n)
        t += (c - n) * DT
        n = c
        op32.unpack(w, x32)
        torch.cuda.synchronize()
        op32.check()
        a, r = x32.cpu().numpy(), x64.cpu().numpy()
        errs[c] = max(float(np.linalg.norm(a[b * L:(b + 1) * L] - r[b * L:(b + 1) * L]) /
                            np.linalg.norm(r[b * L:(b + 1) * L])) for b in range(B64))
    assert op32.defect_refreshes == CHECKPOINTS[-1] // DEFECT_EVERY
    assert all(e <= 1e-5 for e in errs.values()), errs
