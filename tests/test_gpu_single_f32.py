"""Single-instance FP32 form (DGTD_FP32) on the reference layout, for high-order single
solves, with both contraction paths: the tensor-core stage (tcgen05, 3xTF32, 8 elements per
work item; the default) and the plain form's fused stage in FP32 (SIMT).

Bars: one RHS evaluation within FP32 rounding of the oracle (relative L2 <= 2e-6); 200 RK
steps within 1e-5 relative L2 of the FP64 form; the high-order dielectric resonator (p = 6,
random eps_r) likewise.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(7)
WAVE = dict(propagation=[1.0, 0.3, -0.2], polarization=[0.1, 0.0, 1.0], spread=0.2, mean=0.1)


CONTRACTIONS = {"tc": 0, "simt": 1}


@pytest.mark.parametrize("contraction", sorted(CONTRACTIONS))
@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_f32_mult_vs_oracle(torch_cuda, order, contraction):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2), tfsf=((1, 0, 0), (2, 2, 2)), outer_bc=dg.BC_SMA)
    K = m.n_elements
    m.eps = RNG.uniform(1, 4, K); m.mu = RNG.uniform(1, 2, K); m.sigma = RNG.uniform(0, 0.3, K)
    op = dg.Operator(m, order=order, precision=dg.FP32)
    op.set_contraction(CONTRACTIONS[contraction])
    assert op.uses_tensor_cores == (contraction == "tc")
    op.set_planewaves([WAVE])
    orc = po.Oracle.from_mesh(m, order); orc.set_planewaves([WAVE])
    assert op.info["work_word_bytes"] == 4 and op.work_len == op.state_len
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); y = op.new_work()
    op.pack(xd, w)
    op.mult(w, y, 0.3)
    yd = torch.zeros_like(xd)
    op.unpack(y, yd)
    torch.cuda.synchronize()
    xr = x.astype(np.float32).astype(np.float64)
    assert rel_l2(yd.cpu().numpy(), orc.mult(xr, 0.3)) < 2e-6
    op.check()


@pytest.mark.parametrize("order", [2, 4, 6])
def test_f32_tc_mult_many_items_batch_ragged(torch_cuda, order):
    """The tensor-core stage over many work items (more than two per SM, so every CTA cycles
    both buffers many times), two stacked incidences, and an element count that is not a
    multiple of the 8-element work item."""
    torch = torch_cuda
    m = dg.box_mesh((9, 7, 5), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1, 1, 1), (8, 6, 4)), outer_bc=dg.BC_SMA,
                    hole=((4, 3, 2), (5, 4, 3)))
    assert m.n_elements % 8 != 0 and 2 * (m.n_elements // 8) > 2 * 152   # work items over both incidences
    waves = [dict(WAVE, batch=0), dict(WAVE, propagation=[-0.2, 1.0, 0.4], polarization=[1.0, 0.2, 0.0], batch=1)]
    op = dg.Operator(m, order=order, precision=dg.FP32, batch=2)
    assert not op.uses_tensor_cores          # the single-instance default is FP32 SIMT
    op.set_contraction(0)
    assert op.uses_tensor_cores
    op.set_planewaves(waves)
    orc = po.Oracle.from_mesh(m, order)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); y = op.new_work()
    op.pack(xd, w)
    op.mult(w, y, 0.35)
    yd = torch.zeros_like(xd)
    op.unpack(y, yd)
    torch.cuda.synchronize()
    op.check()
    got = yd.cpu().numpy()
    L = op.state_len // 2
    xr = x.astype(np.float32).astype(np.float64)
    for b in range(2):
        orc.set_planewaves([dict(waves[b], batch=0)])
        want = orc.mult(xr[b * L:(b + 1) * L], 0.35, form=po.NODAL)
        assert rel_l2(got[b * L:(b + 1) * L], want) < 2e-6


@pytest.mark.parametrize("contraction", sorted(CONTRACTIONS))
@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_f32_steps_vs_fp64(torch_cuda, integrator, contraction):
    torch = torch_cuda
    m = dg.box_mesh((4, 4, 4), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1,) * 3, (3,) * 3), outer_bc=dg.BC_SMA,
                    hole=((2, 2, 2), (3, 3, 3)))
    w = dict(WAVE, mean=-0.4, spread=0.15)
    o64 = dg.Operator(m, order=3); o64.set_planewaves([w])
    o32 = dg.Operator(m, order=3, precision=dg.FP32); o32.set_planewaves([w])
    o32.set_contraction(CONTRACTIONS[contraction])
    dt = o64.estimate_dt(1.0)
    x64 = torch.zeros(o64.state_len, dtype=torch.float64, device="cuda")
    w32 = o32.new_work()
    o64.step(x64, 0.0, dt, 200, integrator)
    o32.step(w32, 0.0, dt, 200, integrator)
    back = torch.zeros_like(x64)
    o32.unpack(w32, back)
    torch.cuda.synchronize()
    ref = x64.cpu().numpy()
    assert np.linalg.norm(ref) > 1e-3
    assert rel_l2(back.cpu().numpy(), ref) < 1e-5
    # the per-incidence norm agrees too
    assert abs(o32.norm2(w32)[0] / o64.norm2(x64)[0] - 1) < 1e-5


@pytest.mark.parametrize("contraction", sorted(CONTRACTIONS))
def test_f32_high_order_dielectric(torch_cuda, contraction):
    """Order 6, eps_r ~ U[1, 4] per element, PEC walls, smooth random initial E (the
    high-order dielectric workload at small size)."""
    torch = torch_cuda
    rng = np.random.default_rng(20261204)
    m = dg.box_mesh((3, 3, 3))
    m.eps = rng.uniform(1, 4, m.n_elements)
    o64 = dg.Operator(m, order=6)
    o32 = dg.Operator(m, order=6, precision=dg.FP32)
    o32.set_contraction(CONTRACTIONS[contraction])
    xyz = o64.node_coords()
    r2 = np.random.default_rng(20261205)
    E = np.zeros((3, xyz.shape[1]))
    for _ in range(8):
        k = np.pi * r2.integers(1, 4, 3)
        a = r2.standard_normal(3)
        ph = r2.uniform(0, 2 * np.pi)
        E += np.outer(a, np.sin(k @ xyz + ph))
    x0 = np.concatenate([E.ravel(), np.zeros(3 * xyz.shape[1])])
    x64 = torch.from_numpy(x0).cuda()
    w32 = o32.new_work()
    o32.pack(x64, w32)
    o64.step(x64, 0.0, 2e-4, 100)
    o32.step(w32, 0.0, 2e-4, 100)
    back = torch.zeros_like(x64)
    o32.unpack(w32, back)
    torch.cuda.synchronize()
    assert rel_l2(back.cpu().numpy(), x64.cpu().numpy()) < 1e-5


def test_f32_probes_and_noalloc_rejection(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2))
    op = dg.Operator(m, order=3, precision=dg.FP32)
    op.set_probes(points=[[0.3, 0.4, 0.5]], freqs=[0.0], max_records=2)
    xyz = op.node_coords()
    f = 1.0 + 2.0 * xyz[0] - xyz[1] + 0.5 * xyz[2]
    x = torch.from_numpy(np.concatenate([f * (c + 1) for c in range(6)])).cuda()
    w = op.new_work()
    op.pack(x, w)
    op.probe_sample(w, 0.0)
    v = op.probe_read()["series"][0, 0, 0]
    want = (1.0 + 0.6 - 0.4 + 0.25) * np.arange(1, 7)
    assert np.abs(v - want).max() < 1e-5
    with pytest.raises(dg.DgtdError, match="FP64 form only"):
        op.step_noalloc(w, 0.0, 1e-3, 1)
