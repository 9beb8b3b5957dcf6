"""Batched FP32 form (B incidences on one mesh) against the FP64 oracle / FP64 GPU form.

Bar: relative L2 <= 1e-5 against FP64 per incidence, stated for
every result; a single RHS evaluation is checked tighter (FP32 rounding only).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(20261203)


def waves_for(B, seed=20261203, spread=0.1, mean=-0.5):
    rng = np.random.default_rng(seed)
    out = []
    for b in range(B):
        k = rng.standard_normal(3); k /= np.linalg.norm(k)
        g = rng.standard_normal(3); pol = g - g.dot(k) * k; pol /= np.linalg.norm(pol)
        out.append(dict(propagation=k, polarization=pol, spread=spread, mean=mean, batch=b))
    return out


def scatter_mesh(n=6, hole=True):
    # box [-1,1]^3, central PEC cube removed, SMA outer boundary, TF/SF box one cell in from the boundary
    c0, c1 = n // 2 - max(1, n // 6) // 1, n // 2 + max(1, n // 6) // 1
    return dg.box_mesh((n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1),
                       hole=((c0,) * 3, (c1,) * 3) if hole else None,
                       tfsf=((1,) * 3, (n - 1,) * 3), outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)


def test_pack_unpack_roundtrip(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 3))
    B = 5
    op = dg.Operator(m, order=3, precision=dg.FP32_3XTF32, batch=B)
    # working state: the FP32 pair (x_hi, x_lo) of every value, incidences padded to 32
    assert op.info["batch_padded"] == 32 and op.work_len == 2 * 6 * m.n_elements * 20 * 32
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work()
    op.pack(xd, w)
    back = torch.zeros_like(xd)
    op.unpack(w, back)
    torch.cuda.synchronize()
    hi = w[: op.work_len // 2].cpu().numpy()
    assert np.abs(back.cpu().numpy() - x).max() <= 2.0 ** -46 * np.abs(x).max()
    assert np.count_nonzero(hi) == x.size            # x_hi = fl(x) of the B real incidences, 0 in the padding
    # pinned host memory is accepted as the reference-layout buffer (read / written over the host link)
    hx = torch.from_numpy(x).pin_memory()
    w2 = op.new_work()
    op.pack(hx, w2)
    hb = torch.zeros_like(hx).pin_memory()
    op.unpack(w2, hb)
    torch.cuda.synchronize()
    assert torch.equal(w2, w) and np.array_equal(hb.numpy(), back.cpu().numpy())
    with pytest.raises(dg.DgtdError, match="pinned host"):
        op.pack(torch.from_numpy(x), w2)             # pageable host memory is refused


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_batched_mult_vs_oracle(torch_cuda, order):
    torch = torch_cuda
    if order <= 3:
        m = scatter_mesh(6)
    else:
        m = dg.box_mesh((3, 3, 3), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1,) * 3, (2,) * 3), outer_bc=dg.BC_SMA)
    B = 3
    waves = waves_for(B, spread=0.3, mean=-0.2)
    op = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    op.set_planewaves(waves)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); y = op.new_work()
    op.pack(xd, w)
    op.mult(w, y, 0.25)
    yd = torch.zeros_like(xd)
    op.unpack(y, yd)
    torch.cuda.synchronize()
    yv = yd.cpu().numpy()
    L = op.state_len // B
    for b in range(B):
        orc = po.Oracle.from_mesh(m, order)
        orc.set_planewaves([waves[b]])
        xb = x[b * L:(b + 1) * L].astype(np.float32).astype(np.float64)   # same rounded input
        err = rel_l2(yv[b * L:(b + 1) * L], orc.mult(xb, 0.25))
        assert err < 2e-6, (b, err)


def test_batched_materials_boundaries(torch_cuda):
    torch = torch_cuda
    for bc in (dg.BC_PEC, dg.BC_PMC, dg.BC_SMA, dg.BC_OPEN):
        m = dg.box_mesh((2, 3, 2), outer_bc=bc)
        K = m.n_elements
        m.eps = RNG.uniform(1, 4, K); m.mu = RNG.uniform(1, 2, K); m.sigma = RNG.uniform(0, 0.5, K)
        op = dg.Operator(m, order=3, alpha=0.7, precision=dg.FP32_3XTF32, batch=2)
        x = RNG.standard_normal(op.state_len)
        xd = torch.from_numpy(x).cuda()
        w = op.new_work(); y = op.new_work()
        op.pack(xd, w); op.mult(w, y, 0.0)
        yd = torch.zeros_like(xd); op.unpack(y, yd)
        torch.cuda.synchronize()
        orc = po.Oracle.from_mesh(m, 3, alpha=0.7)
        L = op.state_len // 2
        for b in range(2):
            xb = x[b * L:(b + 1) * L].astype(np.float32).astype(np.float64)
            assert rel_l2(yd.cpu().numpy()[b * L:(b + 1) * L], orc.mult(xb, 0.0)) < 2e-6


@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_batched_scattering_vs_fp64_gpu(torch_cuda, integrator):
    """Plane-wave scattering from a PEC cube (TF/SF + SMA), B = 8 incidences, p = 3:
    FP32 batched form vs the FP64 form over 300 steps, relative L2 <= 1e-5 per incidence."""
    torch = torch_cuda
    m = scatter_mesh(6)
    B, order = 8, 3
    waves = waves_for(B)
    op64 = dg.Operator(m, order=order, batch=B)
    op32 = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    op64.set_planewaves(waves); op32.set_planewaves(waves)
    dt = op64.estimate_dt(1.0)
    x0 = torch.zeros(op64.state_len, dtype=torch.float64, device="cuda")
    x64 = x0.clone()
    w = op32.new_work(); op32.pack(x0, w)
    nsteps = 300
    op64.step(x64, 0.0, dt, nsteps, integrator)
    op32.step(w, 0.0, dt, nsteps, integrator)
    x32 = torch.zeros_like(x0); op32.unpack(w, x32)
    torch.cuda.synchronize()
    a, r = x32.cpu().numpy(), x64.cpu().numpy()
    L = op64.state_len // B
    errs = [rel_l2(a[b * L:(b + 1) * L], r[b * L:(b + 1) * L]) for b in range(B)]
    assert np.linalg.norm(r) > 1.0          # the pulse has entered the domain
    assert max(errs) <= 1e-5, errs


def test_batched_norm_and_launch_count(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2))
    op = dg.Operator(m, order=2, precision=dg.FP32_3XTF32, batch=3)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); op.pack(xd, w)
    n = op.norm2(w)
    L = op.state_len // 3
    for b in range(3):
        ref = np.sum(x[b * L:(b + 1) * L].astype(np.float32).astype(np.float64) ** 2)
        assert abs(n[b] - ref) <= 1e-6 * ref
    before = dg.kernel_launches()
    op.step(w, 0.0, 1e-3, 2)
    torch.cuda.synchronize()
    assert dg.kernel_launches() - before == 8          # 4 stage kernels per RK4 step, no sources


# ---------------------------------------------------------------- tensor-core path (tcgen05, 3xTF32)

@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_tensor_core_mult_vs_oracle(torch_cuda, order):
    """B = 64 incidences (one 64-wide chunk): the stage runs on tcgen05; check against the oracle."""
    torch = torch_cuda
    m = scatter_mesh(6) if order <= 2 else dg.box_mesh((3, 3, 3), lo=(-1, -1, -1), hi=(1, 1, 1),
                                                       tfsf=((1,) * 3, (2,) * 3), outer_bc=dg.BC_SMA)
    B = 64
    waves = waves_for(B, spread=0.3, mean=-0.2)
    op = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    assert op.uses_tensor_cores
    op.set_planewaves(waves)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    w = op.new_work(); y = op.new_work()
    op.pack(xd, w)
    op.mult(w, y, 0.25)
    op.check()
    yd = torch.zeros_like(xd)
    op.unpack(y, yd)
    torch.cuda.synchronize()
    yv = yd.cpu().numpy()
    L = op.state_len // B
    for b in (0, 17, 63):
        orc = po.Oracle.from_mesh(m, order)
        orc.set_planewaves([waves[b]])
        xb = x[b * L:(b + 1) * L].astype(np.float32).astype(np.float64)
        err = rel_l2(yv[b * L:(b + 1) * L], orc.mult(xb, 0.25))
        assert err < 2e-6, (b, err)


def test_tensor_core_matches_simt_and_fp64(torch_cuda):
    """Scattering case, B = 64, p = 3, 300 RK4 steps: tensor-core path vs FP32 SIMT path vs FP64 form."""
    torch = torch_cuda
    m = scatter_mesh(6)
    B, order = 64, 3
    waves = waves_for(B)
    op64 = dg.Operator(m, order=order, batch=B)
    tc = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    simt = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    simt.set_contraction(1)
    assert tc.uses_tensor_cores and not simt.uses_tensor_cores
    for o in (op64, tc, simt):
        o.set_planewaves(waves)
    dt = op64.estimate_dt(1.0)
    x0 = torch.zeros(op64.state_len, dtype=torch.float64, device="cuda")
    x64 = x0.clone()
    wt = tc.new_work(); tc.pack(x0, wt)
    ws = simt.new_work(); simt.pack(x0, ws)
    nsteps = 300
    op64.step(x64, 0.0, dt, nsteps)
    tc.step(wt, 0.0, dt, nsteps)
    simt.step(ws, 0.0, dt, nsteps)
    tc.check()
    xt = torch.zeros_like(x0); tc.unpack(wt, xt)
    xs = torch.zeros_like(x0); simt.unpack(ws, xs)
    torch.cuda.synchronize()
    a, s_, r = xt.cpu().numpy(), xs.cpu().numpy(), x64.cpu().numpy()
    L = op64.state_len // B
    e_tc = [rel_l2(a[b * L:(b + 1) * L], r[b * L:(b + 1) * L]) for b in range(B)]
    e_st = [rel_l2(a[b * L:(b + 1) * L], s_[b * L:(b + 1) * L]) for b in range(B)]
    assert np.linalg.norm(r) > 1.0
    assert max(e_tc) <= 1e-5, max(e_tc)
    assert max(e_st) <= 1e-5, max(e_st)


def test_tensor_core_p4_long_run_vs_fp64(torch_cuda):
    """Scattering case at p = 4 with 64 incidences (the tensor-core kernel), 250 RK4 steps:
    relative L2 vs the FP64 form <= 1e-5 for the compared incidences. This bar failed (1.3e-5)
    while the correction products shared the main tensor-memory accumulator."""
    torch = torch_cuda
    n = 12
    m = dg.box_mesh((n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((5,) * 3, (7,) * 3),
                    tfsf=((2,) * 3, (10,) * 3), outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)
    B, Bc, order = 64, 4, 4
    waves = waves_for(B)
    op64 = dg.Operator(m, order=order, batch=Bc)
    tc = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=B)
    assert tc.uses_tensor_cores
    op64.set_planewaves(waves[:Bc])
    tc.set_planewaves(waves)
    dt = op64.estimate_dt(1.0)
    x64 = torch.zeros(op64.state_len, dtype=torch.float64, device="cuda")
    x32 = torch.zeros(tc.state_len, dtype=torch.float64, device="cuda")
    wk = tc.new_work(); tc.pack(x32, wk)
    op64.step(x64, 0.0, dt, 250)
    tc.step(wk, 0.0, dt, 250)
    tc.check()
    tc.unpack(wk, x32)
    torch.cuda.synchronize()
    a, r = x32.cpu().numpy(), x64.cpu().numpy()
    L = op64.state_len // Bc
    errs = [rel_l2(a[b * L:(b + 1) * L], r[b * L:(b + 1) * L]) for b in range(Bc)]
    assert np.linalg.norm(r) > 1.0
    assert max(errs) <= 1e-5, errs
