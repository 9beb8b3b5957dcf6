"""GPU parity of the plain FP64 form against the CPU oracle (through the C ABI).

Bar: relative L2 <= 1e-12 against the oracle's assembled operator on the same
mesh and inputs (FP64 arithmetic, different summation order).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12
RNG = np.random.default_rng(20261203)


def _mesh(cells, bc=dg.BC_PEC, tf=None, mat=False, lo=(0, 0, 0), hi=(1, 1, 1), hole=None):
    m = dg.box_mesh(cells, lo=lo, hi=hi, tfsf=tf, outer_bc=bc, hole=hole)
    if mat:
        K = m.n_elements
        m.eps = RNG.uniform(1, 4, K); m.mu = RNG.uniform(1, 2, K); m.sigma = RNG.uniform(0, 0.5, K)
    return m


def _pair(mesh, order, alpha=1.0, waves=None, batch=1):
    op = dg.Operator(mesh, order=order, alpha=alpha, batch=batch)
    orc = po.Oracle.from_mesh(mesh, order, alpha=alpha)
    if waves:
        op.set_planewaves(waves)
    return op, orc


WAVE = dict(propagation=[1.0, 0.3, -0.2], polarization=[0.1, 0.0, 1.0], spread=0.2, mean=0.1)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_mult_every_order_pec(torch_cuda, order):
    torch = torch_cuda
    m = _mesh((2, 2, 2))
    op, orc = _pair(m, order)
    assert np.allclose(op.node_coords(), orc.nodes(), atol=1e-14)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda(); yd = torch.empty_like(xd)
    op.mult(xd, yd, 0.0)
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), orc.mult(x, 0.0)) < TOL


@pytest.mark.parametrize("bc", [dg.BC_PEC, dg.BC_PMC, dg.BC_SMA, dg.BC_OPEN])
@pytest.mark.parametrize("alpha", [0.0, 1.0, 0.5])
def test_mult_boundaries_and_materials(torch_cuda, bc, alpha):
    torch = torch_cuda
    m = _mesh((2, 3, 2), bc=bc, mat=True)
    op, orc = _pair(m, 3, alpha=alpha)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda(); yd = torch.empty_like(xd)
    op.mult(xd, yd, 0.0)
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), orc.mult(x, 0.0)) < TOL


@pytest.mark.parametrize("t", [0.0, 0.35, 0.8, 5.0])
def test_mult_tfsf_source(torch_cuda, t):
    """TF/SF faces with a plane wave, at times with the source active and skipped (||pw|| < 1e-8)."""
    torch = torch_cuda
    m = _mesh((4, 4, 4), bc=dg.BC_SMA, tf=((1, 1, 1), (3, 3, 3)), lo=(-1, -1, -1), hi=(1, 1, 1))
    wave = dict(WAVE, mean=-0.4, spread=0.1)
    op, orc = _pair(m, 3, waves=[wave])
    orc.set_planewaves([wave])
    x = RNG.standard_normal(op.state_len) * 1e-3
    xd = torch.from_numpy(x).cuda(); yd = torch.empty_like(xd)
    op.mult(xd, yd, t)
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), orc.mult(x, t)) < TOL


def test_mult_interior_pec_sheet_and_hole(torch_cuda):
    torch = torch_cuda
    m = _mesh((4, 4, 4), hole=((1, 1, 1), (2, 2, 2)), bc=dg.BC_SMA)
    V = m.vertices
    faces = set()
    for e in m.elements:
        for f in range(4):
            tri = tuple(sorted(int(v) for q, v in enumerate(e) if q != f))
            if np.allclose(V[list(tri), 2], 0.75):
                faces.add(tri)
    m.int_faces = np.array(sorted(faces), np.int32)
    m.int_codes = np.full(len(faces), dg.BC_PMC, np.int32)
    op, orc = _pair(m, 2)
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda(); yd = torch.empty_like(xd)
    op.mult(xd, yd, 0.0)
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), orc.mult(x, 0.0)) < TOL


@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_fused_steps_match_oracle(torch_cuda, integrator):
    torch = torch_cuda
    m = _mesh((3, 3, 3), bc=dg.BC_SMA, tf=((1, 1, 1), (2, 2, 2)), mat=True)
    wave = dict(WAVE, mean=-0.2)
    op, orc = _pair(m, 3, waves=[wave])
    orc.set_planewaves([wave])
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    op.step(xd, 0.0, 2e-3, 25, integrator)
    torch.cuda.synchronize()
    xr = orc.step(x, 0.0, 2e-3, 25, integrator=integrator)
    assert rel_l2(xd.cpu().numpy(), xr) < TOL


def test_host_run_loop_matches_reference_loop(torch_cuda):
    """dgtd_op_run_host follows Solver::run (truncated last step) like the oracle's loop."""
    m = _mesh((2, 2, 2))
    op, orc = _pair(m, 2)
    x = RNG.standard_normal(op.state_len)
    xg, n1 = op.run_host(x, 0.0, 0.03, 0.1)
    xr, n2 = orc.run(x, 0.0, 0.03, 0.1)
    assert n1 == n2 == 4
    assert rel_l2(xg, xr) < TOL
    yh = op.mult_host(x, 0.0)
    assert rel_l2(yh, orc.mult(x, 0.0)) < TOL


def test_batched_fp64_incidences(torch_cuda):
    """B incidences on one mesh (stacked reference vectors), each with its own plane wave."""
    torch = torch_cuda
    B = 3
    m = _mesh((3, 3, 3), bc=dg.BC_SMA, tf=((1, 1, 1), (2, 2, 2)), lo=(-1, -1, -1), hi=(1, 1, 1))
    waves = []
    for b in range(B):
        k = RNG.standard_normal(3); k /= np.linalg.norm(k)
        g = RNG.standard_normal(3); pol = g - g.dot(k) * k
        waves.append(dict(propagation=k, polarization=pol, spread=0.15, mean=-0.3, batch=b))
    op = dg.Operator(m, order=2, batch=B)
    op.set_planewaves(waves)
    L = op.state_len // B
    x = RNG.standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda(); yd = torch.empty_like(xd)
    op.mult(xd, yd, 0.2)
    op.step(xd, 0.0, 5e-3, 10)
    torch.cuda.synchronize()
    y = yd.cpu().numpy(); xs = xd.cpu().numpy()
    for b in range(B):
        orc = po.Oracle.from_mesh(m, 2)
        orc.set_planewaves([waves[b]])
        xb = x[b * L:(b + 1) * L]
        assert rel_l2(y[b * L:(b + 1) * L], orc.mult(xb, 0.2)) < TOL
        assert rel_l2(xs[b * L:(b + 1) * L], orc.step(xb, 0.0, 5e-3, 10)) < TOL


def te110(xyz, t):
    w = np.pi * np.sqrt(2.0)
    x, y = xyz[0], xyz[1]
    z = np.zeros_like(x)
    return np.concatenate([z, z, np.sin(np.pi * x) * np.sin(np.pi * y) * np.cos(w * t),
                           -(np.pi / w) * np.sin(np.pi * x) * np.cos(np.pi * y) * np.sin(w * t),
                           (np.pi / w) * np.cos(np.pi * x) * np.sin(np.pi * y) * np.sin(w * t), z])


def test_cubic_resonator_full_size(torch_cuda):
    """The 3D PEC cubic resonator: 8^3 hexes x 6 tets (3,072), p = 3, dt = 1e-3, TE110 mode.

    - all 2,000 RK4 steps (T = 2) vs the oracle's RK4 loop (<= 1e-12 relative L2), checked after
      100 steps and at the end;
    - error vs the analytic mode at discretisation level.
    """
    torch = torch_cuda
    m = dg.box_mesh((8, 8, 8))
    op = dg.Operator(m, order=3)
    orc = po.Oracle.from_mesh(m, 3)
    xyz = op.node_coords()
    x0 = te110(xyz, 0.0)
    xd = torch.from_numpy(x0).cuda()
    op.step(xd, 0.0, 1e-3, 100)
    torch.cuda.synchronize()
    xr = orc.step(x0, 0.0, 1e-3, 100, form=po.NODAL)
    assert rel_l2(xd.cpu().numpy(), xr) < TOL
    op.step(xd, 0.1, 1e-3, 1900)
    torch.cuda.synchronize()
    xT = xd.cpu().numpy()
    assert np.all(np.isfinite(xT))
    xr = orc.step(xr, 0.1, 1e-3, 1900, form=po.NODAL)
    assert rel_l2(xT, xr) < TOL
    err = rel_l2(xT, te110(xyz, 2.0))
    assert err < 2e-3, err
