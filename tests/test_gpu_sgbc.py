"""Thin-layer boundaries (SGBC) on the GPU against the oracle (its restatement of the reference's
SGBC path, GlobalEvolution.cpp:48-1001 and SolverExtension.cpp:49-559).

Bars: Mult 1e-12 relative L2; whole runs 1e-10 (the product composes each stage's sub-steps into
one map, the oracle steps them; both FP64); a stack closed by PEC sheets equals an interior PEC
sheet to 1e-12; in a TEM waveguide the slab's reflected and transmitted pulses follow its
analytic S11 / S21 as the oracle's do (1.2e-2 / 4.2e-3 of the incident amplitude measured there).
"""
import math
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import FREE_SPACE_IMPEDANCE as Z0, rel_l2, sgbc_box, slab_pulse, tem_waveguide

pytestmark = pytest.mark.gpu
REF_SGBC = Path(__file__).resolve().parent / "golden" / "cases" / "reference" / "3D_SGBC"

LOSSY = {"layers": [{"eps": 3.0, "mu": 1.0, "sigma": 2.0, "width": 0.05, "segments": 2, "order": 2}],
         "left": 0, "right": 0, "sub_dt": 2.5e-3}
TWO_LAYERS_PEC = {"layers": [{"eps": 2.0, "mu": 1.5, "sigma": 1.0, "width": 0.02, "segments": 2, "order": 2},
                             {"eps": 4.0, "mu": 1.0, "sigma": 0.0, "width": 0.01, "segments": 1, "order": 1}],
                  "left": 1, "right": 0, "sub_dt": 4e-3}
PMC_SMA = {"layers": [{"eps": 1.5, "mu": 1.0, "sigma": 0.5, "width": 0.03, "segments": 2, "order": 2}],
           "left": 2, "right": 3, "sub_dt": 0.0}
WAVE = {"propagation": [1, 0, 0], "polarization": [0, 1, 0], "spread": 0.1, "mean": 0.2}


def _mesh(m, faces, code=dg.BC_SGBC, bdr_codes=None, tfsf=True):
    return dg.Mesh(np.asarray(m.vertices), np.asarray(m.elements), np.asarray(m.bdr_faces),
                   np.asarray(m.bdr_codes if bdr_codes is None else bdr_codes),
                   np.asarray(m.tfsf_faces) if tfsf else np.zeros((0, 3), np.int32),
                   faces, np.full(len(faces), code, np.int32))


def _pair(m, faces, order, stacks, face_stack, waves=(), tfsf=True, code=dg.BC_SGBC, bdr_codes=None):
    """The product operator and the oracle on the same mesh, stacks and sources."""
    mesh = _mesh(m, faces, code, bdr_codes, tfsf)
    op = dg.Operator(mesh, order=order)
    orc = po.Oracle(mesh.vertices, mesh.elements, order, 1.0, 3, mesh.bdr_faces, mesh.bdr_codes,
                    mesh.tfsf_faces if tfsf else None, faces, np.full(len(faces), code, np.int32))
    if waves:
        op.set_planewaves(list(waves))
        orc.set_planewaves(list(waves))
    if code == dg.BC_SGBC:
        op.set_sgbc(stacks, face_stack)
        orc.set_sgbc(stacks, face_stack)
    return op, orc


def _bump(X, x0, s=0.15):
    """Ey = Hz = Gaussian around x = x0 (a right-moving pulse)."""
    N = X.shape[1]
    u = np.zeros(6 * N)
    g = np.exp(-((X[0] - x0) ** 2) / (2 * s * s))
    u[N:2 * N] = g
    u[5 * N:6 * N] = g
    return u


@pytest.mark.parametrize("t", [0.0, 0.004])
def test_mult_matches_oracle(torch_cuda, t):
    """Mult at time t advances the sub-solvers from their start (zero states, time 0) over t with
    the input's ghost values, then injects (GlobalEvolution::Mult, GlobalEvolution.cpp:639-1001)."""
    m, _, F = sgbc_box(n=(4, 2, 2))
    op, orc = _pair(m, F, 2, [LOSSY], np.zeros(len(F), np.int32), [WAVE])
    x = np.random.default_rng(7).standard_normal(op.state_len)
    y = op.mult_host(x, t)
    yo = orc.mult(x, t)
    assert np.linalg.norm(yo) > 0 and rel_l2(y, yo) <= 1e-12


def test_run_matches_oracle(torch_cuda):
    """A TF/SF pulse reaching the layer: 120 RK4 steps with sub-stepped stages (4 sub-steps per
    step, 2 per half step), through dgtd_op_run_host."""
    m, _, F = sgbc_box(n=(4, 2, 2))
    op, orc = _pair(m, F, 2, [LOSSY], np.zeros(len(F), np.int32), [WAVE])
    x0 = np.zeros(op.state_len)
    x, n = op.run_host(x0, 0.0, 0.01, 1.2)
    xo, no = orc.run(x0, 0.0, 0.01, 1.2)
    assert n == no == 120
    assert np.linalg.norm(xo) > 0.1 and rel_l2(x, xo) <= 1e-10
    assert np.linalg.norm(op.sgbc_states()) > 0


def test_mult_after_steps_restarts_from_the_checkpoint(torch_cuda):
    """After steps, a Mult restarts the sub-solvers from the last step's checkpoint (its start
    states) and advances them over t minus that step's start, as GlobalEvolution::Mult does."""
    torch = torch_cuda
    m, _, F = sgbc_box(n=(4, 2, 2), tfsf=False)
    op, orc = _pair(m, F, 2, [LOSSY], np.zeros(len(F), np.int32), tfsf=False)
    x0 = _bump(orc.nodes(), 1.0)
    u = torch.from_numpy(x0.copy()).cuda()
    op.step(u, 0.0, 0.01, 5)
    xo = orc.step(x0, 0.0, 0.01, 5)
    torch.cuda.synchronize()
    assert rel_l2(u.cpu().numpy(), xo) <= 1e-11
    y = op.mult_host(xo, 0.047)
    assert rel_l2(y, orc.mult(xo, 0.047)) <= 1e-11


def test_adapter_step_hooks_match_the_fused_step(torch_cuda):
    """An integrator driving mult itself with the step hooks (the GpuEvolution adapter under the
    reference's RK4Solver and Solver::step) gives dgtd_op_step's result."""
    torch = torch_cuda
    m, _, F = sgbc_box(n=(4, 2, 2), tfsf=False)
    op, orc = _pair(m, F, 2, [LOSSY], np.zeros(len(F), np.int32), tfsf=False)
    other = dg.Operator(_mesh(m, F, tfsf=False), order=2)
    other.set_sgbc([LOSSY], np.zeros(len(F), np.int32))
    x0 = _bump(orc.nodes(), 1.0)
    fused = torch.from_numpy(x0.copy()).cuda()
    op.step(fused, 0.0, 0.01, 8)
    x = torch.from_numpy(x0.copy()).cuda()
    k = [torch.empty_like(x) for _ in range(4)]
    dt = 0.01
    for s in range(8):
        t = s * dt
        other.sgbc_commit(x, t, dt)
        other.mult(x, k[0], t)
        other.mult(x + dt / 2 * k[0], k[1], t + dt / 2)
        other.mult(x + dt / 2 * k[1], k[2], t + dt / 2)
        other.mult(x + dt * k[2], k[3], t + dt)
        x = x + dt / 6 * (k[0] + 2 * k[1] + 2 * k[2] + k[3])
        other.sgbc_finalize(x)
    torch.cuda.synchronize()
    assert rel_l2(x.cpu().numpy(), fused.cpu().numpy()) <= 1e-12
    assert rel_l2(other.sgbc_states(), op.sgbc_states()) <= 1e-12
    assert rel_l2(fused.cpu().numpy(), orc.step(x0, 0.0, dt, 8)) <= 1e-11


def test_two_stacks_and_sheets_match_oracle(torch_cuda):
    """Two sheets with their own stacks: two layers closed by PEC on the left, and PMC / SMA sides
    with one sub-step per span; a pulse between them, 60 steps."""
    m, sheets, F = sgbc_box(n=(6, 2, 2), hi=(3.0, 1.0, 1.0), planes=(1.0, 2.0), tfsf=False)
    fs = np.concatenate([np.zeros(len(sheets[0]), np.int32), np.ones(len(sheets[1]), np.int32)])
    op, orc = _pair(m, F, 2, [TWO_LAYERS_PEC, PMC_SMA], fs, tfsf=False)
    x0 = _bump(orc.nodes(), 1.5, 0.3)
    x, _ = op.run_host(x0, 0.0, 0.01, 0.6)
    xo, _ = orc.run(x0, 0.0, 0.01, 0.6)
    assert rel_l2(x, xo) <= 1e-10


def test_pec_closed_stack_is_a_pec_sheet(torch_cuda):
    m, _, F = sgbc_box(n=(4, 2, 2), tfsf=False)
    closed = {"layers": [{"eps": 3.0, "sigma": 2.0, "width": 0.05, "segments": 2, "order": 2}],
              "left": 1, "right": 1, "sub_dt": 0.004}
    layer = dg.Operator(_mesh(m, F, tfsf=False), order=2)
    layer.set_sgbc([closed], np.zeros(len(F), np.int32))
    sheet = dg.Operator(_mesh(m, F, code=dg.BC_PEC, tfsf=False), order=2)
    x0 = _bump(layer.node_coords(), 1.0)
    a, _ = sheet.run_host(x0, 0.0, 0.01, 0.4)
    b, _ = layer.run_host(x0, 0.0, 0.01, 0.4)
    assert np.linalg.norm(a) > 1.0 and rel_l2(b, a) <= 1e-12


def test_reference_3d_sgbc_mesh_matches_oracle(torch_cuda):
    """The reference's 3D_SGBC mesh and layer (eps 20, 0.2 S/m, 5 mm; 288-unknown sub-solvers on
    240 pairs) with a pulse started on the layer, 40 steps of 2.5e-3 (one sub-step per span)."""
    c = dg.Case(REF_SGBC / "3D_SGBC.json")
    mesh = c.mesh()
    stacks, fs = c.sgbc()
    op = dg.Operator(mesh, order=c.info["order"], alpha=c.info["alpha"])
    op.set_sgbc(stacks, fs)
    orc = po.Oracle.from_mesh(mesh, c.info["order"], alpha=c.info["alpha"])
    orc.set_sgbc(stacks, fs)
    assert orc.sgbc_pairs() == 240
    x0 = _bump(orc.nodes(), 1.9)
    x, n = op.run_host(x0, 0.0, 2.5e-3, 0.1)
    xo, no = orc.run(x0, 0.0, 2.5e-3, 0.1)
    assert n == no == 40 and rel_l2(x, xo) <= 1e-10


def test_reference_3d_sgbc_case_runs(torch_cuda, tmp_path):
    """The reference's 3D_SGBC case through dgtd_case_run: 100,000 steps to t = 10 with its
    plane wave, layer and three point probes."""
    c = dg.Case(REF_SGBC / "3D_SGBC.json")
    _, res = c.run(out_dir=tmp_path, want_state=False)
    assert res["steps"] == 100000 and res["unstable_step"] == -1
    from conftest import read_point_probe
    rows = [read_point_probe(tmp_path / f"PointProbe{k}.dat") for k in range(3)]
    assert all(np.all(np.isfinite(r)) for r in rows)
    assert np.abs(rows[2][:, 2]).max() > 0.05   # Ey beyond the layer: the pulse went through


def test_waveguide_slab_matches_analytic(torch_cuda):
    """The oracle's analytic-slab check on the GPU path (order 3, 450 steps)."""
    torch = torch_cuda
    m, codes, F = tem_waveguide()
    eps, mu, sig, d = 4.0, 1.0, 0.05 * Z0, 0.02
    st = {"layers": [{"eps": eps, "mu": mu, "sigma": sig, "width": d, "segments": 4, "order": 2}],
          "sub_dt": 0.5 * (d / 4) * math.sqrt(eps * mu)}
    op = dg.Operator(_mesh(m, F, bdr_codes=codes), order=3)
    op.set_planewaves([{"propagation": [1, 0, 0], "polarization": [0, 1, 0], "spread": 0.15, "mean": 0.5}])
    op.set_sgbc([st], np.zeros(len(F), np.int32))
    X = op.node_coords()
    N = X.shape[1]
    node = lambda x: int(np.argmin((X[0] - x) ** 2 + (X[1] - 0.25) ** 2 + (X[2] - 0.25) ** 2))
    ir, it = N + node(0.5), N + node(3.5)
    u = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    dt, ts, rr, tr = 0.01, [], [], []
    for s in range(450):
        op.step(u, s * dt, dt, 1)
        v = u[[ir, it]].cpu().numpy()
        ts.append((s + 1) * dt); rr.append(v[0]); tr.append(v[1])
    ts = np.array(ts)
    pt = slab_pulse(ts, 2.5, 3.5, 0.15, 0.5, eps, mu, sig, d, "t")
    pr = slab_pulse(ts, 2.5, 0.5, 0.15, 0.5, eps, mu, sig, d, "r")
    assert np.abs(np.array(tr) - pt).max() <= 0.02
    assert np.abs(np.array(rr) - pr).max() <= 0.01


def test_sgbc_refusals(torch_cuda):
    torch = torch_cuda
    m, _, F = sgbc_box(n=(4, 2, 2), tfsf=False)
    mesh = _mesh(m, F, tfsf=False)
    with pytest.raises(dg.DgtdError, match="FP64 form with one incidence"):
        dg.Operator(mesh, order=2, precision=dg.FP32)
    with pytest.raises(dg.DgtdError, match="FP64 form with one incidence"):
        dg.Operator(mesh, order=2, batch=2)
    op = dg.Operator(mesh, order=2)
    u = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DgtdError, match="dgtd_op_set_sgbc") as e:
        op.step(u, 0.0, 0.01, 1)
    assert e.value.code == -3
    with pytest.raises(dg.DgtdError, match="stack index out of range"):
        op.set_sgbc([LOSSY], np.full(len(F), 3, np.int32))
    op.set_sgbc([LOSSY], np.zeros(len(F), np.int32))
    with pytest.raises(dg.DgtdError, match="classical RK4") as e:
        op.step(u, 0.0, 0.01, 1, integrator=dg.LSERK4)
    assert e.value.code == -3
    with pytest.raises(dg.DgtdError, match="dgtd_op_step_noalloc") as e:
        op.step_noalloc(u, 0.0, 0.01, 1)
    assert e.value.code == -3
    op.step(u, 0.0, 0.01, 2)
    torch.cuda.synchronize()
    assert torch.count_nonzero(u).item() == 0   # zero fields stay zero


def _curved_sheet_mesh(code):
    from conftest import curved_box, plane_faces
    m, Vc, E, els, nodes = curved_box(mode="all", bump=0.03)
    F = plane_faces(np.asarray(m.vertices), E, 0.5)
    mesh = dg.Mesh(Vc, E, np.asarray(m.bdr_faces), np.asarray(m.bdr_codes), np.zeros((0, 3), np.int32), F,
                   np.full(len(F), code, np.int32), curved_elems=els, curved_nodes=nodes)
    return mesh, F


def test_sgbc_on_a_curved_sheet_matches_oracle(torch_cuda):
    """Every element curved, the layer on the bent sheet x = 1/2: the curved elements' injection
    blocks (per-point normals) and the pairs' per-node rotations, 40 steps."""
    mesh, F = _curved_sheet_mesh(dg.BC_SGBC)
    op = dg.Operator(mesh, order=2)
    op.set_sgbc([LOSSY], np.zeros(len(F), np.int32))
    orc = po.Oracle(mesh.vertices, mesh.elements, 2, 1.0, 3, mesh.bdr_faces, mesh.bdr_codes, None, F,
                    np.full(len(F), 4, np.int32))
    orc.set_curved(mesh.curved_elems, mesh.curved_nodes)
    orc.set_sgbc([LOSSY], np.zeros(len(F), np.int32))
    x0 = _bump(orc.nodes(), 0.5)
    x, n = op.run_host(x0, 0.0, 0.005, 0.2)
    xo, no = orc.run(x0, 0.0, 0.005, 0.2)
    assert n == no == 40 and rel_l2(x, xo) <= 1e-10


def test_pec_closed_stack_on_a_curved_sheet_is_a_pec_sheet(torch_cuda):
    closed = {"layers": [{"eps": 3.0, "sigma": 2.0, "width": 0.05, "segments": 2, "order": 2}],
              "left": 1, "right": 1, "sub_dt": 0.004}
    mesh, F = _curved_sheet_mesh(dg.BC_SGBC)
    layer = dg.Operator(mesh, order=2)
    layer.set_sgbc([closed], np.zeros(len(F), np.int32))
    sheet = dg.Operator(_curved_sheet_mesh(dg.BC_PEC)[0], order=2)
    x0 = _bump(layer.node_coords(), 0.5)
    a, _ = sheet.run_host(x0, 0.0, 0.005, 0.2)
    b, _ = layer.run_host(x0, 0.0, 0.005, 0.2)
    assert np.linalg.norm(a) > 1.0 and rel_l2(b, a) <= 1e-12


def test_reference_curved_sgbc_sphere_matches_oracle(torch_cuda):
    """The reference's 3D_RCS_Sphere_Box_05m_G2: an SGBC layer on a curved sphere of radius 0.5
    (9,103 tetrahedra, 724 curved, 62 SGBC faces), a pulse started on the sphere; 20 steps of the
    case's estimated dt."""
    d = Path(__file__).resolve().parent / "golden" / "cases" / "reference" / "3D_RCS_Sphere_Box_05m_G2"
    c = dg.Case(d / "3D_RCS_Sphere_Box_05m_G2.json")
    mesh = c.mesh()
    stacks, fs = c.sgbc()
    assert len(mesh.curved_elems) == 724 and len(fs) == 62
    op = dg.Operator(mesh, order=c.info["order"], alpha=c.info["alpha"])
    op.set_sgbc(stacks, fs)
    orc = po.Oracle.from_mesh(mesh, c.info["order"], alpha=c.info["alpha"])
    orc.set_curved(mesh.curved_elems, mesh.curved_nodes)
    orc.set_sgbc(stacks, fs)
    X = orc.nodes()
    N = X.shape[1]
    x0 = np.zeros(6 * N)
    g = np.exp(-np.sum((X - np.array([[0.5], [0.0], [0.0]])) ** 2, axis=0) / (2 * 0.1 ** 2))
    x0[N:2 * N] = g
    x0[5 * N:6 * N] = g
    dt = c.auto_dt()
    x, n = op.run_host(x0, 0.0, dt, 20 * dt)
    xo, no = orc.run(x0, 0.0, dt, 20 * dt)
    assert n == no and np.linalg.norm(xo) > 0.1 and rel_l2(x, xo) <= 1e-10
