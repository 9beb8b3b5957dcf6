"""Curved (second-order) tetrahedra on the GPU against the oracle's assembly on the curved map
(the reference's global operator on curved elements; HesthavenEvolution copies those rows,
src/evolution/HesthavenEvolution.cpp:207-241, 411-435, 538-540).

Bars: Mult 1e-12 relative L2; runs 1e-11 (FP64 both; the straight elements run the fused stage,
the curved ones their block rows); the reference's 3D_Curved_Element_Test (122 curved of 1,151
tetrahedra) 1e-10 over its first 200 steps and stable to its final time.
"""
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import curved_box, rel_l2

pytestmark = pytest.mark.gpu
REF_CURVED = Path(__file__).resolve().parent / "golden" / "cases" / "reference" / "3D_Curved_Element_Test"


def _pair(mode, p, alpha=1.0, bc=1):
    m, V, E, els, nodes = curved_box(mode=mode, bump=0.03 if mode == "all" else 0.05, bc=bc)
    mesh = dg.Mesh(V, E, m.bdr_faces, m.bdr_codes, curved_elems=els, curved_nodes=nodes)
    op = dg.Operator(mesh, order=p, alpha=alpha)
    orc = po.Oracle(V, E, p, alpha, 3, m.bdr_faces, m.bdr_codes)
    orc.set_curved(els, nodes)
    return op, orc


@pytest.mark.parametrize("mode,p,alpha", [("all", 2, 1.0), ("edge", 3, 0.0), ("edge", 2, 0.5)])
def test_curved_mult_matches_oracle(torch_cuda, mode, p, alpha):
    op, orc = _pair(mode, p, alpha)
    x = np.random.default_rng(3).standard_normal(op.state_len)
    assert rel_l2(op.mult_host(x, 0.0), orc.mult(x)) <= 1e-12


@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_curved_run_matches_oracle(torch_cuda, integrator):
    op, orc = _pair("all", 2, bc=3)
    X = orc.nodes()
    N = X.shape[1]
    x0 = np.zeros(op.state_len)
    x0[N:2 * N] = np.exp(-np.sum((X - 0.5) ** 2, axis=0) / 0.02)   # Ey bump in the curved box
    x, n = op.run_host(x0, 0.0, 0.01, 0.5, integrator)
    xo, no = orc.run(x0, 0.0, 0.01, 0.5, integrator)
    assert n == no == 50 and np.linalg.norm(xo) > 0.1 and rel_l2(x, xo) <= 1e-11


def test_curved_cavity_keeps_its_energy(torch_cuda):
    """Centred flux, PEC walls, every element curved: the semi-discrete operator conserves the
    discrete energy, so 400 RK4 steps change it by RK4's own dissipation only."""
    torch = torch_cuda
    op, orc = _pair("all", 2, alpha=0.0)
    X = orc.nodes()
    N = X.shape[1]
    x0 = np.zeros(op.state_len)
    x0[2 * N:3 * N] = np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])   # Ez of the TE110 shape
    u = torch.from_numpy(x0.copy()).cuda()
    op.step(u, 0.0, 0.005, 400)
    torch.cuda.synchronize()
    x = u.cpu().numpy()
    xo = orc.step(x0, 0.0, 0.005, 400)
    assert rel_l2(x, xo) <= 1e-11
    assert abs(np.linalg.norm(x) / np.linalg.norm(x0) - 1.0) < 0.05


def test_reference_curved_case_matches_oracle(torch_cuda):
    """The reference's 3D_Curved_Element_Test: centred flux (alpha 0), PEC/PMC walls on a
    cylinder-like surface of curved tetrahedra, SMA ends, a TF/SF plane wave; 200 steps of 0.01."""
    c = dg.Case(REF_CURVED / "3D_Curved_Element_Test.json")
    mesh = c.mesh()
    assert len(mesh.curved_elems) == 122
    op = dg.Operator(mesh, order=c.info["order"], alpha=c.info["alpha"])
    op.set_planewaves(c.planewaves())
    orc = po.Oracle.from_mesh(mesh, c.info["order"], alpha=c.info["alpha"])
    orc.set_curved(mesh.curved_elems, mesh.curved_nodes)
    orc.set_planewaves(c.planewaves())
    x0 = np.zeros(op.state_len)
    x, n = op.run_host(x0, 0.0, c.info["time_step"], 2.0)
    xo, no = orc.run(x0, 0.0, c.info["time_step"], 2.0)
    assert n == no == 200 and np.linalg.norm(xo) > 0.1 and rel_l2(x, xo) <= 1e-10


def test_reference_curved_case_runs(torch_cuda, tmp_path):
    c = dg.Case(REF_CURVED / "3D_Curved_Element_Test.json")
    state, res = c.run(out_dir=tmp_path)
    assert res["steps"] == 4500 and res["unstable_step"] == -1 and np.all(np.isfinite(state))


def test_curved_refusals(torch_cuda):
    m, V, E, els, nodes = curved_box(mode="edge")
    mesh = dg.Mesh(V, E, m.bdr_faces, m.bdr_codes, curved_elems=els, curved_nodes=nodes)
    with pytest.raises(dg.DgtdError, match="curved .* FP64"):
        dg.Operator(mesh, order=2, precision=dg.FP32)
    bad = nodes.copy()
    bad[0, 0] += 1e-3   # a corner that is not the element's vertex
    with pytest.raises(dg.DgtdError, match="corners must be the element's vertices"):
        dg.Operator(dg.Mesh(V, E, m.bdr_faces, m.bdr_codes, curved_elems=els, curved_nodes=bad), order=2)


REF_CYL = Path(__file__).resolve().parent / "golden" / "cases" / "reference" / "3D_Resonant_Cylinder"


def _cylinder_error(torch, curved: bool, steps: int = 370):
    """The reference's 3D_Resonant_Cylinder (PEC cylinder of radius 1, one refinement, order 3,
    dt 2.5e-3): its initial Ez = J6(alpha rho) cos(6 phi) is the TM(6,2) cavity mode, so every node
    oscillates as cos(alpha t), alpha = 13.589290170541217. Returns the largest deviation from that
    over `steps` steps (two periods) at the node nearest (0, 0.52, 0), relative to its amplitude."""
    c = dg.Case(REF_CYL / "3D_Resonant_Cylinder.json")
    mesh = c.mesh()
    if not curved:
        mesh.curved_elems = np.zeros(0, np.int32)
        mesh.curved_nodes = np.zeros((0, 10, 3))
    op = dg.Operator(mesh, order=c.info["order"], alpha=c.info["alpha"])
    X = op.node_coords()
    N = X.shape[1]
    x0 = c.initial_state(X)
    k = int(np.argmin(X[0] ** 2 + (X[1] - 0.52) ** 2 + X[2] ** 2))
    amp = x0[2 * N + k]
    u = torch.from_numpy(x0).cuda()
    dt, alpha, worst = c.info["time_step"], 13.589290170541217, 0.0
    for s in range(steps):
        op.step(u, s * dt, dt, 1)
        v = float(u[2 * N + k].item())
        worst = max(worst, abs(v - amp * np.cos(alpha * (s + 1) * dt)))
    op.close()
    return worst / abs(amp)


def test_reference_resonant_cylinder_follows_its_cavity_mode(torch_cuda):
    """Curved walls matter: on the refined cylinder (6,648 of 17,152 tetrahedra curved) the mode
    stays within 3.5 % of cos(alpha t) over two periods (the unrefined mesh at order 3 gives 3.7 %
    in the oracle), and closer than with the same mesh taken as straight-sided."""
    e_curved = _cylinder_error(torch_cuda, True)
    e_straight = _cylinder_error(torch_cuda, False)
    assert e_curved <= 0.035 and e_curved < e_straight


@pytest.mark.parametrize("name", ["3D_Resonant_Cylinder", "3D_Resonant_Sphere"])
def test_reference_resonators_run(torch_cuda, tmp_path, name):
    c = dg.Case(Path(__file__).resolve().parent / "golden" / "cases" / "reference" / name / f"{name}.json")
    state, res = c.run(out_dir=tmp_path)
    assert res["unstable_step"] == -1 and np.all(np.isfinite(state))
    assert res["steps"] == round(c.info["final_time"] / c.info["time_step"])
