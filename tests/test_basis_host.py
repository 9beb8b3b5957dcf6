"""The Gauss-Legendre basis (the reference's solver_options.basis_type 0) on the host: the product's
node set and change of basis against the oracle, which assembles the global operator directly on
the Gauss-Legendre node set (its own Bernstein-based Lagrange basis and quadrature).

The reference's integration rules are exact on straight tetrahedra (faces: order 2p + 1,
src/mfemExtension/IntegratorFunctions.cpp:7-35; volume: 2p - 1 and 2p), so its operator in either
basis is one semi-discrete system: A_legendre = M(lobatto -> legendre) A_lobatto M(legendre ->
lobatto) element by element. Bars: node sets 1e-13; operators 1e-12 relative.
"""
import json
import shutil
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

REF = Path(__file__).resolve().parent / "golden" / "cases" / "reference"
BLEG = "3D_Resonant_Box_BLEG_TM55_H0_P2_PERF"


def _blocks(x, M):
    """Apply the per-element matrix M to every (component, element) block of a state."""
    Np = M.shape[0]
    return (x.reshape(-1, Np) @ M.T).reshape(-1)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_legendre_nodes_match_oracle(p):
    """The product's node set of basis 0 on one tetrahedron equals the oracle's (the same MFEM
    construction restated separately), node for node in DOF order; no node lies on a face."""
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    orc = po.Oracle(V, np.array([[0, 1, 2, 3]], np.int32), p, 1.0, 3, np.zeros((0, 3), np.int32),
                    np.zeros(0, np.int32))
    orc.set_basis(0)
    b = dg.tet_nodes(p, dg.BASIS_GAUSS_LEGENDRE)
    X = orc.nodes()
    assert np.abs(b[:, 1:].T - X).max() <= 1e-13
    assert b.min() > 0.0 and np.abs(b.sum(axis=1) - 1).max() <= 1e-15
    bl = dg.tet_nodes(p, dg.BASIS_GAUSS_LOBATTO)
    orc_l = po.Oracle(V, np.array([[0, 1, 2, 3]], np.int32), p, 1.0, 3, np.zeros((0, 3), np.int32),
                      np.zeros(0, np.int32))
    assert np.abs(bl[:, 1:].T - orc_l.nodes()).max() <= 1e-13


@pytest.mark.parametrize("p", [1, 3, 6])
def test_basis_change_reproduces_polynomials(p):
    """M(from -> to) maps the nodal values of any degree-p polynomial on one node set to its values
    on the other, and the two directions are inverse."""
    rng = np.random.default_rng(p)
    bg, bl = dg.tet_nodes(p, 0), dg.tet_nodes(p, 1)
    exps = [(i, j, k) for i in range(p + 1) for j in range(p + 1 - i) for k in range(p + 1 - i - j)]
    coef = rng.standard_normal(len(exps))
    f = lambda b: sum(c * b[:, 1] ** i * b[:, 2] ** j * b[:, 3] ** k for c, (i, j, k) in zip(coef, exps))
    M = dg.tet_basis_change(p, 0, 1)
    Mi = dg.tet_basis_change(p, 1, 0)
    assert np.abs(M @ f(bg) - f(bl)).max() <= 1e-12 * np.abs(f(bl)).max()
    assert np.abs(M @ Mi - np.eye(M.shape[0])).max() <= 1e-13


@pytest.mark.parametrize("p,alpha,bc", [(1, 1.0, po.BC_PEC), (2, 1.0, po.BC_SMA), (3, 0.0, po.BC_PMC),
                                        (4, 0.5, po.BC_SMA)])
def test_legendre_operator_is_the_lobatto_operator_in_another_basis(p, alpha, bc):
    """The oracle's global operator assembled on the Gauss-Legendre nodes equals M A M^-1 of its
    Gauss-Lobatto operator with the product's change of basis, on a box with random materials
    and conductivity."""
    m = po.box_mesh((2, 2, 2), outer_bc=bc)
    K = np.asarray(m.elements).shape[0]
    rng = np.random.default_rng(7 + p)
    eps, mu, sig = 1 + rng.random(K), 1 + rng.random(K), 0.3 * rng.random(K)
    args = (m.vertices, m.elements, p, alpha, 3, m.bdr_faces, m.bdr_codes)
    gll = po.Oracle(*args, eps=eps, mu=mu, sigma=sig)
    gl = po.Oracle(*args, eps=eps, mu=mu, sigma=sig)
    gl.set_basis(0)
    x = rng.standard_normal(6 * K * dg.tet_nodes(p).shape[0])
    y = _blocks(gll.mult(_blocks(x, dg.tet_basis_change(p, 0, 1))), dg.tet_basis_change(p, 1, 0))
    assert rel_l2(gl.mult(x), y) <= 1e-12


def test_legendre_oracle_refuses_face_node_paths():
    m = po.box_mesh((1, 1, 1))
    o = po.Oracle(m.vertices, m.elements, 2, 1.0, 3, m.bdr_faces, m.bdr_codes)
    o.set_basis(0)
    x = np.zeros(6 * o.nodes().shape[1])
    with pytest.raises(RuntimeError, match="face nodes"):
        o.mult(x, form=po.NODAL)


def test_bleg_case_loads():
    """The reference's Performance input with basis_type 0 loads; its info says so."""
    c = dg.Case(REF / BLEG / f"{BLEG}.json")
    assert c.info["basis_type"] == dg.BASIS_GAUSS_LEGENDRE and c.info["order"] == 2
    assert c.mesh().n_elements == 350


@pytest.mark.parametrize("case,extra,match", [
    ("3D_TFSF", {"solver_options": {"basis_type": 0}}, "plane-wave"),
    (BLEG, {"solver_options": {"evolution_operator": "hesthaven"}}, "hesthaven"),
    (BLEG, {"solver_options": {"basis_type": 2}}, "basis_type 2"),
])
def test_legendre_case_refusals(tmp_path, case, extra, match):
    """Where the change of basis would not be exact the loader refuses basis_type 0: a plane wave
    (sampled at the case's nodes), the Hesthaven evolution (built on face nodes); other basis
    types are refused as before."""
    src = REF / case
    js = json.loads((src / f"{case}.json").read_text())
    for k, v in extra.items():
        js.setdefault(k, {}).update(v)
    d = tmp_path / case
    d.mkdir()
    (d / f"{case}.json").write_text(json.dumps(js))
    shutil.copyfile(src / f"{case}.msh", d / f"{case}.msh")
    with pytest.raises(dg.DgtdError, match=match):
        dg.Case(d / f"{case}.json")


def test_bleg_run_through_change_of_basis_is_the_legendre_run():
    """What the case runner does for the reference's BLEG input, restated on the oracle: the
    Gauss-Lobatto system started from M(GL -> GLL) x0 and mapped back after 500 RK4 steps (dt 1e-4)
    equals the Gauss-Legendre system run directly, to rounding (1e-13 relative L2)."""
    c = dg.Case(REF / BLEG / f"{BLEG}.json")
    m = c.mesh()
    gl = po.Oracle.from_mesh(m, 2, alpha=c.info["alpha"])
    gl.set_basis(0)
    x0 = c.initial_state(gl.nodes())
    xo, no = gl.run(x0, 0.0, c.info["time_step"], 0.05)
    gll = po.Oracle.from_mesh(m, 2, alpha=c.info["alpha"])
    x1, n1 = gll.run(_blocks(x0, dg.tet_basis_change(2, 0, 1)), 0.0, c.info["time_step"], 0.05)
    assert no == n1 == 500 and np.linalg.norm(xo) > 1.0
    assert rel_l2(_blocks(x1, dg.tet_basis_change(2, 1, 0)), xo) <= 1e-13
