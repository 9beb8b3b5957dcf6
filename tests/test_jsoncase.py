"""JSON-case front end on the host: the reference's case schema and gmsh 2.2 meshes
read into the library's tables (no GPU needed).

Fixtures: tests/golden/cases/ (written by tests/golden/make_cases.py from the
library's box mesher, so every expected count is known exactly).
"""
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg

CASES = Path(__file__).resolve().parent / "golden" / "cases"
REFERENCE_INPUTS = CASES / "reference"   # copied by tests/golden/copy_reference_cases.py


def orient(V, t):
    a, b, c, d = V[t[0]], V[t[1]], V[t[2]], V[t[3]]
    return np.dot(b - a, np.cross(c - a, d - a))


def test_resonant_case_tables():
    c = dg.Case(CASES / "box_resonant.json")
    inf = c.info
    assert inf["order"] == 2 and inf["time_step"] == 1e-2 and inf["final_time"] == 0.3 and inf["alpha"] == 1.0
    assert inf["n_elements"] == 162 and inf["n_point_probes"] == 2 and inf["n_waves"] == 0
    m = c.mesh()
    assert all(orient(m.vertices, t) > 0 for t in m.elements)
    # PEC on the 4 x/y walls, PMC on the 2 z walls, 18 triangles per wall
    assert (m.bdr_codes == dg.BC_PEC).sum() == 4 * 18 and (m.bdr_codes == dg.BC_PMC).sum() == 2 * 18
    assert np.allclose(c.point_probes(), [[0.5, 0.5, 0.5], [0.25, 0.5, 0.75]])
    info = dg.validate_mesh(m, order=2)
    assert info["n_elements"] == 162
    # resonant mode (1, 1): Ez = sin(pi x) sin(pi y) at the nodes
    xyz = np.random.default_rng(1).uniform(0, 1, (3, 50))
    u = c.initial_state(xyz).reshape(6, -1)
    assert np.allclose(u[2], np.sin(np.pi * xyz[0]) * np.sin(np.pi * xyz[1]), atol=1e-15)
    assert np.abs(np.delete(u, 2, axis=0)).max() == 0.0


def test_tfsf_case_orientation_and_auto_delay():
    c = dg.Case(CASES / "box_tfsf.json")
    m = c.mesh()
    assert (m.bdr_codes == dg.BC_SMA).sum() == 6 * 32
    nt = m.tfsf_faces.shape[0]
    assert nt == 6 * 4 * 2
    # the winding normal of every TF/SF face points into the total-field box [-0.5, 0.5]^3
    V = m.vertices
    for f in m.tfsf_faces:
        n = np.cross(V[f[1]] - V[f[0]], V[f[2]] - V[f[0]])
        assert np.dot(n, -V[f].mean(axis=0)) > 0
    # the mesh tables accept the faces (validation builds the TF/SF submesh)
    assert dg.validate_mesh(m, order=2)["n_tfsf_faces"] == 2 * nt
    (w,) = c.planewaves()
    assert w["propagation"] == [1.0, 0.0, 0.0] and w["frequency"] == 0.0
    # automatic delay: earliest TF/SF face centroid along k is x = -0.5
    assert w["mean"] == pytest.approx(-0.5 - 5.0 * 0.2 * np.sqrt(2.0), abs=1e-14)
    faces = c.surface(0)
    assert faces.shape == (nt, 3)
    for f in faces:                               # surface faces oriented outwards
        n = np.cross(V[f[1]] - V[f[0]], V[f[2]] - V[f[0]])
        assert np.dot(n, V[f].mean(axis=0)) > 0


def test_refined_dielectric_case():
    c = dg.Case(CASES / "box_dielectric.json")
    inf = c.info
    assert inf["n_elements"] == 48 * 8 and inf["integrator"] == dg.LSERK4 and inf["alpha"] == 0.5
    assert inf["time_step"] == 0.0 and inf["cfl"] == 0.5
    m = c.mesh()
    assert all(orient(m.vertices, t) > 0 for t in m.elements)
    vol = sum(orient(m.vertices, t) for t in m.elements) / 6.0
    assert vol == pytest.approx(1.0, abs=1e-13)
    assert m.bdr_codes.shape[0] == 6 * 8 * 4 and (m.bdr_codes == dg.BC_PEC).all()
    cen = m.vertices[m.elements].mean(axis=1)
    low = cen[:, 2] < 0.5
    assert np.all(m.eps[low] == 2.0) and np.all(m.eps[~low] == 1.0)
    assert np.allclose(m.sigma[low], 0.001 * 376.730313668) and np.all(m.sigma[~low] == 0.0)
    assert dg.validate_mesh(m, order=3)["n_elements"] == 384
    xyz = np.random.default_rng(2).uniform(0, 1, (3, 20))
    u = c.initial_state(xyz).reshape(6, -1)
    g = np.exp(-((xyz - 0.5) ** 2).sum(axis=0) / (2 * 0.2 ** 2))
    assert np.allclose(u[3], g) and np.abs(u[[0, 1, 2, 4, 5]]).max() == 0.0


def test_rejects_unsupported_and_malformed(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('{"solver_options": {"order": 2}, "model": {"filename": "box.msh", "materials": []')
    with pytest.raises(dg.DgtdError, match="JSON parse error"):
        dg.Case(bad)
    src = (CASES / "box_resonant.json").read_text().replace('"PMC"', '"SGBC"')
    (tmp_path / "box_resonant.msh").write_text((CASES / "box_resonant.msh").read_text())
    sg = tmp_path / "sgbc.json"
    sg.write_text(src)
    with pytest.raises(dg.DgtdError, match="not supported"):
        dg.Case(sg)
    nomesh = tmp_path / "nomesh.json"
    nomesh.write_text(src.replace("box_resonant.msh", "missing.msh"))
    with pytest.raises(dg.DgtdError, match="cannot open mesh"):
        dg.Case(nomesh)


@pytest.mark.parametrize("name", ["3D_PEC", "3D_TFSF", "3D_TFSF_InteriorPEC"])
def test_reference_cases_load(name):
    """The reference's own 3D case files load."""
    c = dg.Case(REFERENCE_INPUTS / name / f"{name}.json")
    m = c.mesh()
    assert m.n_elements > 0 and c.info["order"] >= 1
    dg.validate_mesh(m, order=1)
