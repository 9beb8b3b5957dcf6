"""JSON-case front end on the host: the reference's case schema and gmsh 2.2 meshes
read into the library's tables (no GPU needed).

Fixtures: tests/golden/cases/<case>/ (written by tests/golden/make_cases.py from the
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
    c = dg.Case(CASES / "box_resonant" / "box_resonant.json")
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
    c = dg.Case(CASES / "box_tfsf" / "box_tfsf.json")
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
    c = dg.Case(CASES / "box_dielectric" / "box_dielectric.json")
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
    # the reference's conversion: sigma * mu0_SI * c_SI, mu0_SI = 4 pi 1e-7 (PhysicalConstants.h)
    z0 = 4.0 * np.pi * 1e-7 * 299792458.0
    assert np.all(m.sigma[low] == 0.001 * z0) and np.all(m.sigma[~low] == 0.0)
    assert dg.validate_mesh(m, order=3)["n_elements"] == 384
    xyz = np.random.default_rng(2).uniform(0, 1, (3, 20))
    u = c.initial_state(xyz).reshape(6, -1)
    g = np.exp(-((xyz - 0.5) ** 2).sum(axis=0) / (2 * 0.2 ** 2))
    assert np.allclose(u[3], g) and np.abs(u[[0, 1, 2, 4, 5]]).max() == 0.0


def _case_copy(tmp_path, src: str, name: str, edit=None, mesh=None) -> Path:
    """A copy of fixture case `src` as case `name` in the reference's layout
    (<tmp>/<name>/<name>.json and <name>.msh); edit(dict) may change the JSON."""
    import json
    d = tmp_path / name
    d.mkdir()
    case = json.loads((CASES / src / f"{src}.json").read_text())
    case["model"]["filename"] = f"{name}.msh"
    if edit:
        edit(case)
    (d / f"{name}.json").write_text(json.dumps(case))
    if mesh is None:
        (d / f"{name}.msh").write_text((CASES / src / f"{src}.msh").read_text())
    else:
        mesh(CASES / src / f"{src}.msh", d / f"{name}.msh")
    return d / f"{name}.json"


def test_rejects_unsupported_and_malformed(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('{"solver_options": {"order": 2}, "model": {"filename": "box.msh", "materials": []')
    with pytest.raises(dg.DgtdError, match="JSON parse error"):
        dg.Case(bad)

    def sgbc(c):
        for b in c["model"]["boundaries"]:
            if b["type"] == "PMC":
                b["type"] = "SGBC"
    with pytest.raises(dg.DgtdError, match="must define either 'material' or 'layers'"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "sgbc", sgbc))

    def unknown(c):
        c["model"]["boundaries"][0]["type"] = "SIBC"
    with pytest.raises(dg.DgtdError, match="not supported"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "unknown_bc", unknown))

    # a plane wave's Gaussian mean is a position (the reference fails on a plain number too)
    def scalar_mean(c):
        c["sources"][0]["magnitude"]["mean"] = 5.0
    with pytest.raises(dg.DgtdError, match="magnitude.mean must be a 3-vector"):
        dg.Case(_case_copy(tmp_path, "box_tfsf", "scalar_mean", scalar_mean))


def test_case_naming_style(tmp_path):
    """The reference's case layout (driver.cpp:1487-1543, and its DriverTest
    throwsWhenCaseNamingStyleIsInconsistent): a folder named as the case holding <case>.json
    and <case>.msh, with model.filename = "<case>.msh"."""
    import json
    ok = _case_copy(tmp_path, "box_resonant", "named_ok")
    assert dg.Case(ok).info["n_elements"] == 162
    # model.filename naming another mesh (the reference test's case)
    d = tmp_path / "DriverStyleCheckMismatch"
    d.mkdir()
    (d / "DriverStyleCheckMismatch.json").write_text(json.dumps({"model": {"filename": "WrongMeshName.msh"}}))
    with pytest.raises(dg.DgtdError, match="naming style"):
        dg.Case(d / "DriverStyleCheckMismatch.json")
    # folder not named as the case
    other = tmp_path / "elsewhere"
    other.mkdir()
    (other / "named_ok.json").write_text(ok.read_text())
    (other / "named_ok.msh").write_text((ok.parent / "named_ok.msh").read_text())
    with pytest.raises(dg.DgtdError, match="naming style"):
        dg.Case(other / "named_ok.json")
    # mesh file missing
    (ok.parent / "named_ok.msh").unlink()
    with pytest.raises(dg.DgtdError, match="naming style"):
        dg.Case(ok)
    # model.filename absent
    (d / "DriverStyleCheckMismatch.json").write_text(json.dumps({"model": {}}))
    with pytest.raises(dg.DgtdError, match="model.filename is required"):
        dg.Case(d / "DriverStyleCheckMismatch.json")


@pytest.mark.parametrize("name", ["3D_PEC", "3D_TFSF", "3D_TFSF_InteriorPEC", "3D_Resonant_Box_TM55_H1_P3",
                                  "3D_Resonant_Box_TM55_H0_P2_PERF"])
def test_reference_cases_load(name):
    """The reference's own 3D case files load."""
    c = dg.Case(REFERENCE_INPUTS / name / f"{name}.json")
    m = c.mesh()
    assert m.n_elements > 0 and c.info["order"] >= 1
    dg.validate_mesh(m, order=1)


@pytest.mark.parametrize("name,tets,order,final", [("3D_Resonant_Box_TM55_H1_P3", 2800, 3, 10.0),
                                                   ("3D_Resonant_Box_TM55_H0_P2_PERF", 350, 2, 2.0)])
def test_reference_tm55_cases(name, tets, order, final):
    """The resonant-box inputs (the TM55 convergence study and the Performance set): the unit cube of
    350 tetrahedra, one uniform refinement in H1, PEC walls, and the initial field Ez = sin(5 pi x)
    sin(5 pi y) of the TM(5,5) cavity mode (the exact solution the reference's L2 error analysis
    uses, test/cases/L2ErrorAnalysis.cpp:32-54) at every node, the other components zero."""
    c = dg.Case(REFERENCE_INPUTS / name / f"{name}.json")
    m = c.mesh()
    assert m.n_elements == tets and c.info["order"] == order
    assert c.info["time_step"] == 1e-4 and c.info["final_time"] == final and c.info["alpha"] == 1.0
    V = np.asarray(m.vertices)
    assert np.allclose(V.min(0), 0.0) and np.allclose(V.max(0), 1.0)
    assert set(np.unique(m.bdr_codes).tolist()) == {dg.BC_PEC}
    from oracle import pyoracle as po
    orc = po.Oracle.from_mesh(m, order)
    X = orc.nodes()
    N = X.shape[1]
    x0 = c.initial_state(X)
    ez = np.sin(5 * np.pi * X[0]) * np.sin(5 * np.pi * X[1])
    assert np.abs(x0[2 * N:3 * N] - ez).max() <= 1e-14
    assert np.count_nonzero(x0[:2 * N]) == 0 and np.count_nonzero(x0[3 * N:]) == 0


def _second_order_copy(src: Path, dst: Path, bump: float = 0.0) -> None:
    """Rewrite a linear gmsh 2.2 mesh with second-order elements: a node at every edge midpoint
    (shared by the elements of the edge), tetrahedra as type 11, triangles as type 9. bump > 0
    moves the first edge node off its edge by that distance."""
    lines = src.read_text().splitlines()
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    nodes = {}
    for ln in lines[i + 2:i + 2 + n]:
        k, x, y, z = ln.split()
        nodes[int(k)] = np.array([float(x), float(y), float(z)])
    j = lines.index("$Elements")
    ne = int(lines[j + 1])
    mids, elems = {}, []
    next_id = max(nodes) + 1

    def mid(a, b):
        nonlocal next_id
        key = (min(a, b), max(a, b))
        if key not in mids:
            mids[key] = next_id
            nodes[next_id] = 0.5 * (nodes[a] + nodes[b])
            next_id += 1
        return mids[key]

    for ln in lines[j + 2:j + 2 + ne]:
        f = [int(v) for v in ln.split()]
        eid, typ, ntag = f[0], f[1], f[2]
        tags, vs = f[3:3 + ntag], f[3 + ntag:]
        if typ == 4:
            a, b, c, d = vs
            extra = [mid(a, b), mid(b, c), mid(a, c), mid(a, d), mid(c, d), mid(b, d)]
            elems.append((eid, 11, tags, vs + extra))
        elif typ == 2:
            a, b, c = vs
            elems.append((eid, 9, tags, vs + [mid(a, b), mid(b, c), mid(a, c)]))
        else:
            elems.append((eid, typ, tags, vs))
    if bump:
        first = next(iter(mids.values()))
        nodes[first] = nodes[first] + np.array([bump, 0.0, 0.0])
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(len(nodes))]
    out += [f"{k} {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}" for k, v in sorted(nodes.items())]
    out += ["$EndNodes", "$Elements", str(len(elems))]
    out += [" ".join(map(str, [e, t, len(g)] + g + v)) for e, t, g, v in elems]
    out += ["$EndElements"]
    dst.write_text("\n".join(out) + "\n")


def test_straight_second_order_mesh_loads_as_linear(tmp_path):
    """A second-order mesh whose edge nodes sit on the straight edges (the reference's
    curved-element test: high-order nodes within 1e-5 of the linear positions) loads as its
    linear elements: same tables as the linear mesh."""
    lin = dg.Case(CASES / "box_resonant" / "box_resonant.json")
    quad = dg.Case(_case_copy(tmp_path, "box_resonant", "box_p2", mesh=_second_order_copy))
    ml, mq = lin.mesh(), quad.mesh()
    assert quad.info["n_elements"] == lin.info["n_elements"]
    assert np.array_equal(ml.vertices[ml.elements], mq.vertices[mq.elements])
    assert {k: v for k, v in quad.info.items() if k not in ("mesh_path", "name")} == \
        {k: v for k, v in lin.info.items() if k not in ("mesh_path", "name")}


def test_curved_second_order_mesh_keeps_its_geometry(tmp_path):
    """A second-order mesh with an edge node moved off its edge: the tetrahedra on that edge are
    curved (the reference's test, HesthavenEvolution.cpp:207-241) and keep their ten geometry nodes
    (corners in the element's vertex order, then the edges (0,1) (0,2) (0,3) (1,2) (1,3) (2,3))."""
    bumped = dg.Case(_case_copy(tmp_path, "box_resonant", "box_p2c",
                                mesh=lambda src, dst: _second_order_copy(src, dst, bump=1e-3)))
    m = bumped.mesh()
    assert 1 <= len(m.curved_elems) <= 8 and m.curved_nodes.shape == (len(m.curved_elems), 10, 3)
    pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    devs = []
    for i, e in enumerate(m.curved_elems):
        G = m.curved_nodes[i]
        assert np.array_equal(G[:4], m.vertices[m.elements[e]])
        devs += [np.linalg.norm(G[4 + q] - 0.5 * (G[a] + G[b])) for q, (a, b) in enumerate(pairs)]
    assert max(devs) == pytest.approx(1e-3, rel=1e-9) and sorted(devs)[-len(m.curved_elems) - 1] < 1e-12
    # the reference's own curved case: 122 curved tetrahedra, edge nodes up to 8.8e-3 off
    c = dg.Case(REFERENCE_INPUTS / "3D_Curved_Element_Test" / "3D_Curved_Element_Test.json")
    mc = c.mesh()
    assert len(mc.curved_elems) == 122
    dev = max(np.linalg.norm(G[4 + q] - 0.5 * (G[a] + G[b])) for G in mc.curved_nodes for q, (a, b) in enumerate(pairs))
    assert 8.8e-3 < dev < 8.9e-3
    assert dg.validate_mesh(mc, order=2)["n_elements"] == 1151

    # refinement: children on the parent's second-order map; the bumped edge's node becomes a
    # vertex, and the children along that edge stay curved
    def refine(cj):
        cj["model"]["refinement"] = 1
    r = dg.Case(_case_copy(tmp_path, "box_resonant", "box_p2r", refine,
                           mesh=lambda src, dst: _second_order_copy(src, dst, bump=1e-3))).mesh()
    assert r.n_elements == 8 * m.n_elements and len(r.curved_elems) > len(m.curved_elems)
    bumped = [G[4 + q] for G in m.curved_nodes for q, (a, b) in enumerate(pairs)
              if np.linalg.norm(G[4 + q] - 0.5 * (G[a] + G[b])) > 1e-6]
    assert np.min(np.linalg.norm(r.vertices - bumped[0], axis=1)) < 1e-14
    assert dg.validate_mesh(r, order=3)["n_elements"] == r.n_elements


def test_material_rules_follow_the_reference(tmp_path):
    """driver.cpp:946-982 and Model.cpp:61-66: the first material entry of a tag wins; a
    material tag the mesh does not have is an error; no materials at all means vacuum on
    attribute 1."""
    def dup(c):
        c["model"]["materials"] = [{"tags": [1], "relative_permittivity": 2.0},
                                   {"tags": [1], "relative_permittivity": 3.0}]
    m = dg.Case(_case_copy(tmp_path, "box_resonant", "dup_tag", dup)).mesh()
    assert np.all(m.eps == 2.0)

    def absent(c):
        c["model"]["materials"] = [{"tags": [1]}, {"tags": [99], "relative_permittivity": 4.0}]
    with pytest.raises(dg.DgtdError, match="no attribute 99 defined in the mesh"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "absent_tag", absent))

    def none(c):
        c["model"]["materials"] = []
    m = dg.Case(_case_copy(tmp_path, "box_resonant", "no_materials", none)).mesh()
    assert np.all(m.eps == 1.0) and np.all(m.mu == 1.0) and np.all(m.sigma == 0.0)


def test_boundary_rules_follow_the_reference(tmp_path):
    """driver.cpp:985-1049: every boundary entry needs non-empty tags and a type, and the first
    entry of a tag wins (the resonant box: tags 1-4 PEC, 5-6 PMC, 18 triangles per wall)."""
    def dup(c):
        c["model"]["boundaries"] = [{"tags": [1, 2, 3, 4], "type": "PEC"}, {"tags": [5, 6], "type": "PMC"},
                                    {"tags": [5], "type": "SMA"}]
    m = dg.Case(_case_copy(tmp_path, "box_resonant", "dup_bdr", dup)).mesh()
    codes, counts = np.unique(m.bdr_codes, return_counts=True)
    assert dict(zip(codes.tolist(), counts.tolist())) == {dg.BC_PEC: 72, dg.BC_PMC: 36}

    def no_tags(c):
        c["model"]["boundaries"][1]["tags"] = []
    with pytest.raises(dg.DgtdError, match="boundary 1 'tags' are empty"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "no_tags", no_tags))

    def no_type(c):
        del c["model"]["boundaries"][0]["type"]
    with pytest.raises(dg.DgtdError, match="boundary 0 does not have a defined 'type'"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "no_type", no_type))


def _with_interior_triangle(src: Path, dst: Path, tag: int) -> None:
    """Copy a gmsh 2.2 mesh and add one triangle with physical tag `tag` on a face shared by
    two tetrahedra."""
    lines = src.read_text().splitlines()
    j = lines.index("$Elements")
    ne = int(lines[j + 1])
    faces = {}
    for ln in lines[j + 2:j + 2 + ne]:
        f = [int(v) for v in ln.split()]
        if f[1] != 4:
            continue
        vs = f[3 + f[2]:]
        for q in range(4):
            key = tuple(sorted(vs[:q] + vs[q + 1:]))
            faces[key] = faces.get(key, 0) + 1
    shared = next(k for k, n in faces.items() if n == 2)
    eid = max(int(ln.split()[0]) for ln in lines[j + 2:j + 2 + ne]) + 1
    new = f"{eid} 2 2 {tag} {tag} {shared[0]} {shared[1]} {shared[2]}"
    lines = lines[:j + 1] + [str(ne + 1)] + lines[j + 2:j + 2 + ne] + [new] + lines[j + 2 + ne:]
    dst.write_text("\n".join(lines) + "\n")


def test_mixed_interior_exterior_tag_is_an_interior_boundary(tmp_path):
    """A tag with any face between two elements is an interior boundary as a whole: its interior
    faces get the condition and its faces on the domain boundary keep none (the reference's
    per-tag classification, driver.cpp:1024-1048)."""
    m = dg.Case(_case_copy(tmp_path, "box_resonant", "mixed_tag",
                           mesh=lambda s, d: _with_interior_triangle(s, d, 1))).mesh()
    codes, counts = np.unique(m.bdr_codes, return_counts=True)
    assert dict(zip(codes.tolist(), counts.tolist())) == {dg.BC_PEC: 54, dg.BC_PMC: 36}
    assert m.int_codes.tolist() == [dg.BC_PEC]


def test_solver_option_names_follow_the_reference(tmp_path):
    """SolverOptions.h:8-16 / Solver.cpp:41-77: ode_type is a number, 0 = RK4 and 1-6 the
    implicit solvers; driver.cpp:679-691: evolution_operator is maxwell, global or hesthaven."""
    def ode(n):
        return lambda c: c.setdefault("solver_options", {}).__setitem__("ode_type", n)
    c = dg.Case(_case_copy(tmp_path, "box_resonant", "ode0", ode(0)))
    assert c.info["integrator"] == dg.RK4
    with pytest.raises(dg.DgtdError, match="implicit ode_type 2 is not supported"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "ode2", ode(2)))
    with pytest.raises(dg.DgtdError, match="wrong ode type"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "ode9", ode(9)))
    c = dg.Case(_case_copy(tmp_path, "box_resonant", "odes", ode("LSERK4")))
    assert c.info["integrator"] == dg.LSERK4

    def evo(name):
        return lambda c: c.setdefault("solver_options", {}).__setitem__("evolution_operator", name)
    for name in ("maxwell", "global", "hesthaven"):
        dg.Case(_case_copy(tmp_path, "box_resonant", f"evo_{name}", evo(name)))
    with pytest.raises(dg.DgtdError, match="wrong type of evolution operator"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "evo_bad", evo("spectral")))


def test_basis_types(tmp_path):
    """The reference's basis_type is MFEM's BasisType number: Gauss-Lobatto (1) and Gauss-Legendre
    (0) load (the case info keeps which), others (e.g. 2, positive) are refused, not ignored."""
    def bt(n):
        return lambda c: c.setdefault("solver_options", {}).__setitem__("basis_type", n)
    assert dg.Case(_case_copy(tmp_path, "box_resonant", "bt1", bt(1))).info["basis_type"] == 1
    assert dg.Case(_case_copy(tmp_path, "box_resonant", "bt0", bt(0))).info["basis_type"] == 0
    with pytest.raises(dg.DgtdError, match="basis_type 2 is not supported"):
        dg.Case(_case_copy(tmp_path, "box_resonant", "bt2", bt(2)))


def test_point_probe_file_format(tmp_path):
    """The case runner's point-probe files follow the reference's layout; this writes one with the
    runner's format strings (case_api.cu) and reads it back with the tests' parser."""
    from conftest import read_point_probe
    c = 299792458.0
    x = (0.5, 0.25, 0.75)
    lines = ["PointProbe ID 0", "Spatial Position (X, Y, Z) ", "%f %f %f" % x,
             "Time (s) // Ex // Ey // Ez // Hx // Hy // Hz "]
    t = np.array([0.0, 0.01, 0.02])
    v = np.arange(18, dtype=float).reshape(3, 6) * 0.1
    lines += ["%.10e %.10e %.10e %.10e %.10e %.10e %.10e" % ((t[r] / c,) + tuple(v[r])) for r in range(3)]
    (tmp_path / "PointProbe0.dat").write_text("\n".join(lines) + "\n")
    rows = read_point_probe(tmp_path / "PointProbe0.dat")
    assert rows.shape == (3, 7)
    assert np.allclose(rows[:, 0], t, rtol=1e-9, atol=1e-14) and np.allclose(rows[:, 1:], v)


def test_solver_option_defaults_follow_the_reference(tmp_path):
    """Without solver_options the reference runs order 2, upwind alpha 1, final time 2, an
    automatic time step at cfl 1 (SolverOptions.h, EvolutionOptions.h)."""
    def bare(c):
        c.pop("solver_options", None)
    inf = dg.Case(_case_copy(tmp_path, "box_resonant", "bare", bare)).info
    assert inf["order"] == 2 and inf["alpha"] == 1.0 and inf["final_time"] == 2.0
    assert inf["time_step"] == 0.0 and inf["cfl"] == 1.0


def test_automatic_time_step_follows_the_reference(tmp_path):
    """Solver::estimateTimeStep (Solver.cpp:289-345) for the three 3D evolution operators, on
    the host: global = the oracle's restatement (base / 0.8); maxwell = base; hesthaven =
    cfl / (max Fscale p^2) with Fscale = 2 sJ / J = (2/3) area / volume per face."""
    from oracle import pyoracle as po

    def opts(op, cfl=0.7):
        def edit(c):
            so = c.setdefault("solver_options", {})
            so["time_step"] = 0.0
            so["cfl"] = cfl
            if op:
                so["evolution_operator"] = op
        return edit
    glob_ = dg.Case(_case_copy(tmp_path, "box_tfsf", "dt_global", opts(None)))
    mesh = glob_.mesh()
    p = glob_.info["order"]
    want = po.estimate_dt_3d(mesh, p, 0.7)
    assert abs(glob_.auto_dt() - want) <= 1e-15 * want
    mx = dg.Case(_case_copy(tmp_path, "box_tfsf", "dt_maxwell", opts("maxwell"))).auto_dt()
    assert abs(mx - 0.8 * want) <= 1e-14 * want
    P = mesh.vertices[mesh.elements]
    vol = np.abs(np.einsum("ki,ki->k", P[:, 1] - P[:, 0], np.cross(P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]))) / 6.0
    fmax = 0.0
    for f in ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)):
        area = 0.5 * np.linalg.norm(np.cross(P[:, f[1]] - P[:, f[0]], P[:, f[2]] - P[:, f[0]]), axis=1)
        fmax = max(fmax, float(np.max(2.0 / 3.0 * area / vol)))
    he = dg.Case(_case_copy(tmp_path, "box_tfsf", "dt_hesthaven", opts("hesthaven"))).auto_dt()
    assert abs(he - 0.7 / (fmax * p * p)) <= 1e-12 * he


def test_oracle_tm55_mode_one_period():
    """The oracle on the reference's TM55 box (H1: 2,800 tetrahedra) at order 2 follows the exact
    TM(5,5) mode (test/cases/L2ErrorAnalysis.cpp:32-54) over one period of 200 steps to 0.214
    relative L2 in Ez: the figure the GPU test holds the product to."""
    from oracle import pyoracle as po
    name = "3D_Resonant_Box_TM55_H1_P3"
    c = dg.Case(REFERENCE_INPUTS / name / f"{name}.json")
    orc = po.Oracle.from_mesh(c.mesh(), 2, alpha=c.info["alpha"])
    X = orc.nodes()
    N = X.shape[1]
    w = 5 * np.pi * np.sqrt(2.0)
    period = 2 * np.pi / w
    x, n = orc.run(c.initial_state(X), 0.0, period / 200, period)
    ez = np.sin(5 * np.pi * X[0]) * np.sin(5 * np.pi * X[1])
    err = np.linalg.norm(x[2 * N:3 * N] - ez * np.cos(w * period)) / np.linalg.norm(ez)
    assert n == 200 and 0.20 <= err <= 0.22
