"""Writes the small JSON cases and gmsh 2.2 meshes under tests/golden/cases/<case>/.

The cases follow the reference's case-file schema (solver_options / model /
sources / probes, as read by driver::buildSolverJson) and are built from this
library's structured box mesher, so their content is known exactly:
  box_resonant     unit cube, 3^3 hexes x 6 tets, PEC on x and y walls, PMC on z
                   walls, TE110 resonant initial field, order 2, two point probes;
  box_tfsf         [-1,1]^3, 4^3 hexes x 6 tets, SMA outer walls, TF/SF surface
                   around the central 2^3 hexes (tag 7, automatic delay), point and
                   rcssurface probes;
  box_dielectric   unit cube, 2^3 hexes x 6 tets refined once, two materials
                   (eps_r 2 with conductivity in the lower half), PEC walls,
                   3D Gaussian initial field.
Run: python tests/golden/make_cases.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent / "cases"


def case_dir(name: str) -> Path:
    """<cases>/<name>/: the reference's case layout (a folder named as the case holding
    <name>.json and <name>.msh)."""
    d = OUT / name
    d.mkdir(parents=True, exist_ok=True)
    return d


def write_msh(path, V, E, etag, F, ftag):
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(V))
        for i, v in enumerate(V):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, v[0], v[1], v[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % (len(F) + len(E)))
        k = 1
        for t, tag in zip(F, ftag):
            f.write("%d 2 2 %d %d %d %d %d\n" % (k, tag, tag, t[0] + 1, t[1] + 1, t[2] + 1)); k += 1
        for t, tag in zip(E, etag):
            f.write("%d 4 2 %d %d %d %d %d %d\n" % (k, tag, tag, t[0] + 1, t[1] + 1, t[2] + 1, t[3] + 1)); k += 1
        f.write("$EndElements\n")


def side_tags(V, F, lo, hi):
    """Tag of each boundary triangle by the box side it lies on: x-lo 1, x-hi 2, y-lo 3, y-hi 4, z-lo 5, z-hi 6."""
    tags = []
    for t in F:
        c = V[t].mean(axis=0)
        for d in range(3):
            if abs(c[d] - lo[d]) < 1e-12:
                tags.append(1 + 2 * d); break
            if abs(c[d] - hi[d]) < 1e-12:
                tags.append(2 + 2 * d); break
        else:
            raise RuntimeError("face not on the box boundary")
    return tags


def main():
    import dgtd_gb300 as dg
    OUT.mkdir(exist_ok=True)

    # ---- box_resonant
    m = dg.box_mesh((3, 3, 3))
    tags = side_tags(m.vertices, m.bdr_faces, (0, 0, 0), (1, 1, 1))
    write_msh(case_dir("box_resonant") / "box_resonant.msh", m.vertices, m.elements, [1] * m.n_elements, m.bdr_faces, tags)
    case = {
        "solver_options": {"upwind_alpha": 1.0, "time_step": 1e-2, "final_time": 0.3, "order": 2,
                           "evolution_operator": "global"},
        "model": {"filename": "box_resonant.msh",
                  "materials": [{"tags": [1], "type": "vacuum"}],
                  "boundaries": [{"tags": [1, 2, 3, 4], "type": "PEC"}, {"tags": [5, 6], "type": "PMC"}]},
        "probes": {"exporter": {"steps": 10},
                   "point": [{"position": [0.5, 0.5, 0.5], "steps": 1}, {"position": [0.25, 0.5, 0.75], "steps": 1}]},
        "sources": [{"type": "initial", "field_type": "electric", "polarization": [0.0, 0.0, 1.0],
                     "magnitude": {"type": "resonant", "modes": [1, 1]}}],
    }
    (case_dir("box_resonant") / "box_resonant.json").write_text(json.dumps(case, indent=2) + "\n")

    # ---- box_tfsf
    m = dg.box_mesh((4, 4, 4), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1, 1, 1), (3, 3, 3)), outer_bc=dg.BC_SMA)
    tags = side_tags(m.vertices, m.bdr_faces, (-1, -1, -1), (1, 1, 1))
    cen = m.vertices[m.elements].mean(axis=1)
    etag = [2 if np.all(np.abs(c) < 0.5) else 1 for c in cen]
    F = np.concatenate([m.bdr_faces, m.tfsf_faces[:, ::-1]])      # reversed: the file's winding carries no meaning
    write_msh(case_dir("box_tfsf") / "box_tfsf.msh", m.vertices, m.elements, etag, F, tags + [7] * len(m.tfsf_faces))
    case = {
        "solver_options": {"upwind_alpha": 1.0, "time_step": 2e-2, "final_time": 0.4, "order": 2},
        "model": {"filename": "box_tfsf.msh",
                  "materials": [{"tags": [1, 2], "type": "vacuum"}],
                  "boundaries": [{"tags": [1, 2, 3, 4, 5, 6], "type": "SMA"}]},
        "probes": {"point": [{"position": [0.0, 0.1, 0.2], "steps": 2}],
                   "rcssurface": [{"name": "box", "tags": [7], "steps": 1}]},
        "sources": [{"type": "planewave", "polarization": [0.0, 0.0, 1.0], "propagation": [1.0, 0.0, 0.0],
                     "tags": [7], "magnitude": {"type": "gaussian", "spread": 0.2}}],
    }
    (case_dir("box_tfsf") / "box_tfsf.json").write_text(json.dumps(case, indent=2) + "\n")

    # ---- box_dielectric
    m = dg.box_mesh((2, 2, 2))
    tags = side_tags(m.vertices, m.bdr_faces, (0, 0, 0), (1, 1, 1))
    cen = m.vertices[m.elements].mean(axis=1)
    etag = [3 if c[2] < 0.5 else 4 for c in cen]
    write_msh(case_dir("box_dielectric") / "box_dielectric.msh", m.vertices, m.elements, etag, m.bdr_faces, tags)
    case = {
        "solver_options": {"upwind_alpha": 0.5, "final_time": 0.1, "cfl": 0.5, "order": 3, "ode_type": "LSERK4"},
        "model": {"filename": "box_dielectric.msh", "refinement": 1,
                  "materials": [{"tags": [3], "type": "dielectric", "relative_permittivity": 2.0,
                                 "bulk_conductivity": 0.001},
                                {"tags": [4], "type": "vacuum"}],
                  "boundaries": [{"tags": [1, 2, 3, 4, 5, 6], "type": "PEC"}]},
        "sources": [{"type": "initial", "field_type": "magnetic", "center": [0.5, 0.5, 0.5],
                     "polarization": [1.0, 0.0, 0.0], "dimension": 3,
                     "magnitude": {"type": "gaussian", "spread": 0.2}}],
    }
    (case_dir("box_dielectric") / "box_dielectric.json").write_text(json.dumps(case, indent=2) + "\n")
    print("wrote", sorted(p.name for p in OUT.iterdir()))


if __name__ == "__main__":
    main()
