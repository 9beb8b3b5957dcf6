"""A Gauss-Legendre case (the reference's basis_type 0) run on the GPU through dgtd_case_run
against the oracle's global operator assembled on the Gauss-Legendre nodes.

The runner interpolates the initial fields at the case's Gauss-Legendre nodes, moves the state to
the operator's Gauss-Lobatto nodes (the same polynomial), runs the FP64 form and moves the final
state back; the oracle runs the Gauss-Legendre system itself. Bar: 1e-11 relative L2 after 500
RK4 steps (both FP64; the change of basis is exact up to rounding).
"""
import json
import shutil
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import read_point_probe, rel_l2

pytestmark = pytest.mark.gpu
REF = Path(__file__).resolve().parent / "golden" / "cases" / "reference"
BLEG = "3D_Resonant_Box_BLEG_TM55_H0_P2_PERF"


def _short_case(tmp_path, final_time):
    """The BLEG Performance input (350 tetrahedra, order 2, dt 1e-4, the TM(5,5) initial field)
    with an earlier final time."""
    js = json.loads((REF / BLEG / f"{BLEG}.json").read_text())
    js["solver_options"]["final_time"] = final_time
    d = tmp_path / BLEG
    d.mkdir()
    (d / f"{BLEG}.json").write_text(json.dumps(js))
    shutil.copyfile(REF / BLEG / f"{BLEG}.msh", d / f"{BLEG}.msh")
    return dg.Case(d / f"{BLEG}.json")


def test_bleg_case_matches_legendre_oracle(torch_cuda, tmp_path):
    case = _short_case(tmp_path, 0.05)
    assert case.info["basis_type"] == dg.BASIS_GAUSS_LEGENDRE
    out = tmp_path / "out"
    out.mkdir()
    state, res = case.run(out_dir=out)
    m = case.mesh()
    orc = po.Oracle.from_mesh(m, 2, alpha=case.info["alpha"])
    orc.set_basis(0)
    x0 = case.initial_state(orc.nodes())
    xo, no = orc.run(x0, 0.0, case.info["time_step"], 0.05)
    assert res["steps"] == no == 500 and res["unstable_step"] == -1
    assert np.linalg.norm(xo) > 1.0 and rel_l2(state, xo) <= 1e-11
    for f in sorted(out.glob("PointProbe*.dat")):
        rows = read_point_probe(f)
        assert rows.shape == (res["n_records"], 7) and np.all(np.isfinite(rows))


def test_bleg_performance_case_runs(torch_cuda, tmp_path):
    """The whole BLEG input (20,000 steps to t = 2) runs stable to its end."""
    state, res = dg.Case(REF / BLEG / f"{BLEG}.json").run(out_dir=tmp_path)
    assert res["steps"] == 20000 and res["unstable_step"] == -1 and np.all(np.isfinite(state))
