"""JSON cases run on the GPU (dgtd_case_run) against the operator path and the oracle.

Bar: the case runner's final state is bit-identical to the same solve through
dgtd_op_run_host (same operator, same loop), and within 1e-12 relative L2 of the
oracle's RK4 loop; point-probe files hold one record per sampled step.
"""
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu
CASES = Path(__file__).resolve().parent / "golden" / "cases"


def operator_run(case):
    m = case.mesh()
    inf = case.info
    op = dg.Operator(m, order=inf["order"], alpha=inf["alpha"])
    waves = case.planewaves()
    if waves:
        op.set_planewaves(waves)
    dt = inf["time_step"] if inf["time_step"] > 0 else op.estimate_dt(inf["cfl"])
    x0 = case.initial_state(op.node_coords())
    x, n = op.run_host(x0, 0.0, dt, inf["final_time"], inf["integrator"])
    return m, op, x0, dt, x, n


@pytest.mark.parametrize("name", ["box_resonant", "box_tfsf", "box_dielectric"])
def test_case_run_matches_operator_and_oracle(torch_cuda, tmp_path, name):
    case = dg.Case(CASES / f"{name}.json")
    state, res = case.run(freqs=[0.5, 1.0], out_dir=tmp_path)
    m, op, x0, dt, ref, n = operator_run(case)
    assert res["steps"] == n and res["dt"] == dt
    assert np.linalg.norm(ref) > 0
    assert np.array_equal(state, ref)
    inf = case.info
    orc = po.Oracle.from_mesh(m, inf["order"], alpha=inf["alpha"])
    if case.planewaves():
        orc.set_planewaves(case.planewaves())
    xo, no = orc.run(x0, 0.0, dt, inf["final_time"], inf["integrator"])
    assert no == n and rel_l2(state, xo) <= 1e-12
    npts = inf["n_point_probes"]
    files = sorted(tmp_path.glob("PointProbe*.dat"))
    assert len(files) == npts
    for f in files:
        rows = np.loadtxt(f, ndmin=2)
        assert rows.shape == (res["n_records"], 7)
        assert rows[-1, 0] == pytest.approx(res["final_time"])


def test_resonant_case_probe_values(torch_cuda, tmp_path):
    """The probe at the cavity centre follows the TE110 mode: Ez(t) ~ cos(w t) with w = pi sqrt(2)."""
    case = dg.Case(CASES / "box_resonant.json")
    _, res = case.run(out_dir=tmp_path, want_state=False)
    rows = np.loadtxt(tmp_path / "PointProbe0.dat")
    t, ez = rows[:, 0], rows[:, 3]
    w = np.pi * np.sqrt(2.0)
    # order 2 on 3^3 hexes: a few percent of discretisation error
    assert np.abs(ez - np.cos(w * t)).max() < 0.05
