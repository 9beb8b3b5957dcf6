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
from conftest import read_point_probe, rel_l2

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
    case = dg.Case(CASES / name / f"{name}.json")
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
        rows = read_point_probe(f)
        assert rows.shape == (res["n_records"], 7)
        assert rows[-1, 0] == pytest.approx(res["final_time"])


def test_resonant_case_probe_values(torch_cuda, tmp_path):
    """The probe at the cavity centre follows the TE110 mode: Ez(t) ~ cos(w t) with w = pi sqrt(2)."""
    case = dg.Case(CASES / "box_resonant" / "box_resonant.json")
    _, res = case.run(out_dir=tmp_path, want_state=False)
    rows = read_point_probe(tmp_path / "PointProbe0.dat")
    t, ez = rows[:, 0], rows[:, 3]
    w = np.pi * np.sqrt(2.0)
    # order 2 on 3^3 hexes: a few percent of discretisation error
    assert np.abs(ez - np.cos(w * t)).max() < 0.05


REFERENCE_CASES = CASES / "reference"    # the reference's own inputs (tests/golden/copy_reference_cases.py)


@pytest.mark.parametrize("name", ["3D_TFSF", "3D_TFSF_InteriorPEC"])
def test_reference_case_end_to_end(torch_cuda, tmp_path, name):
    """The reference's 3D_TFSF (plane wave through a TF/SF surface, one uniform refinement, PEC/PMC
    walls, 6,000 steps) and 3D_TFSF_InteriorPEC (TF/SF, interior PEC sheets, SMA, estimated dt) run
    to their final times through dgtd_case_run, with the reference's loop (driver.cpp:1545 ->
    Solver::run). Bar: the final state within 1e-12 relative L2 of the oracle's RK4 loop on the same
    case tables, the same step count, one probe record per sampled step, and no instability."""
    case = dg.Case(REFERENCE_CASES / name / f"{name}.json")
    state, res = case.run(out_dir=tmp_path)
    inf = case.info
    m = case.mesh()
    orc = po.Oracle.from_mesh(m, inf["order"], alpha=inf["alpha"])
    if case.planewaves():
        orc.set_planewaves(case.planewaves())
    x0 = case.initial_state(orc.nodes())
    xo, no = orc.run(x0, 0.0, res["dt"], inf["final_time"], inf["integrator"], form=po.NODAL)
    assert res["steps"] == no and res["final_time"] == pytest.approx(inf["final_time"])
    assert res["unstable_step"] == -1
    assert np.linalg.norm(xo) > 0 and np.all(np.isfinite(state))
    assert rel_l2(state, xo) <= 1e-12
    files = sorted(tmp_path.glob("PointProbe*.dat"))
    assert len(files) == inf["n_point_probes"]
    for f in files:
        rows = read_point_probe(f)
        assert rows.shape == (res["n_records"], 7) and np.all(np.isfinite(rows))


def test_reference_case_3d_pec_is_unstable_as_given(torch_cuda, tmp_path):
    """The reference's 3D_PEC case asks for dt = 1e-2 at order 3 on its mesh, about 5x the
    reference's own 3D estimate (Solver.cpp:289-300, 349-351), and the explicit RK4 solution grows
    without bound: the oracle's restatement of the reference loop overflows too. The case runner's
    instability detector (Solver.cpp:500-516) reports it and the run goes on, as the reference's
    does. Parity holds on the first steps, before the growth reaches overflow: the first 5 steps
    through the operator path are within 1e-12 relative L2 of the oracle."""
    torch = torch_cuda
    case = dg.Case(REFERENCE_CASES / "3D_PEC" / "3D_PEC.json")
    inf = case.info
    _, res = case.run(out_dir=tmp_path, want_state=False)
    assert res["steps"] == 1000 and res["unstable_step"] > 0 and res["unstable_step"] % 10 == 0
    m = case.mesh()
    orc = po.Oracle.from_mesh(m, inf["order"], alpha=inf["alpha"])
    x0 = case.initial_state(orc.nodes())
    xo = orc.step(x0, 0.0, inf["time_step"], res["unstable_step"], form=po.NODAL)
    assert not (np.linalg.norm(xo) <= 1e20)          # the reference loop's norm is past 1e20 there too
    op = dg.Operator(m, order=inf["order"], alpha=inf["alpha"])
    assert inf["time_step"] > 4 * op.estimate_dt(1.0)
    xd = torch.from_numpy(x0.copy()).cuda()
    op.step(xd, 0.0, inf["time_step"], 5)
    torch.cuda.synchronize()
    assert rel_l2(xd.cpu().numpy(), orc.step(x0, 0.0, inf["time_step"], 5, form=po.NODAL)) <= 1e-12
