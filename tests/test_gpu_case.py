"""JSON cases run on the GPU (dgtd_case_run) against the operator path and the oracle.

Bar: the case runner's final state is bit-identical to the same solve through
dgtd_op_run_host (same operator, same loop), and within 1e-12 relative L2 of the
oracle's RK4 loop; point-probe files hold one record per sampled step.
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


TM55 = REFERENCE_CASES / "3D_Resonant_Box_TM55_H1_P3" / "3D_Resonant_Box_TM55_H1_P3.json"
TM55_W = 5 * np.pi * np.sqrt(2.0)


def _tm55_case(tmp_path, refinement):
    """The H1_P3 input with its refinement level changed (the reference's H<k> inputs differ in
    nothing else but the order), in a folder named as the case."""
    if refinement == 1:
        return dg.Case(TM55)
    name = f"3D_Resonant_Box_TM55_H{refinement}"
    d = tmp_path / name
    d.mkdir()
    js = json.loads(TM55.read_text())
    js["model"]["refinement"] = refinement
    js["model"]["filename"] = f"{name}.msh"
    (d / f"{name}.json").write_text(json.dumps(js))
    shutil.copyfile(TM55.with_suffix(".msh"), d / f"{name}.msh")
    return dg.Case(d / f"{name}.json")


@pytest.mark.parametrize("refinement,order,bar", [(1, 2, 0.22), (1, 3, 0.09), (2, 2, 0.045)])
def test_reference_tm55_mode_converges(torch_cuda, tmp_path, refinement, order, bar):
    """The reference's TM55 resonant box (the unit PEC cube of 350 tetrahedra, refined once, H1,
    or twice, H2) started on the TM(5,5) mode Ez = sin(5 pi x) sin(5 pi y) follows Ez cos(w t),
    Hx = -(5 pi / w) sin(5 pi x) cos(5 pi y) sin(w t), Hy = (5 pi / w) cos(5 pi x) sin(5 pi y)
    sin(w t), w = 5 pi sqrt(2) (test/cases/L2ErrorAnalysis.cpp:32-54) over one period of 200
    steps. The bars are the oracle's own errors at the node set (H1: 0.214 at order 2, 0.083 at
    order 3; H2 order 2: 0.043, five times below H1), so they pin the discretisation, and the first
    20 steps match the oracle to 1e-12."""
    case = _tm55_case(tmp_path, refinement)
    m = case.mesh()
    assert m.n_elements == 350 * 8 ** refinement
    op = dg.Operator(m, order=order, alpha=case.info["alpha"])
    X = op.node_coords()
    N = X.shape[1]
    x0 = case.initial_state(X)
    period = 2 * np.pi / TM55_W
    dt = period / 200
    orc = po.Oracle.from_mesh(m, order, alpha=case.info["alpha"])
    x20, n20 = op.run_host(x0, 0.0, dt, 20 * dt)
    assert n20 == 20 and rel_l2(x20, orc.run(x0, 0.0, dt, 20 * dt)[0]) <= 1e-12
    x, n = op.run_host(x0, 0.0, dt, period)
    assert n == 200
    sx, cx = np.sin(5 * np.pi * X[0]), np.cos(5 * np.pi * X[0])
    sy, cy = np.sin(5 * np.pi * X[1]), np.cos(5 * np.pi * X[1])
    ez = sx * sy
    assert np.linalg.norm(x[2 * N:3 * N] - ez * np.cos(TM55_W * period)) / np.linalg.norm(ez) <= bar
    amp = 5 * np.pi / TM55_W
    hx = -amp * sx * cy * np.sin(TM55_W * period)
    hy = amp * cx * sy * np.sin(TM55_W * period)
    # sin(w T) = 0 after one period: the magnetic field is back to zero up to the same error
    assert np.linalg.norm(x[3 * N:4 * N] - hx) / np.linalg.norm(ez) <= bar
    assert np.linalg.norm(x[4 * N:5 * N] - hy) / np.linalg.norm(ez) <= bar


def test_reference_tm55_performance_case_runs(torch_cuda, tmp_path):
    """The reference's Performance input 3D_Resonant_Box_TM55_H0_P2_PERF (350 tetrahedra, order 2,
    dt 1e-4 to t = 2: 20,000 steps) runs end to end through dgtd_case_run: the step count, no
    instability, one record per sampled step in both probe files, their Ez varying,
    and the field decaying as the upwind flux damps the under-resolved mode."""
    name = "3D_Resonant_Box_TM55_H0_P2_PERF"
    case = dg.Case(REFERENCE_CASES / name / f"{name}.json")
    state, res = case.run(out_dir=tmp_path)
    assert res["steps"] == 20000 and res["unstable_step"] == -1 and np.all(np.isfinite(state))
    files = sorted(tmp_path.glob("PointProbe*.dat"))
    assert len(files) == 2
    for f in files:
        rows = read_point_probe(f)
        assert rows.shape == (res["n_records"], 7) and np.all(np.isfinite(rows))
        assert np.ptp(rows[:, 3]) > 0.1
    # Five half-wavelengths on seven elements per side at order 2 are under-resolved, and the
    # upwind flux takes about two thirds of the nodal norm by t = 2 (the oracle: 0.35 of it).
    x0 = case.initial_state(dg.Operator(case.mesh(), order=2).node_coords())
    assert 0.2 < np.linalg.norm(state) / np.linalg.norm(x0) < 0.5
