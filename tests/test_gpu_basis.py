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


@pytest.mark.parametrize("p", [2, 3])
def test_op_change_basis_and_legendre_mult(torch_cuda, p):
    """dgtd_op_change_basis on the device equals the host matrix applied per element block, and
    change(GL -> GLL), Mult, change(GLL -> GL) equals the oracle's operator assembled on the
    Gauss-Legendre nodes (1e-12)."""
    torch = torch_cuda
    m = po.box_mesh((2, 2, 2), outer_bc=po.BC_SMA)
    mesh = dg.Mesh(m.vertices, m.elements, m.bdr_faces, m.bdr_codes)
    op = dg.Operator(mesh, order=p, alpha=1.0)
    x = np.random.default_rng(p).standard_normal(op.state_len)
    xd = torch.from_numpy(x).cuda()
    yd, zd, wd = torch.empty_like(xd), torch.empty_like(xd), torch.empty_like(xd)
    op.change_basis(xd, yd, dg.BASIS_GAUSS_LEGENDRE, dg.BASIS_GAUSS_LOBATTO)
    torch.cuda.synchronize()
    M = dg.tet_basis_change(p, 0, 1)
    host = (x.reshape(-1, M.shape[0]) @ M.T).reshape(-1)
    assert np.abs(yd.cpu().numpy() - host).max() <= 1e-13 * np.abs(host).max()
    op.mult(yd, zd, 0.0)
    op.change_basis(zd, wd, dg.BASIS_GAUSS_LOBATTO, dg.BASIS_GAUSS_LEGENDRE)
    torch.cuda.synchronize()
    gl = po.Oracle(m.vertices, m.elements, p, 1.0, 3, m.bdr_faces, m.bdr_codes)
    gl.set_basis(0)
    assert rel_l2(wd.cpu().numpy(), gl.mult(x)) <= 1e-12
    with pytest.raises(dg.DgtdError, match="alias"):
        op.change_basis(xd, xd, 0, 1)
