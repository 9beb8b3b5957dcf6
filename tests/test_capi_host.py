"""C-ABI library: loads on a machine without a GPU, exports every declared
symbol, and its host-only parts (mesh generation, table validation,
reference element) behave."""
import re
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w \*]*?\b(dgtd_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = dg.lib()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"missing export {n}"
    # and the binding covers all of them
    assert set(names) <= set(dg.SIGNATURES), set(names) - set(dg.SIGNATURES)


def test_box_mesh_counts():
    m = dg.box_mesh((8, 8, 8))
    assert m.n_elements == 6 * 8 ** 3 == 3072
    assert m.bdr_faces.shape[0] == 6 * 8 * 8 * 2
    m3 = dg.box_mesh((24, 24, 24), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((10,) * 3, (14,) * 3),
                     tfsf=((3,) * 3, (21,) * 3), outer_bc=dg.BC_SMA)
    assert m3.n_elements == 6 * (24 ** 3 - 4 ** 3) == 82560
    assert m3.tfsf_faces.shape[0] == 6 * 18 * 18 * 2
    codes = m3.bdr_codes
    assert (codes == dg.BC_SMA).sum() == 6 * 24 * 24 * 2
    assert (codes == dg.BC_PEC).sum() == 6 * 4 * 4 * 2


def test_validate_reports_tables():
    m = dg.box_mesh((3, 3, 3), tfsf=((1, 1, 1), (2, 2, 2)))
    info = dg.validate_mesh(m, order=3)
    assert info["n_elements"] == 162 and info["np"] == 20 and info["nfp"] == 10
    assert info["n_tfsf_faces"] == 2 * 6 * 2          # 12 TF/SF triangles, both sides counted
    assert info["state_len"] == 6 * 162 * 20
    assert info["min_edge"] == pytest.approx(1.0 / 3.0)


def test_validate_rejects_bad_meshes():
    m = dg.box_mesh((1, 1, 1))
    bad = dg.Mesh(m.vertices, m.elements[:, [1, 0, 2, 3]].copy(), m.bdr_faces, m.bdr_codes)
    with pytest.raises(dg.DgtdError, match="Jacobian"):
        dg.validate_mesh(bad)
    dup = dg.Mesh(m.vertices, np.concatenate([m.elements, m.elements[:1]]), m.bdr_faces, m.bdr_codes)
    with pytest.raises(dg.DgtdError, match="more than two"):
        dg.validate_mesh(dup)
    wrong = dg.Mesh(m.vertices, m.elements, np.array([[0, 1, 2]], np.int32), np.array([1], np.int32))
    with pytest.raises(dg.DgtdError):
        dg.validate_mesh(wrong)
    with pytest.raises(dg.DgtdError, match="order"):
        dg.validate_mesh(m, order=9)


def test_reference_tet_tables():
    for p in range(1, 7):
        R = dg.ref_tet(p)
        Np = (p + 1) * (p + 2) * (p + 3) // 6
        # derivative of a linear function is exact; of a constant zero
        assert np.abs(R["Dr"] @ np.ones(Np)).max() < 1e-12
        assert np.abs(R["Dr"] @ R["r"] - 1).max() < 1e-12
        assert np.abs(R["Ds"] @ R["r"]).max() < 1e-12
        # each face has Nfp nodes on it
        F = R["Fmask"]
        assert F.shape == (4, (p + 1) * (p + 2) // 2)
        assert np.allclose(R["t"][F[3]], -1) and np.allclose(R["s"][F[2]], -1) and np.allclose(R["r"][F[1]], -1)
        assert np.allclose(R["r"][F[0]] + R["s"][F[0]] + R["t"][F[0]], -1)


def test_operator_rejects_bad_options_before_touching_the_device():
    """Argument checks of dgtd_op_create run before any CUDA call, so they work without a GPU."""
    m = dg.box_mesh((1, 1, 1))
    for kw, msg in [(dict(order=0), "order"), (dict(order=7), "order"), (dict(batch=0), "batch"),
                    (dict(alpha=-1.0), "alpha"), (dict(precision=9), "precision")]:
        args = dict(order=2, alpha=1.0, precision=dg.FP64, batch=1)
        args.update(kw)
        with pytest.raises(dg.DgtdError, match=msg):
            dg.Operator(m, **args)
    empty = dg.Mesh(np.zeros((0, 3)), np.zeros((0, 4), np.int32))
    with pytest.raises(dg.DgtdError):
        dg.validate_mesh(empty)


def test_server_and_case_argument_checks():
    with pytest.raises(dg.DgtdError, match="memory_budget"):
        dg.Server(memory_budget=0)
    with pytest.raises(dg.DgtdError, match="max_active"):
        dg.Server(max_active=1000)
    with pytest.raises(dg.DgtdError, match="precision"):
        dg.Server(precision=dg.FP32_3XTF32)
    with pytest.raises(dg.DgtdError, match="cannot open case"):
        dg.Case("/nonexistent/case.json")


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """There is no CPU fallback: without the CUDA library every entry point raises."""
    monkeypatch.setattr(dg, "LIB_PATH", tmp_path / "libdgtd_gb300.so")
    monkeypatch.setattr(dg, "_lib_handle", None)
    with pytest.raises(ImportError, match="missing"):
        dg.lib()
    with pytest.raises(ImportError):
        dg.box_mesh((1, 1, 1))
