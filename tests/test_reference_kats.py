"""Known-answer tests: the oracle and the product's reference element against the
reference's own element-matrix tests (test/hesthavenComparison/*.cpp), read
from tests/golden/reference_kats.json (made by extract_reference_kats.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def kat(name):
    return np.array(KATS[name]["matrix"], dtype=float)


def seg_oracle(n_el, order):
    x = np.linspace(0.0, 1.0, n_el + 1)
    V = np.stack([x, 0 * x, 0 * x], 1)
    E = np.stack([np.arange(n_el), np.arange(1, n_el + 1)], 1)
    return po.Oracle(V, E, order, 1.0, dim=1, bdr_faces=np.array([[0], [n_el]]), bdr_codes=np.array([3, 3]))


# Hesthaven1DTest.cpp:38-110 (unit segment, MakeCartesian1D(1))
def test_1d_mass_inverse_mass_stiffness_o1():
    m = po.element_matrices(1, 1, [[0.0], [1.0]])
    assert np.allclose(m["M"], kat("1d_mass_o1"), atol=1e-14)
    # InverseIntegrator(MassIntegrator(2.0))
    assert np.allclose(m["Minv"] / 2.0, kat("1d_invmass_o1"), atol=1e-13)
    S = m["M"] @ m["Dx"]
    assert np.allclose(S, kat("1d_stiffness_o1"), atol=1e-14)


@pytest.mark.parametrize("order,key", [(1, "1d_D_o1"), (2, "1d_D_o2"), (4, "1d_D_o4")])
def test_1d_derivative(order, key):
    m = po.element_matrices(1, order, [[0.0], [1.0]])
    # D = (2 M)^-1 S on the unit segment: the (-1,1) reference derivative
    D = 0.5 * m["Dx"]
    assert np.allclose(D, kat(key), atol=1e-12)


def test_1d_MS_operator():
    # Hesthaven1DTest.cpp:112-146: -M^-1 S on 3 and 4 elements of order 2
    o3 = seg_oracle(3, 2)
    MS3 = o3.subop(kind=3, d=0)
    assert np.allclose(-MS3, kat("1d_MS_3E"), atol=1e-11)
    o4 = seg_oracle(4, 2)
    MS4 = o4.subop(kind=3, d=0)
    blk = kat("1d_MS4E_block")
    ref4 = np.kron(np.eye(4), blk)
    assert np.allclose(-MS4, ref4, atol=1e-11)


def test_1d_MF_operator_sma():
    # Hesthaven1DTest.cpp:148-187: (2M)^-1 * one-normal trace-jump (beta 1, interior and SMA boundary) = 0.5 MF_H
    for n_el, key in ((4, "1d_MF_4E"), (3, "1d_MF_3E")):
        o = seg_oracle(n_el, 2)
        MF = o.subop(kind=1, d=0, beta_int=1.0, beta_bdr=1.0, minv_coef=2.0)
        assert np.allclose(MF, 0.5 * kat(key), atol=1e-11), key


def _unit_tet_mass(order):
    return po.element_matrices(3, order, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])["M"]


def test_3d_mass_order2():
    # Hesthaven3DTest.cpp:77-108: first tet of the 1x1x1 cube (volume 1/6), M = (V V^T)^-1 J with J = 1/8;
    # the table is quoted to 5 significant digits, the test uses isApprox(.., 1e-4).
    M = _unit_tet_mass(2)
    ref = kat("3d_mass_o2_vvt_inv") / 8.0
    assert np.linalg.norm(M - ref) <= 1e-4 * np.linalg.norm(ref)
    # the product's reference element: M_ref = (V V^T)^-1 on the (-1,1) tet
    R = dg.ref_tet(2)
    Mp = np.linalg.inv(R["Minv"]) / 8.0
    assert np.linalg.norm(Mp - ref) <= 1e-4 * np.linalg.norm(ref)


def test_3d_derivatives_onetetra_order1():
    # Hesthaven3DTest.cpp:110-152 on testData/mfemMeshes/3D/onetetra.mesh: unit tet, MFEM reorders the
    # element's vertices to (v3, v2, v1, v0); D_{r,s,t} = (2 M)^-1 S_{z,y,x} = R^T D_H R.
    verts = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0], [0, 0, 0]], dtype=float)
    m = po.element_matrices(3, 1, verts)
    Rm = kat("3d_rotator_o1")
    assert np.allclose(0.5 * m["Dz"], Rm.T @ kat("3d_Dr_o1") @ Rm, atol=1e-13)
    assert np.allclose(0.5 * m["Dy"], Rm.T @ kat("3d_Ds_o1") @ Rm, atol=1e-13)
    assert np.allclose(0.5 * m["Dx"], Rm.T @ kat("3d_Dt_o1") @ Rm, atol=1e-13)


def test_3d_emat_order1():
    # Hesthaven3DTest.cpp:232-265 (table printed to 4 decimals, EXPECT_NEAR 1e-3)
    E = po.ref_emat(1)
    assert np.allclose(E, kat("3d_emat_o1"), atol=1e-3)
    # product LIFT = M_ref^-1 Emat
    R = dg.ref_tet(1)
    assert np.allclose(R["Minv"] @ E, R["LIFT"], atol=1e-13)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_product_reference_element_matches_oracle(order):
    """Product tables (orthonormal Vandermonde) vs oracle (Bernstein basis + quadrature)."""
    R = dg.ref_tet(order)
    m = po.element_matrices(3, order, [[-1, -1, -1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    scale = max(1.0, np.abs(R["Dr"]).max())
    for a, b in (("Dr", "Dx"), ("Ds", "Dy"), ("Dt", "Dz")):
        assert np.abs(R[a] - m[b]).max() <= 1e-13 * scale
    assert np.abs(R["Minv"] - m["Minv"]).max() <= 1e-13 * np.abs(R["Minv"]).max()
    E = po.ref_emat(order)
    L = R["Minv"] @ E
    assert np.abs(L - R["LIFT"]).max() <= 1e-13 * np.abs(R["LIFT"]).max()


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_node_set_gauss_lobatto(order):
    """Oracle and product 1D Gauss-Lobatto points and tet node sets agree."""
    g = po.lobatto(order)
    R = dg.ref_tet(order)
    # edge nodes of the tet along r (s = t = -1) are the GLL points
    on_edge = np.isclose(R["s"], -1) & np.isclose(R["t"], -1)
    r = np.sort(R["r"][on_edge])
    assert np.allclose((r + 1) / 2, g, atol=1e-15)


def _pw_oracle(waves):
    """An oracle on one reference tetrahedron with the given plane waves installed (the source
    evaluation does not depend on the mesh)."""
    V = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]
    o = po.Oracle(V, [[0, 1, 2, 3]], 1)
    o.set_planewaves(waves)
    return o


def test_planewave_source_kats():
    """The reference's SourcesTest.planewave (test/maxwell/solver/SourcesTest.cpp:18-36): a
    Gaussian plane wave (spread 0.2, mean -1.5) polarised along y and travelling along x peaks
    at (x = -1.5, t = 0) and at (x = 0, t = 1.5), and its H_z equals its E_y."""
    o = _pw_oracle([dict(propagation=[1, 0, 0], polarization=[0, 1, 0], spread=0.2, mean=-1.5)])
    e, _ = o.pw_eval([-1.5, 0, 0], 0.0)
    assert abs(e[1] - 1.0) <= 1e-6
    e, _ = o.pw_eval([0.0, 0, 0], 1.5)
    assert abs(e[1] - 1.0) <= 1e-6
    for x in np.arange(0.0, 3.0, 0.1):
        e, h = o.pw_eval([x, 0, 0], 0.0)
        assert abs(e[1] - h[2]) <= 1e-6


def test_modulated_gaussian_kats():
    """The reference's FunctionTest.ModulatedGaussian_atMean / _zeroCrossing
    (test/maxwell/math/FunctionTest.cpp:81-102), as the plane wave's time profile: 1 at the
    mean; 0 a quarter period from it under a wide envelope."""
    o = _pw_oracle([dict(propagation=[1, 0, 0], polarization=[0, 0, 1], spread=0.2, mean=0.5, frequency=3.0)])
    e, _ = o.pw_eval([0.5, 0, 0], 0.0)
    assert e[2] == 1.0
    o = _pw_oracle([dict(propagation=[1, 0, 0], polarization=[0, 0, 1], spread=10.0, mean=0.0, frequency=1.0)])
    e, _ = o.pw_eval([0.25, 0, 0], 0.0)
    assert abs(e[2]) <= 1e-10
