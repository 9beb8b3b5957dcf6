"""The oracle's two restatements (assembled CSR vs nodal) agree, and the
oracle reproduces the reference tests' physics (PEC cavity round trip, cavity
mode, TF/SF plane wave)."""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

RNG = np.random.default_rng(20261203)

CASES = [
    # (cells, order, outer bc, tf box, materials)
    ((2, 2, 2), 1, dg.BC_PEC, None, False),
    ((2, 2, 2), 2, dg.BC_PMC, None, True),
    ((2, 1, 2), 3, dg.BC_SMA, None, True),
    ((3, 3, 3), 2, dg.BC_SMA, ((1, 1, 1), (2, 2, 2)), True),
    ((2, 2, 2), 4, dg.BC_OPEN, None, False),
]


def _mesh(cells, bc, tf, mat):
    m = dg.box_mesh(cells, tfsf=tf, outer_bc=bc)
    if mat:
        K = m.n_elements
        m.eps = RNG.uniform(1, 4, K); m.mu = RNG.uniform(1, 2, K); m.sigma = RNG.uniform(0, 0.5, K)
    return m


@pytest.mark.parametrize("cells,order,bc,tf,mat", CASES)
def test_global_equals_nodal(cells, order, bc, tf, mat):
    m = _mesh(cells, bc, tf, mat)
    o = po.Oracle.from_mesh(m, order, alpha=1.0)
    if tf is not None:
        o.set_planewaves([dict(propagation=[1, 0.3, 0.2], polarization=[0, 0, 1], spread=0.2, mean=-0.2)])
    x = RNG.standard_normal(o.state_len)
    yg = o.mult(x, 0.35, po.GLOBAL)
    yn = o.mult(x, 0.35, po.NODAL)
    assert rel_l2(yn, yg) < 1e-13


def test_centered_flux_alpha0():
    m = _mesh((2, 2, 2), dg.BC_PEC, None, False)
    o = po.Oracle.from_mesh(m, 2, alpha=0.0)
    x = RNG.standard_normal(o.state_len)
    assert rel_l2(o.mult(x, 0, po.NODAL), o.mult(x, 0, po.GLOBAL)) < 1e-13
    # centered flux with PEC conserves the discrete energy: <x, M L x> = 0 is not directly
    # available; use the skew property of the centered operator in the (element-mass) inner product
    # indirectly: the energy of a short RK4 run stays constant to high order.
    x0 = RNG.standard_normal(o.state_len) * 0.0
    xyz = o.nodes()
    x0[2 * o.ndofs:3 * o.ndofs] = np.sin(np.pi * xyz[0]) * np.sin(np.pi * xyz[1])
    x1 = o.step(x0, 0, 1e-3, 50, form=po.NODAL)
    assert abs(np.linalg.norm(x1) - np.linalg.norm(x0)) / np.linalg.norm(x0) < 5e-3


def test_interior_pec_sheet():
    """An interior PEC sheet behaves like a PEC wall on both sides (assembled IBFI rules)."""
    m = dg.box_mesh((2, 2, 2))
    # the x = 0.5 plane between the two cell layers
    V = m.vertices
    pick = np.where(np.all(np.isclose(V[m.elements][:, :, 0], 0.5) | True, axis=1))[0]
    # collect triangles lying on x = 0.5
    faces = set()
    for e in m.elements:
        for f in range(4):
            tri = tuple(sorted(int(v) for q, v in enumerate(e) if q != f))
            if np.allclose(V[list(tri), 0], 0.5):
                faces.add(tri)
    m.int_faces = np.array(sorted(faces), np.int32)
    m.int_codes = np.full(len(faces), dg.BC_PEC, np.int32)
    o = po.Oracle.from_mesh(m, 2)
    x = RNG.standard_normal(o.state_len)
    assert rel_l2(o.mult(x, 0, po.NODAL), o.mult(x, 0, po.GLOBAL)) < 1e-13
    # decoupled: fields on the left do not influence the right half
    xyz = o.nodes()
    left = xyz[0] < 0.5 - 1e-12
    xl = x.copy()
    for c in range(6):
        xl[c * o.ndofs:(c + 1) * o.ndofs][~left] = 0.0
    y = o.mult(xl, 0, po.GLOBAL)
    right = xyz[0] > 0.5 + 1e-12
    for c in range(6):
        assert np.abs(y[c * o.ndofs:(c + 1) * o.ndofs][right]).max() < 1e-13


def _segment(n_el, bc_left, bc_right):
    x = np.linspace(0.0, 1.0, n_el + 1)
    V = np.stack([x, 0 * x, 0 * x], 1)
    E = np.stack([np.arange(n_el), np.arange(1, n_el + 1)], 1)
    return V, E, np.array([[0], [n_el]]), np.array([bc_left, bc_right])


def test_1d_pec_cavity_round_trip():
    """1D PEC cavity: 100 elements, p = 3, alpha = 1, Ey Gaussian (sigma 0.05) at 0.5, T = 2.

    After one period the field returns (reference Solver1DTest.cpp:150-160 checks ||E(T)-E(0)|| < 1e-2);
    the mid-run field matches d'Alembert with odd reflection at the PEC walls.
    """
    n_el, p = 100, 3
    V, E, bf, bc = _segment(n_el, dg.BC_PEC, dg.BC_PEC)
    o = po.Oracle(V, E, p, 1.0, dim=1, bdr_faces=bf, bdr_codes=bc)
    X = o.nodes()[0]
    f0 = lambda s: np.exp(-((s - 0.5) ** 2) / (2 * 0.05 ** 2))
    x0 = np.zeros(o.state_len)
    x0[o.ndofs:2 * o.ndofs] = f0(X)
    g = po.lobatto(p)
    dt = 0.5 * (g[1] - g[0]) * (1.0 / n_el) / p ** 1.5      # Solver.cpp:311-320 with cfl 0.5
    xT, steps = o.run(x0, 0.0, dt, 2.0, form=po.NODAL)
    ey0, eyT = x0[o.ndofs:2 * o.ndofs], xT[o.ndofs:2 * o.ndofs]
    assert np.linalg.norm(eyT - ey0) / np.linalg.norm(ey0) < 1e-2
    # half period: the pulse split and reflected with odd images -> E(x,1) = -E0(1-x) ... compare d'Alembert
    x_half, _ = o.run(x0, 0.0, dt, 0.25, form=po.NODAL)

    def odd_periodic(s):
        s = np.mod(s, 2.0)
        return np.where(s <= 1.0, f0(s), -f0(2.0 - s))
    exact = 0.5 * (odd_periodic(X - 0.25) + odd_periodic(X + 0.25))
    assert np.abs(x_half[o.ndofs:2 * o.ndofs] - exact).max() < 1e-3


def test_1d_global_equals_nodal():
    V, E, bf, bc = _segment(7, dg.BC_SMA, dg.BC_PEC)
    o = po.Oracle(V, E, 3, 1.0, dim=1, bdr_faces=bf, bdr_codes=bc)
    x = RNG.standard_normal(o.state_len)
    assert rel_l2(o.mult(x, 0, po.NODAL), o.mult(x, 0, po.GLOBAL)) < 1e-13


def te110(xyz, t):
    w = np.pi * np.sqrt(2.0)
    x, y = xyz[0], xyz[1]
    ez = np.sin(np.pi * x) * np.sin(np.pi * y) * np.cos(w * t)
    hx = -(np.pi / w) * np.sin(np.pi * x) * np.cos(np.pi * y) * np.sin(w * t)
    hy = (np.pi / w) * np.cos(np.pi * x) * np.sin(np.pi * y) * np.sin(w * t)
    z = np.zeros_like(x)
    return np.concatenate([z, z, ez, hx, hy, z])


def test_te110_cavity_mode_small():
    """Unit-cube PEC resonator, TE110 mode: error vs the analytic mode converges with h."""
    errs = []
    for n in (2, 4):
        m = dg.box_mesh((n, n, n))
        o = po.Oracle.from_mesh(m, 3)
        xyz = o.nodes()
        x0 = te110(xyz, 0.0)
        T = 0.2
        xT, _ = o.run(x0, 0.0, 2e-3, T, form=po.NODAL)
        errs.append(rel_l2(xT, te110(xyz, T)))
    assert errs[1] < errs[0] / 4
    assert errs[1] < 5e-3


def test_tfsf_plane_wave_in_empty_box():
    """TF/SF box inside an SMA-terminated domain: the total-field region carries the incident
    plane wave, the scattered-field region stays (nearly) empty."""
    n = 6
    m = dg.box_mesh((n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1, 1, 1), (5, 5, 5)), outer_bc=dg.BC_SMA)
    o = po.Oracle.from_mesh(m, 3)
    k = np.array([1.0, 0.0, 0.0]); pol = np.array([0.0, 0.0, 1.0])
    spread = 0.25
    # driver auto mean: min phase on the TF/SF surface minus 5 sigma sqrt 2 (driver.cpp:576-589)
    mean = -2.0 / 3.0 - 5 * spread * np.sqrt(2.0)
    wave = dict(propagation=k, polarization=pol, spread=spread, mean=mean)
    o.set_planewaves([wave])
    x0 = np.zeros(o.state_len)
    T = 2.4
    xT, _ = o.run(x0, 0.0, 5e-3, T, form=po.NODAL)
    xyz = o.nodes()
    s = xyz[0] - T
    g = np.exp(-((s - mean) ** 2) / (2 * spread ** 2))
    inside = np.all(np.abs(xyz) < 2.0 / 3.0 - 1e-9, axis=0)
    outside = np.any(np.abs(xyz) > 2.0 / 3.0 + 1e-9, axis=0)
    ez = xT[2 * o.ndofs:3 * o.ndofs]
    hy = xT[4 * o.ndofs:5 * o.ndofs]
    assert np.abs(ez[inside] - g[inside]).max() < 0.05
    assert np.abs(hy[inside] + g[inside]).max() < 0.05     # H = k x pol g = -y g
    assert np.abs(ez[outside]).max() < 0.05


def test_tfsf_skip_when_source_negligible():
    """Before the pulse reaches the TF/SF surface (||pw|| < 1e-8) the source term is skipped."""
    m = dg.box_mesh((3, 3, 3), tfsf=((1, 1, 1), (2, 2, 2)), outer_bc=dg.BC_SMA)
    o = po.Oracle.from_mesh(m, 2)
    o.set_planewaves([dict(propagation=[1, 0, 0], polarization=[0, 1, 0], spread=0.05, mean=-3.0)])
    x = np.zeros(o.state_len)
    assert np.abs(o.mult(x, 0.0, po.GLOBAL)).max() == 0.0
    assert np.abs(o.mult(x, 0.0, po.NODAL)).max() == 0.0
    # at the crossing time the source is active
    assert np.abs(o.mult(x, 3.0 + 0.5, po.GLOBAL)).max() > 1e-3
