"""Curved (second-order) tetrahedra on the host, no GPU.

- The product's block rows of the curved elements (curved.cpp: the upwind flux at each face point
  with its own normal, M^-1 int phi F dS) against the oracle's assembled operator (integrator
  modes of the reference's face integrators on the curved map): bar 1e-13 relative to the rows'
  largest entry.
- The oracle's curved assembly: straight elements given as curved reproduce the affine operator;
  with centred flux and PEC walls the curved operator is skew in the mass inner product
  (eigenvalues on the imaginary axis).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import curved_box


def _oracle(m, V, E, els, nodes, p, alpha=1.0):
    o = po.Oracle(V, E, p, alpha, 3, m.bdr_faces, m.bdr_codes)
    o.set_curved(els, nodes)
    return o


def _column(o, k):
    u = np.zeros(o.state_len)
    u[k] = 1.0
    return o.mult(u)


@pytest.mark.parametrize("p,mode,alpha", [(1, "all", 1.0), (2, "all", 1.0), (2, "edge", 0.0), (3, "edge", 1.0)])
def test_curved_rows_match_oracle(p, mode, alpha):
    m, V, E, els, nodes = curved_box(mode=mode, bump=0.03 if mode == "all" else 0.05)
    mesh = dg.Mesh(V, E, m.bdr_faces, m.bdr_codes, curved_elems=els, curved_nodes=nodes)
    R = dg.curved_block_rows(mesh, p, alpha)
    o = _oracle(m, V, E, els, nodes, p, alpha)
    Np, N = o.np, o.ndofs
    dofs = lambda e: [c * N + e * Np + j for c in range(6) for j in range(Np)]
    check = range(0, len(R["elems"]), max(1, len(R["elems"]) // 6))
    for c in check:
        e = int(R["elems"][c])
        blocks = [(e, R["blocks"][c, 0])] + [(int(R["nbr"][c, f]), R["blocks"][c, 1 + f])
                                             for f in range(4) if R["nbr"][c, f] >= 0]
        rows = dofs(e)
        scale = max(np.abs(B).max() for _, B in blocks)
        for el, B in blocks:
            for jj, k in enumerate(dofs(el)):
                col = _column(o, k)[rows]
                assert np.abs(col - B[:, jj]).max() <= 1e-13 * scale


def test_oracle_straight_elements_given_as_curved_are_affine():
    m = po.box_mesh((2, 2, 2), outer_bc=po.BC_PEC)
    V, E = np.asarray(m.vertices, dtype=np.float64), np.asarray(m.elements)
    els = np.arange(0, E.shape[0], 3)
    pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    nodes = np.array([np.vstack([V[E[e]]] + [0.5 * (V[E[e][a]] + V[E[e][b]]) for a, b in pairs]) for e in els])
    a = po.Oracle(V, E, 2, 1.0, 3, m.bdr_faces, m.bdr_codes)
    b = _oracle(m, V, E, els, nodes, 2)
    x = np.random.default_rng(1).standard_normal(a.state_len)
    ya, yb = a.mult(x), b.mult(x)
    assert np.linalg.norm(ya - yb) <= 1e-13 * np.linalg.norm(ya)


def test_oracle_curved_centred_flux_is_skew():
    m, V, E, els, nodes = curved_box(mode="all")
    o = _oracle(m, V, E, els, nodes, 2, alpha=0.0)
    n = o.state_len
    A = np.stack([_column(o, k) for k in range(n)], axis=1)
    ev = np.linalg.eigvals(A)
    assert np.abs(ev).max() > 10 and ev.real.max() <= 1e-11
