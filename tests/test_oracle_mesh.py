"""The oracle's numpy box meshes and 3D time-step estimate against the product's.

The CPU baselines of bench.py build their meshes and dt with oracle/pyoracle.py only, so
that nothing of the product library runs on that side. These checks pin that the two
sides step the same workload: identical vertex, element and face tables, and the same dt
(the reference's 3D Global estimate, src/solver/Solver.cpp:289-300, 349-351).
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po

CASES = [
    dict(n=(3, 4, 5)),
    dict(n=(6, 6, 6), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((2, 2, 2), (4, 4, 4)), tfsf=((1, 1, 1), (5, 5, 5)),
         outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC),
    dict(n=(12, 12, 12), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((5, 5, 5), (7, 7, 7)), tfsf=((2, 2, 2), (10, 10, 10)),
         outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC),
    dict(n=(2, 3, 2), lo=(0.5, -0.25, 0.0), hi=(1.5, 2.0, 0.4), tfsf=((0, 1, 0), (2, 2, 1)), outer_bc=dg.BC_PMC),
]


@pytest.mark.parametrize("case", CASES)
def test_box_mesh_tables_identical(case):
    kw = dict(case)
    n = kw.pop("n")
    a = dg.box_mesh(n, **kw)
    b = po.box_mesh(n, **kw)
    for f in ("vertices", "elements", "bdr_faces", "bdr_codes", "tfsf_faces"):
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape, f
        assert np.array_equal(x, y), f


@pytest.mark.parametrize("case", CASES[:3])
@pytest.mark.parametrize("order", [1, 3, 4, 6])
def test_dt_estimate_identical(case, order):
    kw = dict(case)
    n = kw.pop("n")
    a = dg.box_mesh(n, **kw)
    b = po.box_mesh(n, **kw)
    info = dg.validate_mesh(a, order)
    assert po.dt_scale_min(b.vertices, b.elements) == pytest.approx(info["dt_scale_min"], rel=1e-14)
    g = po.lobatto(order)
    want = info["dt_scale_min"] * 2.0 * (g[1] - g[0]) * 2.0 / 3.0 * 0.75 / 0.8
    assert po.estimate_dt_3d(b, order) == pytest.approx(want, rel=1e-14)
