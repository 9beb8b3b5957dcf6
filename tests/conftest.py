"""Shared test setup: the `gpu` marker, library builds, common fixtures."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# Modules whose GPU paths are the newest (change of basis, thin layers, curved elements) run after
# the others, so that with -x a failure there does not keep the rest of the suite from running.
RUN_LAST = ("test_gpu_basis.py", "test_gpu_sgbc.py", "test_gpu_curved.py")


def pytest_collection_modifyitems(session, config, items):
    items.sort(key=lambda it: 1 if Path(str(it.fspath)).name in RUN_LAST else 0)


def _ensure_built():
    from dgtd_gb300 import build as pkg_build
    from oracle import pyoracle
    pkg_build.build()
    pyoracle.build()


_ensure_built()


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_l2(a, b):
    import numpy as np
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


SPEED_OF_LIGHT_SI = 299792458.0


def read_point_probe(path):
    """A point-probe file in the reference's format (ProbesManager.cpp:203-215, 400-407): four
    header lines (ID, "Spatial Position (X, Y, Z)", the position, the column names), then rows
    t[s] Ex Ey Ez Hx Hy Hz. Returned as an array with t back in normalised units (t[s] * c)."""
    import numpy as np
    lines = Path(path).read_text().splitlines()
    assert lines[0].startswith("PointProbe ID ")
    assert lines[1].startswith("Spatial Position (X, Y, Z)")
    assert len(lines[2].split()) == 3
    assert lines[3].startswith("Time (s) // Ex // Ey // Ez // Hx // Hy // Hz")
    rows = np.loadtxt(path, skiprows=4, ndmin=2)
    rows[:, 0] *= SPEED_OF_LIGHT_SI
    return rows


def plane_faces(vertices, elements, x0, tol=1e-12):
    """Interior faces (vertex triples) of a tetrahedral mesh lying on the plane x = x0."""
    import numpy as np
    from collections import Counter
    V = np.asarray(vertices)
    cnt = Counter()
    for t in np.asarray(elements):
        for f in range(4):
            fv = tuple(sorted(int(v) for v in np.delete(t, f)))
            if all(abs(V[v, 0] - x0) < tol for v in fv):
                cnt[fv] += 1
    return np.array([list(k) for k, c in sorted(cnt.items()) if c == 2], dtype=np.int32).reshape(-1, 3)


def sgbc_box(n=(4, 3, 3), hi=(2.0, 1.0, 1.0), planes=(1.0,), tfsf=True):
    """A box with SMA walls, a TF/SF box from the second cell on, and thin-layer (SGBC) sheets on
    the planes x = planes[i] (interior faces with code 4). Returns (mesh tables as the oracle's
    BoxMesh fields, the sheet faces per plane)."""
    import numpy as np
    from oracle import pyoracle as po
    m = po.box_mesh(n, hi=hi, outer_bc=po.BC_SMA, tfsf=((1, 0, 0), tuple(n)) if tfsf else None)
    sheets = [plane_faces(m.vertices, m.elements, x) for x in planes]
    faces = np.concatenate(sheets) if sheets else np.zeros((0, 3), np.int32)
    return m, sheets, faces


FREE_SPACE_IMPEDANCE = 4e-7 * 3.141592653589793 * SPEED_OF_LIGHT_SI


def tem_waveguide(n=(16, 2, 2), hi=(4.0, 0.5, 0.5), tf_cell=4, sheet_x=2.5):
    """A TEM waveguide along x: PEC walls at y = 0, hi[1], PMC walls at z = 0, hi[2], SMA ends;
    the TF/SF plane at cell tf_cell (total field beyond), and the interior faces on x = sheet_x.
    An Ey/Hz plane wave along x travels in it as in free space. Returns (box mesh, boundary codes,
    sheet faces)."""
    import numpy as np
    from oracle import pyoracle as po
    m = po.box_mesh(n, hi=hi, outer_bc=po.BC_SMA, tfsf=((tf_cell, 0, 0), tuple(n)))
    V = np.asarray(m.vertices)
    codes = []
    for f in np.asarray(m.bdr_faces):
        P = V[f]
        on = lambda a, v: bool(np.all(np.abs(P[:, a] - v) < 1e-12))
        if on(1, 0.0) or on(1, hi[1]):
            codes.append(1)
        elif on(2, 0.0) or on(2, hi[2]):
            codes.append(2)
        else:
            codes.append(3)
    return m, np.array(codes, np.int32), plane_faces(V, m.elements, sheet_x)


def slab_pulse(times, x_sheet, x_probe, spread, mean, eps, mu, sigma, width, kind):
    """Analytic response of a homogeneous slab (relative eps, mu, conductivity sigma in solver
    units, thickness width) of zero extent in the mesh at x_sheet to the Gaussian plane wave
    exp(-(x - t - mean)^2 / (2 spread^2)) at normal incidence: the transmitted ('t', probe beyond
    the sheet) or reflected ('r', probe before it) field at x_probe, from the slab's S21 / S11
    (transmission-line matrix of the slab, fields referred to its faces)."""
    import numpy as np
    dt = times[1] - times[0]
    N = 1 << 16
    t = np.arange(N) * dt - 20.0
    F = np.fft.fft(np.exp(-((x_sheet - t - mean) ** 2) / (2 * spread ** 2)))
    w = 2 * np.pi * np.fft.fftfreq(N, dt)
    wa = np.where(w == 0, 1e-30, np.abs(w))
    ec = eps - 1j * sigma / wa                       # e^{+i w t}: eps_c = eps - i sigma / w
    k = wa * np.sqrt(mu * ec)
    Z = np.sqrt(mu / ec)
    den = np.cos(k * width) + 0.5j * (Z + 1 / Z) * np.sin(k * width)
    S = (1 / den) if kind == "t" else (0.5j * (Z - 1 / Z) * np.sin(k * width) / den)
    S = np.where(w >= 0, S, np.conj(S))
    lag = (x_probe - x_sheet) if kind == "t" else (x_sheet - x_probe)
    out = np.real(np.fft.ifft(F * S * np.exp(-1j * w * lag)))
    return np.interp(times, t, out)


EDGE_PAIRS = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def curved_box(n=(2, 2, 2), bump=0.03, bc=1, mode="all"):
    """Box meshes with second-order (curved) tetrahedra for the curved-element tests.
    mode "all": every vertex and edge node through x -> x + bump sin(pi x) sin(pi y) sin(pi z)
    (1, 0.6, 0.3), every element curved (the map vanishes on the box's faces);
    mode "edge": one interior edge's node moved by `bump` across it, the tetrahedra on that edge
    curved, the rest straight. Returns (box mesh, vertices, elements, curved ids, [n, 10, 3] nodes)."""
    import numpy as np
    from oracle import pyoracle as po
    m = po.box_mesh(n, outer_bc=bc)
    V = np.asarray(m.vertices, dtype=np.float64)
    E = np.asarray(m.elements)
    if mode == "all":
        f = lambda P: P + bump * np.sin(np.pi * P[..., [0]]) * np.sin(np.pi * P[..., [1]]) * \
            np.sin(np.pi * P[..., [2]]) * np.array([1.0, 0.6, 0.3])
        Vc = f(V)
        els = np.arange(E.shape[0])
        nodes = np.array([np.vstack([Vc[E[e]]] + [f(0.5 * (V[E[e][a]] + V[E[e][b]])) for a, b in EDGE_PAIRS])
                          for e in els])
        return m, Vc, E, els, nodes
    # the edge from the box's centre vertex along +x
    c = np.argmin(np.linalg.norm(V - 0.5 * (V.min(0) + V.max(0)), axis=1))
    nb = [v for v in range(len(V)) if np.allclose(V[v] - V[c], [np.ptp(V[:, 0]) / n[0], 0, 0])]
    a, b = c, nb[0]
    els = np.array([e for e in range(E.shape[0]) if a in E[e] and b in E[e]], dtype=np.int32)
    nodes = []
    for e in els:
        t = E[e]
        mids = []
        for p, q in EDGE_PAIRS:
            mid = 0.5 * (V[t[p]] + V[t[q]])
            if {t[p], t[q]} == {a, b}:
                mid = mid + np.array([0.0, bump, 0.4 * bump])
            mids.append(mid)
        nodes.append(np.vstack([V[t]] + mids))
    return m, V, E, els, np.array(nodes)
