"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference's DG Maxwell operator on the CPU; see
dgtd_oracle.cpp for what it follows. Only tests/, __graft_entry__.smoke() and
the cpu_baseline leg of bench.py use it, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libdgtd_oracle.so"
GLOBAL, NODAL = 0, 1

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_lib = None


def build(verbose: bool = False) -> Path:
    res = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(res.stdout)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        h = C.CDLL(str(LIB))
        h.orc_last_error.restype = C.c_char_p
        h.orc_create.restype = C.c_void_p
        h.orc_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int64, _D, C.c_int64, _I32, _D, _D, _D,
                                 C.c_int64, _I32, _I32, C.c_int64, _I32, C.c_int64, _I32, _I32]
        h.orc_destroy.argtypes = [C.c_void_p]
        h.orc_ndofs.restype = C.c_int64; h.orc_ndofs.argtypes = [C.c_void_p]
        h.orc_np.restype = C.c_int; h.orc_np.argtypes = [C.c_void_p]
        h.orc_nodes.argtypes = [C.c_void_p, _D]
        h.orc_set_planewaves.argtypes = [C.c_void_p, C.c_int, _D]
        h.orc_mult.restype = C.c_int; h.orc_mult.argtypes = [C.c_void_p, C.c_int, _D, _D, C.c_double]
        h.orc_step.restype = C.c_int
        h.orc_step.argtypes = [C.c_void_p, C.c_int, _D, C.c_double, C.c_double, C.c_int, C.c_int]
        h.orc_run.restype = C.c_int
        h.orc_run.argtypes = [C.c_void_p, C.c_int, _D, C.c_double, C.c_double, C.c_double, C.c_int,
                              C.POINTER(C.c_int64)]
        h.orc_nnz.restype = C.c_int64; h.orc_nnz.argtypes = [C.c_void_p]
        h.orc_element_matrices.restype = C.c_int
        h.orc_element_matrices.argtypes = [C.c_int, C.c_int, _D, _D, _D, _D, _D, _D]
        h.orc_ref_emat.restype = C.c_int; h.orc_ref_emat.argtypes = [C.c_int, _D]
        h.orc_lobatto.restype = C.c_int; h.orc_lobatto.argtypes = [C.c_int, _D]
        h.orc_pw_eval.restype = None; h.orc_pw_eval.argtypes = [C.c_void_p, _D, C.c_double, _D, _D]
        h.orc_threads.restype = C.c_int
        h.orc_subop.restype = C.c_int
        h.orc_subop.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _D]
        h.orc_set_curved.restype = C.c_int
        h.orc_set_curved.argtypes = [C.c_void_p, C.c_int64, _I32, _D]
        h.orc_set_basis.restype = C.c_int
        h.orc_set_basis.argtypes = [C.c_void_p, C.c_int]
        h.orc_set_sgbc.restype = C.c_int
        h.orc_set_sgbc.argtypes = [C.c_void_p, C.c_int, _I32, _D, _I32, _D, _I32]
        h.orc_sgbc_pairs.restype = C.c_int64; h.orc_sgbc_pairs.argtypes = [C.c_void_p]
        h.orc_sgbc_stack_create.restype = C.c_void_p
        h.orc_sgbc_stack_create.argtypes = [C.c_int, _D, C.c_int, C.c_int, C.c_double]
        h.orc_sgbc_stack_destroy.argtypes = [C.c_void_p]
        h.orc_sgbc_stack_size.restype = C.c_int64; h.orc_sgbc_stack_size.argtypes = [C.c_void_p]
        h.orc_sgbc_stack_matrix.argtypes = [C.c_void_p, _D]
        h.orc_sgbc_stack_advance.argtypes = [C.c_void_p, _D, _D, _D, C.c_double, C.c_double, C.c_int]
        h.orc_sgbc_stack_iface.restype = C.c_int64; h.orc_sgbc_stack_iface.argtypes = [C.c_void_p, C.c_int]
        _lib = h
    return _lib


def _d(a):
    return a.ctypes.data_as(_D) if a is not None else _D()


def _i(a):
    return a.ctypes.data_as(_I32) if a is not None else _I32()


class Oracle:
    """CPU restatement of the reference operator on a mesh.

    form GLOBAL: assembled CSR (GlobalEvolution); form NODAL: matrix-free
    nodal form (HesthavenEvolution).
    """

    def __init__(self, vertices, elements, order: int, alpha: float = 1.0, dim: int = 3,
                 bdr_faces=None, bdr_codes=None, tfsf_faces=None, int_faces=None, int_codes=None,
                 eps=None, mu=None, sigma=None):
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.int32)
        V = f64(vertices)
        if V.ndim == 1 or V.shape[1] != 3:
            V3 = np.zeros((V.shape[0], 3)); V3[:, : V.reshape(V.shape[0], -1).shape[1]] = V.reshape(V.shape[0], -1)
            V = V3
        self._keep = [V, i32(elements), f64(eps), f64(mu), f64(sigma), i32(bdr_faces), i32(bdr_codes),
                      i32(tfsf_faces), i32(int_faces), i32(int_codes)]
        V, E, ep, mu_, sg, bf, bc, tf, itf, ic = self._keep
        nb = 0 if bc is None else bc.size
        nt = 0 if tf is None else (tf.shape[0] if tf.ndim > 1 else tf.size // (2 if dim == 1 else 3))
        ni = 0 if ic is None else ic.size
        self.h = lib().orc_create(dim, order, alpha, V.shape[0], _d(V), E.shape[0], _i(E), _d(ep), _d(mu_), _d(sg),
                                  nb, _i(bf), _i(bc), nt, _i(tf), ni, _i(itf), _i(ic))
        if not self.h:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        self.dim, self.order = dim, order
        self.ndofs = int(lib().orc_ndofs(self.h))
        self.np = int(lib().orc_np(self.h))
        self.state_len = 6 * self.ndofs

    @classmethod
    def from_mesh(cls, mesh, order: int, alpha: float = 1.0) -> "Oracle":
        """Build from a dgtd_gb300.Mesh-like object (same flat tables)."""
        return cls(mesh.vertices, mesh.elements, order, alpha, 3, mesh.bdr_faces, mesh.bdr_codes,
                   mesh.tfsf_faces, mesh.int_faces, mesh.int_codes, mesh.eps, mesh.mu, mesh.sigma)

    def __del__(self):
        try:
            if self.h:
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def nodes(self) -> np.ndarray:
        xyz = np.zeros((3, self.ndofs))
        lib().orc_nodes(self.h, _d(xyz))
        return xyz

    def set_planewaves(self, waves: Sequence[dict]) -> None:
        prm = np.zeros((max(1, len(waves)), 11))
        for i, w in enumerate(waves):
            prm[i, 0:3] = w["propagation"]; prm[i, 3:6] = w["polarization"]
            prm[i, 6] = w["spread"]; prm[i, 7] = w["mean"]; prm[i, 8] = w.get("frequency", 0.0)
        lib().orc_set_planewaves(self.h, len(waves), _d(prm))

    def pw_eval(self, x, t: float):
        """Incident (E, H) of the installed plane waves at point x (3) and time t."""
        xx = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(3))
        e, h = np.zeros(3), np.zeros(3)
        lib().orc_pw_eval(self.h, _d(xx), float(t), _d(e), _d(h))
        return e, h

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())

    def mult(self, x: np.ndarray, t: float = 0.0, form: int = GLOBAL) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._chk(lib().orc_mult(self.h, form, _d(x), _d(y), float(t)))
        return y

    def step(self, x: np.ndarray, t0: float, dt: float, nsteps: int, integrator: int = 0, form: int = GLOBAL):
        x = np.array(x, dtype=np.float64, copy=True)
        self._chk(lib().orc_step(self.h, form, _d(x), float(t0), float(dt), int(nsteps), int(integrator)))
        return x

    def run(self, x: np.ndarray, t0: float, dt: float, final_time: float, integrator: int = 0, form: int = GLOBAL):
        x = np.array(x, dtype=np.float64, copy=True)
        n = C.c_int64()
        self._chk(lib().orc_run(self.h, form, _d(x), float(t0), float(dt), float(final_time), int(integrator),
                                C.byref(n)))
        return x, int(n.value)

    def nnz(self) -> int:
        return int(lib().orc_nnz(self.h))

    def set_curved(self, elems, nodes) -> None:
        """Second-order geometry of the listed elements: nodes [n, 10, 3] = corners (the element's
        vertex order) then edge nodes of (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)."""
        el = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1)
        nd = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1)
        self._keep += [el, nd]
        self._chk(lib().orc_set_curved(self.h, el.size, _i(el), _d(nd)))

    def set_basis(self, basis_type: int) -> None:
        """MFEM basis type of the node set: 0 Gauss-Legendre, 1 Gauss-Lobatto (the default). Set
        before the first product; the Gauss-Legendre set runs the global form only."""
        self._chk(lib().orc_set_basis(self.h, int(basis_type)))

    def set_sgbc(self, stacks: Sequence[dict], face_stack) -> None:
        """Thin-layer (SGBC) sub-solvers for the interior faces given with code 4, in their order:
        face_stack[i] is the stack of the i-th such face (stack dicts: see sgbc_stack_arrays)."""
        counts, prm, bcs, subs = sgbc_stack_arrays(stacks)
        fs = np.ascontiguousarray(face_stack, dtype=np.int32)
        self._keep += [counts, prm, bcs, subs, fs]
        self._chk(lib().orc_set_sgbc(self.h, len(stacks), _i(counts), _d(prm), _i(bcs), _d(subs), _i(fs)))

    def sgbc_pairs(self) -> int:
        return int(lib().orc_sgbc_pairs(self.h))

    def subop(self, kind: int, d: int = 0, d2: int = 0, beta_int: float = 1.0, beta_bdr: float = 1.0,
              minv_coef: float = 1.0) -> np.ndarray:
        """Dense (M^-1/minv_coef) F for one integrator (see orc_subop)."""
        out = np.zeros((self.ndofs, self.ndofs))
        self._chk(lib().orc_subop(self.h, kind, d, d2, beta_int, beta_bdr, minv_coef, _d(out)))
        return out


def sgbc_stack_arrays(stacks: Sequence[dict]):
    """Flat arrays of SGBC stacks. A stack is {"layers": [{"eps", "mu", "sigma", "width", "segments",
    "order"}], "left": bc, "right": bc, "sub_dt": s}; sigma in solver units, bc 0 (none), 1 PEC,
    2 PMC, 3 SMA."""
    counts = np.array([len(s["layers"]) for s in stacks], dtype=np.int32)
    prm = np.array([[L.get("eps", 1.0), L.get("mu", 1.0), L.get("sigma", 0.0), L["width"], L["segments"], L["order"]]
                    for s in stacks for L in s["layers"]], dtype=np.float64).reshape(-1, 6)
    bcs = np.array([[s.get("left", 0), s.get("right", 0)] for s in stacks], dtype=np.int32).reshape(-1, 2)
    subs = np.array([s.get("sub_dt", 0.0) for s in stacks], dtype=np.float64)
    return counts, prm, bcs, subs


class SgbcStack:
    """One SGBC sub-solver on its own (tests of the 1D operator and of the sub-stepping)."""

    def __init__(self, stack: dict):
        counts, prm, bcs, subs = sgbc_stack_arrays([stack])
        self._keep = (prm,)
        self.h = lib().orc_sgbc_stack_create(int(counts[0]), _d(prm), int(bcs[0, 0]), int(bcs[0, 1]), float(subs[0]))
        if not self.h:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        self.n = int(lib().orc_sgbc_stack_size(self.h))
        self.idx_left = int(lib().orc_sgbc_stack_iface(self.h, 0))
        self.idx_right = int(lib().orc_sgbc_stack_iface(self.h, 1))

    def __del__(self):
        try:
            if self.h:
                lib().orc_sgbc_stack_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def matrix(self) -> np.ndarray:
        A = np.zeros((self.n, self.n))
        lib().orc_sgbc_stack_matrix(self.h, _d(A))
        return A

    def advance(self, x, g_old, g_new=None, t0: float = 0.0, span: float = 0.0) -> np.ndarray:
        """x advanced by span from t0: ghosts g_old (12 face-local values) held, or interpolated
        towards g_new when it is given."""
        x = np.array(x, dtype=np.float64, copy=True)
        go = np.ascontiguousarray(g_old, dtype=np.float64)
        gn = np.ascontiguousarray(go if g_new is None else g_new, dtype=np.float64)
        lib().orc_sgbc_stack_advance(self.h, _d(x), _d(go), _d(gn), float(t0), float(span), int(g_new is not None))
        return x


def element_matrices(dim: int, order: int, verts) -> dict:
    v = np.zeros((dim + 1, 3)); vv = np.asarray(verts, dtype=np.float64); v[:, : vv.shape[1]] = vv
    n = order + 1 if dim == 1 else (order + 1) * (order + 2) * (order + 3) // 6
    out = {k: np.zeros((n, n)) for k in ("M", "Minv", "Dx", "Dy", "Dz")}
    rc = lib().orc_element_matrices(dim, order, _d(v), *(_d(out[k]) for k in ("M", "Minv", "Dx", "Dy", "Dz")))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return out


def ref_emat(order: int) -> np.ndarray:
    n = (order + 1) * (order + 2) * (order + 3) // 6
    nfp = (order + 1) * (order + 2) // 2
    e = np.zeros((n, 4 * nfp))
    lib().orc_ref_emat(order, _d(e))
    return e


def lobatto(p: int) -> np.ndarray:
    g = np.zeros(p + 1)
    lib().orc_lobatto(p, _d(g))
    return g


def threads() -> int:
    return int(lib().orc_threads())


# ----------------------------------------------------------------------------- meshes and dt (numpy)
# Structured box meshes and the reference's 3D time-step estimate, restated in numpy so
# that the CPU baselines need nothing from the product library. The construction is the
# product's box generator (dgtd_box_mesh_*): same vertex numbering, element order,
# orientation and face lists; tests/test_oracle_mesh.py checks that they are identical.
BC_OPEN, BC_PEC, BC_PMC, BC_SMA = 0, 1, 2, 3

# 6 tetrahedra of a hex (corners 0..7 in the i-fastest order of the cell) sharing the
# 0-6 diagonal, all positively oriented
_KUHN = np.array([[0, 1, 2, 6], [0, 5, 1, 6], [0, 4, 5, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6]])


class BoxMesh:
    """Flat mesh tables with the fields Oracle.from_mesh reads."""

    def __init__(self, vertices, elements, bdr_faces, bdr_codes, tfsf_faces):
        self.vertices = vertices
        self.elements = elements
        self.bdr_faces = bdr_faces
        self.bdr_codes = bdr_codes
        self.tfsf_faces = tfsf_faces
        self.int_faces = np.zeros((0, 3), np.int32)
        self.int_codes = np.zeros((0,), np.int32)
        self.eps = self.mu = self.sigma = None
        self.dim = 3

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])


def box_mesh(n, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), hole=None, tfsf=None, outer_bc: int = BC_PEC,
             hole_bc: int = BC_PEC) -> BoxMesh:
    """n[0] x n[1] x n[2] hexes, each split into 6 tets; hole / tfsf: half-open cell ranges."""
    nx, ny, nz = (int(v) for v in n)
    vid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    V = np.stack([lo[0] + (hi[0] - lo[0]) * ii.ravel() / nx, lo[1] + (hi[1] - lo[1]) * jj.ravel() / ny,
                  lo[2] + (hi[2] - lo[2]) * kk.ravel() / nz], axis=1)
    hole_lo, hole_hi = (hole if hole is not None else ((0, 0, 0), (0, 0, 0)))
    tf_lo, tf_hi = (tfsf if tfsf is not None else ((0, 0, 0), (0, 0, 0)))

    def in_range(i, j, k, a, b):
        return a[0] <= i < b[0] and a[1] <= j < b[1] and a[2] <= k < b[2]

    def exists(i, j, k):
        return 0 <= i < nx and 0 <= j < ny and 0 <= k < nz and not in_range(i, j, k, hole_lo, hole_hi)

    cells = [(i, j, k) for k in range(nz) for j in range(ny) for i in range(nx)
             if not in_range(i, j, k, hole_lo, hole_hi)]
    c = np.array([[vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k), vid(i, j, k + 1),
                   vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)] for i, j, k in cells],
                 dtype=np.int64).reshape(-1, 8)
    E = c[:, _KUHN].reshape(-1, 4).astype(np.int32)
    have_tf = all(tf_hi[d] > tf_lo[d] for d in range(3))
    bf, bc, tf = [], [], []

    def quad(dst, a, b, cc, d, flip):            # quad a-b-c-d, diagonal a-c
        dst.extend([[a, cc, b], [a, d, cc]] if flip else [[a, b, cc], [a, cc, d]])

    lim0 = (nx, ny, nz)
    for axis in range(3):
        lim = list(lim0)
        lim[axis] += 1
        for k in range(lim[2]):
            for j in range(lim[1]):
                for i in range(lim[0]):
                    im = [i, j, k]
                    im[axis] -= 1
                    a_ex, b_ex = exists(*im), exists(i, j, k)
                    if not a_ex and not b_ex:
                        continue
                    if axis == 0:
                        q = (vid(i, j, k), vid(i, j + 1, k), vid(i, j + 1, k + 1), vid(i, j, k + 1))
                    elif axis == 1:
                        q = (vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j, k + 1), vid(i, j, k + 1))
                    else:
                        q = (vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k))
                    if a_ex != b_ex:
                        on_outer = (i in (0, nx)) if axis == 0 else ((j in (0, ny)) if axis == 1 else (k in (0, nz)))
                        quad(bf, *q, False)
                        bc.extend([outer_bc if on_outer else hole_bc] * 2)
                    elif have_tf:
                        a_tf, b_tf = in_range(*im, tf_lo, tf_hi), in_range(i, j, k, tf_lo, tf_hi)
                        if a_tf != b_tf:
                            nrm = np.cross(V[q[1]] - V[q[0]], V[q[2]] - V[q[0]])
                            quad(tf, *q, bool(nrm[axis] > 0.0) != b_tf)
    as3 = lambda a: np.asarray(a, dtype=np.int32).reshape(-1, 3)
    return BoxMesh(V, E, as3(bf), np.asarray(bc, dtype=np.int32), as3(tf))


def dt_scale_min(vertices, elements) -> float:
    """min over elements of volume / (half the sum of its face areas) (reference getTimeStepScale
    restated for straight-sided tets, src/solver/Solver.cpp:289-300)."""
    P = np.asarray(vertices, dtype=np.float64)[np.asarray(elements)]          # [K, 4, 3]
    vol = np.abs(np.einsum("ki,ki->k", P[:, 1] - P[:, 0], np.cross(P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]))) / 6.0
    area = np.zeros(len(P))
    for f in ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)):
        a, b, cc = P[:, f[0]], P[:, f[1]], P[:, f[2]]
        area += 0.5 * np.linalg.norm(np.cross(b - a, cc - a), axis=1)
    return float(np.min(vol / (0.5 * area)))


def estimate_dt_3d(mesh, order: int, cfl: float = 1.0) -> float:
    """The reference's 3D estimate for the Global operator (Solver.cpp:289-300, 349-351):
    dtscale_min * rmin * 2/3 * 0.75 * cfl / 0.8, rmin the smallest Gauss-Lobatto spacing
    on [-1, 1] (lobatto() gives the nodes on [0, 1])."""
    g = lobatto(order)
    rmin = 2.0 * float(abs(g[1] - g[0]))
    return dt_scale_min(mesh.vertices, mesh.elements) * rmin * 2.0 / 3.0 * 0.75 * cfl / 0.8
