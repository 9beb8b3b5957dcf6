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
        h.orc_threads.restype = C.c_int
        h.orc_subop.restype = C.c_int
        h.orc_subop.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _D]
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

    def subop(self, kind: int, d: int = 0, d2: int = 0, beta_int: float = 1.0, beta_bdr: float = 1.0,
              minv_coef: float = 1.0) -> np.ndarray:
        """Dense (M^-1/minv_coef) F for one integrator (see orc_subop)."""
        out = np.zeros((self.ndofs, self.ndofs))
        self._chk(lib().orc_subop(self.h, kind, d, d2, beta_int, beta_bdr, minv_coef, _d(out)))
        return out


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
