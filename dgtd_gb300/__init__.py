"""dgtd_gb300 — GB300-native DG time-domain Maxwell step (Python binding).

The product is the CUDA shared library ``libdgtd_gb300.so`` built from
``dgtd_gb300/csrc`` (C ABI in ``include/dgtd_gb300.h``). This module is a thin
ctypes binding over it, used by the tests and the benchmark; there is no
Python or CPU compute path. Loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libdgtd_gb300.so"

DGTD_OK = 0
BC_OPEN, BC_PEC, BC_PMC, BC_SMA, BC_SGBC = 0, 1, 2, 3, 4
FP64, FP32_3XTF32, FP32 = 0, 1, 2
RK4, LSERK4 = 0, 1


class DgtdError(RuntimeError):
    """A C-ABI call returned an error status (``code``: the DGTD_ERR_* value)."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("n_vertices", C.c_int64), ("vertices", C.POINTER(C.c_double)),
        ("n_elements", C.c_int64), ("elements", C.POINTER(C.c_int32)),
        ("eps_r", C.POINTER(C.c_double)), ("mu_r", C.POINTER(C.c_double)), ("sigma", C.POINTER(C.c_double)),
        ("n_bdr_faces", C.c_int64), ("bdr_faces", C.POINTER(C.c_int32)), ("bdr_codes", C.POINTER(C.c_int32)),
        ("n_tfsf_faces", C.c_int64), ("tfsf_faces", C.POINTER(C.c_int32)),
        ("n_int_faces", C.c_int64), ("int_faces", C.POINTER(C.c_int32)), ("int_codes", C.POINTER(C.c_int32)),
        ("n_curved", C.c_int64), ("curved_elems", C.POINTER(C.c_int32)), ("curved_nodes", C.POINTER(C.c_double)),
    ]


class OpOpts(C.Structure):
    _fields_ = [("order", C.c_int32), ("alpha", C.c_double), ("precision", C.c_int32), ("batch", C.c_int32)]


class PlaneWave(C.Structure):
    _fields_ = [("propagation", C.c_double * 3), ("polarization", C.c_double * 3), ("spread", C.c_double),
                ("mean", C.c_double), ("frequency", C.c_double), ("batch", C.c_int32)]


class OpInfo(C.Structure):
    _fields_ = [("n_elements", C.c_int64), ("order", C.c_int32), ("np", C.c_int32), ("nfp", C.c_int32),
                ("batch", C.c_int32), ("precision", C.c_int32), ("ndofs", C.c_int64), ("state_len", C.c_int64),
                ("n_tfsf_faces", C.c_int64), ("min_edge", C.c_double), ("dt_scale_min", C.c_double),
                ("device_bytes", C.c_int64), ("work_len", C.c_int64), ("work_word_bytes", C.c_int32),
                ("batch_padded", C.c_int32)]


class BoxSpec(C.Structure):
    _fields_ = [("n", C.c_int32 * 3), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("hole_lo", C.c_int32 * 3), ("hole_hi", C.c_int32 * 3),
                ("tf_lo", C.c_int32 * 3), ("tf_hi", C.c_int32 * 3),
                ("outer_bc", C.c_int32), ("hole_bc", C.c_int32)]


class ProbeSpec(C.Structure):
    _fields_ = [("n_points", C.c_int32), ("points", C.POINTER(C.c_double)), ("n_surface_faces", C.c_int64),
                ("surface_faces", C.POINTER(C.c_int32)), ("n_freqs", C.c_int32), ("freqs", C.POINTER(C.c_double)),
                ("every", C.c_int32), ("max_records", C.c_int32)]


class SgbcLayer(C.Structure):
    _fields_ = [("eps_r", C.c_double), ("mu_r", C.c_double), ("sigma", C.c_double), ("width", C.c_double),
                ("segments", C.c_int32), ("order", C.c_int32)]


class SgbcStack(C.Structure):
    _fields_ = [("n_layers", C.c_int32), ("layers", C.POINTER(SgbcLayer)), ("left_bc", C.c_int32),
                ("right_bc", C.c_int32), ("sub_dt", C.c_double)]


class CaseInfo(C.Structure):
    _fields_ = [("order", C.c_int32), ("integrator", C.c_int32), ("alpha", C.c_double), ("time_step", C.c_double),
                ("final_time", C.c_double), ("cfl", C.c_double), ("n_waves", C.c_int32),
                ("n_initial_fields", C.c_int32), ("n_point_probes", C.c_int32), ("n_surfaces", C.c_int32),
                ("n_elements", C.c_int64), ("n_vertices", C.c_int64), ("n_sgbc_stacks", C.c_int32),
                ("n_sgbc_layers", C.c_int32), ("n_sgbc_faces", C.c_int64), ("basis_type", C.c_int32)]


class CaseRunOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("freqs", C.POINTER(C.c_double)), ("n_freqs", C.c_int32),
                ("out_dir", C.c_char_p)]


class CaseResult(C.Structure):
    _fields_ = [("steps", C.c_int64), ("dt", C.c_double), ("final_time", C.c_double), ("n_records", C.c_int64),
                ("seconds", C.c_double), ("unstable_step", C.c_int64)]


class ServerOpts(C.Structure):
    _fields_ = [("memory_budget", C.c_int64), ("max_active", C.c_int32), ("steps_per_round", C.c_int32),
                ("device", C.c_int32), ("precision", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("mesh", C.POINTER(MeshDesc)), ("order", C.c_int32), ("alpha", C.c_double),
                ("waves", C.POINTER(PlaneWave)), ("n_waves", C.c_int32), ("h_init", C.POINTER(C.c_double)),
                ("t0", C.c_double), ("final_time", C.c_double), ("dt", C.c_double), ("cfl", C.c_double)]


class RequestStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("order", C.c_int32), ("n_elements", C.c_int64), ("state_len", C.c_int64),
                ("steps", C.c_int64), ("region_bytes", C.c_int64), ("dt", C.c_double), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_first_launch", C.c_double), ("t_done", C.c_double),
                ("unstable", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("active", C.c_int64),
                ("queued", C.c_int64), ("stage_launches", C.c_int64), ("slot_stage_updates", C.c_int64),
                ("max_active_seen", C.c_int64), ("bytes_in_use", C.c_int64), ("peak_bytes_in_use", C.c_int64),
                ("memory_budget", C.c_int64), ("dof_updates", C.c_int64)]


REQ_QUEUED, REQ_ACTIVE, REQ_DONE, REQ_FAILED = 0, 1, 2, 3
SERVER_MAX_ACTIVE = 128
DGTD_ERR_TIMEOUT = -5
DGTD_ERR_UNSTABLE = -6

_lib_handle: Optional[C.CDLL] = None

# Every symbol the C ABI declares, with (restype, argtypes).
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_D_F = C.POINTER(C.c_float)
SIGNATURES = {
    "dgtd_last_error": (C.c_char_p, []),
    "dgtd_kernel_launches": (C.c_uint64, []),
    "dgtd_op_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(OpOpts), C.POINTER(_P)]),
    "dgtd_op_destroy": (None, [_P]),
    "dgtd_op_get_info": (C.c_int, [_P, C.POINTER(OpInfo)]),
    "dgtd_op_node_coords": (C.c_int, [_P, _D]),
    "dgtd_op_set_planewaves": (C.c_int, [_P, C.POINTER(PlaneWave), C.c_int32]),
    "dgtd_op_mult": (C.c_int, [_P, _P, _P, C.c_double, _P]),
    "dgtd_op_change_basis": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, _P]),
    "dgtd_op_mult_host": (C.c_int, [_P, _D, _D, C.c_double]),
    "dgtd_op_pack": (C.c_int, [_P, _P, _P, _P]),
    "dgtd_op_unpack": (C.c_int, [_P, _P, _P, _P]),
    "dgtd_op_step": (C.c_int, [_P, _P, C.c_double, C.c_double, C.c_int32, C.c_int32, _P]),
    "dgtd_op_run_host": (C.c_int, [_P, _D, C.c_double, C.c_double, C.c_double, C.c_int32, _I64]),
    "dgtd_op_step_noalloc": (C.c_int, [_P, _P, C.c_double, C.c_double, C.c_int32, C.c_int32, _P]),
    "dgtd_noalloc_max_state": (C.c_int64, []),
    "dgtd_op_norm2": (C.c_int, [_P, _P, _D, _P]),
    "dgtd_op_set_stability_check": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "dgtd_op_stability": (C.c_int, [_P, _I64, _D, _D, _I64]),
    "dgtd_op_stability_check": (C.c_int, [_P, _P, C.c_int64, C.c_double, _P]),
    "dgtd_op_stability_reset": (C.c_int, [_P]),
    "dgtd_op_set_contraction": (C.c_int, [_P, C.c_int32]),
    "dgtd_op_uses_tensor_cores": (C.c_int, [_P]),
    "dgtd_op_set_graph_steps": (C.c_int, [_P, C.c_int32]),
    "dgtd_op_set_defect_correction": (C.c_int, [_P, C.c_int32]),
    "dgtd_op_defect_refreshes": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "dgtd_op_autotune": (C.c_int, [_P, _P, _P, _D, _I32]),
    "dgtd_op_check": (C.c_int, [_P, _P]),
    "dgtd_op_estimate_dt": (C.c_int, [_P, C.c_double, _D]),
    "dgtd_box_mesh_size": (C.c_int, [C.POINTER(BoxSpec), _I64, _I64, _I64, _I64]),
    "dgtd_box_mesh_fill": (C.c_int, [C.POINTER(BoxSpec), _D, _I32, _I32, _I32, _I32]),
    "dgtd_ref_tet": (C.c_int, [C.c_int32, _D, _D, _D, _D, _D, _D, _D, _D, _I32]),
    "dgtd_mesh_validate": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(OpOpts), C.POINTER(OpInfo)]),
    "dgtd_tc_selftest": (C.c_int, [_D_F, _D_F, _D_F, C.c_int32, _I32]),
    "dgtd_op_set_probes": (C.c_int, [_P, C.POINTER(ProbeSpec)]),
    "dgtd_op_set_sgbc": (C.c_int, [_P, C.POINTER(SgbcStack), C.c_int32, _I32]),
    "dgtd_op_sgbc_states": (C.c_int, [_P, _I64, _I64, _D, C.c_int64]),
    "dgtd_op_sgbc_commit": (C.c_int, [_P, _P, C.c_double, C.c_double, _P]),
    "dgtd_op_sgbc_finalize": (C.c_int, [_P, _P, _P]),
    "dgtd_sgbc_stack_operator": (C.c_int, [C.POINTER(SgbcStack), _I64, _I64, _I64, _D, C.c_int64]),
    "dgtd_sgbc_stack_maps": (C.c_int, [C.POINTER(SgbcStack), C.c_double, C.c_int32, _D, _D, _D, _D, _D]),
    "dgtd_curved_block_rows": (C.c_int, [C.POINTER(MeshDesc), C.c_int32, C.c_double, _I32, _I32, _D, C.c_int64]),
    "dgtd_tet_nodes": (C.c_int, [C.c_int32, C.c_int32, _D]),
    "dgtd_tet_basis_change": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _D]),
    "dgtd_op_clear_probes": (C.c_int, [_P]),
    "dgtd_op_probe_reset": (C.c_int, [_P, _P]),
    "dgtd_op_probe_info": (C.c_int, [_P, _I64, _I64, _I64]),
    "dgtd_op_probe_surface": (C.c_int, [_P, _D, _D, _D]),
    "dgtd_op_probe_sample": (C.c_int, [_P, _P, C.c_double, _P]),
    "dgtd_op_probe_read": (C.c_int, [_P, _D, _D, _D, _D, _P]),
    "dgtd_case_load": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "dgtd_case_destroy": (None, [_P]),
    "dgtd_case_get_info": (C.c_int, [_P, C.POINTER(CaseInfo)]),
    "dgtd_case_auto_dt": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dgtd_case_sgbc": (C.c_int, [_P, C.POINTER(SgbcStack), C.POINTER(SgbcLayer), _I32]),
    "dgtd_case_mesh": (C.c_int, [_P, C.POINTER(MeshDesc)]),
    "dgtd_case_planewaves": (C.c_int, [_P, C.POINTER(PlaneWave), C.c_int32]),
    "dgtd_case_point_probes": (C.c_int, [_P, _D]),
    "dgtd_case_surface": (C.c_int, [_P, C.c_int32, _I32, _I64]),
    "dgtd_case_initial_state": (C.c_int, [_P, _D, C.c_int64, _D]),
    "dgtd_case_run": (C.c_int, [_P, C.POINTER(CaseRunOpts), _D, C.POINTER(CaseResult)]),
    "dgtd_server_create": (C.c_int, [C.POINTER(ServerOpts), C.POINTER(_P)]),
    "dgtd_server_destroy": (None, [_P]),
    "dgtd_server_submit": (C.c_int, [_P, C.POINTER(Request), _I64]),
    "dgtd_server_wait": (C.c_int, [_P, C.c_int64, C.c_double, _D, C.POINTER(RequestStats)]),
    "dgtd_server_query": (C.c_int, [_P, C.c_int64, C.POINTER(RequestStats)]),
    "dgtd_server_get_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "dgtd_arena_create": (C.c_int, [C.c_int64, C.c_int64, C.POINTER(_P)]),
    "dgtd_arena_destroy": (None, [_P]),
    "dgtd_arena_alloc": (C.c_int64, [_P, C.c_int64]),
    "dgtd_arena_release": (C.c_int, [_P, C.c_int64]),
    "dgtd_arena_usage": (C.c_int, [_P, _I64, _I64, _I64]),
}


def lib() -> C.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib_handle
    if _lib_handle is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib_handle = h
    return _lib_handle


def kernel_launches() -> int:
    """Kernels launched by the CUDA library in this process so far."""
    return int(lib().dgtd_kernel_launches())


def noalloc_max_state() -> int:
    """Largest reference-layout state (6*K*Np*B entries) Operator.step_noalloc accepts."""
    return int(lib().dgtd_noalloc_max_state())


def _check(rc: int, what: str) -> None:
    if rc != DGTD_OK:
        msg = lib().dgtd_last_error().decode(errors="replace")
        raise DgtdError(f"{what} failed ({rc}): {msg}", rc)


def _waves_array(waves: Sequence[dict]):
    arr = (PlaneWave * max(1, len(waves)))()
    for i, w in enumerate(waves):
        arr[i].propagation[:] = list(map(float, w["propagation"]))
        arr[i].polarization[:] = list(map(float, w["polarization"]))
        arr[i].spread = float(w["spread"]); arr[i].mean = float(w["mean"])
        arr[i].frequency = float(w.get("frequency", 0.0)); arr[i].batch = int(w.get("batch", 0))
    return arr


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_I32)


@dataclass
class Mesh:
    """Flat mesh tables (vertices [nv,3], tets [ne,4], boundary/TF-SF faces)."""
    vertices: np.ndarray
    elements: np.ndarray
    bdr_faces: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    bdr_codes: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))
    tfsf_faces: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    int_faces: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    int_codes: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))
    eps: Optional[np.ndarray] = None
    mu: Optional[np.ndarray] = None
    sigma: Optional[np.ndarray] = None
    dim: int = 3
    # second-order (curved) elements: ids and [n, 10, 3] geometry nodes (corners, then the edge
    # nodes of (0,1) (0,2) (0,3) (1,2) (1,3) (2,3))
    curved_elems: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))
    curved_nodes: np.ndarray = field(default_factory=lambda: np.zeros((0, 10, 3), np.float64))

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])

    def normalized(self) -> "Mesh":
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        return Mesh(f64(self.vertices), i32(self.elements), i32(self.bdr_faces).reshape(-1, 3),
                    i32(self.bdr_codes).reshape(-1), i32(self.tfsf_faces).reshape(-1, 3),
                    i32(self.int_faces).reshape(-1, 3), i32(self.int_codes).reshape(-1),
                    f64(self.eps), f64(self.mu), f64(self.sigma), self.dim,
                    i32(self.curved_elems).reshape(-1), f64(self.curved_nodes).reshape(-1, 10, 3))


def box_mesh(n: Sequence[int], lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), hole=None, tfsf=None,
             outer_bc: int = BC_PEC, hole_bc: int = BC_PEC) -> Mesh:
    """Structured box of n[0] x n[1] x n[2] hexes, each split into 6 tets.

    hole / tfsf: ((i0, j0, k0), (i1, j1, k1)) cell-index ranges (half open).
    """
    s = BoxSpec()
    for d in range(3):
        s.n[d] = int(n[d]); s.lo[d] = float(lo[d]); s.hi[d] = float(hi[d])
        if hole is not None:
            s.hole_lo[d] = int(hole[0][d]); s.hole_hi[d] = int(hole[1][d])
        if tfsf is not None:
            s.tf_lo[d] = int(tfsf[0][d]); s.tf_hi[d] = int(tfsf[1][d])
    s.outer_bc = outer_bc; s.hole_bc = hole_bc
    nv, ne, nb, nt = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    L = lib()
    _check(L.dgtd_box_mesh_size(C.byref(s), C.byref(nv), C.byref(ne), C.byref(nb), C.byref(nt)), "box_mesh_size")
    V = np.zeros((nv.value, 3)); E = np.zeros((ne.value, 4), np.int32)
    BF = np.zeros((nb.value, 3), np.int32); BC = np.zeros((nb.value,), np.int32)
    TF = np.zeros((nt.value, 3), np.int32)
    _check(L.dgtd_box_mesh_fill(C.byref(s), _dp(V), _ip(E), _ip(BF), _ip(BC), _ip(TF)), "box_mesh_fill")
    return Mesh(V, E, BF, BC, TF)


def ref_tet(order: int) -> dict:
    """The product's reference-element tables (host), for known-answer tests."""
    np_ = (order + 1) * (order + 2) * (order + 3) // 6
    nfp = (order + 1) * (order + 2) // 2
    out = {k: np.zeros(np_) for k in ("r", "s", "t")}
    for k in ("Dr", "Ds", "Dt", "Minv"):
        out[k] = np.zeros((np_, np_))
    out["LIFT"] = np.zeros((np_, 4 * nfp))
    out["Fmask"] = np.zeros((4, nfp), np.int32)
    _check(lib().dgtd_ref_tet(order, *(_dp(out[k]) for k in ("r", "s", "t", "Dr", "Ds", "Dt", "Minv", "LIFT")),
                              _ip(out["Fmask"])), "ref_tet")
    return out


def tc_selftest(a: np.ndarray, b: np.ndarray):
    """Run the device tensor-core self-check: returns (D = A B^T in 3xTF32, status)."""
    a = np.ascontiguousarray(a, dtype=np.float32); b = np.ascontiguousarray(b, dtype=np.float32)
    assert a.shape[0] == 128 and b.shape[0] == 48 and a.shape[1] == b.shape[1]
    d = np.zeros((128, 48), np.float32)
    st = C.c_int32()
    fp = C.POINTER(C.c_float)
    _check(lib().dgtd_tc_selftest(a.ctypes.data_as(fp), b.ctypes.data_as(fp), d.ctypes.data_as(fp),
                                  a.shape[1], C.byref(st)), "dgtd_tc_selftest")
    return d, int(st.value)


def _ptr(x) -> int:
    """Device pointer of a torch tensor or a raw integer address."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError("expected a torch CUDA tensor or a device address")


def _stream(s) -> Optional[int]:
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return int(s.cuda_stream) if hasattr(s, "cuda_stream") else int(s)


def _sgbc_structs(stacks: Sequence[dict]):
    """ctypes stacks (and the layer arrays they point to) from dicts {"layers": [{"eps", "mu",
    "sigma", "width", "segments", "order"}], "left": bc, "right": bc, "sub_dt": s}."""
    keep = []
    arr = (SgbcStack * max(1, len(stacks)))()
    for i, st in enumerate(stacks):
        L = (SgbcLayer * len(st["layers"]))()
        for j, l in enumerate(st["layers"]):
            L[j] = SgbcLayer(float(l.get("eps", 1.0)), float(l.get("mu", 1.0)), float(l.get("sigma", 0.0)),
                             float(l["width"]), int(l["segments"]), int(l["order"]))
        keep.append(L)
        arr[i] = SgbcStack(len(st["layers"]), C.cast(L, C.POINTER(SgbcLayer)), int(st.get("left", 0)),
                           int(st.get("right", 0)), float(st.get("sub_dt", 0.0)))
    return arr, keep


def sgbc_stack_operator(stack: dict) -> dict:
    """The thin-layer sub-solver of one stack, built on the host: its operator A [n, n] and its
    interface rows (no GPU)."""
    arr, keep = _sgbc_structs([stack])
    n, il, ir = C.c_int64(), C.c_int64(), C.c_int64()
    _check(lib().dgtd_sgbc_stack_operator(arr, C.byref(n), C.byref(il), C.byref(ir), None, 0), "sgbc_stack_operator")
    A = np.zeros((n.value, n.value))
    _check(lib().dgtd_sgbc_stack_operator(arr, None, None, None, _dp(A), A.size), "sgbc_stack_operator")
    return {"A": A, "n": n.value, "idx_left": il.value, "idx_right": ir.value}


def sgbc_stack_maps(stack: dict, span: float, nsteps: int) -> dict:
    """Composed sub-step maps of one stack (no GPU): interface values R x + G g with ghosts held,
    state F x + Vo g_old + Vn g_new with ghosts interpolated."""
    n = sgbc_stack_operator(stack)["n"]
    arr, keep = _sgbc_structs([stack])
    out = {"R": np.zeros((12, n)), "G": np.zeros((12, 12)), "F": np.zeros((n, n)), "Vo": np.zeros((n, 12)),
           "Vn": np.zeros((n, 12))}
    _check(lib().dgtd_sgbc_stack_maps(arr, float(span), int(nsteps), *(_dp(out[k]) for k in ("R", "G", "F", "Vo", "Vn"))),
           "sgbc_stack_maps")
    return out


def _mesh_desc(m: Mesh) -> MeshDesc:
    d = MeshDesc()
    d.dim = 3
    d.n_vertices = m.vertices.shape[0]; d.vertices = _dp(m.vertices)
    d.n_elements = m.elements.shape[0]; d.elements = _ip(m.elements)
    null_d = C.POINTER(C.c_double)()
    d.eps_r = _dp(m.eps) if m.eps is not None else null_d
    d.mu_r = _dp(m.mu) if m.mu is not None else null_d
    d.sigma = _dp(m.sigma) if m.sigma is not None else null_d
    d.n_bdr_faces = m.bdr_codes.shape[0]; d.bdr_faces = _ip(m.bdr_faces); d.bdr_codes = _ip(m.bdr_codes)
    d.n_tfsf_faces = m.tfsf_faces.shape[0]; d.tfsf_faces = _ip(m.tfsf_faces)
    d.n_int_faces = m.int_codes.shape[0]; d.int_faces = _ip(m.int_faces); d.int_codes = _ip(m.int_codes)
    d.n_curved = m.curved_elems.shape[0]
    d.curved_elems = _ip(m.curved_elems) if d.n_curved else C.POINTER(C.c_int32)()
    d.curved_nodes = _dp(m.curved_nodes) if d.n_curved else null_d
    return d


def curved_block_rows(mesh: Mesh, order: int, alpha: float = 1.0) -> dict:
    """The curved elements' rows of the operator, built on the host (no GPU): blocks
    [n, 5, 6 Np, 6 Np] over the element's own state (block 0) and its face neighbours'."""
    m = mesh.normalized()
    d = _mesh_desc(m)
    n = m.curved_elems.shape[0]
    Np = (order + 1) * (order + 2) * (order + 3) // 6
    el, nb = np.zeros(n, np.int32), np.zeros((n, 4), np.int32)
    B = np.zeros((n, 5, 6 * Np, 6 * Np))
    _check(lib().dgtd_curved_block_rows(C.byref(d), order, alpha, _ip(el), _ip(nb), _dp(B), B.size), "curved_block_rows")
    return {"elems": el, "nbr": nb, "blocks": B}


BASIS_GAUSS_LEGENDRE, BASIS_GAUSS_LOBATTO = 0, 1


def tet_nodes(order: int, basis_type: int = BASIS_GAUSS_LOBATTO) -> np.ndarray:
    """Barycentric coordinates [Np, 4] of the order-p tetrahedron's nodes of an MFEM basis type
    (1 Gauss-Lobatto: the operator's node set; 0 Gauss-Legendre), in DOF order."""
    Np = (order + 1) * (order + 2) * (order + 3) // 6
    out = np.zeros((Np, 4))
    _check(lib().dgtd_tet_nodes(order, basis_type, _dp(out)), "dgtd_tet_nodes")
    return out


def tet_basis_change(order: int, from_basis: int, to_basis: int) -> np.ndarray:
    """[Np, Np] matrix M with v_to = M v_from for the nodal values of a degree-p polynomial."""
    Np = (order + 1) * (order + 2) * (order + 3) // 6
    out = np.zeros((Np, Np))
    _check(lib().dgtd_tet_basis_change(order, from_basis, to_basis, _dp(out)), "dgtd_tet_basis_change")
    return out


def validate_mesh(mesh: Mesh, order: int = 3, batch: int = 1) -> dict:
    """Build the mesh tables on the host only (no GPU) and return the op info."""
    m = mesh.normalized()
    d = _mesh_desc(m)
    o = OpOpts(order=order, alpha=1.0, precision=FP64, batch=batch)
    inf = OpInfo()
    _check(lib().dgtd_mesh_validate(C.byref(d), C.byref(o), C.byref(inf)), "dgtd_mesh_validate")
    return {k: getattr(inf, k) for k, _ in OpInfo._fields_}


class Operator:
    """DG Maxwell evolution operator on the GPU (the reference's
    ``GlobalEvolution : mfem::TimeDependentOperator``, GlobalEvolution.h:14-111).

    ``mult(x, y, t)`` is ``Mult`` with ``SetTime(t)``; ``step`` fuses the RK
    stages; all compute runs in the CUDA library.
    """

    def __init__(self, mesh: Mesh, order: int = 3, alpha: float = 1.0, precision: int = FP64, batch: int = 1):
        m = mesh.normalized()
        self._keep = m
        d = _mesh_desc(m)
        o = OpOpts(order=order, alpha=alpha, precision=precision, batch=batch)
        h = C.c_void_p()
        _check(lib().dgtd_op_create(C.byref(d), C.byref(o), C.byref(h)), "dgtd_op_create")
        self._h = h
        inf = OpInfo()
        _check(lib().dgtd_op_get_info(self._h, C.byref(inf)), "get_info")
        self.info = {k: getattr(inf, k) for k, _ in OpInfo._fields_}
        self.order = order
        self.batch = batch
        self.precision = precision

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().dgtd_op_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def state_len(self) -> int:
        """Entries of the reference-layout state (6 K Np B)."""
        return int(self.info["state_len"])

    @property
    def work_len(self) -> int:
        """Entries of the working state used by mult/step (FP64: reference layout; FP32: internal)."""
        return int(self.info["work_len"])

    def work_dtype(self):
        import torch
        return torch.float64 if int(self.info["work_word_bytes"]) == 8 else torch.float32

    def new_work(self, device="cuda"):
        import torch
        return torch.zeros(self.work_len, dtype=self.work_dtype(), device=device)

    def pack(self, ref, work, stream=None) -> None:
        """Reference-layout FP64 device state -> working state."""
        _check(lib().dgtd_op_pack(self._h, _ptr(ref), _ptr(work), _stream(stream)), "dgtd_op_pack")

    def unpack(self, work, ref, stream=None) -> None:
        _check(lib().dgtd_op_unpack(self._h, _ptr(work), _ptr(ref), _stream(stream)), "dgtd_op_unpack")

    @property
    def ndofs(self) -> int:
        return int(self.info["ndofs"])

    def node_coords(self) -> np.ndarray:
        xyz = np.zeros((3, self.ndofs))
        _check(lib().dgtd_op_node_coords(self._h, _dp(xyz)), "node_coords")
        return xyz

    def set_planewaves(self, waves: Sequence[dict]) -> None:
        _check(lib().dgtd_op_set_planewaves(self._h, _waves_array(waves), len(waves)), "set_planewaves")

    def estimate_dt(self, cfl: float = 1.0) -> float:
        v = C.c_double()
        _check(lib().dgtd_op_estimate_dt(self._h, cfl, C.byref(v)), "estimate_dt")
        return v.value

    def set_sgbc(self, stacks: Sequence[dict], face_stack) -> None:
        """Thin-layer stacks of the mesh's SGBC interior faces (code BC_SGBC), face_stack[i] the
        stack of the i-th such face in mesh order (see sgbc_stack_operator for the stack dicts)."""
        arr, keep = _sgbc_structs(stacks)
        fs = np.ascontiguousarray(face_stack, dtype=np.int32)
        _check(lib().dgtd_op_set_sgbc(self._h, arr, len(stacks), _ip(fs)), "dgtd_op_set_sgbc")

    def sgbc_commit(self, x, t: float, dt: float, stream=None) -> None:
        """Start of a step driven through mult (the reference's commitSGBCCheckpoint)."""
        _check(lib().dgtd_op_sgbc_commit(self._h, _ptr(x), float(t), float(dt), _stream(stream)), "dgtd_op_sgbc_commit")

    def sgbc_finalize(self, x, stream=None) -> None:
        """End of a step driven through mult, x the step's end state (finalizeSGBCStep)."""
        _check(lib().dgtd_op_sgbc_finalize(self._h, _ptr(x), _stream(stream)), "dgtd_op_sgbc_finalize")

    def sgbc_states(self) -> np.ndarray:
        """The sub-solver states, pair after pair (empty without SGBC)."""
        npair, sl = C.c_int64(), C.c_int64()
        _check(lib().dgtd_op_sgbc_states(self._h, C.byref(npair), C.byref(sl), None, 0), "sgbc_states")
        out = np.zeros(sl.value)
        if sl.value:
            _check(lib().dgtd_op_sgbc_states(self._h, None, None, _dp(out), out.size), "sgbc_states")
        return out

    # -- device API (torch tensors or raw device addresses)
    def mult(self, x, y, t: float = 0.0, stream=None) -> None:
        _check(lib().dgtd_op_mult(self._h, _ptr(x), _ptr(y), float(t), _stream(stream)), "dgtd_op_mult")

    def change_basis(self, x, y, from_basis: int, to_basis: int, stream=None) -> None:
        """FP64 form: y = the state x moved between nodal bases (BASIS_GAUSS_LEGENDRE,
        BASIS_GAUSS_LOBATTO) element by element on the device; x and y distinct."""
        _check(lib().dgtd_op_change_basis(self._h, _ptr(x), _ptr(y), int(from_basis), int(to_basis),
                                          _stream(stream)), "dgtd_op_change_basis")

    def step(self, state, t0: float, dt: float, nsteps: int, integrator: int = RK4, stream=None) -> None:
        _check(lib().dgtd_op_step(self._h, _ptr(state), float(t0), float(dt), int(nsteps), int(integrator),
                                  _stream(stream)), "dgtd_op_step")

    def step_noalloc(self, state, t0: float, dt: float, nsteps: int, integrator: int = RK4, stream=None) -> None:
        """FP64 form: dgtd_op_step with the RK registers in the library's fixed device
        scratch (no device allocation; calls overlapping on the GPU race)."""
        _check(lib().dgtd_op_step_noalloc(self._h, _ptr(state), float(t0), float(dt), int(nsteps), int(integrator),
                                          _stream(stream)), "dgtd_op_step_noalloc")

    def set_contraction(self, mode: int) -> None:
        """FP32 forms: 0 = tensor cores (tcgen05 3xTF32) where supported, 1 = FP32 SIMT
        (defaults: 0 for the batched form, 1 for the single-instance form)."""
        _check(lib().dgtd_op_set_contraction(self._h, int(mode)), "dgtd_op_set_contraction")

    TUNE_CANDIDATES = ("tensor cores (3xTF32, 64 incidences x 1 element per work item)",
                       "FP32 SIMT, 4 warps x 32 incidences per block", "FP32 SIMT, 8 warps x 32 incidences per block",
                       "FP32 SIMT, 16 warps x 32 incidences per block")

    def autotune(self, work, stream=None) -> dict:
        """Batched FP32 form: time the candidate stage kernels and keep the fastest."""
        ms = np.zeros(4)
        ch = C.c_int32()
        _check(lib().dgtd_op_autotune(self._h, _ptr(work), _stream(stream), _dp(ms), C.byref(ch)), "dgtd_op_autotune")
        return {"choice": int(ch.value), "kernel": self.TUNE_CANDIDATES[ch.value],
                "ms_per_launch": {self.TUNE_CANDIDATES[i]: float(ms[i]) for i in range(4) if ms[i] >= 0}}

    def set_graph_steps(self, steps: int) -> None:
        """Batched FP32 form: replay blocks of `steps` RK4 steps from one captured CUDA graph (0: off)."""
        _check(lib().dgtd_op_set_graph_steps(self._h, int(steps)), "dgtd_op_set_graph_steps")

    def set_defect_correction(self, every: int) -> None:
        """Batched FP32 form, classical RK4: every `every` steps (0: off) form c = L64(x) - L32(x)
        with the FP64 operator, keep it where the state has not moved since the previous refresh,
        and add its RK4 step increment to the state after every step."""
        _check(lib().dgtd_op_set_defect_correction(self._h, int(every)), "dgtd_op_set_defect_correction")

    @property
    def defect_refreshes(self) -> int:
        n = C.c_int64()
        _check(lib().dgtd_op_defect_refreshes(self._h, C.byref(n)), "dgtd_op_defect_refreshes")
        return int(n.value)

    @property
    def uses_tensor_cores(self) -> bool:
        return bool(lib().dgtd_op_uses_tensor_cores(self._h))

    def check(self, stream=None) -> None:
        """Synchronise and raise if a kernel reported a timed-out device wait."""
        _check(lib().dgtd_op_check(self._h, _stream(stream)), "dgtd_op_check")

    def norm2(self, state, stream=None) -> np.ndarray:
        out = np.zeros(self.batch)
        _check(lib().dgtd_op_norm2(self._h, _ptr(state), _dp(out), _stream(stream)), "dgtd_op_norm2")
        return out

    def set_stability_check(self, every: int = 10, stop: bool = False) -> None:
        """Instability detector of run_host (reference Solver.cpp:500-516): a device norm check
        every `every` steps (0: off); stop=True ends the run with DGTD_ERR_UNSTABLE, else a
        warning is printed on stderr and the run goes on (the reference's behaviour)."""
        _check(lib().dgtd_op_set_stability_check(self._h, int(every), 1 if stop else 0),
               "dgtd_op_set_stability_check")

    def stability(self) -> dict:
        st, t, nrm, ch = C.c_int64(), C.c_double(), C.c_double(), C.c_int64()
        _check(lib().dgtd_op_stability(self._h, C.byref(st), C.byref(t), C.byref(nrm), C.byref(ch)),
               "dgtd_op_stability")
        return {"first_step": st.value, "t": t.value, "norm": nrm.value, "checks": ch.value,
                "unstable": st.value >= 0}

    # -- probes (point probes, near-to-far surface, running FP64 DFT sums)
    def set_probes(self, points=None, surface_faces=None, freqs=(), every: int = 1, max_records: int = 0) -> None:
        pts = np.ascontiguousarray(np.zeros((0, 3)) if points is None else points, dtype=np.float64).reshape(-1, 3)
        fcs = np.ascontiguousarray(np.zeros((0, 3)) if surface_faces is None else surface_faces,
                                   dtype=np.int32).reshape(-1, 3)
        fr = np.ascontiguousarray(freqs, dtype=np.float64).reshape(-1)
        self._probe_keep = (pts, fcs, fr)
        sp = ProbeSpec(n_points=pts.shape[0], points=_dp(pts), n_surface_faces=fcs.shape[0], surface_faces=_ip(fcs),
                       n_freqs=fr.shape[0], freqs=_dp(fr), every=int(every), max_records=int(max_records))
        _check(lib().dgtd_op_set_probes(self._h, C.byref(sp)), "dgtd_op_set_probes")
        self._probe_shape = (pts.shape[0], fr.shape[0], int(max_records))

    def clear_probes(self) -> None:
        _check(lib().dgtd_op_clear_probes(self._h), "dgtd_op_clear_probes")

    def probe_reset(self, stream=None) -> None:
        _check(lib().dgtd_op_probe_reset(self._h, _stream(stream)), "dgtd_op_probe_reset")

    def probe_sample(self, state, t: float, stream=None) -> None:
        _check(lib().dgtd_op_probe_sample(self._h, _ptr(state), float(t), _stream(stream)), "dgtd_op_probe_sample")

    def probe_info(self) -> dict:
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().dgtd_op_probe_info(self._h, C.byref(a), C.byref(b), C.byref(c)), "dgtd_op_probe_info")
        return {"n_surface_nodes": a.value, "n_samples": b.value, "n_records": c.value}

    def probe_surface(self):
        n = self.probe_info()["n_surface_nodes"]
        xyz, nrm, w = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        _check(lib().dgtd_op_probe_surface(self._h, _dp(xyz), _dp(nrm), _dp(w)), "dgtd_op_probe_surface")
        return xyz, nrm, w

    def probe_read(self, stream=None) -> dict:
        """Raw DFT sums as complex arrays: points [B, n_points, 6, nf], surface [B, n_surf, 6, nf];
        series [n_records, B, n_points, 6] and its times."""
        npts, nf, _ = self._probe_shape
        info = self.probe_info()
        ns, nr = info["n_surface_nodes"], info["n_records"]
        B = self.batch
        pd = np.zeros((B, npts, 6, nf, 2)); sd = np.zeros((B, ns, 6, nf, 2))
        se = np.zeros((nr, B, npts, 6)); st = np.zeros(nr)
        _check(lib().dgtd_op_probe_read(self._h, _dp(pd), _dp(sd), _dp(se), _dp(st), _stream(stream)),
               "dgtd_op_probe_read")
        return {"points": pd[..., 0] + 1j * pd[..., 1], "surface": sd[..., 0] + 1j * sd[..., 1], "series": se,
                "times": st, "n_samples": info["n_samples"]}

    # -- host API
    def mult_host(self, x: np.ndarray, t: float = 0.0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        _check(lib().dgtd_op_mult_host(self._h, _dp(x), _dp(y), float(t)), "dgtd_op_mult_host")
        return y

    def run_host(self, x: np.ndarray, t0: float, dt: float, final_time: float, integrator: int = RK4):
        x = np.array(x, dtype=np.float64, copy=True)
        n = C.c_int64()
        _check(lib().dgtd_op_run_host(self._h, _dp(x), float(t0), float(dt), float(final_time), int(integrator),
                                      C.byref(n)), "dgtd_op_run_host")
        return x, int(n.value)


class Server:
    """Continuous-batching server of independent solves (C ABI ``dgtd_server_*``).

    Each request is one ``Solver::run`` of its own mesh, order, plane waves and
    final time (plain FP64 operator, classical RK4). ``submit`` returns at once;
    ``wait`` returns the final state (reference layout) and the request's timing.
    """

    def __init__(self, memory_budget: int = 4 << 30, max_active: int = 64, steps_per_round: int = 4, device: int = 0,
                 precision: int = FP64):
        o = ServerOpts(memory_budget=int(memory_budget), max_active=int(max_active),
                       steps_per_round=int(steps_per_round), device=int(device), precision=int(precision))
        h = C.c_void_p()
        _check(lib().dgtd_server_create(C.byref(o), C.byref(h)), "dgtd_server_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().dgtd_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, mesh: Mesh, order: int, final_time: float, waves: Sequence[dict] = (), init=None,
               dt: float = 0.0, cfl: float = 1.0, alpha: float = 1.0, t0: float = 0.0) -> int:
        m = mesh.normalized()
        d = _mesh_desc(m)
        arr = _waves_array(waves)
        q = Request()
        q.mesh = C.pointer(d)
        q.order = int(order); q.alpha = float(alpha)
        q.waves = arr; q.n_waves = len(waves)
        keep = None
        if init is not None:
            keep = np.ascontiguousarray(init, dtype=np.float64)
            q.h_init = _dp(keep)
        q.t0 = float(t0); q.final_time = float(final_time); q.dt = float(dt); q.cfl = float(cfl)
        rid = C.c_int64()
        _check(lib().dgtd_server_submit(self._h, C.byref(q), C.byref(rid)), "dgtd_server_submit")
        return int(rid.value)

    def wait(self, rid: int, timeout: float = -1.0, want_state: bool = True):
        """(final state in the reference layout or None, stats dict) of a request, which is then
        released. Raises DgtdError (code -5 when the timeout expires, the request stays pending)."""
        st = RequestStats()
        out = None
        if want_state:
            _check(lib().dgtd_server_query(self._h, int(rid), C.byref(st)), "dgtd_server_query")
            out = np.zeros(int(st.state_len))
        _check(lib().dgtd_server_wait(self._h, int(rid), float(timeout), _dp(out) if out is not None else None,
                                      C.byref(st)), "dgtd_server_wait")
        return out, {k: getattr(st, k) for k, _ in RequestStats._fields_}

    def query(self, rid: int) -> dict:
        st = RequestStats()
        _check(lib().dgtd_server_query(self._h, int(rid), C.byref(st)), "dgtd_server_query")
        return {k: getattr(st, k) for k, _ in RequestStats._fields_}

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().dgtd_server_get_stats(self._h, C.byref(st)), "dgtd_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}


class Arena:
    """Host-side first-fit range allocator the server uses for its device budget."""

    def __init__(self, capacity: int, align: int = 256):
        h = C.c_void_p()
        _check(lib().dgtd_arena_create(int(capacity), int(align), C.byref(h)), "dgtd_arena_create")
        self._h = h

    def alloc(self, nbytes: int) -> int:
        return int(lib().dgtd_arena_alloc(self._h, int(nbytes)))

    def release(self, off: int) -> None:
        _check(lib().dgtd_arena_release(self._h, int(off)), "dgtd_arena_release")

    def usage(self) -> dict:
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().dgtd_arena_usage(self._h, C.byref(a), C.byref(b), C.byref(c)), "dgtd_arena_usage")
        return {"in_use": a.value, "largest_free": b.value, "n_free_ranges": c.value}

    def __del__(self):
        try:
            if self._h.value:
                lib().dgtd_arena_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass


class Case:
    """A reference JSON case (``driver::buildSolverJson`` input) and its gmsh 2.2 mesh."""

    def __init__(self, json_path):
        h = C.c_void_p()
        _check(lib().dgtd_case_load(str(json_path).encode(), C.byref(h)), "dgtd_case_load")
        self._h = h
        inf = CaseInfo()
        _check(lib().dgtd_case_get_info(self._h, C.byref(inf)), "dgtd_case_get_info")
        self.info = {k: getattr(inf, k) for k, _ in CaseInfo._fields_}

    def __del__(self):
        try:
            if self._h.value:
                lib().dgtd_case_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def auto_dt(self) -> float:
        """The time step of a run with time_step 0: the reference's estimate for the case's
        evolution operator (computed on the host)."""
        v = C.c_double()
        _check(lib().dgtd_case_auto_dt(self._h, C.byref(v)), "dgtd_case_auto_dt")
        return float(v.value)

    def mesh(self) -> Mesh:
        d = MeshDesc()
        _check(lib().dgtd_case_mesh(self._h, C.byref(d)), "dgtd_case_mesh")
        nv, ne, nb, nt, ni = d.n_vertices, d.n_elements, d.n_bdr_faces, d.n_tfsf_faces, d.n_int_faces
        arr = lambda p, n, dt: np.ctypeslib.as_array(p, shape=(n,)).astype(dt).copy() if n > 0 else np.zeros(0, dt)
        nc = d.n_curved
        return Mesh(arr(d.vertices, 3 * nv, np.float64).reshape(-1, 3), arr(d.elements, 4 * ne, np.int32).reshape(-1, 4),
                    arr(d.bdr_faces, 3 * nb, np.int32).reshape(-1, 3), arr(d.bdr_codes, nb, np.int32),
                    arr(d.tfsf_faces, 3 * nt, np.int32).reshape(-1, 3), arr(d.int_faces, 3 * ni, np.int32).reshape(-1, 3),
                    arr(d.int_codes, ni, np.int32), arr(d.eps_r, ne, np.float64), arr(d.mu_r, ne, np.float64),
                    arr(d.sigma, ne, np.float64), 3, arr(d.curved_elems, nc, np.int32),
                    arr(d.curved_nodes, 30 * nc, np.float64).reshape(-1, 10, 3))

    def planewaves(self) -> list:
        n = self.info["n_waves"]
        a = (PlaneWave * max(1, n))()
        _check(lib().dgtd_case_planewaves(self._h, a, n), "dgtd_case_planewaves")
        return [dict(propagation=list(a[i].propagation), polarization=list(a[i].polarization), spread=a[i].spread,
                     mean=a[i].mean, frequency=a[i].frequency, batch=a[i].batch) for i in range(n)]

    def sgbc(self):
        """The case's thin-layer stacks (dicts as Operator.set_sgbc takes them) and the stack of each
        SGBC interior face in mesh order."""
        ns, nl, nf = self.info["n_sgbc_stacks"], self.info["n_sgbc_layers"], self.info["n_sgbc_faces"]
        st = (SgbcStack * max(1, ns))()
        ly = (SgbcLayer * max(1, nl))()
        fs = np.zeros(nf, np.int32)
        _check(lib().dgtd_case_sgbc(self._h, st, ly, _ip(fs) if nf else None), "dgtd_case_sgbc")
        stacks = []
        for i in range(ns):
            layers = [dict(eps=st[i].layers[j].eps_r, mu=st[i].layers[j].mu_r, sigma=st[i].layers[j].sigma,
                           width=st[i].layers[j].width, segments=st[i].layers[j].segments, order=st[i].layers[j].order)
                      for j in range(st[i].n_layers)]
            stacks.append(dict(layers=layers, left=st[i].left_bc, right=st[i].right_bc, sub_dt=st[i].sub_dt))
        return stacks, fs

    def point_probes(self) -> np.ndarray:
        p = np.zeros((self.info["n_point_probes"], 3))
        if p.size:
            _check(lib().dgtd_case_point_probes(self._h, _dp(p)), "dgtd_case_point_probes")
        return p

    def surface(self, s: int) -> np.ndarray:
        n = C.c_int64()
        _check(lib().dgtd_case_surface(self._h, int(s), None, C.byref(n)), "dgtd_case_surface")
        f = np.zeros((n.value, 3), np.int32)
        _check(lib().dgtd_case_surface(self._h, int(s), _ip(f), C.byref(n)), "dgtd_case_surface")
        return f

    def initial_state(self, xyz: np.ndarray) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        n = xyz.shape[1]
        out = np.zeros(6 * n)
        _check(lib().dgtd_case_initial_state(self._h, _dp(xyz), n, _dp(out)), "dgtd_case_initial_state")
        return out

    def run(self, freqs=(), out_dir=None, want_state: bool = True):
        fr = np.ascontiguousarray(freqs, dtype=np.float64).reshape(-1)
        o = CaseRunOpts(precision=FP64, freqs=_dp(fr) if fr.size else None, n_freqs=fr.size,
                        out_dir=str(out_dir).encode() if out_dir else None)
        r = CaseResult()
        state = None
        if want_state:
            Np = (self.info["order"] + 1) * (self.info["order"] + 2) * (self.info["order"] + 3) // 6
            state = np.zeros(6 * self.info["n_elements"] * Np)
        _check(lib().dgtd_case_run(self._h, C.byref(o), _dp(state) if state is not None else None, C.byref(r)),
               "dgtd_case_run")
        return state, {k: getattr(r, k) for k, _ in CaseResult._fields_}
