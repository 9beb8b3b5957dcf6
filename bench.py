"""Benchmark of the DG Maxwell time step (DOF-updates/s) on GB300.

Contract: ``python bench.py --gpus N --steps K --warmup W [--impl ours|reference]``
prints ONE JSON line on rank 0.

A "step" is one full RK4 time step (all stages) of the workload over its mesh.
``value`` is the device-timed rate with inputs resident in HBM; ``e2e`` is the
same metric through the C ABI with host buffers: every step's host->device copy
of its whole state, the step and the device->host read of the result are inside
the timed region, with consecutive steps pipelined (upload of step k+1 and
download of step k-1 overlap step k's compute).

N > 1: the path is replicas only (independent solves, no collective); every
rank runs its own copy of the workload on its GPU and ``value`` sums them.

``--impl reference`` times the reference algorithm's CPU implementation on the
host cores: the reference cannot be built here (its MFEM fork is not vendored),
so this is the CPU restatement in oracle/ (assembled CSR + RK4, OpenMP),
stepped on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DOF-updates/s"
UNIT = "DOF-updates/s"


# ----------------------------------------------------------------------------- workloads
def te110_state(xyz: np.ndarray) -> np.ndarray:
    x, y = xyz[0], xyz[1]
    z = np.zeros_like(x)
    return np.concatenate([z, z, np.sin(np.pi * x) * np.sin(np.pi * y), z, z, z])


def plane_waves(B: int, seed: int = 20261203, spread: float = 0.1, mean: float = -0.5):
    """B Gaussian plane waves: k from normalised N(0, I3) draws, polarisation = normalised
    (g - (g.k) k) with g ~ N(0, I3); Gaussian mean -0.5 along k (peak crosses the origin at t = 0.5)."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(B):
        k = rng.standard_normal(3); k /= np.linalg.norm(k)
        g = rng.standard_normal(3); pol = g - g.dot(k) * k; pol /= np.linalg.norm(pol)
        out.append(dict(propagation=k.tolist(), polarization=pol.tolist(), spread=spread, mean=mean, batch=b))
    return out


WORKLOADS = {
    "scattering_batched_fp32": dict(
        desc="Batched plane-wave scattering: box [-1,1]^3 as 24^3 hexes x 6 tets minus the central 4^3 hexes "
             "(PEC cube [-1/6,1/6]^3) = 82,560 tets, p=4 (Np=35), first-order SMA outer boundary, TF/SF box at "
             "|x|=0.75, B=64 Gaussian plane waves (spread 0.1, delay 0.5, seed 20261203), FP32 state, RK4, "
             "dt from the reference 3D estimator at cfl=1",
        cells=(24, 24, 24), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((10, 10, 10), (14, 14, 14)),
        tfsf=((3, 3, 3), (21, 21, 21)), order=4, batch=64, dt=None, cfl=1.0, precision="fp32",
        outer_bc="SMA", init="zero", dtype="f32", waves=64,
        accuracy=dict(cells=(12, 12, 12), hole=((5, 5, 5), (7, 7, 7)), tfsf=((2, 2, 2), (10, 10, 10)), batch=4,
                      checkpoints=(250, 1000, 2000, 4000))),
    "scattering_batched_fp32_small": dict(
        desc="Profiling size of the batched scattering workload: 12^3 hexes x 6 tets minus the central 2^3 "
             "(10,320 tets), p=4, SMA, TF/SF box at |x|=2/3, B=64, FP32, RK4",
        cells=(12, 12, 12), lo=(-1, -1, -1), hi=(1, 1, 1), hole=((5, 5, 5), (7, 7, 7)),
        tfsf=((2, 2, 2), (10, 10, 10)), order=4, batch=64, dt=None, cfl=1.0, precision="fp32",
        outer_bc="SMA", init="zero", dtype="f32", waves=64),
    "dielectric_p6_fp32": dict(
        desc="High-order heterogeneous dielectric: unit cube 32^3 hexes x 6 tets (196,608), p=6 (Np=84), eps_r ~ "
             "U[1,4] per element (seed 20261204), mu=1, PEC walls, E = sum of 8 Fourier modes (seed 20261205), H=0, "
             "dt=2e-4, classical RK4; single-instance FP32 form",
        cells=(32, 32, 32), lo=(0, 0, 0), hi=(1, 1, 1), order=6, batch=1, dt=2e-4, precision="fp32s",
        outer_bc="PEC", init="fourier8", eps_seed=20261204, dtype="f32"),
    "dielectric_p6_fp32_small": dict(
        desc="Profiling size of the high-order dielectric: 20^3 hexes x 6 tets (48,000), p=6, same fields "
             "(97 MB per FP32 state copy: a stage's registers exceed the 129 MB L2); single-instance FP32 form",
        cells=(20, 20, 20), lo=(0, 0, 0), hi=(1, 1, 1), order=6, batch=1, dt=2e-4, precision="fp32s",
        outer_bc="PEC", init="fourier8", eps_seed=20261204, dtype="f32"),
    "cubic_resonator_fp64": dict(
        desc="3D PEC cubic resonator: unit cube 8^3 hexes x 6 tets (3,072), p=3 (Np=20), eps=mu=1, "
             "upwind, TE110 initial mode, classical RK4, dt=1e-3; plain FP64 form",
        cells=(8, 8, 8), lo=(0, 0, 0), hi=(1, 1, 1), order=3, batch=1, dt=1e-3, precision="fp64",
        outer_bc="PEC", init="te110", dtype="f64"),
}
DEFAULT_WORKLOAD = "scattering_batched_fp32"


def build_mesh(w: dict):
    import dgtd_gb300 as dg
    bc = {"PEC": dg.BC_PEC, "SMA": dg.BC_SMA, "PMC": dg.BC_PMC}[w["outer_bc"]]
    m = dg.box_mesh(w["cells"], lo=w["lo"], hi=w["hi"], hole=w.get("hole"), tfsf=w.get("tfsf"), outer_bc=bc,
                    hole_bc=dg.BC_PEC)
    if w.get("eps_seed"):
        m.eps = np.random.default_rng(w["eps_seed"]).uniform(1.0, 4.0, m.n_elements)
    return m


def initial_state(w: dict, xyz: np.ndarray) -> np.ndarray:
    if w["init"] == "te110":
        return te110_state(xyz)
    if w["init"] == "zero":
        return np.zeros(6 * xyz.shape[1])
    if w["init"] == "fourier8":
        return high_order_state(xyz)
    raise ValueError(w["init"])


def workload_dt(w: dict, op) -> float:
    return w["dt"] if w.get("dt") else op.estimate_dt(w.get("cfl", 1.0))


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.path is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------- helpers
def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "bf16_tflops": d.get("bf16_tflops", 1900.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def profile_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if present."""
    f = ROOT / "profiles" / f"{kernel}__{workload}.md"
    if f.exists():
        import re
        m = re.search(r"^dram_bytes_per_launch:\s*([0-9.eE+]+)", f.read_text(), flags=re.M)
        if m:
            return float(m.group(1))
    return None


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def max_over_ranks(v: float, world: int, device=None) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------------------- CPU side
def host_mesh(w: dict):
    """The workload's mesh built by the oracle's numpy generator (identical tables to the
    product's box generator, tests/test_oracle_mesh.py): the CPU legs load nothing of the
    product library."""
    from oracle import pyoracle as po
    bc = {"PEC": po.BC_PEC, "SMA": po.BC_SMA, "PMC": po.BC_PMC}[w["outer_bc"]]
    m = po.box_mesh(w["cells"], lo=w["lo"], hi=w["hi"], hole=w.get("hole"), tfsf=w.get("tfsf"), outer_bc=bc,
                    hole_bc=po.BC_PEC)
    if w.get("eps_seed"):
        m.eps = np.random.default_rng(w["eps_seed"]).uniform(1.0, 4.0, m.n_elements)
    return m


def host_dt(w: dict, mesh) -> float:
    """dt of the workload: explicit, or the reference 3D Global estimator (Solver.cpp:289-300,
    349-351) restated in the oracle."""
    if w.get("dt"):
        return w["dt"]
    from oracle import pyoracle as po
    return po.estimate_dt_3d(mesh, w["order"], w.get("cfl", 1.0))


def workload_config(w: dict, workload: str, world: int) -> dict:
    """The `config` object of the JSON line, the same on both arms (computed on the host)."""
    m = host_mesh(w)
    Np = (w["order"] + 1) * (w["order"] + 2) * (w["order"] + 3) // 6
    return {"workload": workload, "description": w["desc"], "elements": m.n_elements, "order": w["order"],
            "incidences": w["batch"], "dt": host_dt(w, m), "integrator": "RK4",
            "dofs_per_step": 6 * m.n_elements * Np * w["batch"],
            "l2": "flushed between timed steps (256 MB write); inputs larger than L2",
            "parallelism": f"replicas x{world}"}


def cpu_rate(w: dict, budget_s: float, max_steps: int | None = None, warmup: int = 1) -> dict:
    """Time the oracle on a bounded sample of the workload (one incidence).

    Meshes whose assembled operator fits in host memory use the assembled-CSR RK4
    restatement of the reference's default GlobalEvolution; larger ones the
    matrix-free nodal restatement (HesthavenEvolution form), OpenMP over elements.
    """
    from oracle import pyoracle as po
    mesh = host_mesh(w)
    orc = po.Oracle.from_mesh(mesh, w["order"])
    if w.get("waves"):
        orc.set_planewaves([plane_waves(1)[0]])
    x = initial_state(w, orc.nodes())
    dt = host_dt(w, mesh)
    form = po.GLOBAL if orc.ndofs * 6 <= 2_000_000 else po.NODAL
    t_build0 = time.perf_counter()
    nnz = orc.nnz() if form == po.GLOBAL else None   # assemble outside the timed sample
    t_build = time.perf_counter() - t_build0
    t = 0.0
    for _ in range(max(1, warmup)):                   # warm-up (page-in, nodal tables)
        x = orc.step(x, t, dt, 1, form=form)
        t += dt
    steps, t0 = 0, time.perf_counter()
    while True:
        x = orc.step(x, t, dt, 1, form=form)
        t += dt; steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_steps is not None and steps >= max_steps):
            break
    dofs = 6 * orc.ndofs
    kind = (f"assembled CSR operator ({nnz} nnz, GlobalEvolution restatement)" if form == po.GLOBAL
            else "matrix-free nodal operator (HesthavenEvolution restatement; the assembled CSR does not fit in host memory)")
    return {"value": dofs * steps / el, "seconds": el, "steps": steps, "dofs": dofs, "cores": po.threads(),
            "assembly_s": t_build, "kind": kind, "warmup": max(1, warmup)}


# ----------------------------------------------------------------------------- GPU side
def make_op(w: dict, mesh, precision: int, batch: int):
    import dgtd_gb300 as dg
    op = dg.Operator(mesh, order=w["order"], alpha=1.0, precision=precision, batch=batch)
    if w.get("waves"):
        op.set_planewaves(plane_waves(batch))
    return op


def time_steps(op, state, dt, t0, steps, stream, flush, dev):
    """Per-step CUDA-event times (ms) of `steps` fused RK4 steps, L2 flushed between steps."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t = t0
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        op.step(state, t, dt, 1, stream=stream)
        ev[k][1].record(stream)
        t += dt
    torch.cuda.synchronize(dev)
    return [a.elapsed_time(b) for a, b in ev], t


def accuracy_vs_fp64(w: dict, dev, contraction: int, dt: float, defect: int = 0) -> dict:
    """Error of the timed FP32 kernel against the FP64 form over the configuration's full length.

    A reduced mesh (12^3 hexes instead of 24^3: same order, boundaries, sources and the timed
    run's dt, so the same 4,000 steps reach the same final time T = 9.9) is stepped by the FP32
    batched operator with the workload's 64 incidences and the timed run's contraction path,
    and by the FP64 form for the first `batch` incidences (same waves); the relative L2 of each
    compared incidence is reported at checkpoints. defect: the timed run's defect-correction
    period (0: off)."""
    import torch
    import dgtd_gb300 as dg
    acc = w["accuracy"]
    wr = dict(w, cells=acc["cells"], hole=acc["hole"], tfsf=acc["tfsf"])
    mesh = build_mesh(wr)
    B = acc["batch"]
    op64 = make_op(wr, mesh, dg.FP64, B)
    op32 = make_op(wr, mesh, dg.FP32_3XTF32, w["batch"])
    op32.set_contraction(contraction)
    if defect:
        op32.set_defect_correction(defect)
    x64 = torch.zeros(op64.state_len, dtype=torch.float64, device=dev)
    x32 = torch.zeros(op32.state_len, dtype=torch.float64, device=dev)
    wk = op32.new_work(dev)
    op32.pack(x32, wk)
    L = op64.state_len // B
    points, n, t = [], 0, 0.0
    for c in acc["checkpoints"]:
        op64.step(x64, t, dt, c - n)
        op32.step(wk, t, dt, c - n)
        t += (c - n) * dt
        n = c
        op32.unpack(wk, x32)
        torch.cuda.synchronize(dev)
        op32.check()
        a, r = x32.cpu().numpy(), x64.cpu().numpy()
        errs = [float(np.linalg.norm(a[b * L:(b + 1) * L] - r[b * L:(b + 1) * L]) /
                      np.linalg.norm(r[b * L:(b + 1) * L])) for b in range(B)]
        points.append({"steps": c, "t": c * dt, "rel_l2_max": max(errs)})
    return {"rel_l2_vs_fp64_max": points[-1]["rel_l2_max"], "steps": n, "t_end": n * dt, "dt": dt,
            "checkpoints": points, "incidences_compared": B, "fp32_batch": w["batch"],
            "fp32_kernel": "tensor cores (stage_tc)" if op32.uses_tensor_cores else "FP32 SIMT (stage_f32)",
            "defect_correction_every": defect,
            "case": f"{acc['cells'][0]}^3 hexes x 6 tets, same order/sources/boundaries and the timed run's dt"}


def run_ours(args, world, rank, local):
    import torch
    import dgtd_gb300 as dg

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]
    mesh = build_mesh(w)
    prec = {"fp64": dg.FP64, "fp32": dg.FP32_3XTF32, "fp32s": dg.FP32}[w["precision"]]
    t_setup0 = time.perf_counter()
    op = make_op(w, mesh, prec, w["batch"])
    setup_s = time.perf_counter() - t_setup0
    dt = workload_dt(w, op)
    xyz = op.node_coords()
    x0 = np.tile(initial_state(w, xyz), w["batch"])
    ref = torch.from_numpy(x0).to(dev)
    state = op.new_work(dev)
    op.pack(ref, state)
    del ref
    stream = torch.cuda.current_stream(dev)
    tune = None
    if prec == dg.FP32_3XTF32:
        if args.contraction == "auto":
            tune = op.autotune(state, stream=stream)
        else:
            op.set_contraction(0 if args.contraction == "tc" else 1)
    elif prec == dg.FP32 and args.contraction != "auto":
        op.set_contraction(0 if args.contraction == "tc" else 1)
    dofs = 6 * op.ndofs * w["batch"]
    flush = torch.empty(int(256 * 2 ** 20) // 4, dtype=torch.float32, device=dev)   # 256 MB > 129 MB L2

    # FP64 defect correction (batched form): refreshed every `defect` steps. Timed segments start
    # right after a refresh, and each adds the refreshes its length calls for beyond those that
    # fell inside it (K / defect - refreshes inside, times the measured refresh time), so a
    # segment shorter than the period still pays its share.
    defect = args.defect_every if prec == dg.FP32_3XTF32 else 0
    if defect:
        op.set_defect_correction(defect)

    t = 0.0
    for i in range(args.warmup):
        if defect and i == args.warmup - 1:
            op.set_defect_correction(defect)        # refresh in the last warm-up step
        op.step(state, t, dt, 1, stream=stream); t += dt
    torch.cuda.synchronize(dev)

    n_launch0 = dg.kernel_launches()
    r_timed0 = op.defect_refreshes if defect else 0
    barrier(world)
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        step_ms, t = time_steps(op, state, dt, t, args.steps, stream, flush, dev)
    barrier(world)
    launches = dg.kernel_launches() - n_launch0
    defect_info = None
    timed_s = sum(step_ms) / 1e3
    stage_step_s = None
    if defect:
        r_in = op.defect_refreshes - r_timed0
        # one refresh timed alone: a step that refreshes minus a step that does not (L2 flushed before each)
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        flush.zero_()
        op.set_defect_correction(defect)
        evs[0].record(stream); op.step(state, t, dt, 1, stream=stream); evs[1].record(stream); t += dt
        flush.zero_()
        evs[2].record(stream); op.step(state, t, dt, 1, stream=stream); evs[3].record(stream); t += dt
        torch.cuda.synchronize(dev)
        refresh_s = max(0.0, (evs[0].elapsed_time(evs[1]) - evs[2].elapsed_time(evs[3])) / 1e3)
        extra_s = max(0.0, args.steps / defect - r_in) * refresh_s
        # the stage kernel alone (the roofline's launch time): steps without the correction's
        # own kernels (refresh, per-step increment)
        op.set_defect_correction(0)
        k_stage = max(3, min(args.steps, 10))
        stage_ms, t = time_steps(op, state, dt, t, k_stage, stream, flush, dev)
        stage_step_s = max_over_ranks(sum(stage_ms) / 1e3, world, dev) / k_stage
        op.set_defect_correction(defect)
        defect_info = {"every": defect, "refresh_ms": refresh_s * 1e3, "refreshes_in_timed_region": r_in,
                       "added_ms": extra_s * 1e3, "amortised_ms_per_step": refresh_s * 1e3 / defect,
                       "stage_kernels_ms_per_step": stage_step_s * 1e3,
                       "note": "FP64 operator correction (dgtd_op_set_defect_correction): value includes "
                               "max(0, steps/every - refreshes inside) refreshes at the measured refresh time"}
        timed_s += extra_s
    total_s = max_over_ranks(timed_s, world, dev)
    value = world * dofs * args.steps / total_s
    ms_per_step = total_s * 1e3 / args.steps
    if not bool(torch.isfinite(state).all()):
        raise RuntimeError("non-finite state after the timed steps")

    # --- end to end through the drop-in boundary: a caller that holds the reference-layout FP64
    # state (the reference's Fields vector) in pinned host memory and advances it one RK4 step per
    # call, as the TimeDependentOperator adapter would. Every step moves the state host -> device,
    # converts it to the working layout (dgtd_op_pack; the FP64 form steps it in place), advances
    # it (dgtd_op_step), converts it back (dgtd_op_unpack) and moves it device -> host into the
    # same host vector, which the next step uploads: a dependent chain, nothing overlaps across
    # steps. Two ways of moving the data are timed and the faster is the line's e2e.
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    ref_dev = torch.empty(op.state_len, dtype=torch.float64, device=dev)
    op.unpack(state, ref_dev, stream=stream)
    host = torch.empty(op.state_len, dtype=torch.float64, pin_memory=True)
    host.copy_(ref_dev)

    def e2e_chain(zero_copy: bool):
        """One dependent chain of e2e_steps steps; returns (seconds, launches). zero_copy: the pack
        and unpack kernels read and write the pinned host vector directly (the transfer and the
        layout conversion in one pass over the host link); else cudaMemcpy H2D / D2H into a device
        reference-layout buffer around device-side pack / unpack."""
        t_ = t
        if defect:                                   # start right after a refresh (untimed step)
            op.set_defect_correction(defect)
            op.step(state, t_, dt, 1, stream=stream)
            t_ += dt
        r0 = op.defect_refreshes if defect else 0
        e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = dg.kernel_launches()
        torch.cuda.synchronize(dev)
        e_start.record(stream)
        with torch.cuda.stream(stream):
            for k in range(e2e_steps):
                flush.zero_()
                if prec == dg.FP64:
                    ref_dev.copy_(host, non_blocking=True)
                    op.step(ref_dev, t_, dt, 1, stream=stream)
                    host.copy_(ref_dev, non_blocking=True)
                elif zero_copy:
                    op.pack(host, state, stream=stream)
                    op.step(state, t_, dt, 1, stream=stream)
                    op.unpack(state, host, stream=stream)
                else:
                    ref_dev.copy_(host, non_blocking=True)
                    op.pack(ref_dev, state, stream=stream)
                    op.step(state, t_, dt, 1, stream=stream)
                    op.unpack(state, ref_dev, stream=stream)
                    host.copy_(ref_dev, non_blocking=True)
                t_ += dt
        e_end.record(stream)
        torch.cuda.synchronize(dev)
        sec = e_start.elapsed_time(e_end) / 1e3
        if defect:
            sec += max(0.0, e2e_steps / defect - (op.defect_refreshes - r0)) * defect_info["refresh_ms"] / 1e3
        return max_over_ranks(sec, world, dev), dg.kernel_launches() - n0

    variants = {"copy_engine": e2e_chain(False)}
    if prec != dg.FP64:
        variants["zero_copy"] = e2e_chain(True)
    if not bool(torch.isfinite(host).all()):
        raise RuntimeError("non-finite state after the end-to-end steps")
    best = min(variants, key=lambda v: variants[v][0])
    e2e_s, e2e_launches = variants[best]
    ref_bytes = int(host.numel() * host.element_size())
    paths = {
        "copy_engine": "pinned host FP64 reference-layout state -> cudaMemcpy H2D -> dgtd_op_pack -> dgtd_op_step "
                       "(1 RK4 step) -> dgtd_op_unpack -> cudaMemcpy D2H into the same host vector, step after step",
        "zero_copy": "pinned host FP64 reference-layout state -> dgtd_op_pack reading the host vector over the host "
                     "link -> dgtd_op_step (1 RK4 step) -> dgtd_op_unpack writing the host vector, step after step",
    }
    if prec == dg.FP64:
        paths["copy_engine"] = ("pinned host FP64 reference-layout state -> H2D -> dgtd_op_step (1 RK4 step) -> D2H "
                                "into the same host vector, step after step")
    e2e = {"value": world * dofs * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": ref_bytes,
           "d2h_bytes_per_step": ref_bytes, "steps": e2e_steps, "ms_per_step": e2e_s * 1e3 / e2e_steps,
           "gpu_launches": e2e_launches, "path": paths[best] + " (a dependent chain: nothing overlaps across steps)",
           "variants_ms_per_step": {v: variants[v][0] * 1e3 / e2e_steps for v in variants}}
    t += (e2e_steps + (1 if defect else 0)) * dt * len(variants)
    del host, ref_dev
    if defect:
        op.set_defect_correction(0)       # the streaming leg steps independent states

    # --- streaming variant: independent jobs of the private working layout, pipelined (step k+1's
    # upload and step k-1's download on their own streams under step k's compute, three device
    # buffers): how far copies hide under compute when a caller streams independent states.
    t2 = t
    host = state.detach().cpu().pin_memory()
    out = torch.empty_like(host).pin_memory()
    nbuf = 3
    dbufs = [torch.empty_like(state) for _ in range(nbuf)]
    s_up, s_down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev = lambda: torch.cuda.Event(enable_timing=False)
    up_done = [ev() for _ in range(e2e_steps)]
    comp_done = [ev() for _ in range(e2e_steps)]
    down_done = [ev() for _ in range(e2e_steps)]
    e2e_start, e2e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e2e_start.record(s_up)
    for k in range(e2e_steps):
        buf = dbufs[k % nbuf]
        if k >= nbuf:
            s_up.wait_event(down_done[k - nbuf])          # the buffer's previous result is downloaded
        with torch.cuda.stream(s_up):
            buf.copy_(host, non_blocking=True)
            up_done[k].record(s_up)
        stream.wait_event(up_done[k])
        flush.zero_()
        op.step(buf, t2, dt, 1, stream=stream)
        comp_done[k].record(stream)
        s_down.wait_event(comp_done[k])
        with torch.cuda.stream(s_down):
            out.copy_(buf, non_blocking=True)
            down_done[k].record(s_down)
        t2 += dt
    stream.wait_event(down_done[e2e_steps - 1])
    e2e_end.record(stream)
    torch.cuda.synchronize(dev)
    st_s = max_over_ranks(e2e_start.elapsed_time(e2e_end) / 1e3, world, dev)
    work_bytes = int(host.numel() * host.element_size())
    e2e_streaming = {"value": world * dofs * e2e_steps / st_s, "unit": UNIT, "h2d_bytes_per_step": work_bytes,
                     "d2h_bytes_per_step": work_bytes, "steps": e2e_steps,
                     "path": "independent states in the working layout (no defect correction: every step is "
                             "another state), pinned host buffers, uploads/downloads "
                             "pipelined under the previous/next step's compute"}
    del dbufs, host, out

    # --- roofline of the dominant kernel (the fused stage kernel; RK4 = 4 launches per step)
    peaks = measured_peaks()
    stage_launches = 4
    # mean stage-launch time: the timed steps / 4, or, with the defect correction on, steps timed
    # without the correction's own kernels (the stage kernel is the same in both)
    avg_launch_s = (stage_step_s if stage_step_s is not None else total_s / args.steps) / stage_launches
    word = 8 if prec == dg.FP64 else 4
    K, Np, nfp = op.info["n_elements"], op.info["np"], op.info["nfp"]
    # algorithmic bytes per DOF per RK4 step: 16 words over the 4 stages (x, y, z registers: 3+5+5+3);
    # the batched form's compensated update adds 3 (stage 4 reads x_hi, x_lo and writes x_lo). The
    # defect correction's per-step increment is a separate elementwise kernel, not counted here.
    words = 19 if prec == dg.FP32_3XTF32 else 16
    alg_bytes_launch = words * word * dofs / stage_launches
    achieved_gbs = alg_bytes_launch / avg_launch_s / 1e9
    flops_per_dof_step = 4 * (6 * Np + 8 * nfp)          # contraction terms, FMA = 2
    achieved_tflops = flops_per_dof_step * dofs / (avg_launch_s * stage_launches) / 1e12
    if prec == dg.FP64:
        kname = "stage_fp64"
    elif prec == dg.FP32:
        kname = "stage_tc1" if op.uses_tensor_cores else "stage_f32s"
    else:
        kname = "stage_tc" if op.uses_tensor_cores else "stage_f32"
    traffic = profile_traffic(kname, args.workload)
    roofline = {"bound": "hbm", "achieved": round(achieved_gbs, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved_gbs / peaks["hbm_gbs"], 4), "traffic": traffic,
                "peak_source": peaks["source"] + " (MEASURED_PEAKS.json hbm_gbs)" if peaks["source"] == "measured" else peaks["source"],
                "kernel": kname, "algorithmic_bytes_per_launch": alg_bytes_launch, "words_per_dof_step": words,
                "avg_launch_ms": avg_launch_s * 1e3,
                "contraction_tflops": round(achieved_tflops, 4)}
    if prec == dg.FP32:
        roofline["fp32_pipe"] = {"achieved_tflops": round(achieved_tflops, 4),
                                 "note": "single-instance FP32 form: contraction flops on the FP32 pipe (FMA = 2)"}
    if prec == dg.FP64:
        roofline["fp64_pipe"] = {"achieved_tflops": round(achieved_tflops, 4), "nominal_peak_tflops": 1.25,
                                 "frac_of_nominal": round(achieved_tflops / 1.25, 4),
                                 "note": "plain FP64 form is FP64-issue bound; nominal GB300 FP64 peak, not measured"}
    res = dict(value=value, ms_per_step=ms_per_step, e2e=e2e, e2e_streaming=e2e_streaming, tune=tune,
               defect=defect_info,
               launches=launches, uses_tc=bool(getattr(op, "uses_tensor_cores", False)), clocks=clk.summary(), roofline=roofline,
               setup_s=setup_s, w=w, dofs=dofs, K=K, Np=Np, dt=dt)
    del state, op

    if prec != dg.FP64 and not args.no_fp64_compare:
        # the plain FP64 GPU path on the same workload (metric: DOF-updates/s vs the plain FP64 path)
        op64 = make_op(w, mesh, dg.FP64, w["batch"])
        s64 = torch.from_numpy(x0).to(dev)
        op64.step(s64, 0.0, dt, 1, stream=stream)
        torch.cuda.synchronize(dev)
        ms64, _ = time_steps(op64, s64, dt, dt, args.fp64_steps, stream, flush, dev)
        v64 = dofs * args.fp64_steps / (sum(ms64) / 1e3)
        res["plain_fp64"] = {"value": v64, "unit": UNIT, "ms_per_step": sum(ms64) / args.fp64_steps,
                             "steps": args.fp64_steps, "speedup": value / v64}
        del s64, op64
        torch.cuda.empty_cache()
        if w.get("accuracy") and not args.no_accuracy:
            res["accuracy"] = accuracy_vs_fp64(w, dev, 0 if res["uses_tc"] else 1, dt, defect)
    return res


# ----------------------------------------------------------------------------- high order (single instance)
HIGH_ORDER_DESC = ("High-order heterogeneous dielectric: unit cube 32^3 hexes x 6 tets (196,608), p=6 (Np=84), "
                   "eps_r ~ U[1,4] per element (seed 20261204), mu=1, PEC walls, E = sum of 8 Fourier modes "
                   "a_m sin(k_m.x + phi_m) with a ~ N(0,1)^3, k_m in pi*{1..3}^3, phi_m ~ U[0,2pi) (seed 20261205), "
                   "H=0, dt=2e-4, classical RK4; single-instance FP32 form (contractions on the tensor cores, "
                   "3xTF32, or FP32 SIMT: the faster of the two is the value)")


def high_order_mesh(n: int):
    import dgtd_gb300 as dg
    m = dg.box_mesh((n, n, n))
    m.eps = np.random.default_rng(20261204).uniform(1.0, 4.0, m.n_elements)
    return m


def high_order_state(xyz: np.ndarray) -> np.ndarray:
    rng = np.random.default_rng(20261205)
    E = np.zeros((3, xyz.shape[1]))
    for _ in range(8):
        k = np.pi * rng.integers(1, 4, 3)
        a = rng.standard_normal(3)
        ph = rng.uniform(0.0, 2.0 * np.pi)
        E += np.outer(a, np.sin(k @ xyz + ph))
    return np.concatenate([E.ravel(), np.zeros(3 * xyz.shape[1])])


def run_high_order(steps: int, dev) -> dict:
    """C4 on the single-instance FP32 form: both contraction paths timed (tensor cores and FP32
    SIMT; the faster is the value), the FP64 form's rate on the same mesh, and each FP32 path's
    error against the FP64 form on a reduced mesh (8^3 hexes) over the configuration's 1,000 steps."""
    import torch
    import dgtd_gb300 as dg
    dt = 2e-4
    m = high_order_mesh(32)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(int(256 * 2 ** 20) // 4, dtype=torch.float32, device=dev)
    paths = {}
    for name, mode in (("tensor_cores", 0), ("simt", 1)):
        op = dg.Operator(m, order=6, precision=dg.FP32)
        op.set_contraction(mode)
        x0 = torch.from_numpy(high_order_state(op.node_coords())).to(dev)
        w = op.new_work(dev)
        op.pack(x0, w)
        op.step(w, 0.0, dt, 3, stream=stream)
        torch.cuda.synchronize(dev)
        n0 = dg.kernel_launches()
        ms, _ = time_steps(op, w, dt, 3 * dt, steps, stream, flush, dev)
        op.check(stream)
        launches = dg.kernel_launches() - n0
        dofs = 6 * op.ndofs
        step_s = sum(ms) / 1e3 / steps
        paths[name] = {"value": dofs / step_s, "ms_per_step": step_s * 1e3, "ms_per_launch": step_s * 1e3 / 4,
                       "gpu_launches": launches, "uses_tensor_cores": op.uses_tensor_cores}
        Np, Nfp = op.info["np"], op.info["nfp"]
        del w, x0, op
        torch.cuda.empty_cache()
    best = "tensor_cores" if paths["tensor_cores"]["value"] >= paths["simt"]["value"] else "simt"
    step_s = paths[best]["ms_per_step"] / 1e3
    flops = 4 * (6 * Np + 8 * Nfp) * dofs / step_s
    out = {"workload": HIGH_ORDER_DESC, "elements": m.n_elements, "dofs_per_step": dofs, "steps": steps,
           "value": dofs / step_s, "unit": UNIT, "ms_per_step": step_s * 1e3, "stage_kernel": best,
           "gpu_launches": paths[best]["gpu_launches"], "paths": paths,
           "contraction_tflops": flops / 1e12,
           "hbm_gbs_algorithmic": 16 * 4 * dofs / step_s / 1e9}
    op64 = dg.Operator(m, order=6)
    x64 = torch.from_numpy(high_order_state(op64.node_coords())).to(dev)
    op64.step(x64, 0.0, dt, 1, stream=stream)
    torch.cuda.synchronize(dev)
    ms64, _ = time_steps(op64, x64, dt, dt, 2, stream, flush, dev)
    out["plain_fp64"] = {"value": dofs * 2 / (sum(ms64) / 1e3), "ms_per_step": sum(ms64) / 2, "steps": 2}
    out["speedup_vs_fp64"] = out["value"] / out["plain_fp64"]["value"]
    del x64, op64
    torch.cuda.empty_cache()
    ms_ = high_order_mesh(8)
    a64 = dg.Operator(ms_, order=6)
    xa = torch.from_numpy(high_order_state(a64.node_coords())).to(dev)
    x0a = xa.clone()
    a64.step(xa, 0.0, dt, 1000, stream=stream)
    torch.cuda.synchronize(dev)
    r = xa.cpu().numpy()
    acc = {}
    for name, mode in (("tensor_cores", 0), ("simt", 1)):
        a32 = dg.Operator(ms_, order=6, precision=dg.FP32)
        a32.set_contraction(mode)
        wa = a32.new_work(dev)
        a32.pack(x0a, wa)
        a32.step(wa, 0.0, dt, 1000, stream=stream)
        back = torch.zeros_like(xa)
        a32.unpack(wa, back)
        torch.cuda.synchronize(dev)
        acc[name] = float(np.linalg.norm(back.cpu().numpy() - r) / np.linalg.norm(r))
    out["accuracy"] = {"rel_l2_vs_fp64": acc[best], "by_path": acc, "steps": 1000, "t_end": 1000 * dt,
                       "case": "8^3 hexes x 6 tets, same order, materials, initial field and dt"}
    return out


# ----------------------------------------------------------------------------- serving
SERVING_N = (8, 16)          # hexes per axis, U{lo..hi}
SERVING_T = (1.0, 4.0)       # final time, U[lo, hi]
SERVING_DESC = ("Serving stream (C5 with a smaller mesh range): Poisson arrivals; each request a box [-1,1]^3 of "
                "n^3 hexes x 6 tets, n ~ U{8..16} (configuration: U{8..32}), central PEC cube of round(n/6) hexes, SMA "
                "outer boundary, TF/SF box one cell in, order p ~ U{2..5}, one Gaussian plane wave (spread 0.1, delay "
                "0.5) with random direction and orthogonal polarisation, final time T ~ U[1, 4], dt from the reference "
                "3D estimator at cfl=1; classical RK4; request parameters seed 20261206, arrival times seed 20261207")


def serving_requests(n_req: int, rate: float, seed: int = 20261206):
    """The request stream: parameters from one RNG stream and arrival times from another, so the
    first k requests are the same at every arrival rate and in the one-at-a-time sample."""
    import dgtd_gb300 as dg
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(np.random.default_rng(seed + 1).exponential(1.0 / rate, n_req))
    reqs = []
    for _ in range(n_req):
        n = int(rng.integers(SERVING_N[0], SERVING_N[1] + 1))
        p = int(rng.integers(2, 6))
        T = float(rng.uniform(*SERVING_T))
        k = rng.standard_normal(3); k /= np.linalg.norm(k)
        g = rng.standard_normal(3); pol = g - g.dot(k) * k; pol /= np.linalg.norm(pol)
        c = max(1, int(np.floor(n / 6 + 0.5)))
        lo = (n - c) // 2
        hole = ((lo,) * 3, (lo + c,) * 3)
        m = dg.box_mesh((n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), hole=hole, tfsf=((1,) * 3, (n - 1,) * 3),
                        outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)
        reqs.append(dict(mesh=m, order=p, final_time=T, n=n,
                         waves=[dict(propagation=k, polarization=pol, spread=0.1, mean=-0.5)]))
    return reqs, arrivals


def serving_point(reqs, arrivals, srv) -> dict:
    """Feed one request stream into a running server at its arrival times; time-to-solution
    per request = result on the host minus submission."""
    n_req = len(reqs)
    base = srv.stats()
    ids = [None] * n_req
    t0 = time.perf_counter()

    def feeder():
        for i, r in enumerate(reqs):
            d = t0 + arrivals[i] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids[i] = srv.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0)

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    stats = [srv.wait(ids[i], timeout=3600, want_state=False)[1] for i in range(n_req)]
    wall = time.perf_counter() - t0
    end = srv.stats()
    tts = np.array([s["t_done"] - s["t_submit"] for s in stats])
    span = max(s["t_done"] for s in stats) - min(s["t_submit"] for s in stats)
    launches = end["stage_launches"] - base["stage_launches"]
    return {"requests": n_req, "solves_per_s": n_req / span,
            "p50_time_to_solution_s": float(np.percentile(tts, 50)),
            "p99_time_to_solution_s": float(np.percentile(tts, 99)), "mean_time_to_solution_s": float(tts.mean()),
            "makespan_s": span, "wall_s": wall,
            "dof_updates_per_s": (end["dof_updates"] - base["dof_updates"]) / span, "stage_launches": launches,
            "requests_per_stage_launch": (end["slot_stage_updates"] - base["slot_stage_updates"]) / max(1, launches),
            "max_active": end["max_active_seen"], "failed": end["failed"] - base["failed"],
            "unstable": int(sum(s["unstable"] for s in stats))}


def run_serving(n_req: int, rates, serial_sample: int, device: int, precision: str = "fp32") -> dict:
    """Continuous-batching runs of the request stream through dgtd_server_* at each arrival rate
    (a light load and a saturating one), and the stream's first `serial_sample` requests run one
    at a time through the single-operator path on the plain FP64 form (the configuration's
    comparison) and on the server's own form."""
    import dgtd_gb300 as dg
    free = 0
    try:
        import torch
        free, _ = torch.cuda.mem_get_info(device)
    except Exception:
        pass
    budget = int(min(32 << 30, max(1 << 30, free // 4)))
    prec = dg.FP32 if precision == "fp32" else dg.FP64
    points = []
    with dg.Server(memory_budget=budget, max_active=64, steps_per_round=8, device=device, precision=prec) as srv:
        reqs, _ = serving_requests(1, 1.0)
        w = srv.submit(reqs[0]["mesh"], reqs[0]["order"], 0.05, waves=reqs[0]["waves"], cfl=1.0)   # warm-up
        srv.wait(w, timeout=600, want_state=False)
        for rate in rates:
            reqs, arrivals = serving_requests(n_req, rate)
            pt = serving_point(reqs, arrivals, srv)
            pt["arrival_rate_per_s"] = rate
            points.append(pt)
        peak = srv.stats()["peak_bytes_in_use"]
    out = {"workload": SERVING_DESC, "points": points, "memory_budget": budget, "peak_device_bytes": peak,
           "precision": (("fp32 (single-instance FP32 form" if prec == dg.FP32 else "fp64 (plain form") +
                         "; bit-identical alone and in the mix, tests/test_gpu_serve.py)")}
    # headline figures, all from one operating point: the saturating rate (the capacity)
    cap = max(points, key=lambda p: p["solves_per_s"])
    out["operating_point"] = {"arrival_rate_per_s": cap["arrival_rate_per_s"], "solves_per_s": cap["solves_per_s"],
                              "p50_time_to_solution_s": cap["p50_time_to_solution_s"],
                              "p99_time_to_solution_s": cap["p99_time_to_solution_s"]}
    out["solves_per_s"] = cap["solves_per_s"]
    out["p50_time_to_solution_s"] = cap["p50_time_to_solution_s"]
    out["p99_time_to_solution_s"] = cap["p99_time_to_solution_s"]
    if serial_sample > 0:
        reqs, _ = serving_requests(serial_sample, 1.0)       # the stream's first requests (same parameters)
        ser = {}
        for name, pr in (("fp64", dg.FP64), ("server_form", prec)):
            t1 = time.perf_counter()
            dofs = 0.0
            for r in reqs:
                op = dg.Operator(r["mesh"], order=r["order"], precision=pr)
                if pr == dg.FP32:
                    op.set_contraction(1)        # the server's FP32 stage body (SIMT)
                op.set_planewaves(r["waves"])
                _, n = op.run_host(np.zeros(op.state_len), 0.0, op.estimate_dt(1.0), r["final_time"])
                dofs += op.state_len * n
                op.close()
            sec = time.perf_counter() - t1
            ser[name] = {"requests": serial_sample, "seconds": sec, "solves_per_s": serial_sample / sec,
                         "dof_updates_per_s": dofs / sec}
        out["serial_sample"] = {"path": "dgtd_op_run_host, one request at a time, the stream's first requests",
                                **ser}
        # the stream's requests are not all the sample's size, so capacity is compared per DOF-update
        out["capacity_vs_serial_fp64_dof_rate"] = cap["dof_updates_per_s"] / ser["fp64"]["dof_updates_per_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the 4,000-step accuracy leg")
    ap.add_argument("--e2e-steps", type=int, default=20, help="steps of the end-to-end legs (at most --steps)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--serving-requests", type=int, default=256, help="requests of the serving stream (0: skip)")
    ap.add_argument("--high-order-steps", type=int, default=10, help="timed steps of the p=6 dielectric (0: skip)")
    ap.add_argument("--serving-rates", default="4,64",
                    help="Poisson arrival rates of the serving stream (1/s): a light load and a saturating one "
                         "(capacity)")
    ap.add_argument("--serving-serial", type=int, default=6, help="requests also run one at a time for comparison")
    ap.add_argument("--serving-precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--defect-every", type=int, default=100,
                    help="batched form: refresh period (steps) of the FP64 defect correction (0: off)")
    ap.add_argument("--contraction", choices=["auto", "tc", "simt"], default="auto",
                    help="batched form: autotuned stage kernel (default), or force tensor cores / FP32 SIMT; "
                         "single-instance FP32 form: the library default (auto), tensor cores or FP32 SIMT")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init(args)
    w = WORKLOADS[args.workload]
    config = workload_config(w, args.workload, world)

    if args.impl == "reference":
        if rank != 0:
            return
        n_steps = max(1, args.steps)
        # bounded: each step is one RK4 step of one incidence of the workload on the host cores
        r = cpu_rate(w, budget_s=min(args.cpu_budget * 4, 120.0), max_steps=n_steps, warmup=args.warmup)
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": r["steps"],
                "warmup": r["warmup"], "ms_per_step": r["seconds"] * 1e3 / r["steps"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": config,
                "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
                                 "sample": f"{r['steps']} RK4 steps of one incidence of the workload (same mesh, "
                                           f"order, dt and sources as the config; the rate is per DOF-update, "
                                           f"so one incidence stands for the {w['batch']} of the config) with "
                                           f"the oracle's {r['kind']}; setup ({r['assembly_s']:.1f} s) excluded"},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    r = run_ours(args, world, rank, local)
    if (r["K"], r["dofs"]) != (config["elements"], config["dofs_per_step"]) or abs(r["dt"] - config["dt"]) > 1e-15:
        raise RuntimeError("device operator and host config disagree on the workload")
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        c = cpu_rate(w, budget_s=args.cpu_budget)
        cpu = {"value": c["value"], "unit": UNIT, "cores": c["cores"], "kind": "port",
               "sample": f"{c['steps']} RK4 steps ({c['seconds']:.1f} s) of one incidence of the same workload with "
                         f"the oracle's {c['kind']}, OpenMP"}
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r["w"]["dtype"], "data": "synthetic", "config": config,
            "e2e": r["e2e"], "gpu_launches": r["launches"], "clocks": r["clocks"], "roofline": r["roofline"],
            "cpu_baseline": cpu, "setup_s": r["setup_s"]}
    if r.get("tune"):
        line["stage_kernel"] = {"choice": r["tune"]["kernel"], "ms_per_launch": r["tune"]["ms_per_launch"]}
    if r.get("e2e_streaming"):
        line["e2e_streaming"] = r["e2e_streaming"]
    if r.get("defect"):
        line["defect_correction"] = r["defect"]
    if "plain_fp64" in r:
        line["plain_fp64"] = r["plain_fp64"]
    if "accuracy" in r:
        line["accuracy"] = r["accuracy"]
    if args.high_order_steps > 0 and world == 1:
        import torch
        line["high_order"] = run_high_order(args.high_order_steps, torch.device("cuda", local))
    if args.serving_requests > 0 and world == 1:
        rates = [float(r) for r in args.serving_rates.split(",") if r]
        line["serving"] = run_serving(args.serving_requests, rates, args.serving_serial, local, args.serving_precision)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
