"""Serving engine (dgtd_server_*): continuous batching of independent solves.

Bars:
- a served request equals the same solve through the single-operator path
  (dgtd_op_run_host) and the oracle's RK4 loop: bit-identical to the former
  (same per-block arithmetic), <= 1e-12 relative L2 to the latter;
- every request's result is the same alone and in the mix: bit-identical,
  tolerance 0, because a block's arithmetic does not depend on which other
  requests share its launch;
- requests that arrive while others run are admitted and stepped in shared
  launches (packing and overlap visible in the server counters and timings);
- admission respects the memory budget; an oversize request fails cleanly.
"""
import time

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def scatter_request(n, order, seed, T):
    """Box [-1,1]^3 of n^3 hexes x 6 tets, SMA outer boundary, TF/SF box one cell in, and (n >= 5)
    a central PEC cube of max(1, round(n/6)) hexes."""
    rng = np.random.default_rng(seed)
    hole = None
    if n >= 5:
        c = max(1, int(np.floor(n / 6 + 0.5)))
        lo = (n - c) // 2
        hole = ((lo,) * 3, (lo + c,) * 3)
    m = dg.box_mesh((n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), hole=hole, tfsf=((1,) * 3, (n - 1,) * 3),
                    outer_bc=dg.BC_SMA, hole_bc=dg.BC_PEC)
    k = rng.standard_normal(3); k /= np.linalg.norm(k)
    g = rng.standard_normal(3); pol = g - g.dot(k) * k; pol /= np.linalg.norm(pol)
    wave = dict(propagation=k, polarization=pol, spread=0.1, mean=-0.5)
    return dict(mesh=m, order=order, waves=[wave], final_time=T)


def alone(req, **kw):
    with dg.Server(memory_budget=1 << 30, max_active=4, steps_per_round=kw.get("spr", 4)) as s:
        rid = s.submit(req["mesh"], req["order"], req["final_time"], waves=req["waves"], cfl=1.0)
        x, st = s.wait(rid, timeout=300)
    return x, st


def test_served_request_matches_operator_and_oracle(torch_cuda):
    req = scatter_request(3, 3, seed=1, T=0.12)
    x, st = alone(req)
    assert st["status"] == dg.REQ_DONE and st["steps"] > 0
    op = dg.Operator(req["mesh"], order=3)
    op.set_planewaves(req["waves"])
    dt = op.estimate_dt(1.0)
    assert st["dt"] == dt
    ref, n = op.run_host(np.zeros(op.state_len), 0.0, dt, req["final_time"])
    assert n == st["steps"]
    assert np.linalg.norm(ref) > 0
    assert np.array_equal(x, ref)
    orc = po.Oracle.from_mesh(req["mesh"], 3)
    orc.set_planewaves(req["waves"])
    xo, no = orc.run(np.zeros(op.state_len), 0.0, dt, req["final_time"])
    assert no == n
    assert rel_l2(x, xo) <= 1e-12


def test_alone_equals_in_the_mix(torch_cuda):
    reqs = [scatter_request(n, p, seed=10 + i, T=T)
            for i, (n, p, T) in enumerate([(3, 2, 0.3), (4, 3, 0.2), (3, 3, 0.25), (4, 4, 0.1), (5, 2, 0.2),
                                           (3, 4, 0.15)])]
    ref = [alone(r)[0] for r in reqs]
    with dg.Server(memory_budget=2 << 30, max_active=16, steps_per_round=2) as s:
        ids = [s.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0) for r in reqs]
        got = [s.wait(i, timeout=300) for i in ids]
        stats = s.stats()
    for (x, st), xr in zip(got, ref):
        assert st["status"] == dg.REQ_DONE
        assert np.array_equal(x, xr)
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["max_active_seen"] >= 2
    # packing: on average a stage launch advanced more than one request
    assert stats["slot_stage_updates"] > stats["stage_launches"]
    assert stats["bytes_in_use"] == 0


def test_arrivals_while_running_are_admitted_and_overlap(torch_cuda):
    long = scatter_request(5, 3, seed=21, T=1.0)
    short = [scatter_request(3, 3, seed=30 + i, T=0.1) for i in range(3)]
    ref_short = [alone(r)[0] for r in short]
    with dg.Server(memory_budget=2 << 30, max_active=8, steps_per_round=2) as s:
        lid = s.submit(long["mesh"], long["order"], long["final_time"], waves=long["waves"], cfl=1.0)
        # wait until the long solve is on the device, then send the short ones
        t0 = time.time()
        while s.query(lid)["t_first_launch"] == 0.0 and time.time() - t0 < 60:
            time.sleep(0.005)
        sids = [s.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0) for r in short]
        outs = [s.wait(i, timeout=300) for i in sids]
        xl, stl = s.wait(lid, timeout=300)
    for (x, st), xr in zip(outs, ref_short):
        assert np.array_equal(x, xr)
        # admitted and finished while the long request was still running
        assert st["t_first_launch"] < stl["t_done"]
        assert st["t_done"] < stl["t_done"]
    assert np.array_equal(xl, alone(long)[0])


def test_memory_budget_admission(torch_cuda):
    reqs = [scatter_request(4, 3, seed=40 + i, T=0.1) for i in range(5)]
    ref = [alone(r)[0] for r in reqs]
    # measure one region, then give the server room for two at a time
    with dg.Server(memory_budget=1 << 30, max_active=4) as s:
        rid = s.submit(reqs[0]["mesh"], 3, 0.0, waves=reqs[0]["waves"], cfl=1.0)
        _, st = s.wait(rid, timeout=300, want_state=False)
        region = st["region_bytes"]
    assert region > 0
    budget = int(2.5 * region)
    with dg.Server(memory_budget=budget, max_active=8, steps_per_round=2) as s:
        ids = [s.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0) for r in reqs]
        got = [s.wait(i, timeout=300) for i in ids]
        stats = s.stats()
    for (x, st), xr in zip(got, ref):
        assert np.array_equal(x, xr)
    assert stats["peak_bytes_in_use"] <= budget
    assert stats["max_active_seen"] <= 2


def test_oversize_request_fails_cleanly(torch_cuda):
    req = scatter_request(4, 3, seed=50, T=0.1)
    with dg.Server(memory_budget=1 << 20, max_active=2) as s:
        rid = s.submit(req["mesh"], req["order"], req["final_time"], waves=req["waves"], cfl=1.0)
        with pytest.raises(dg.DgtdError, match="budget"):
            s.wait(rid, timeout=120)
        # the server keeps serving requests that fit
        small = scatter_request(2, 1, seed=51, T=0.05)
        rid2 = s.submit(small["mesh"], small["order"], small["final_time"], waves=small["waves"], cfl=1.0)
        x, st = s.wait(rid2, timeout=120)
        assert st["status"] == dg.REQ_DONE


def test_initial_state_and_no_sources(torch_cuda):
    """A resonator request (TE110 initial field, PEC, no sources) against the operator path."""
    m = dg.box_mesh((3, 3, 3))
    op = dg.Operator(m, order=3)
    xyz = op.node_coords()
    z = np.zeros(op.ndofs)
    x0 = np.concatenate([z, z, np.sin(np.pi * xyz[0]) * np.sin(np.pi * xyz[1]), z, z, z])
    with dg.Server(memory_budget=1 << 28, max_active=2) as s:
        rid = s.submit(m, 3, 0.05, init=x0, dt=1e-3)
        x, st = s.wait(rid, timeout=120)
    ref, n = op.run_host(x0, 0.0, 1e-3, 0.05)
    assert st["steps"] == n == 50
    assert np.array_equal(x, ref)


def test_unstable_request_is_flagged(torch_cuda):
    """The run loop's instability detector (reference Solver.cpp:500-516) on served requests: a
    NaN planted in one request's initial state flags that request only."""
    m = dg.box_mesh((3, 3, 3))
    op = dg.Operator(m, order=2)
    xyz = op.node_coords()
    z = np.zeros(op.ndofs)
    good = np.concatenate([z, z, np.sin(np.pi * xyz[0]) * np.sin(np.pi * xyz[1]), z, z, z])
    bad = good.copy()
    bad[7] = np.nan
    with dg.Server(memory_budget=1 << 28, max_active=4) as s:
        ids = [s.submit(m, 2, 0.02, init=x, dt=1e-3) for x in (good, bad)]
        res = [s.wait(i, timeout=120) for i in ids]
    assert res[0][1]["unstable"] == 0 and np.all(np.isfinite(res[0][0]))
    assert res[1][1]["unstable"] == 1 and not np.all(np.isfinite(res[1][0]))
    assert res[1][1]["status"] == dg.REQ_DONE


def test_fp32_serving_matches_fp32_operator_and_mix(torch_cuda):
    """FP32 serving runs the single-instance FP32 form's stage: bit-identical to
    dgtd_op_run_host of that form, alone and in the mix, and within 1e-5 of FP64."""
    reqs = [scatter_request(n, p, seed=60 + i, T=0.2) for i, (n, p) in enumerate([(4, 3), (5, 2), (4, 4)])]
    with dg.Server(memory_budget=1 << 30, max_active=8, steps_per_round=3, precision=dg.FP32) as s:
        ids = [s.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0) for r in reqs]
        mix = [s.wait(i, timeout=300)[0] for i in ids]
    for r, xm in zip(reqs, mix):
        with dg.Server(memory_budget=1 << 30, max_active=2, precision=dg.FP32) as s:
            alone_x, st = s.wait(s.submit(r["mesh"], r["order"], r["final_time"], waves=r["waves"], cfl=1.0), 300)
        assert np.array_equal(xm, alone_x)
        op = dg.Operator(r["mesh"], order=r["order"], precision=dg.FP32)
        op.set_contraction(1)          # the server steps the FP32 SIMT stage body
        op.set_planewaves(r["waves"])
        ref32, n = op.run_host(np.zeros(op.state_len), 0.0, op.estimate_dt(1.0), r["final_time"])
        assert n == st["steps"] and np.array_equal(xm, ref32)
        op64 = dg.Operator(r["mesh"], order=r["order"])
        op64.set_planewaves(r["waves"])
        ref64, _ = op64.run_host(np.zeros(op64.state_len), 0.0, op64.estimate_dt(1.0), r["final_time"])
        assert rel_l2(xm, ref64) < 1e-5
