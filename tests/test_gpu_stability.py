"""Instability detector of the run loop (reference Solver::run, src/solver/Solver.cpp:500-516).

The reference checks the field norm after every step and warns when it is not finite or
above 1e20. Here a device reduction runs every `every` steps inside dgtd_op_run_host and
its record is read back on the host. The failures are made on the host: a NaN written into
the initial state, a state above the threshold, and a time step far above the stability
limit that makes the solution grow until it trips the threshold.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg

pytestmark = pytest.mark.gpu


def _op(precision=dg.FP64, batch=1, order=2):
    m = dg.box_mesh((3, 3, 3), outer_bc=dg.BC_PEC)
    return dg.Operator(m, order=order, precision=precision, batch=batch)


def _te110(op):
    xyz = op.node_coords()
    z = np.zeros(xyz.shape[1])
    one = np.concatenate([z, z, np.sin(np.pi * xyz[0]) * np.sin(np.pi * xyz[1]), z, z, z])
    return np.tile(one, op.batch)


@pytest.mark.parametrize("precision,batch", [(dg.FP64, 1), (dg.FP32, 1), (dg.FP32_3XTF32, 64)])
def test_stable_run_is_not_flagged(torch_cuda, precision, batch):
    op = _op(precision, batch)
    op.set_stability_check(every=3)
    dt = op.estimate_dt(1.0)
    _, n = op.run_host(_te110(op), 0.0, dt, 20 * dt)
    st = op.stability()
    assert n == 20
    assert not st["unstable"] and st["first_step"] == -1
    assert st["checks"] == 20 // 3 + 1      # every third step and the final state


@pytest.mark.parametrize("precision,batch", [(dg.FP64, 1), (dg.FP32, 1), (dg.FP32_3XTF32, 64)])
def test_nan_in_initial_state_is_flagged(torch_cuda, precision, batch):
    op = _op(precision, batch)
    op.set_stability_check(every=1)
    x = _te110(op)
    x[len(x) // 3 + 5] = np.nan
    dt = op.estimate_dt(1.0)
    out, n = op.run_host(x, 0.0, dt, 4 * dt)      # warning mode: the run goes on
    st = op.stability()
    assert n == 4 and st["unstable"] and st["first_step"] == 1
    assert not np.isfinite(st["norm"])
    assert abs(st["t"] - dt) < 1e-12
    op.set_stability_check(every=1, stop=True)
    with pytest.raises(dg.DgtdError) as ei:
        op.run_host(x, 0.0, dt, 4 * dt)
    assert ei.value.code == dg.DGTD_ERR_UNSTABLE
    assert "potentially unstable" in str(ei.value)


def test_norm_above_threshold_is_flagged(torch_cuda):
    op = _op()
    op.set_stability_check(every=2)
    x = _te110(op) * 1e21          # ||x|| well above 1e20 from the start
    dt = op.estimate_dt(1.0)
    op.run_host(x, 0.0, dt, 5 * dt)
    st = op.stability()
    assert st["unstable"] and st["first_step"] == 2 and st["norm"] > 1e20
    x = _te110(op)                 # the record is cleared by the next run
    op.run_host(x, 0.0, dt, 5 * dt)
    assert not op.stability()["unstable"]


def test_time_step_above_the_limit_trips_the_detector(torch_cuda):
    """An explicit RK4 step 40x above the estimate grows the discrete solution
    exponentially; the detector reports the first check past 1e20 and stop mode ends
    the run early."""
    op = _op(order=3)
    dt = 40.0 * op.estimate_dt(1.0)
    op.set_stability_check(every=5, stop=True)
    with pytest.raises(dg.DgtdError) as ei:
        op.run_host(_te110(op), 0.0, dt, 5000 * dt)
    assert ei.value.code == dg.DGTD_ERR_UNSTABLE
    st = op.stability()
    assert st["unstable"] and st["first_step"] % 5 == 0 and st["first_step"] < 5000
    assert not (st["norm"] <= 1e20)


def test_detector_off(torch_cuda):
    op = _op()
    op.set_stability_check(every=0)
    x = _te110(op)
    x[3] = np.nan
    dt = op.estimate_dt(1.0)
    op.run_host(x, 0.0, dt, 3 * dt)
    st = op.stability()
    assert st["checks"] == 0 and not st["unstable"]
