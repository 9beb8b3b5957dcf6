"""CUDA-graph replay of blocks of RK4 steps (batched FP32 form).

Bars: without sources the replay runs the same kernels on the same data, so the
state is bit-identical to direct launches; with a TF/SF plane wave the stage
times come from a device scalar (block start + offset) instead of the host, so
the source term can differ in the last FP32 bit of the time: relative L2 <= 1e-6.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _run(op, torch, steps, graph, x0, dt, stream):
    op.set_graph_steps(graph)
    w = op.new_work()
    with torch.cuda.stream(stream):
        op.pack(torch.from_numpy(x0).cuda(), w, stream=stream)
        op.step(w, 0.0, dt, steps, stream=stream)
        out = torch.zeros(op.state_len, dtype=torch.float64, device="cuda")
        op.unpack(w, out, stream=stream)
    stream.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("order,tc", [(2, True), (4, True), (3, False)])
def test_graph_matches_direct_without_sources(torch_cuda, order, tc):
    torch = torch_cuda
    m = dg.box_mesh((3, 3, 3), outer_bc=dg.BC_PEC)
    op = dg.Operator(m, order=order, precision=dg.FP32_3XTF32, batch=64)
    op.set_contraction(0 if tc else 1)
    x0 = np.random.default_rng(5).standard_normal(op.state_len)
    s = torch.cuda.Stream()
    direct = _run(op, torch, 23, 0, x0, 1e-3, s)
    graph = _run(op, torch, 23, 5, x0, 1e-3, s)
    assert np.array_equal(direct, graph)


def test_graph_with_tfsf_source(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((4, 4, 4), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1,) * 3, (3,) * 3), outer_bc=dg.BC_SMA)
    B = 64
    rng = np.random.default_rng(3)
    waves = []
    for b in range(B):
        k = rng.standard_normal(3); k /= np.linalg.norm(k)
        g = rng.standard_normal(3); pol = g - g.dot(k) * k
        waves.append(dict(propagation=k, polarization=pol, spread=0.15, mean=-0.5, batch=b))
    op = dg.Operator(m, order=3, precision=dg.FP32_3XTF32, batch=B)
    op.set_planewaves(waves)
    dt = op.estimate_dt(1.0)
    x0 = np.zeros(op.state_len)
    s = torch.cuda.Stream()
    direct = _run(op, torch, 60, 0, x0, dt, s)
    graph = _run(op, torch, 60, 8, x0, dt, s)
    assert np.linalg.norm(direct) > 0
    assert rel_l2(graph, direct) <= 1e-6
    # replaying again from a new start reuses the captured graph
    again = _run(op, torch, 60, 8, x0, dt, s)
    assert np.array_equal(again, graph)


def test_graph_rejected_on_other_forms(torch_cuda):
    m = dg.box_mesh((2, 2, 2))
    op = dg.Operator(m, order=2)
    with pytest.raises(dg.DgtdError, match="batched"):
        op.set_graph_steps(4)
