"""Point probes, near-to-far surface nodes and running FP64 DFT sums (dgtd_op_*probe*).

Bars: interpolation of fields the element space represents exactly (linear in x)
to 1e-12; DFT sums equal sum_n u(t_n) exp(-i 2 pi f t_n) of the recorded samples
to 1e-12 (FP64 form) and are bit-identical between automatic sampling inside
dgtd_op_step and explicit sampling of the same states; the FP32 batched form
agrees with the FP64 form to its FP32 tolerance.
"""
import numpy as np
import pytest

import dgtd_gb300 as dg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(99)
COEF = RNG.standard_normal((6, 4))   # component c: a + b.x


def linear_state(xyz, B=1, scale=None):
    comps = [COEF[c, 0] + COEF[c, 1:] @ xyz for c in range(6)]
    one = np.concatenate(comps)
    return np.concatenate([one * (1.0 + b if scale is None else scale[b]) for b in range(B)])


def linear_at(p, b=0):
    return np.array([(COEF[c, 0] + COEF[c, 1:] @ p) * (1.0 + b) for c in range(6)])


def test_point_probes_interpolate_and_dft(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((2, 2, 2))
    op = dg.Operator(m, order=3)
    pts = np.array([[0.31, 0.42, 0.77], [0.5, 0.5, 0.5], [0.0, 0.0, 0.0], [1.0, 0.25, 0.6], [0.12, 0.9, 0.33]])
    freqs = np.array([0.0, 1.5, 3.25])
    op.set_probes(points=pts, freqs=freqs, max_records=4)
    x = torch.from_numpy(linear_state(op.node_coords())).cuda()
    t = 0.3
    op.probe_sample(x, t)
    r = op.probe_read()
    assert r["n_samples"] == 1 and r["series"].shape == (1, 1, len(pts), 6)
    for k, p in enumerate(pts):
        want = linear_at(p)
        assert np.abs(r["series"][0, 0, k] - want).max() < 1e-12
        for f, fr in enumerate(freqs):
            ph = np.exp(-2j * np.pi * fr * t)
            assert np.abs(r["points"][0, k, :, f] - want * ph).max() < 1e-12
    with pytest.raises(dg.DgtdError, match="outside"):
        op.set_probes(points=[[1.5, 0.5, 0.5]])


@pytest.mark.parametrize("integrator", [dg.RK4, dg.LSERK4])
def test_sampling_inside_step_matches_explicit_samples(torch_cuda, integrator):
    torch = torch_cuda
    m = dg.box_mesh((3, 3, 3), tfsf=((1, 1, 1), (2, 2, 2)), outer_bc=dg.BC_SMA)
    wave = dict(propagation=[1, 0.2, 0], polarization=[0, 0, 1], spread=0.15, mean=-0.3)
    pts = np.array([[0.5, 0.5, 0.5], [0.1, 0.2, 0.3], [0.9, 0.8, 0.45]])
    freqs = np.array([0.5, 1.3])
    auto = dg.Operator(m, order=2); auto.set_planewaves([wave])
    auto.set_probes(points=pts, surface_faces=m.tfsf_faces[:, ::-1], freqs=freqs, every=2, max_records=16)
    plain = dg.Operator(m, order=2); plain.set_planewaves([wave])
    manual = dg.Operator(m, order=2)
    manual.set_probes(points=pts, surface_faces=m.tfsf_faces[:, ::-1], freqs=freqs, every=1, max_records=16)
    dt = auto.estimate_dt(1.0)
    a = torch.zeros(auto.state_len, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    auto.step(a, 0.0, dt, 10, integrator)
    t = 0.0
    for n in range(1, 11):
        plain.step(b, t, dt, 1, integrator)
        t += dt
        if n % 2 == 0:
            manual.probe_sample(b, t)
    ra, rm = auto.probe_read(), manual.probe_read()
    assert ra["n_samples"] == rm["n_samples"] == 5
    assert np.array_equal(ra["points"], rm["points"]) and np.array_equal(ra["surface"], rm["surface"])
    assert np.array_equal(ra["series"], rm["series"]) and np.array_equal(ra["times"], rm["times"])
    assert np.abs(ra["series"]).max() > 0
    # the sums are the DFT of the recorded samples
    ph = np.exp(-2j * np.pi * np.outer(ra["times"], freqs))             # [n, nf]
    ref = np.einsum("nbpc,nf->bpcf", ra["series"], ph)
    assert np.abs(ra["points"] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_surface_nodes_weights_normals_and_side(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((4, 4, 4), tfsf=((1, 1, 1), (3, 3, 3)))
    op = dg.Operator(m, order=3)
    outward = m.tfsf_faces[:, ::-1]       # TF/SF faces wind into the total-field box: reverse them
    op.set_probes(surface_faces=outward, freqs=[0.0])
    xyz, nrm, w = op.probe_surface()
    assert xyz.shape[0] == outward.shape[0] * 10
    assert abs(w.sum() - 6 * 0.5 ** 2) < 1e-12                      # area of the box [0.25, 0.75]^3
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0)
    assert (np.einsum("ij,ij->i", nrm, xyz - 0.5) > 0).all()        # outward
    # a field that is 1 in elements inside the box and 0 outside: the inner element is sampled
    nodes = op.node_coords()
    Np = 20
    cen = nodes.reshape(3, -1, Np).mean(axis=2)
    inside = np.all((cen > 0.25) & (cen < 0.75), axis=0)
    f = np.repeat(inside.astype(float), Np)
    x = torch.from_numpy(np.concatenate([f] * 6)).cuda()
    op.probe_sample(x, 0.0)
    s = op.probe_read()["surface"]
    assert np.allclose(s.real, 1.0, atol=1e-14) and np.allclose(s.imag, 0.0, atol=1e-14)


def test_batched_fp32_probes_match_fp64(torch_cuda):
    torch = torch_cuda
    m = dg.box_mesh((3, 3, 3), lo=(-1, -1, -1), hi=(1, 1, 1), tfsf=((1, 1, 1), (2, 2, 2)), outer_bc=dg.BC_SMA)
    B = 3
    waves = [dict(propagation=[1, 0.1 * b, 0.2], polarization=[0, 1, 0], spread=0.2, mean=-0.4, batch=b)
             for b in range(B)]
    pts = np.array([[0.05, 0.1, -0.2], [0.6, -0.3, 0.4]])
    freqs = np.array([0.4, 0.9])
    faces = m.tfsf_faces[:, ::-1]
    o64 = dg.Operator(m, order=3, batch=B); o64.set_planewaves(waves)
    o32 = dg.Operator(m, order=3, batch=B, precision=dg.FP32_3XTF32); o32.set_planewaves(waves)
    for o in (o64, o32):
        o.set_probes(points=pts, surface_faces=faces, freqs=freqs, every=1, max_records=40)
    dt = o64.estimate_dt(1.0)
    x64 = torch.zeros(o64.state_len, dtype=torch.float64, device="cuda")
    w32 = o32.new_work()
    o64.step(x64, 0.0, dt, 40)
    o32.step(w32, 0.0, dt, 40)
    r64, r32 = o64.probe_read(), o32.probe_read()
    assert r64["n_samples"] == r32["n_samples"] == 40
    assert np.abs(r64["points"]).max() > 1e-3
    for key in ("points", "surface", "series"):
        assert rel_l2(r32[key], r64[key]) < 1e-5, key
    # a linear field through pack: interpolation exact to FP32 rounding
    xs = torch.from_numpy(linear_state(o32.node_coords(), B=B)).cuda()
    o32.probe_reset()
    o32.pack(xs, w32)
    o32.probe_sample(w32, 0.0)
    r = o32.probe_read()
    for b in range(B):
        for k, p in enumerate(pts):
            assert np.abs(r["series"][0, b, k] - linear_at(p, b)).max() < 1e-5 * (1 + b) * 10
