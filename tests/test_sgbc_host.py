"""Thin-layer boundaries (SGBC) on the host, no GPU.

- The product's sub-solver operator (nodal DG, sgbc.cpp) against the oracle's assembled 1D
  operator (weak form, exact quadrature): bar 1e-13 relative to max |A|.
- The product's composed sub-step maps against the oracle's stepwise SDIRK33 sub-steps: 1e-12.
- The oracle's coupling (a restatement of GlobalEvolution's SGBC path, GlobalEvolution.cpp:48-1001):
  a stack closed by PEC sheets on both sides is an interior PEC sheet (1e-12); in a TEM waveguide
  the reflected and transmitted pulses follow the analytic S11/S21 of the slab.
- The case loader's SGBC rules (driver.cpp:1293-1466, SolverExtension.cpp:509-541) on the
  reference's own 3D_SGBC case and edited copies of it.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import dgtd_gb300 as dg
from oracle import pyoracle as po
from conftest import FREE_SPACE_IMPEDANCE as Z0, SPEED_OF_LIGHT_SI as C0, rel_l2, sgbc_box, slab_pulse, tem_waveguide

REF_SGBC = Path(__file__).resolve().parent / "golden" / "cases" / "reference" / "3D_SGBC"

STACKS = [
    # the reference 3D_SGBC layer (eps 20, 0.2 S/m, 5 mm; automatic order 3 and 4 segments)
    {"layers": [{"eps": 20.0, "mu": 1.0, "sigma": 0.2 * Z0, "width": 5e-3, "segments": 4, "order": 3}],
     "left": 0, "right": 0, "sub_dt": 2.795e-3},
    # two layers of different order, a PEC sheet on the left
    {"layers": [{"eps": 2.0, "mu": 1.5, "sigma": 1.0, "width": 0.02, "segments": 2, "order": 2},
                {"eps": 4.0, "mu": 1.0, "sigma": 0.0, "width": 0.01, "segments": 3, "order": 1}],
     "left": 1, "right": 0, "sub_dt": 1e-3},
    # PMC left, SMA right
    {"layers": [{"eps": 1.0, "mu": 1.0, "sigma": 0.0, "width": 0.01, "segments": 2, "order": 4}],
     "left": 2, "right": 3, "sub_dt": 1e-3},
]


@pytest.mark.parametrize("k", range(len(STACKS)))
def test_stack_operator_matches_oracle(k):
    P = dg.sgbc_stack_operator(STACKS[k])
    S = po.SgbcStack(STACKS[k])
    A = S.matrix()
    assert P["n"] == S.n and P["idx_left"] == S.idx_left and P["idx_right"] == S.idx_right
    assert np.abs(P["A"] - A).max() <= 1e-13 * np.abs(A).max()


@pytest.mark.parametrize("k", range(len(STACKS)))
def test_stack_maps_match_oracle_substeps(k):
    st = STACKS[k]
    S = po.SgbcStack(st)
    rng = np.random.default_rng(10 + k)
    L = S.n // 6
    for span in (5e-4, 2.5e-3, 7.3e-3):
        ns = math.ceil(span / st["sub_dt"]) if 0 < st["sub_dt"] < span else 1
        M = dg.sgbc_stack_maps(st, span, ns)
        x, go, gn = rng.standard_normal(S.n), rng.standard_normal(12), rng.standard_normal(12)
        y = S.advance(x, go, None, 0.0, span)   # ghosts held (a stage's sub-solve)
        iface = np.array([y[c * L + S.idx_left] for c in range(6)] + [y[c * L + S.idx_right] for c in range(6)])
        assert np.abs(M["R"] @ x + M["G"] @ go - iface).max() <= 1e-12 * np.abs(iface).max()
        y = S.advance(x, go, gn, 0.0, span)     # ghosts interpolated (the step's finalisation)
        assert np.abs(M["F"] @ x + M["Vo"] @ go + M["Vn"] @ gn - y).max() <= 1e-12 * np.abs(y).max()


def test_stack_above_dense_limit_is_refused():
    big = {"layers": [{"eps": 1.0, "mu": 1.0, "sigma": 0.0, "width": 0.01, "segments": 2, "order": 6}]}
    with pytest.raises(dg.DgtdError, match="dense limit"):
        dg.sgbc_stack_operator(big)
    with pytest.raises(dg.DgtdError, match="needs segments >= 1"):
        dg.sgbc_stack_operator({"layers": [{"width": 0.01, "segments": 0, "order": 2}]})


def _bump(o, x0=1.0, s=0.15):
    """Ey = Hz = Gaussian across x = x0: a right-moving pulse already on the sheet, so that no pair
    is ever quiescent."""
    X = o.nodes()
    N = X.shape[1]
    u = np.zeros(6 * N)
    g = np.exp(-((X[0] - x0) ** 2) / (2 * s * s))
    u[1 * N:2 * N] = g
    u[5 * N:6 * N] = g
    return u


def test_oracle_pec_closed_stack_is_a_pec_sheet():
    """Both sides closed by PEC: the injection's slot values are the PEC mirrors of the two
    elements' own traces, which is the interior PEC sheet's integrator (DGOperatorFactory.h:577-675)."""
    m, _, F = sgbc_box(n=(4, 2, 2), tfsf=False)
    mk = lambda code: po.Oracle(m.vertices, m.elements, 2, 1.0, 3, m.bdr_faces, m.bdr_codes, None, F,
                                np.full(len(F), code, np.int32))
    sheet, layer = mk(1), mk(4)
    layer.set_sgbc([{"layers": [{"eps": 3.0, "sigma": 2.0, "width": 0.05, "segments": 2, "order": 2}],
                     "left": 1, "right": 1, "sub_dt": 0.004}], np.zeros(len(F), np.int32))
    assert layer.sgbc_pairs() == len(F) * 6
    u0 = _bump(sheet)
    a, b = sheet.step(u0, 0.0, 0.01, 40), layer.step(u0, 0.0, 0.01, 40)
    assert np.linalg.norm(a) > 1.0 and rel_l2(b, a) <= 1e-12


def test_oracle_slab_matches_analytic_s_parameters():
    """A 2 cm slab (eps 4, 0.05 S/m) as an SGBC sheet in a TEM waveguide, order 3: the reflected
    field before the TF/SF plane and the transmitted field beyond the sheet follow the slab's
    analytic S11 and S21 applied to the incident Gaussian. Measured: 1.2e-2 / 4.2e-3 of the incident
    amplitude (the same mesh without a sheet carries 4.8e-3 against free propagation)."""
    m, codes, F = tem_waveguide()
    eps, mu, sig, d = 4.0, 1.0, 0.05 * Z0, 0.02
    st = {"layers": [{"eps": eps, "mu": mu, "sigma": sig, "width": d, "segments": 4, "order": 2}],
          "sub_dt": 0.5 * (d / 4) * math.sqrt(eps * mu)}
    o = po.Oracle(m.vertices, m.elements, 3, 1.0, 3, m.bdr_faces, codes, m.tfsf_faces, F, np.full(len(F), 4, np.int32))
    o.set_planewaves([{"propagation": [1, 0, 0], "polarization": [0, 1, 0], "spread": 0.15, "mean": 0.5}])
    o.set_sgbc([st], np.zeros(len(F), np.int32))
    X = o.nodes()
    N = X.shape[1]
    node = lambda x: int(np.argmin((X[0] - x) ** 2 + (X[1] - 0.25) ** 2 + (X[2] - 0.25) ** 2))
    ir, it = node(0.5), node(3.5)
    u, dt, ts, rr, tr = np.zeros(6 * N), 0.01, [], [], []
    for s in range(450):
        u = o.step(u, s * dt, dt, 1)
        ts.append((s + 1) * dt); rr.append(u[N + ir]); tr.append(u[N + it])
    ts = np.array(ts)
    pt = slab_pulse(ts, 2.5, 3.5, 0.15, 0.5, eps, mu, sig, d, "t")
    pr = slab_pulse(ts, 2.5, 0.5, 0.15, 0.5, eps, mu, sig, d, "r")
    assert 0.8 < np.abs(pt).max() < 0.9 and 0.15 < np.abs(pr).max() < 0.3
    assert np.abs(np.array(tr) - pt).max() <= 0.02
    assert np.abs(np.array(rr) - pr).max() <= 0.01


# ---------------------------------------------------------------- case loader rules

def _ref_sgbc_copy(tmp_path, name, edit=None):
    d = tmp_path / name
    d.mkdir()
    case = json.loads((REF_SGBC / "3D_SGBC.json").read_text())
    case["model"]["filename"] = f"{name}.msh"
    if edit:
        edit(case)
    (d / f"{name}.json").write_text(json.dumps(case))
    (d / f"{name}.msh").write_text((REF_SGBC / "3D_SGBC.msh").read_text())
    return d / f"{name}.json"


def _expected_layer(eps, mu, sigma_si, width, fmax):
    """driver.cpp:1298-1405 and SolverExtension.cpp:509-541, restated for the check."""
    mu_si, eps_si = mu * 4e-7 * math.pi, eps * 8.8541878188e-12
    pe = sigma_si / (fmax * eps_si) if sigma_si > 0 else 0.0
    order = 2 if pe > 100 else (4 if (pe < 0.1 and sigma_si < 1e-3) else 3)
    wl = 1.0 / (fmax * math.sqrt(mu_si * eps_si))
    dxw = wl / math.ceil(20.0 / order)
    skin = 1.0 / math.sqrt(math.pi * fmax * mu_si * sigma_si) if sigma_si > 0 else 0.0
    dxs = skin / 2 if sigma_si > 0 else float("inf")
    seg = min(max(math.ceil(width / min(dxw, dxs)), 4), 1000)
    nd = width / skin if sigma_si > 0 else 0.0
    dtl = (width / seg * math.sqrt(eps * mu)) / C0 * 0.5
    if nd > 3:
        dtl *= min(nd * nd, 50.0)
    return order, seg, dtl * C0


def test_reference_3d_sgbc_case_stack():
    c = dg.Case(REF_SGBC / "3D_SGBC.json")
    assert c.info["n_sgbc_stacks"] == 1 and c.info["n_sgbc_faces"] == 40
    stacks, fs = c.sgbc()
    assert list(fs) == [0] * 40
    (L,) = stacks[0]["layers"]
    order, seg, sub = _expected_layer(20.0, 1.0, 0.2, 5e-3, C0 / (2 * 0.2))
    assert (L["order"], L["segments"]) == (order, seg) == (3, 4)
    assert L["eps"] == 20.0 and L["mu"] == 1.0 and L["width"] == 5e-3
    assert L["sigma"] == pytest.approx(0.2 * Z0, rel=1e-15)
    assert stacks[0]["sub_dt"] == pytest.approx(sub, rel=1e-15) and stacks[0]["left"] == stacks[0]["right"] == 0
    m = c.mesh()
    assert list(np.unique(m.int_codes)) == [dg.BC_SGBC] and len(m.int_codes) == 40
    assert dg.sgbc_stack_operator(stacks[0])["n"] == 288


@pytest.mark.parametrize("eps,sigma", [(20.0, 1e4), (1.0, 0.0), (4.0, 1e-4), (2.0, 5.0)])
def test_sgbc_automatic_order_and_segments(tmp_path, eps, sigma):
    def edit(c):
        mat = c["model"]["boundaries"][3]["material"]
        mat["relative_permittivity"] = eps
        mat["bulk_conductivity"] = sigma
    c = dg.Case(_ref_sgbc_copy(tmp_path, "auto", edit))
    (L,) = c.sgbc()[0][0]["layers"]
    order, seg, sub = _expected_layer(eps, 1.0, sigma, 5e-3, C0 / (2 * 0.2))
    assert (L["order"], L["segments"]) == (order, seg)
    assert c.sgbc()[0][0]["sub_dt"] == pytest.approx(sub, rel=1e-14)


def test_sgbc_modulated_source_frequency_and_overrides(tmp_path):
    def edit(c):
        c["sources"][0]["magnitude"]["frequency"] = 2e9
        mat = c["model"]["boundaries"][3]["material"]
        mat["bulk_conductivity"] = 3.0
    c = dg.Case(_ref_sgbc_copy(tmp_path, "modulated", edit))
    (L,) = c.sgbc()[0][0]["layers"]
    order, seg, _ = _expected_layer(20.0, 1.0, 3.0, 5e-3, 2e9 + C0 / (2 * 0.2))
    assert (L["order"], L["segments"]) == (order, seg)

    def override(c):
        c["model"]["boundaries"][3]["material"].update({"num_of_segments": 7, "order": 2})
    c = dg.Case(_ref_sgbc_copy(tmp_path, "override", override))
    (L,) = c.sgbc()[0][0]["layers"]
    assert (L["order"], L["segments"]) == (2, 7)


def test_sgbc_layers_and_sheet_sides(tmp_path):
    def layers(c):
        b = c["model"]["boundaries"][3]
        del b["material"]
        b["layers"] = [{"relative_permittivity": 2.0, "bulk_conductivity": 0.0, "material_width": 1e-3,
                        "num_of_segments": 2, "order": 2},
                       {"relative_permeability": 3.0, "bulk_conductivity": 1.0, "material_width": 2e-3,
                        "num_of_segments": 3, "order": 1}]
        b["sgbc_boundaries"] = {"left": "PEC"}
    st = dg.Case(_ref_sgbc_copy(tmp_path, "layers", layers)).sgbc()[0][0]
    assert [(L["eps"], L["mu"], L["segments"], L["order"]) for L in st["layers"]] == [(2.0, 1.0, 2, 2), (1.0, 3.0, 3, 1)]
    assert (st["left"], st["right"]) == (dg.BC_PEC, 0)

    def material_sides(c):   # sides in the material when the entry has none (driver.cpp:1447-1452)
        c["model"]["boundaries"][3]["material"]["sgbc_boundaries"] = {"left": "SMA", "right": "PMC"}
    st = dg.Case(_ref_sgbc_copy(tmp_path, "msides", material_sides)).sgbc()[0][0]
    assert (st["left"], st["right"]) == (dg.BC_SMA, dg.BC_PMC)


@pytest.mark.parametrize("edit,msg", [
    (lambda b: b["material"].pop("bulk_conductivity"), "without 'bulk_conductivity'"),
    (lambda b: b["material"].pop("material_width"), "must define 'material_width'"),
    (lambda b: b.pop("material"), "must define either 'material' or 'layers'"),
    (lambda b: b.update({"sgbc_boundaries": {"left": "XYZ"}}), "Incorrect sgbc_bdr_type"),
])
def test_sgbc_malformed_entries(tmp_path, edit, msg):
    def e(c):
        edit(c["model"]["boundaries"][3])
    with pytest.raises(dg.DgtdError, match=msg):
        dg.Case(_ref_sgbc_copy(tmp_path, "bad", e))


def test_sgbc_on_the_domain_boundary_and_operator_rules(tmp_path):
    # the SMA end walls (tags 19, 30) as an SGBC entry: exterior faces, SMA coefficients
    def outer(c):
        b = c["model"]["boundaries"]
        b[2]["type"] = "SGBC"
        b[2]["material"] = {"bulk_conductivity": 1.0, "material_width": 1e-3}
    c = dg.Case(_ref_sgbc_copy(tmp_path, "outer", outer))
    m = c.mesh()
    assert c.info["n_sgbc_stacks"] == 2 and c.info["n_sgbc_faces"] == 40
    assert int(np.sum(m.bdr_codes == dg.BC_SMA)) == 56

    def outer_alpha(c):
        outer(c)
        c["solver_options"]["upwind_alpha"] = 0.5
    with pytest.raises(dg.DgtdError, match="upwind_alpha 1 only"):
        dg.Case(_ref_sgbc_copy(tmp_path, "outer_alpha", outer_alpha))

    def hesthaven(c):
        c["solver_options"]["evolution_operator"] = "hesthaven"
    with pytest.raises(dg.DgtdError, match="evolution_operator 'global' only"):
        dg.Case(_ref_sgbc_copy(tmp_path, "hest", hesthaven))


def test_oracle_pec_closed_stack_on_a_curved_sheet_is_a_pec_sheet():
    """The same identity on a curved sheet (every element curved, the sheet x = 1/2 bent by the
    map): per-point normals in the injection's face integrals and per-node normals in the pairs'
    rotations."""
    from conftest import curved_box, plane_faces
    m, Vc, E, els, nodes = curved_box(mode="all", bump=0.03)
    F = plane_faces(np.asarray(m.vertices), E, 0.5)
    mk = lambda code: po.Oracle(Vc, E, 2, 1.0, 3, m.bdr_faces, m.bdr_codes, None, F, np.full(len(F), code, np.int32))
    sheet, layer = mk(1), mk(4)
    for o in (sheet, layer):
        o.set_curved(els, nodes)
    layer.set_sgbc([{"layers": [{"eps": 3.0, "sigma": 2.0, "width": 0.05, "segments": 2, "order": 2}],
                     "left": 1, "right": 1, "sub_dt": 0.004}], np.zeros(len(F), np.int32))
    u0 = _bump(sheet, 0.5)
    a, b = sheet.step(u0, 0.0, 0.005, 40), layer.step(u0, 0.0, 0.005, 40)
    assert np.linalg.norm(a) > 1.0 and rel_l2(b, a) <= 1e-12
