"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no golden vectors for these functions, so the oracle is
pinned by identities that the reference code satisfies by construction:
searchsortedlast semantics, partition of unity of the bilinear weights,
constant-field averages, exact gathers of bilinear grid fields, RK4 under a
uniform velocity, rotation invariance of the stress invariant, the Drucker-
Prager cap after yielding and the viscous limit of the visco-elastic
bisection.
"""
import math

import numpy as np
import pytest


def _model(eb, name="sinking_block"):
    return eb.synthetic.config(name)


def test_searchsortedlast_edges(oracle):
    lib = oracle.lib()
    g = np.array([0.0, 1.0, 2.5, 2.5000000000000004, 4.0, 10.0])
    n = len(g)
    pts = [-1.0, -0.0, 0.0, 0.5, 1.0, 2.5, np.nextafter(2.5, 3), 2.5000000000000004, 3.9999999, 4.0, 10.0, 11.0]
    for x in pts:
        want = int(np.searchsorted(g, x, side="right"))  # Julia searchsortedlast
        want = min(max(want, 1), n - 1)
        got = lib.o_index_of_left_node(float(x), g.ctypes.data, n)
        assert got == want, (x, got, want)


def test_weights_partition_of_unity(eb, oracle):
    ref = oracle.OracleMIC(_model(eb))
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    inside = ref.mk["inside"] == 1
    s = ref.mk["wUL"] + ref.mk["wLL"] + ref.mk["wUR"] + ref.mk["wLR"]
    assert np.max(np.abs(s[inside] - 1.0)) < 1e-15
    svy = ref.mk["wULvy"] + ref.mk["wLLvy"] + ref.mk["wURvy"] + ref.mk["wLRvy"]
    assert np.max(np.abs(svy[inside] - 1.0)) < 1e-15
    assert np.all((ref.mk["dx"][inside] >= 0) & (ref.mk["dx"][inside] <= 1))


def test_constant_field_averages_to_constant(eb, oracle):
    m = _model(eb)
    m.markers["rho"][:] = 2975.0
    m.markers["eta"][:] = 3.3e21
    ref = oracle.OracleMIC(m)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_stokes_parameters_to_grid()
    for name, val, w in (("rho1", 2975.0, "wtnodes"), ("etas1", 3.3e21, "wtetas"), ("etan1", 3.3e21, "wtetan"),
                         ("rho1_vy", 2975.0, "wtnodes_vy")):
        nz = ref.gr[w] != 0
        assert nz.any()
        assert np.max(np.abs(ref.gr[name][nz] / val - 1.0)) < 1e-14, name


def test_bilinear_field_gathers_exactly(eb, oracle):
    m = _model(eb)
    ref = oracle.OracleMIC(m)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    X, Y = np.meshgrid(m.grid.gridx_b, m.grid.gridy_b)
    ref.gr["tk1"][:] = np.asfortranarray(300.0 + 1e-3 * X + 2e-3 * Y)
    ref.interpolate_temperature_to_markers()
    inside = ref.mk["inside"] == 1
    want = 300.0 + 1e-3 * ref.mk["x"] + 2e-3 * ref.mk["y"]
    assert np.max(np.abs(ref.mk["tk"][inside] / want[inside] - 1.0)) < 1e-13


def test_rk4_uniform_velocity_moves_by_v_dt(eb, oracle):
    m = _model(eb)
    ref = oracle.OracleMIC(m)
    vx, vy = 3e-10, -2e-10
    ref.gr["vx1"][:] = vx
    ref.gr["vy1"][:] = vy
    ref.gr["esp"][:] = 0.0
    x0, y0 = ref.mk["x"].copy(), ref.mk["y"].copy()
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.advect_markers_and_rotate_stress()
    dt = m.params["timestep"]
    inside = ref.mk["inside"] == 1
    assert np.max(np.abs(ref.mk["x"][inside] - (x0[inside] + dt * vx))) < 1e-9
    assert np.max(np.abs(ref.mk["y"][inside] - (y0[inside] + dt * vy))) < 1e-9


def test_rotation_preserves_stress_invariant(eb, oracle):
    m = _model(eb)
    ref = oracle.OracleMIC(m)
    ref.gr["esp"][:] = np.asfortranarray(np.full(ref.gr["esp"].shape, 1e-13))
    s0 = np.hypot(ref.mk["sxx"], ref.mk["sxy"])
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.advect_markers_and_rotate_stress()
    s1 = np.hypot(ref.mk["sxx"], ref.mk["sxy"])
    inside = ref.mk["inside"] == 1
    assert np.max(np.abs(s1[inside] - s0[inside]) / s0[inside]) < 1e-14


def test_drucker_prager_cap_after_yielding(eb, oracle):
    m = eb.synthetic.config("rift_small")
    m.markers["sxx"] *= 40.0  # push many markers over the yield stress
    m.markers["sxy"] *= 40.0
    ref = oracle.OracleMIC(m)
    ref.get_marker_inside_flags()
    pf0 = ref.mk["pfailure"].copy()
    ref.update_plastic_yielding()
    yielded = (ref.mk["pfailure"] == 1) & (pf0 == 0)
    assert yielded.sum() > 100
    sii = np.hypot(ref.mk["sxx"], ref.mk["sxy"])[yielded]
    coh, sf, p = ref.mk["cohesion"][yielded], ref.mk["fric"][yielded], ref.mk["pr"][yielded]
    sy = coh * np.cos(np.arcsin(sf)) + sf * p
    assert np.max(np.abs(sii - sy) / sy) < 1e-12


def test_bisection_viscous_limit(eb, oracle):
    """With a very large shear modulus the visco-elastic factor -> 0 and the
    bisection must land on the viscous fixed point sigma = 2 eta(sigma) eps
    when the marker stress starts near it (the reference bisects between the
    marker stress and its forecast, CompositeViscosity.jl:234-276)."""
    m = eb.synthetic.config("rift_small")
    m.mats.mat_mu[:] = 1e40
    m.params["powerlaw_stress_min"] = 1.0
    m.params["viscosity_min"], m.params["viscosity_max"] = 1e10, 1e40
    k0 = m.markers
    k0["sr_ratio"][:] = 1.0
    k0["tk"][:] = 1100.0
    A, nexp, Ea = 8.57e-4, 4.0, 223.0
    eii = np.hypot(k0["exx"], k0["exy"])
    E = math.exp(-(Ea * 1000.0) / (m.params["gas_constant"] * 1100.0))
    s_star = (eii / (A * E)) ** (1.0 / nexp) * 1e6     # eps = A E s^n, s in MPa
    k0["sxx"][:] = s_star * 1.05
    k0["sxy"][:] = 0.0
    ref = oracle.OracleMIC(m)
    ref.get_marker_inside_flags()
    ref.update_marker_rheology()
    k = ref.mk
    sel = (k["matid"] == 2) & (k["inside"] == 1)       # wet quartzite: dislocation creep only
    assert sel.sum() > 1000
    assert np.all(ref.iters[sel] < 20)
    eta_star = 0.5 * s_star[sel] / eii[sel]
    got = k["eta_flow"][sel]
    # the loop stops once the bracket is <= 1 Pa wide: eta ~ sigma^(1-n) moves by (n-1)/sigma per Pa
    tol = (nexp - 1.0) * 1.0 / s_star[sel] + 1e-12
    assert np.all(np.abs(got / eta_star - 1.0) <= tol)


def test_oracle_cycle_is_deterministic(eb, oracle):
    m = _model(eb)
    a, b = oracle.OracleMIC(m), oracle.OracleMIC(m)
    a.marker_cycle()
    b.marker_cycle()
    for k in ("x", "y", "sxx", "sxy", "tk"):
        assert np.array_equal(a.mk[k], b.mk[k])
    for k in ("rho1", "etas1", "tk1", "dsxyn"):
        assert np.array_equal(a.gr[k], b.gr[k])
