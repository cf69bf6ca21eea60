"""The analytic profiles and measures the benchmark tests compare against, restated from the
reference's post-processing managers, checked against their defining properties."""
import math

import numpy as np


def test_power_law_channel_profile(eb):
    """ChannelFlowNonNewtonianManager.calc_velocity: zero on the walls, symmetric, and the
    centre value C1 / (n + 1) (-dp/dy)^n (W/2)^(n+1) with C1 = 2 A / 1e6^n."""
    syn = eb.synthetic
    W, ydim = 10e3, 9500.0
    x = np.linspace(0.0, W, 51)
    v = syn.channel_flow_velocity(x, W, ydim, 1e9, 5e-20, 3.0)
    assert v[0] == 0.0 and v[-1] == 0.0
    assert np.allclose(v, v[::-1], rtol=1e-15, atol=0.0)
    c1 = 5e-20 * 2.0 / 1e18
    assert math.isclose(v[25], c1 / 4.0 * (1e9 / ydim) ** 3 * (W / 2.0) ** 4, rel_tol=1e-14)


def test_couette_steady_profile_spans_the_wall_temperatures(eb):
    """CouetteFlowViscousHeatingManager: the profile runs from the left wall (phi = 1, x = 0) to
    the right wall (phi = phi1, x = W) and rises monotonically."""
    x, t = eb.synthetic.couette_temperature_profile(1000.15, 1300.0, 30e3, 150e3)
    assert x[0] == 0.0 and math.isclose(x[-1], 30e3, rel_tol=1e-9)
    assert t[0] == 1000.15 and abs(t[-1] - 1300.0) < 1e-3
    assert np.all(np.diff(t) > 0.0) and np.all(np.diff(x) > 0.0)


def test_variable_conductivity_profile(eb):
    """ChannelFlowVariableConductivityManager: the wall temperature on both walls, symmetric,
    and for b -> 0 the constant-conductivity parabola T_w + W^4 (dp/dy)^2 / (192 k eta)
    (1 - (2x/W - 1)^4)."""
    syn = eb.synthetic
    W, h = 30e3, 11250.0
    x = np.linspace(0.0, W, 51)
    t = syn.channel_flow_variable_conductivity_temperature(x, W, h, 298.15, 3e7, 1e19, 8.0, 1.0)
    assert math.isclose(t[0], 298.15, rel_tol=1e-14) and math.isclose(t[-1], 298.15, rel_tol=1e-14)
    assert np.allclose(t, t[::-1], rtol=1e-13)
    tb = syn.channel_flow_variable_conductivity_temperature(x, W, h, 298.15, 3e7, 1e19, 8.0, 1e-9)
    lin = 298.15 + W ** 4 * (3e7 / h) ** 2 / 192.0 / 8.0 / 1e19 * (1.0 - (2.0 * x / W - 1.0) ** 4)
    assert np.allclose(tb, lin, rtol=1e-6)


def test_non_steady_channel_profile_starts_from_the_initial_temperature(eb):
    """ChannelFlowNonSteadyTemperatureManager: at t = 0 every term vanishes and the profile is the
    initial temperature of the row (Celsius)."""
    t = eb.synthetic.channel_flow_non_steady_temperature_profile(
        np.linspace(0.0, 30e3, 51), 0.0, 30e3, 12.5e3, 11, 11, 727.0, 1227.0, 1e5, 1e19, 2.0, 3000.0, 1000.0)
    assert np.allclose(t, 1227.0, rtol=0.0, atol=1e-9)


def test_box_convection_vrms_of_a_uniform_field(eb):
    """BoxConvection.calculate_nondimensional_rms_velocity: vx = vy = v everywhere gives
    sqrt(2) v H / kappa on any grid."""
    syn = eb.synthetic
    g = syn.box_convection().grid
    v = 3e-11
    vx1 = np.full((g.ynum + 1, g.xnum), v)
    vy1 = np.full((g.ynum, g.xnum + 1), v)
    kappa = 5.0 / 1250.0 / 4000.0
    got = syn.box_convection_vrms(g, vx1, vy1, 5.0, 1250.0, 4000.0)
    assert math.isclose(got, math.sqrt(2.0) * v * (g.ymax - g.ymin) / kappa, rel_tol=1e-12)


def test_benchmark_models_follow_their_configurations(eb):
    """Geometry and material layout of the synthetic benchmark models."""
    syn = eb.synthetic
    slab = syn.elastic_slab()
    x, y, mid = slab.markers["x"], slab.markers["y"], slab.markers["matid"]
    inside = (0.2 < y / 1e6) & (y / 1e6 < 0.8) & (x / 1e6 < 0.8)
    assert np.all(np.isin(mid[inside], (4, 5))) and np.all(np.isin(mid[~inside], (2, 3)))
    box = syn.box_convection().grid
    assert box.xnum == box.ynum == 51 and box.ystp_b.min() > 5e3 and math.isclose(box.ystp_b[20], 30e3)
    rot = syn.solid_body_rotation()
    hot = rot.markers["tk"] == 1500.0
    assert np.all((0.4 <= rot.markers["x"][hot] / 50e3) & (rot.markers["x"][hot] / 50e3 <= 0.6))
    assert rot.grids["vx1"].shape == (52, 51) and rot.grids["vy1"].shape == (51, 52)


def test_pressure_grid_value_reproduces_a_linear_field(eb):
    """GridToMarker.get_marker_value_from_pressure_grid_without_mapping_input: bilinear weights on
    the cell-centre (pressure) nodes, with the index clamped to the interior cells and the
    distance left unclamped, so a linear field comes back exactly everywhere in the box, edges
    included."""
    syn = eb.synthetic
    g = syn.staggered_grid(np.linspace(0.0, 40e3, 41), np.linspace(0.0, 12e3, 13))
    xc = 0.5 * (g.gridx_b[1:] + g.gridx_b[:-1])
    yc = 0.5 * (g.gridy_b[1:] + g.gridy_b[:-1])
    f = 3.0 + 2e-4 * xc[None, :] - 5e-4 * yc[:, None]
    rng = np.random.default_rng(3)
    for x, y in zip(rng.uniform(0.0, 40e3, 200), rng.uniform(0.0, 12e3, 200)):
        assert math.isclose(syn.pressure_grid_value(g, f, x, y), 3.0 + 2e-4 * x - 5e-4 * y, rel_tol=1e-12)
    assert math.isclose(syn.pressure_grid_value(g, f, 0.0, 12e3), 3.0 - 6.0, rel_tol=1e-12)


def test_kaus10_dip_measurement_recovers_a_planted_shear_zone(eb):
    """PlasticityBenchmarkK10: strain-rate bands rising from the notch's top corners at a given
    dip are measured back at that dip to within the sampling (ynum x 10 points over 9.6 km), and
    the target is (Coulomb + Arthur) / 2 = 56.25 degrees for phi = 30, psi = 0."""
    syn = eb.synthetic
    model = syn.plasticity_benchmark_kaus10()
    g, p = model.grid, model.params
    xc = 0.5 * (g.gridx_b[1:] + g.gridx_b[:-1])
    yc = 0.5 * (g.gridy_b[1:] + g.gridy_b[:-1])
    X, Y = np.meshgrid(xc, yc)
    top = g.ymax - p["w_seed"] / 2.0
    xl, xr = p["x_seed"] - p["w_seed"] / 2.0, p["x_seed"] + p["w_seed"] / 2.0
    for dip in (45.0, 52.5, 60.0):
        t = math.tan(math.radians(dip))
        dl = np.abs((Y - top) + t * (xl - X))
        dr = np.abs((Y - top) + t * (X - xr))
        eii = 1e-15 + 1e-13 * np.exp(-np.minimum(dl, dr) ** 2 / (2.0 * 150.0 ** 2))
        r = syn.kaus10_fault_dip(g, eii, p)
        assert r["target"] == 56.25
        # each end of a stick lies on the pressure-node row nearest the band (rows 120 m apart)
        for (x1, y1), (x2, y2) in (r["sticks"]["left"], r["sticks"]["right"]):
            for x, y in ((x1, y1), (x2, y2)):
                centre = top - t * min(abs(x - xl), abs(x - xr))
                assert abs(y - centre) <= 60.0 + 10.0, (dip, x, y, centre)
        assert abs(r["theta_left"] - dip) < 2.0 and abs(r["theta_right"] - dip) < 2.0, (dip, r)


def test_kaus10_model_follows_its_configuration(eb):
    """models/plasticity_benchmark_kaus10: 400 x 100 cells of 3 x 3 markers; sticky air above
    2 km; the seven-layer ids 3-8 below; the 800 x 400 m notch (id 9) at the bottom centre;
    the sides at -/+ 2e-11 m/s, the top letting in 1.2e-11 m/s, free slip at the bottom."""
    model = eb.synthetic.plasticity_benchmark_kaus10()
    mk, g = model.markers, model.grid
    assert model.marknum == 400 * 100 * 9
    air = mk["matid"] == 1
    assert np.all(mk["y"][air] <= 2000.0) and np.all(mk["y"][~air] > 2000.0)
    notch = mk["matid"] == 9
    assert notch.sum() == 24 * 10
    assert mk["x"][notch].min() > 19600.0 and mk["x"][notch].max() < 20400.0 and mk["y"][notch].min() > 11600.0
    assert set(np.unique(mk["matid"])) == {1, 3, 4, 5, 6, 7, 8, 9}
    gr = model.grids
    assert np.allclose(gr["bleftx"][:, 0], -2e-11, rtol=1e-15) and np.allclose(gr["brightx"][:, 0], 2e-11, rtol=1e-15)
    assert np.allclose(gr["btopy"][:, 0], 1.2e-11, rtol=1e-15) and np.all(gr["btopy"][:, 1] == 0.0)
    assert np.all(gr["bbottomy"] == 0.0) and np.all(gr["bbottomx"][:, 1] == 1.0)
    assert model.params["itype_global"] == 1 and model.params["yield_stress_min"] == 2e7
    assert math.isclose(model.mats.mat_rho[2], 2700.0 * (1.0 - 3e-5 * (273.0 - 298.15)), rel_tol=1e-15)


def test_kaus10_oracle_record_is_consistent(eb):
    """tests/golden/kaus10_oracle_9steps.npz (written by make_kaus10_oracle.py): the dip measured
    from the recorded line samples of step 9 is the recorded dip, and that dip meets the
    reference's criterion (within 4 % of 56.25 degrees)."""
    import pathlib
    g = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "kaus10_oracle_9steps.npz")
    model = eb.synthetic.plasticity_benchmark_kaus10()
    xs, ys = eb.synthetic.kaus10_measurement_lines(model.grid, model.params)
    lines = g["lines"]
    assert lines.shape == (4, len(ys))
    yl = [ys[int(np.argmax(v))] for v in lines]
    th_l = math.degrees(math.atan(abs(yl[1] - yl[0]) / abs(xs[1] - xs[0])))
    th_r = math.degrees(math.atan(abs(yl[3] - yl[2]) / abs(xs[3] - xs[2])))
    assert np.allclose(g["dips"][-1], [th_l, th_r, (th_l + th_r) / 2.0], rtol=1e-14)
    assert abs(g["dips"][-1][2] - 56.25) / 56.25 <= 0.04
    assert len(g["iters"]) == 9 and all(len(g[f"nnode_{s}"]) == n for s, n in enumerate(g["iters"], start=1))
