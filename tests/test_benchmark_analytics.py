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
