"""GPU parity: every hot-path entry point, called through the C-ABI, against the CPU oracle.

Contract (tolerances written here, applied entry by entry):
  * inside flags and marker->cell indices (marker_xn/yn, marker_xn_vy/yn_vy): bit-exact;
  * floating-point fields: |gpu - oracle| <= RTOL * S with RTOL = 1e-6, where S is
    the magnitude of what the entry is made of:
      - marker->grid averages: the same step run by the oracle on absolute values
        (|w1 s1| + |w2 s2| + ... over w1 + w2 + ...), the classical bound of a
        weighted sum; for a positive field S is the value itself (plain 1e-6
        relative);
      - grid->marker gathers: the largest |grid value| among the nodes the
        marker interpolates from (a 5x5-node neighbourhood of its cell, which
        covers the staggered and the RK4 intermediate cells), the usual error
        scale of an interpolant;
      - marker stresses: the stress magnitude, plus the local grid stress
        magnitude where a step mixes grid stress into the marker;
  * zero weight sums (empty nodes, which select the backup value) identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def close(got, want, name, scale=None, rtol=RTOL):
    """|got - want| <= rtol * scale entrywise; scale defaults to |want| (plain relative error)."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape, name
    s = np.abs(want) if scale is None else np.maximum(np.abs(np.asarray(scale, dtype=np.float64)), np.abs(want))
    tol = rtol * s
    bad = ~(np.abs(got - want) <= tol)
    if bad.any():
        i = np.flatnonzero(bad.ravel())[0]
        rel = np.max(np.abs(got - want) / np.maximum(s, 1e-300))
        raise AssertionError(f"{name}: {bad.sum()} of {want.size} entries out of tolerance; worst rel {rel:.3g}; "
                             f"first at {i}: gpu {got.ravel()[i]!r} oracle {want.ravel()[i]!r} scale {s.ravel()[i]!r}")


SIGNED_MARKER_FIELDS = ("sxx", "sxy", "exx", "exy", "subgrid_dt")
SIGNED_GRID_FIELDS = ("sxx1", "sxy1", "sxx0", "sxy0", "exx", "exy", "sxx2", "sxy2", "dsxx", "dsxy", "dsxxn", "dsxyn",
                      "dtk1", "dtkn", "vx1", "vy1", "esp", "pr1")


def local_max(grid_values, ref):
    """Largest |value| of a grid field in the 5x5-node neighbourhood of each marker's basic cell."""
    from scipy.ndimage import maximum_filter
    mx = maximum_filter(np.abs(np.asarray(grid_values)), size=5, mode="nearest")
    yn = np.clip(ref.mk["yn"].astype(np.int64) - 1, 0, mx.shape[0] - 1)
    xn = np.clip(ref.mk["xn"].astype(np.int64) - 1, 0, mx.shape[1] - 1)
    out = mx[yn, xn]
    out[ref.mk["inside"] != 1] = 0.0
    return out


def abs_model(model):
    """The same model with every signed marker and grid field replaced by its absolute value:
    the oracle run on it gives the magnitude S of each weighted sum."""
    m = model.copy()
    for k in SIGNED_MARKER_FIELDS:
        if k in m.markers:
            m.markers[k] = np.abs(m.markers[k])
    for k in SIGNED_GRID_FIELDS:
        if k in m.grids:
            m.grids[k] = np.asfortranarray(np.abs(m.grids[k]))
    return m


@pytest.fixture(scope="module", params=["sinking_block", "rift_small", "rift_2p5M"])
def pair(request, eb, oracle):
    eb.build()
    model = eb.synthetic.config(request.param)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    ref = oracle.OracleMIC(model)
    yield model, mic, ref
    mic.close()


def fresh(eb, oracle, model):
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    return mic, oracle.OracleMIC(model)


def locate_both(mic, ref):
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()


def test_inside_flags_and_cell_indices_bit_exact(eb, oracle, pair):
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    inside = ref.mk["inside"]
    assert np.array_equal(mic.download_marker("inside"), inside)
    sel = inside == 1
    for f in ("xn", "yn", "xn_vy", "yn_vy"):
        assert np.array_equal(mic.download_marker(f)[sel], ref.mk[f][sel]), f
    mic.close()


def test_cell_indices_on_grid_lines_and_edges(eb, oracle):
    """Markers exactly on grid lines, on staggered lines and on the domain edges."""
    model = eb.synthetic.config("sinking_block")
    g = model.grid
    rng = np.random.default_rng(5)
    xs = np.concatenate([g.gridx_b, g.gridx_vy[1:-1], np.nextafter(g.gridx_b, -np.inf)[1:],
                         np.nextafter(g.gridx_b, np.inf)[:-1]])
    ys = np.concatenate([g.gridy_b, g.gridy_vx[1:-1], np.nextafter(g.gridy_b, np.inf)[:-1]])
    n = model.marknum
    x = rng.choice(xs, n)
    y = rng.choice(ys, n)
    x[:4] = [g.xmin, g.xmax, g.xmin - 1.0, g.xmax + 1e-9]
    y[:4] = [g.ymin, g.ymax, g.ymax, g.ymin]
    model.markers["x"], model.markers["y"] = x, y
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    assert np.array_equal(mic.download_marker("inside"), ref.mk["inside"])
    sel = ref.mk["inside"] == 1
    for f in ("xn", "yn", "xn_vy", "yn_vy"):
        assert np.array_equal(mic.download_marker(f)[sel], ref.mk[f][sel]), f
    # exclusive quadrants decided exactly: the viscosity scatter is sensitive to them
    mic.interpolate_marker_stokes_parameters_to_grid()
    ref.interpolate_marker_stokes_parameters_to_grid()
    for f in ("wtetas", "etas1"):
        close(mic.download_grid(f), ref.gr[f], f)
    mic.close()


def test_denominators(eb, oracle, pair):
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    for f in ("wtnodes", "wtetas", "wtetan", "wtnodes_vy"):
        got = mic.download_grid(f)
        assert np.array_equal(got == 0, ref.gr[f] == 0), f
        close(got, ref.gr[f], f)
    mic.close()


STOKES_GRIDS = ["rho1", "rho0", "rho1_vy", "rho0_vy", "etas1", "etas0", "eta_flow", "eta_flow0", "mus1", "mus0",
                "sxy1", "sxy0", "plastics", "cohesion_grid", "fric_degrees_grid", "etan1", "etan0", "mun1", "mun0",
                "sxx1", "sxx0", "plasticn", "dilatation_grid", "extractable_meltfrac_grid"]


def oracle_pair(oracle, model, steps):
    """Run the oracle's steps on the model and on its absolute-value twin."""
    ref, refa = oracle.OracleMIC(model), oracle.OracleMIC(abs_model(model))
    for o in (ref, refa):
        for st in steps:
            getattr(o, st)()
    return ref, refa


def stress_scale(ref):
    return np.hypot(ref.mk["sxx"], ref.mk["sxy"])


def subgrid_change_scale(oracle, model, steps_before):
    """Error scales of the averaged subgrid stress changes dsxyn, dsxxn.  A marker's change is
    (gathered grid stress - marker stress) x (1 - exp(-...)): where the two stresses nearly cancel,
    its error is relative to their magnitudes, not to the change.  So the scale of each weighted
    average is the same average of |marker stress before| + |marker stress after| (which bounds
    both terms), from an oracle run of the steps before update_subgrid_stress and of that step."""
    o = oracle.OracleMIC(model)
    for st in steps_before:
        getattr(o, st)()
    sxy0, sxx0 = o.mk["sxy"].copy(), o.mk["sxx"].copy()
    o.update_subgrid_stress()
    return o.excl_cent_average(np.abs(o.mk["sxy"]) + np.abs(sxy0), np.abs(o.mk["sxx"]) + np.abs(sxx0))


def test_scatter_stokes(eb, oracle, pair):
    model, _, _ = pair
    mic = fresh(eb, oracle, model)[0]
    steps = ["get_marker_inside_flags", "initialize_bilinear_interpolation",
             "interpolate_marker_stokes_parameters_to_grid"]
    for st in steps:
        getattr(mic, st)()
    ref, refa = oracle_pair(oracle, model, steps)
    for f in STOKES_GRIDS:
        close(mic.download_grid(f), ref.gr[f], f, scale=refa.gr[f])
    mic.close()


def test_scatter_heat(eb, oracle, pair):
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    mic.interpolate_marker_heat_parameters_to_grid()
    ref.interpolate_marker_heat_parameters_to_grid()
    for f in ("tk1", "tk0", "kt1", "kt0", "rhocp1", "hr1", "ha1"):
        close(mic.download_grid(f), ref.gr[f], f)
    mic.close()


def test_viscosity_rescatter(eb, oracle, pair):
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    eta = model.markers["eta"] * np.exp(np.sin(np.arange(model.marknum)))
    mic.upload_marker("eta", eta)
    ref.mk["eta"][:] = eta
    for o in (mic, ref):
        o.backup_and_clear_viscosity_transport_arrays()
        o.interpolate_viscosity_to_transport_arrays()
    for f in ("etas1", "etas0", "etan1", "etan0"):
        close(mic.download_grid(f), ref.gr[f], f)
    mic.close()


def test_gathers(eb, oracle, pair):
    model, _, _ = pair
    mic = fresh(eb, oracle, model)[0]
    steps = ["get_marker_inside_flags", "initialize_bilinear_interpolation", "post_stokes_marker_gathers"]
    for st in steps:
        getattr(mic, st)()
    ref, refa = oracle_pair(oracle, model, steps)
    for f in ("exx", "exy", "pr"):
        close(mic.download_marker(f), ref.mk[f], f, scale=local_max(model.grids[f if f != "pr" else "pr1"], ref))
    # the strain-rate ratio divides stress-based by velocity-based invariants built from
    # gathers: its error scale is the ratio of the local magnitudes
    # and the stress-based invariant is itself made of gathered stresses: the local stress
    # magnitudes over the marker's viscosity (and dt*mu) set its error scale
    e_loc = np.hypot(local_max(model.grids["exx"], ref), local_max(model.grids["exy"], ref))
    e_here = np.maximum(np.hypot(ref.mk["exx"], ref.mk["exy"]), 1e-300)
    mu = model.mats.mat_mu[ref.mk["matid"].astype(np.int64) - 1]
    tf = 1.0 / (model.params["timestep"] * mu)
    eta = ref.mk["eta"]
    num_loc = 0.5 * np.hypot(local_max(model.grids["sxx2"], ref) / eta + local_max(model.grids["dsxx"], ref) * tf,
                             local_max(model.grids["sxy2"], ref) / eta + local_max(model.grids["dsxy"], ref) * tf)
    close(mic.download_marker("sr_ratio"), ref.mk["sr_ratio"], "sr_ratio",
          scale=ref.mk["sr_ratio"] * e_loc / e_here + num_loc / e_here)
    mic.upload_grid("tk1", model.grids["tk2"])
    ref.gr["tk1"][:] = model.grids["tk2"]
    mic.interpolate_temperature_to_markers()
    ref.interpolate_temperature_to_markers()
    close(mic.download_marker("tk"), ref.mk["tk"], "tk")
    mic.close()


def test_subgrid_stress_and_correction(eb, oracle, pair):
    model, _, _ = pair
    mic = fresh(eb, oracle, model)[0]
    steps = ["get_marker_inside_flags", "initialize_bilinear_interpolation", "update_subgrid_stress"]
    for st in steps:
        getattr(mic, st)()
    ref, refa = oracle_pair(oracle, model, steps)
    # the relaxation moves the marker stress toward the gathered grid stress: the terms are the
    # stress before, the stress after and the local grid stress
    s_loc = (stress_scale(ref) + np.hypot(model.markers["sxx"], model.markers["sxy"]) +
             np.hypot(local_max(model.grids["sxx1"], ref), local_max(model.grids["sxy1"], ref)))
    for f in ("sxx", "sxy"):
        close(mic.download_marker(f), ref.mk[f], f, scale=s_loc)
    sc = dict(zip(("dsxyn", "dsxxn"), subgrid_change_scale(oracle, model, steps[:-1])))
    for f in ("dsxyn", "dsxxn"):
        close(mic.download_grid(f), ref.gr[f], f, scale=sc[f])
    for f, fn in (("dsxy", "dsxyn"), ("dsxx", "dsxxn")):
        close(mic.download_grid(f), ref.gr[f], f, scale=np.abs(model.grids[f]) + sc[fn])
    for f in ("wtetas", "wtetan"):
        close(mic.download_grid(f), ref.gr[f], f)
    mic.apply_marker_stress_correction()
    ref.apply_marker_stress_correction()
    s_loc = s_loc + np.hypot(local_max(ref.gr["dsxx"], ref), local_max(ref.gr["dsxy"], ref))
    for f in ("sxx", "sxy"):
        close(mic.download_marker(f), ref.mk[f], f, scale=s_loc)
    mic.close()


def test_subgrid_heat_and_remaining_dt(eb, oracle, pair):
    """The subgrid temperature change is a correction to the temperature: its
    tolerance is relative to the temperature it corrects."""
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    for o in (mic, ref):
        o.interpolate_marker_heat_parameters_to_grid()
        o.subgrid_heat_diffusion_update()
    close(mic.download_marker("subgrid_dt"), ref.mk["subgrid_dt"], "subgrid_dt", scale=ref.mk["tk"])
    close(mic.download_marker("tk"), ref.mk["tk"], "tk")
    close(mic.download_grid("wtnodes"), ref.gr["wtnodes"], "wtnodes")
    for f in ("dtkn", "dtk1"):
        close(mic.download_grid(f), ref.gr[f], f, scale=ref.gr["tk1"])
    for o in (mic, ref):
        o.add_remaining_grid_change_to_marker_temperature()
    close(mic.download_marker("tk"), ref.mk["tk"], "tk")
    mic.close()


def test_advection_rk4(eb, oracle, pair):
    model, _, _ = pair
    mic = fresh(eb, oracle, model)[0]
    steps = ["get_marker_inside_flags", "initialize_bilinear_interpolation", "advect_markers_and_rotate_stress"]
    for st in steps:
        getattr(mic, st)()
    ref, refa = oracle_pair(oracle, model, steps)
    vscale = {"vx": local_max(model.grids["vx1"], ref), "vy": local_max(model.grids["vy1"], ref),
              "spin": local_max(model.grids["esp"], ref)}
    for f in ("vx", "vy", "spin"):
        close(mic.download_marker(f), ref.mk[f], f, scale=vscale[f])
    # positions: the displacement dt*v within RTOL of dt times the local velocity magnitude
    dt = model.params["timestep"]
    for f, v in (("x", "vx"), ("y", "vy")):
        f0 = model.markers[f]
        close(mic.download_marker(f) - f0, ref.mk[f] - f0, f + " displacement", scale=dt * vscale[v])
    for f in ("sxx", "sxy"):
        close(mic.download_marker(f), ref.mk[f], f, scale=stress_scale(ref))
    mic.close()


def test_strain_update(eb, oracle, pair):
    model, _, _ = pair
    mic, ref = fresh(eb, oracle, model)
    for o in (mic, ref):
        o.get_marker_inside_flags()
        o.update_marker_strain()
    for f in ("gii", "strain_plastic", "strain_rate_plastic"):
        close(mic.download_marker(f), ref.mk[f], f)
    mic.close()


def test_rheology(eb, oracle):
    model = eb.synthetic.config("rift_small")
    mic, ref = fresh(eb, oracle, model)
    for o in (mic, ref):
        o.get_marker_inside_flags()
        o.update_marker_rheology()
    for f in ("cohesion", "fric", "preexp"):
        close(mic.download_marker(f), ref.mk[f], f, rtol=1e-12)
    close(mic.download_marker("eta_flow"), ref.mk["eta_flow"], "eta_flow")
    for o in (mic, ref):
        o.update_marker_viscoplastic_viscosity(use_marker_plasticity=True)
    close(mic.download_marker("eta"), ref.mk["eta"], "eta")
    for f in ("sxx", "sxy"):
        close(mic.download_marker(f), ref.mk[f], f, scale=stress_scale(ref))
    assert np.array_equal(mic.download_marker("pfailure"), ref.mk["pfailure"])
    mic.close()


@pytest.mark.parametrize("name", ["rift_small", "rift_2p5M"])
def test_flow_viscosity_bisection_follows_the_reference(eb, oracle, name):
    """CompositeViscosity.update_marker_flow_viscosity!: the GPU decides each bisection step from
    the root of the decision function and evaluates the creep law only at the last midpoint; the
    decisions, the step count and that midpoint must be the reference's, so eta_flow agrees with
    the oracle's plain FP64 bisection to 1e-11: the last bits of exp and pow differ between CUDA and
    the host's C library (up to ~1.5e-12 here), while one different decision or step would move it
    by at least the final half-interval over the stress, 1e-9 or more.  Checked on the markers as
    generated and after they took the strain rates and pressures of a real Stokes solution."""
    model = eb.synthetic.config(name)
    for stage in ("initial", "after one time step"):
        mic, ref = fresh(eb, oracle, model)
        for o in (mic, ref):
            o.get_marker_inside_flags()
            o.update_marker_rheology()
        sel = ref.mk["inside"] == 1
        got, want = mic.download_marker("eta_flow")[sel], ref.mk["eta_flow"][sel]
        rel = np.abs(got - want) / want
        print(f"{name} {stage}: worst relative eta_flow error {rel.max():.3g}; oracle bisection steps "
              f"{np.bincount(ref.iters[sel])}")
        assert np.all(rel <= 1e-11), (stage, int(np.sum(rel > 1e-11)), rel.max())
        assert np.array_equal(mic.download_marker("preexp"), ref.mk["preexp"])
        if stage == "initial":
            mic.time_step(3, 1e-3, rtol=1e-10)
            model = model.copy()
            for f in ("x", "y", "sxx", "sxy", "exx", "exy", "pr", "sr_ratio", "gii", "strain_plastic", "tk", "eta"):
                model.markers[f] = mic.download_marker(f)
        mic.close()


def test_full_marker_cycle(eb, oracle, pair):
    model, _, _ = pair
    mic = fresh(eb, oracle, model)[0]
    mic.marker_cycle()
    ref, refa = oracle_pair(oracle, model, ["marker_cycle"])
    loc = {f: local_max(model.grids[g], ref) for f, g in (("vx", "vx1"), ("vy", "vy1"), ("exx", "exx"),
                                                           ("exy", "exy"), ("pr", "pr1"))}
    for f in ("vx", "vy", "exx", "exy", "pr"):
        close(mic.download_marker(f), ref.mk[f], f, scale=loc[f])
    s_loc = stress_scale(ref) + np.hypot(model.markers["sxx"], model.markers["sxy"]) + \
        np.hypot(local_max(ref.gr["sxx1"], ref), local_max(ref.gr["sxy1"], ref)) + \
        np.hypot(local_max(ref.gr["dsxx"], ref), local_max(ref.gr["dsxy"], ref))
    for f in ("sxx", "sxy"):
        close(mic.download_marker(f), ref.mk[f], f, scale=s_loc)
    for f in ("tk", "gii"):
        close(mic.download_marker(f), ref.mk[f], f)
    dt = model.params["timestep"]
    for f in ("x", "y"):
        f0 = model.markers[f]
        close(mic.download_marker(f) - f0, ref.mk[f] - f0, f + " displacement", scale=dt * loc["v" + f])
    for f in ("rho1", "etas1", "etan1", "tk1"):
        close(mic.download_grid(f), ref.gr[f], f)
    close(mic.download_grid("dtk1"), ref.gr["dtk1"], "dtk1", scale=ref.gr["tk1"])
    # dsxy = input change - averaged relaxed marker stress change: its terms are the input and
    # the marker stress changes being averaged
    sc_xy, _ = subgrid_change_scale(oracle, model, ["get_marker_inside_flags", "initialize_bilinear_interpolation",
                                                    "interpolate_marker_heat_parameters_to_grid",
                                                    "interpolate_marker_stokes_parameters_to_grid",
                                                    "post_stokes_marker_gathers"])
    # the averaged change is made of gathered grid stresses (FP32 gathers: the local grid magnitude)
    from scipy.ndimage import maximum_filter
    g_loc = maximum_filter(np.abs(ref.gr["sxy1"]), size=5, mode="nearest")
    close(mic.download_grid("dsxy"), ref.gr["dsxy"], "dsxy", scale=np.abs(model.grids["dsxy"]) + sc_xy + g_loc)
    mic.close()


def test_deterministic(eb, oracle):
    model = eb.synthetic.config("rift_small")
    outs = []
    for _ in range(2):
        mic = eb.MarkerInCell(0)
        mic.load_model(model)
        mic.marker_cycle()
        outs.append({f: mic.download_marker(f) for f in ("x", "y", "sxx", "tk")} |
                    {f: mic.download_grid(f) for f in ("rho1", "etas1", "tk1", "dsxyn")})
        mic.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_empty_and_all_outside(eb, oracle):
    model = eb.synthetic.config("sinking_block")
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.upload_marker("x", np.full(model.marknum, -1e9))  # every marker outside the domain
    mic.marker_cycle()
    assert np.all(mic.download_marker("inside") == -1)
    rho_before = model.grids["rho1"]
    np.testing.assert_array_equal(mic.download_grid("rho1"), rho_before)  # empty nodes keep the backup
    mic.resize_markers(0)
    mic.marker_cycle()
    mic.close()


def test_errors_are_reported_not_raised_on_device(eb):
    model = eb.synthetic.config("sinking_block")
    mic = eb.MarkerInCell(0)
    mic.set_grid(model.grid)
    mic.set_params(model.params)
    with pytest.raises(eb.EarthBoxGPUError) as e:
        mic.interpolate_marker_stokes_parameters_to_grid()  # no materials, not located
    assert e.value.code in (3, 5)
    mic.set_materials(model.mats)
    mic.resize_markers(model.marknum)
    bad = model.markers["matid"].copy()
    bad[7] = 99
    with pytest.raises(eb.EarthBoxGPUError):
        mic.upload_marker("matid", bad)
    mic.close()


def test_grid_viscoplastic_viscosity_to_markers(eb, oracle):
    """GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity!: yielding cells take the
    plastic-flag-weighted harmonic average of etas1 when it is below the flow viscosity (eta
    within 1e-6, the failure flags exact); cells without a yielding corner keep eta_flow."""
    model = eb.synthetic.config("rift_small")
    Y, X = model.grid.ynum, model.grid.xnum
    rng = np.random.default_rng(11)
    model.grids["plastic_yield"] = np.asfortranarray((rng.random((Y, X)) < 0.25).astype(float))
    model.grids["etas1"] = np.asfortranarray(10.0 ** rng.uniform(19.0, 24.0, (Y, X)))
    mic, ref = fresh(eb, oracle, model)
    locate_both(mic, ref)
    mic.calc_marker_viscoplastic_viscosity()
    ref.calc_marker_viscoplastic_viscosity()
    sel = ref.mk["inside"] == 1
    close(mic.download_marker("eta")[sel], ref.mk["eta"][sel], "eta")
    pf = mic.download_marker("pfailure")
    assert np.array_equal(pf, ref.mk["pfailure"])
    newly = (ref.mk["pfailure"] == 1) & (model.markers["pfailure"] == 0)
    assert newly.sum() > 100, "the case must make markers fail"
    keep = sel & (ref.mk["eta"] == ref.mk["eta_flow"])
    assert keep.sum() > 100
    mic.close()


def topo_model(eb):
    """rift_small with the topography model on: two extra materials stand for the sticky air
    (1.2 kg/m^3) and sticky water (1025 kg/m^3) of FlattenDensity, and sea level sits 7 km above
    the rock surface, so that both the air and the water branch replace node densities."""
    model = eb.synthetic.config("rift_small")
    m = model.mats
    pad = lambda a, v: np.concatenate([a, np.array(v, dtype=a.dtype)])
    mats = eb.synthetic.Materials(
        mat_mu=pad(m.mat_mu, [1e20, 1e20]), mat_hr=pad(m.mat_hr, [0.0, 0.0]),
        mat_flow_type=pad(m.mat_flow_type, [0, 0]),
        mat_flow=np.asfortranarray(np.vstack([m.mat_flow, np.zeros((2, 12))])),
        mat_plastic=np.asfortranarray(np.vstack([m.mat_plastic, np.zeros((2, 6))])),
        mat_rho=pad(m.mat_rho, [1.2, 1025.0]))
    mats.mat_flow[4:, 0] = 1e18
    model.mats = mats
    model.params.update(iuse_topo=1, y_sealevel=3e3, matid_sticky_air_rho=5, matid_sticky_water_rho=6)
    return model


def test_sticky_layer_density_flattening(eb, oracle):
    """FlattenDensity.flatten_staggered_grid_density_in_sticky_air_layer! (iuse_topo = 1): rho1 and
    rho1_vy of nodes at or below 1100 kg/m^3 become the sticky-air density above sea level and
    the sticky-water density below it (rho1 only where hr1 == 0)."""
    model = topo_model(eb)
    mic = fresh(eb, oracle, model)[0]
    steps = ["get_marker_inside_flags", "initialize_bilinear_interpolation",
             "interpolate_marker_heat_parameters_to_grid", "interpolate_marker_stokes_parameters_to_grid"]
    for st in steps:
        getattr(mic, st)()
    ref, refa = oracle_pair(oracle, model, steps)
    for f in ("rho1", "rho1_vy"):
        got = mic.download_grid(f)
        close(got, ref.gr[f], f, scale=refa.gr[f])
        assert np.sum(ref.gr[f] == 1.2) >= 50 and np.sum(ref.gr[f] == 1025.0) >= 50, f
        assert np.array_equal(got == 1.2, ref.gr[f] == 1.2) and np.array_equal(got == 1025.0, ref.gr[f] == 1025.0), f
    mic.close()


@pytest.mark.parametrize("option", [0, 4, 5, -1])
def test_other_flow_laws_match_oracle(eb, oracle, option):
    """The flow laws the model's largest mat_flow_type selects besides composite creep
    (FlowViscosity.jl:21-44): isoviscous (preexp = viscosity), the temperature-dependent Couette
    law (mat_flow columns 13-14), the Blankenbach law (columns 15-17) and the x-dependent channel
    law, through the rheology entry point and the fused pass, against the oracle."""
    import copy
    model = eb.synthetic.config("rift_small")
    mats = copy.deepcopy(model.mats)
    n = len(mats.mat_mu)
    flow = np.zeros((n, 17))
    flow[:, :12] = mats.mat_flow
    flow[:, 0] = 1e21 * (1.0 + np.arange(n))
    flow[:, 12] = 1e15 * (1.0 + np.arange(n))
    flow[:, 13] = 150.0
    flow[:, 14] = 1e23
    flow[:, 15] = np.log(1000.0)
    flow[:, 16] = 0.5
    mats.mat_flow = np.asfortranarray(flow)
    mats.mat_flow_type = np.full(n, option, np.int64)
    model.mats = mats
    model.params = dict(model.params, temperature_bottom=1603.15, temperature_left=1000.15)
    mic, ref = fresh(eb, oracle, model)
    for o in (mic, ref):
        o.get_marker_inside_flags()
        o.update_marker_rheology()
    close(mic.download_marker("preexp"), ref.mk["preexp"], "preexp", rtol=0.0)
    close(mic.download_marker("eta_flow"), ref.mk["eta_flow"], "eta_flow", rtol=1e-12)
    fused = eb.MarkerInCell(0)
    fused.load_model(model)
    fused.get_marker_inside_flags()
    fused.update_marker_rheology_and_viscoplastic_viscosity(True)
    close(fused.download_marker("eta_flow"), mic.download_marker("eta_flow"), "fused eta_flow", rtol=0.0)
    for m in (mic, fused):
        m.close()
