"""GPU step-boundary updates against the oracle, through the C-ABI: rock properties of the
markers for every density x rhocp x conductivity model (bit-identical where the formula
has no exp; within 2e-16 relative otherwise), the sediment porosity correction, and the
displacement-limited time step in both modes (bit-identical)."""
import numpy as np
import pytest

from boundary_cases import porosity_fields, rock_tables, sediment

pytestmark = pytest.mark.gpu


def setup(eb, name="rift_small", nmat=4):
    model = eb.synthetic.config(name)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    M = model.marknum
    mk = {k: mic.download_marker(k) for k in ("x", "y", "matid", "pr", "tk", "rho", "rhocp", "kt", "ha", "inside")}
    por = porosity_fields(M)
    for k, v in por.items():
        mic.upload_marker(k, v)
    mk.update(por)
    tabs = rock_tables(nmat)
    mic.set_rock_tables(*tabs)
    return model, mic, mk, tabs


@pytest.mark.parametrize("dm,cm,km", [(d, c, k) for d in range(3) for c in range(2) for k in range(6)])
def test_rock_properties_match_oracle(eb, dm, cm, km):
    from oracle import boundary as B
    model, mic, mk, tabs = setup(eb)
    mic.update_marker_rock_properties(dm, cm, km, 0, 1200.0)
    want = B.rock_properties(mk, *tabs, dm, cm, km, model.params["temperature_top"], 1200.0)
    for n in ("rho", "rhocp", "kt", "ha"):
        got = mic.download_marker(n)
        if km == 0 and n == "kt":
            np.testing.assert_allclose(got, want[n], rtol=4e-16, atol=0, err_msg=n)
        else:
            assert np.array_equal(got, want[n]), n
    mic.close()


def test_rock_properties_porosity_match_oracle(eb):
    from oracle import boundary as B
    model, mic, mk, tabs = setup(eb)
    sed = sediment(model.grid)
    mic.set_sediment_porosity(sed["matids"], sed["topo_x"], sed["topo_y"], sed["conductivity_water"],
                              sed["density_water"], sed["heat_capacity_water"])
    mic.update_marker_rock_properties(1, 1, 2, 1, 1200.0)
    want = B.rock_properties(mk, *tabs, 1, 1, 2, model.params["temperature_top"], 1200.0, iuse_por=1, sed=sed)
    for n in ("rho", "rhocp", "kt", "ha"):
        np.testing.assert_allclose(mic.download_marker(n), want[n], rtol=1e-15, atol=0, err_msg=n)
    mic.close()


def test_rock_properties_rejects_unknown_material(eb):
    model, mic, mk, tabs = setup(eb, nmat=4)
    mic.set_rock_tables(tabs[0][:2], tabs[1][:2], tabs[2][:2])  # fewer materials than the markers use
    with pytest.raises(RuntimeError):
        mic.update_marker_rock_properties()
    mic.close()


@pytest.mark.parametrize("local", [0, 1])
def test_timestep_matches_oracle(eb, local):
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    vx, vy = model.grids["vx1"], model.grids["vy1"]
    for dt_old in (1e9, 1e13):
        got, upd = mic.update_model_time_step_using_displacement_limit(dt_old, 0.5, local)
        want = B.timestep_displacement_limit(model.grid, vx, vy, 0.5, local, dt_old)
        assert got == want and upd == (want != dt_old)
    mic.close()


@pytest.mark.parametrize("water,random_fric", [(1, 0), (2, 1)])
def test_recycle_markers_match_oracle(eb, water, random_fric):
    """Markers pushed out through all four sides re-enter bit-identically to the oracle:
    positions, reset properties, the recycled list in marker order and the counts."""
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    g = model.grid
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    M = model.marknum
    rng = np.random.default_rng(17)
    x, y = mic.download_marker("x"), mic.download_marker("y")
    out = rng.random(M) < 0.04
    side = rng.integers(0, 4, M)
    x = np.where(out & (side == 0), g.xmin - rng.uniform(1.0, 5e3, M), x)
    x = np.where(out & (side == 1), g.xmax + rng.uniform(1.0, 5e3, M), x)
    y = np.where(out & (side == 2), g.ymin - rng.uniform(1.0, 5e3, M), y)
    y = np.where(out & (side == 3), g.ymax + rng.uniform(1.0, 5e3, M), y)
    mic.upload_marker("x", x)
    mic.upload_marker("y", y)
    for k in B.RECYCLE_FIELDS[2:]:
        mic.upload_marker(k, rng.uniform(0.5, 2.0, M))
    mic.upload_marker("pfailure", rng.uniform(0, 1, M).astype(np.float32))
    mic.get_marker_inside_flags()
    mk = {k: mic.download_marker(k) for k in (*B.RECYCLE_FIELDS, "matid", "pfailure", "inside")}
    assert np.sum(mk["inside"] != 1) > 100 and np.any(mk["matid"][mk["inside"] != 1] == 1)
    vyu, vyl, tbot, seed, step = -1e-10, 2e-10, 1603.0, 2024, 9
    p = model.params
    want, widx, wfl, wnair = B.recycle_extension(mk, 1, water, 4, g.xmax, g.ymax, vyu, vyl, p["timestep"],
                                                 p["temperature_top"], tbot, g.gridy_b[-1], model.mats.mat_plastic,
                                                 random_fric, 0.1, seed, step)
    nair, nsub = mic.recycle_markers(1, water, 4, g.xmax, g.ymax, vyu, vyl, tbot, seed, step,
                                     iuse_random_fric=random_fric, delta_fric_coef=0.1)
    assert (nair, nsub) == (wnair, len(widx) - wnair)
    idx, fl = mic.recycled_markers()
    assert np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(mic.download_marker(k), want[k]), k
    # every marker is back inside
    mic.get_marker_inside_flags()
    assert np.all(mic.download_marker("inside") == 1)
    mic.close()


def test_recycle_no_bottom_inflow_and_channel_match_oracle(eb):
    """Recycling types 2 (extension without bottom inflow) and 3 (channel) against the oracle."""
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    g = model.grid
    p = model.params
    rng = np.random.default_rng(23)
    # type 2: markers pushed out through the sides and the bottom
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    M = model.marknum
    x, y = mic.download_marker("x"), mic.download_marker("y")
    out = rng.random(M) < 0.03
    x = np.where(out & (rng.random(M) < 0.5), g.xmax + rng.uniform(1.0, 3e3, M), x)
    y = np.where(out & (x <= g.xmax), g.ymax + rng.uniform(1.0, 3e3, M), y)
    mic.upload_marker("x", x)
    mic.upload_marker("y", y)
    mic.get_marker_inside_flags()
    mk = {k: mic.download_marker(k) for k in (*B.RECYCLE_FIELDS, "matid", "pfailure", "inside")}
    want, widx, wfl = B.recycle_no_bottom_inflow(mk, 1, g.xmax, -2e-10, p["timestep"], p["temperature_top"],
                                                 model.mats.mat_plastic, 77, 3)
    nair, nsub = mic.recycle_markers(1, 1, 4, g.xmax, g.ymax, -2e-10, 0.0, 1603.0, 77, 3, recycle_type=2)
    assert (nair, nsub) == (len(widx), 0) and nair > 50
    idx, fl = mic.recycled_markers()
    assert np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(mic.download_marker(k), want[k]), k
    mic.close()
    # type 3: markers below the grid wrap to the top
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    y = mic.download_marker("y")
    y = np.where(rng.random(M) < 0.05, g.ymax + rng.uniform(1.0, 2e3, M), y)
    mic.upload_marker("y", y)
    tk = mic.download_marker("tk")
    wy, wtk, widx = B.recycle_channel(y, tk, g.gridy_b[0], g.gridy_b[-1], p["temperature_top"], 1603.0)
    nair, nsub = mic.recycle_markers(1, 1, 4, g.xmax, g.ymax, 0.0, 0.0, 1603.0, 0, 0, recycle_type=3)
    assert (nair, nsub) == (0, len(widx)) and nsub > 50
    idx, _ = mic.recycled_markers()
    assert np.array_equal(idx, widx)
    assert np.array_equal(mic.download_marker("y"), wy) and np.array_equal(mic.download_marker("tk"), wtk)
    mic.close()


@pytest.mark.parametrize("asym,random_fric", [(0, 1), (1, 0)])
def test_recycle_contraction_matches_oracle(eb, asym, random_fric):
    """Recycling type 4 (ContractionViscoelastic): markers pushed out through all four sides
    re-enter at the two sides bit-identically to the oracle, subsurface ones as the seven-layer
    or strong-zone material of their new position (12 materials, friction per material)."""
    import dataclasses
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    g = model.grid
    p = model.params
    rng = np.random.default_rng(41 + asym)
    m0 = model.mats
    rows = np.arange(12) % len(m0.mat_mu)
    mp = np.asfortranarray(np.asarray(m0.mat_plastic)[rows].copy())
    mp[:, 2] = rng.uniform(0.1, 0.6, 12)
    mats = dataclasses.replace(m0, mat_mu=np.asarray(m0.mat_mu)[rows], mat_hr=np.asarray(m0.mat_hr)[rows],
                               mat_flow_type=np.asarray(m0.mat_flow_type)[rows],
                               mat_flow=np.asfortranarray(np.asarray(m0.mat_flow)[rows]), mat_plastic=mp,
                               mat_rho=np.asarray(m0.mat_rho)[rows])
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.set_materials(mats)
    M = model.marknum
    x, y = mic.download_marker("x"), mic.download_marker("y")
    out = rng.random(M) < 0.05
    side = rng.integers(0, 4, M)
    x = np.where(out & (side == 0), g.xmin - rng.uniform(1.0, 5e3, M), x)
    x = np.where(out & (side == 1), g.xmax + rng.uniform(1.0, 5e3, M), x)
    y = np.where(out & (side == 2), g.ymin - rng.uniform(1.0, 5e3, M), y)
    y = np.where(out & (side == 3), g.ymax + rng.uniform(1.0, 5e3, M), y)
    mic.upload_marker("x", x)
    mic.upload_marker("y", y)
    for k in B.RECYCLE_FIELDS[2:]:
        mic.upload_marker(k, rng.uniform(0.5, 2.0, M))
    mic.upload_marker("pfailure", rng.uniform(0, 1, M).astype(np.float32))
    mic.get_marker_inside_flags()
    mk = {k: mic.download_marker(k) for k in (*B.RECYCLE_FIELDS, "matid", "pfailure", "inside")}
    layers, strong = (1, 5, 6, 7, 8, 9, 10), (11, 12, 4)
    thick = (0.05 * g.ymax, 0.1 * g.ymax, 0.08 * g.ymax, 0.15 * g.ymax, 0.1 * g.ymax, 0.12 * g.ymax)
    hl, hr, vfull, xl, xr, seed, step = 0.05 * g.ymax, 0.06 * g.ymax, 2e-9, -1.0, 0.5 * g.xmax, 515, 12
    want, widx, wfl, wnair = B.recycle_contraction(mk, 1, 2, layers, strong, g.xmax, g.ymax, vfull, p["timestep"], hl,
                                                   hr, p["temperature_top"], thick, xl, xr, mp, random_fric, 0.05,
                                                   seed, step, asym)
    con = dict(asymmetric=asym, full_velocity_contraction=vfull, sticky_thickness_left=hl, sticky_thickness_right=hr,
               layer_thickness=thick, x_left_strong=xl, x_right_strong=xr, matid_layers=layers, matid_strong=strong)
    nair, nsub = mic.recycle_markers(1, 2, 4, g.xmax, g.ymax, 0.0, 0.0, 1603.0, seed, step,
                                     iuse_random_fric=random_fric, delta_fric_coef=0.05, recycle_type=4,
                                     contraction=con)
    assert (nair, nsub) == (wnair, len(widx) - wnair) and nair > 10 and nsub > 10
    idx, fl = mic.recycled_markers()
    assert np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(mic.download_marker(k), want[k]), k
    assert len(set(want["matid"][widx - 1][wfl == 1].tolist())) >= (4 if asym else 8)
    mic.get_marker_inside_flags()
    assert np.all(mic.download_marker("inside") == 1)
    mic.close()


@pytest.mark.parametrize("random_fric", [0, 1])
def test_recycle_side_inflow_matches_oracle(eb, random_fric):
    """Recycling type 5 (ExtensionInflowAndOutflowAlongSides): sticky markers in the top band,
    subsurface ones at the two sides below the plate with the ramp factor, as asthenosphere with
    the adiabatic temperature; bit-identical to the oracle."""
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    g = model.grid
    p = model.params
    rng = np.random.default_rng(71 + random_fric)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    M = model.marknum
    x, y = mic.download_marker("x"), mic.download_marker("y")
    out = rng.random(M) < 0.05
    side = rng.integers(0, 4, M)
    x = np.where(out & (side == 0), g.xmin - rng.uniform(1.0, 5e3, M), x)
    x = np.where(out & (side == 1), g.xmax + rng.uniform(1.0, 5e3, M), x)
    y = np.where(out & (side == 2), g.ymin - rng.uniform(1.0, 5e3, M), y)
    y = np.where(out & (side == 3), g.ymax + rng.uniform(1.0, 5e3, M), y)
    mic.upload_marker("x", x)
    mic.upload_marker("y", y)
    for k in B.RECYCLE_FIELDS[2:]:
        mic.upload_marker(k, rng.uniform(0.5, 2.0, M))
    mic.upload_marker("pfailure", rng.uniform(0, 1, M).astype(np.float32))
    mic.get_marker_inside_flags()
    mk = {k: mic.download_marker(k) for k in (*B.RECYCLE_FIELDS, "matid", "pfailure", "inside")}
    hl, hr, plate, smooth = 0.05 * g.ymax, 0.06 * g.ymax, 0.25 * g.ymax, 0.1 * g.ymax
    vyu, vin_l, vin_r, grad, tbot, seed, step = -1e-10, 1e-9, 2e-9, 0.4, 1603.0, 3131, 2
    want, widx, wfl, wnair = B.recycle_side_inflow(mk, 1, 2, 4, g.xmax, g.ymax, vyu, p["timestep"],
                                                   p["temperature_top"], tbot, hl, hr, plate, smooth, vin_l, vin_r,
                                                   grad, model.mats.mat_plastic, random_fric, 0.05, seed, step)
    side_in = dict(sticky_thickness_left=hl, sticky_thickness_right=hr, plate_thickness=plate,
                   smoothing_thickness=smooth, velocity_inflow_left=vin_l, velocity_inflow_right=vin_r,
                   adiabatic_gradient=grad)
    nair, nsub = mic.recycle_markers(1, 2, 4, g.xmax, g.ymax, vyu, 0.0, tbot, seed, step,
                                     iuse_random_fric=random_fric, delta_fric_coef=0.05, recycle_type=5,
                                     side_inflow=side_in)
    assert (nair, nsub) == (wnair, len(widx) - wnair) and nair > 10 and nsub > 10
    idx, fl = mic.recycled_markers()
    assert np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(mic.download_marker(k), want[k]), k
    mic.get_marker_inside_flags()
    assert np.all(mic.download_marker("inside") == 1)
    mic.close()


@pytest.mark.parametrize("asym", [0, 1])
def test_recycle_fracture_zone_matches_oracle(eb, asym):
    """Recycling type 6 (ContractionFractureZone): contraction positions, fracture-zone material
    and temperature; bit-identical to the oracle except the temperature, within 1e-14 (CUDA's
    erf against libm's)."""
    import dataclasses
    from oracle import boundary as B
    model = eb.synthetic.config("rift_small")
    g = model.grid
    p = model.params
    rng = np.random.default_rng(91 + asym)
    m0 = model.mats
    rows = np.arange(12) % len(m0.mat_mu)
    mp = np.asfortranarray(np.asarray(m0.mat_plastic)[rows].copy())
    mp[:, 2] = rng.uniform(0.1, 0.6, 12)
    mats = dataclasses.replace(m0, mat_mu=np.asarray(m0.mat_mu)[rows], mat_hr=np.asarray(m0.mat_hr)[rows],
                               mat_flow_type=np.asarray(m0.mat_flow_type)[rows],
                               mat_flow=np.asfortranarray(np.asarray(m0.mat_flow)[rows]), mat_plastic=mp,
                               mat_rho=np.asarray(m0.mat_rho)[rows])
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.set_materials(mats)
    M = model.marknum
    x, y = mic.download_marker("x"), mic.download_marker("y")
    out = rng.random(M) < 0.05
    side = rng.integers(0, 4, M)
    x = np.where(out & (side == 0), g.xmin - rng.uniform(1.0, 5e3, M), x)
    x = np.where(out & (side == 1), g.xmax + rng.uniform(1.0, 5e3, M), x)
    y = np.where(out & (side == 2), g.ymin - rng.uniform(1.0, 5e3, M), y)
    y = np.where(out & (side == 3), g.ymax + rng.uniform(1.0, 5e3, M), y)
    mic.upload_marker("x", x)
    mic.upload_marker("y", y)
    for k in B.RECYCLE_FIELDS[2:]:
        mic.upload_marker(k, rng.uniform(0.5, 2.0, M))
    mic.upload_marker("pfailure", rng.uniform(0, 1, M).astype(np.float32))
    mic.get_marker_inside_flags()
    mk = {k: mic.download_marker(k) for k in (*B.RECYCLE_FIELDS, "matid", "pfailure", "inside")}
    fz_ids = (1, 5, 6, 7, 8, 9, 10)
    thick = (0.05 * g.ymax, 0.01 * g.ymax, 0.02 * g.ymax, 0.03 * g.ymax, 0.25 * g.ymax, 0.45 * g.ymax, 0.15 * g.ymax)
    hl, hr, vfull, seed, step, tbot = 0.04 * g.ymax, 0.06 * g.ymax, 2e-9, 616, 4, 1603.0
    x_start, x_end, ages, tld, kappa, grad = -1.0, 0.2 * g.xmax, (15.0, 45.0), (0.4 * g.ymax, 0.6 * g.ymax), 1e-6, 0.4
    want, widx, wfl, wnair = B.recycle_fracture_zone(mk, 1, 2, fz_ids, g.xmax, g.ymax, vfull, p["timestep"], hl, hr,
                                                     p["temperature_top"], tbot, grad, thick, x_start, x_end, *ages,
                                                     *tld, kappa, mp, 1, 0.05, seed, step, asym)
    con = dict(asymmetric=asym, full_velocity_contraction=vfull, sticky_thickness_left=hl, sticky_thickness_right=hr)
    fz = dict(fz_thickness=thick, x_fracture_zone_start=x_start, x_fracture_zone_end=x_end, matid_fz=fz_ids,
              age_lithosphere_left=ages[0], age_lithosphere_right=ages[1], thermal_lithosphere_depth_left=tld[0],
              thermal_lithosphere_depth_right=tld[1], thermal_diffusivity=kappa, adiabatic_gradient=grad)
    nair, nsub = mic.recycle_markers(1, 2, 4, g.xmax, g.ymax, 0.0, 0.0, tbot, seed, step, iuse_random_fric=1,
                                     delta_fric_coef=0.05, recycle_type=6, contraction=con, fracture_zone=fz)
    assert (nair, nsub) == (wnair, len(widx) - wnair) and nair > 10 and nsub > 10
    idx, fl = mic.recycled_markers()
    assert np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        got = mic.download_marker(k)
        if k == "tk":
            np.testing.assert_allclose(got, want[k], rtol=1e-14, atol=0)
        else:
            assert np.array_equal(got, want[k]), k
    lith = (wfl == 1) & np.isin(want["matid"][widx - 1], (8,))
    assert lith.sum() > 5  # markers in the cooling plate (the erf branch)
    mic.get_marker_inside_flags()
    assert np.all(mic.download_marker("inside") == 1)
    mic.close()


def test_rock_property_laws_match_reference_known_answers(eb):
    """The GPU's heat capacity (Waples) and conductivities (Liao14, Sekiguchi-Waples) at the
    conditions of the reference's own rock-property test values (rock_props_tests.jl,
    tolerance 1e-9 as there), on inside markers of a model whose fields are overwritten."""
    from boundary_cases import rock_golden_markers
    g, mk, tabs, (nw, nl, ns) = rock_golden_markers()
    model = eb.synthetic.config("rift_small")
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    idx = np.flatnonzero(mic.download_marker("inside") == 1)[:nw + nl + ns]
    for k in ("tk", "pr", "matid"):
        a = mic.download_marker(k)
        if k == "matid":
            a[:] = 1
        a[idx] = mk[k]
        mic.upload_marker(k, a)
    mic.set_rock_tables(*tabs)
    mic.update_marker_rock_properties(0, 1, 0, 0, 1e30)
    np.testing.assert_allclose(mic.download_marker("rhocp")[idx[:nw]], g["waples"]["expected_cp"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(mic.download_marker("kt")[idx[nw:nw + nl]], g["liao14"]["expected_k"], rtol=0, atol=1e-9)
    mic.update_marker_rock_properties(0, 0, 5, 0, 1e30)
    np.testing.assert_allclose(mic.download_marker("kt")[idx[nw + nl:]], g["sekiguchi_waples"]["expected_k"], rtol=0,
                               atol=1e-9)
    mic.close()
