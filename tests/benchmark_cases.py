"""The reference's solid-body-rotation benchmark stepped through the oracle, for the CPU test
and as the GPU test's comparison."""
import numpy as np

ROTATION_STEPS = 90  # 55344.0275 yr steps per rotation at 3.1536 cm/yr on a 25 km radius
Y_INDEX = 11         # Options.jl: y_index of the compared temperature profile


def rotation_check(model, t_initial, t_final) -> float:
    """SolidBodyRotationManager.get_test_results: the profile after the rotation against the
    step-1 profile, in Celsius, largest relative error (TestResults.calc_relative_error_1d)."""
    a = t_initial - 273.15
    b = t_final - 273.15
    nz = a != 0.0
    return float(np.max(np.abs(b[nz] - a[nz]) / np.abs(a[nz])))


def solid_body_rotation_oracle(eb, rotations: int = 3):
    """TimeLoop.run_loop!'s body for the benchmark (src/time_loop/TimeLoop.jl:181-194) through the
    oracle: inside flags, bilinear set-up and heat averages (the output's TempC is this grid
    temperature), the kinematic velocity (Kinematics.solid_body_rotation!) with its spin, the heat
    step (RHS, heat loop, grid change, subgrid diffusion, remaining change to the markers) and RK4
    advection.  Returns (model, {step: row-11 grid temperature}) for step 1 and the steps that
    follow each full rotation (the reference's outputs 1, 91, 181, 271)."""
    from oracle.heat import HeatOracle
    from oracle.oracle import OracleMIC
    model = eb.synthetic.solid_body_rotation()
    g = model.grid
    mic = OracleMIC(model)
    # spin of the rigid rotation: 0.5 (dvy/dx - dvx/dy) = vrotation / (xsize / 2) everywhere
    omega = model.params["velocity_rotation"] / (0.5 * (g.xmax - g.xmin))
    mic.gr["esp"] = np.asfortranarray(np.full((g.ynum, g.xnum), omega))
    marks = {1 + k * ROTATION_STEPS for k in range(rotations + 1)}
    last = max(marks)
    rows = {}
    for step in range(1, last + 1):
        mic.get_marker_inside_flags()
        mic.initialize_bilinear_interpolation()
        mic.interpolate_marker_heat_parameters_to_grid()
        if step in marks:
            rows[step] = mic.gr["tk1"][Y_INDEX - 1, :].copy()
        if step == last:
            break
        ho = HeatOracle(model, grids=mic.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            mic.gr[k] = np.asfortranarray(ho.gr[k])
        mic.subgrid_heat_diffusion_update()
        mic.add_remaining_grid_change_to_marker_temperature()
        mic.advect_markers_and_rotate_stress()
    return model, rows


COUETTE_STEPS = 99   # Options.jl: output 100 (its grid temperature is the one after 99 steps)
COUETTE_ROW = 11     # Options.jl: y_index


def couette_error(eb, model, row) -> float:
    """CouetteFlowViscousHeatingManager.get_test_results: the numerical profile (row 11 of the grid
    temperature) interpolated linearly at the analytic profile's positions, against the steady
    analytic temperature built from its own wall temperatures; largest relative error in K."""
    g = model.grid
    xs, ts = eb.synthetic.couette_temperature_profile(row[0], row[-1], g.xmax - g.xmin, 150e3)
    num = np.interp(xs, g.gridx_b, row)
    return float(np.max(np.abs(num - ts) / ts))


def couette_oracle(eb, nsteps: int = COUETTE_STEPS):
    """The Couette viscous-heating benchmark through the oracle, step by step as
    TimeLoop.run_loop! runs it (src/time_loop/TimeLoop.jl:181-194): pre-solver averages and the
    temperature-dependent flow law, one nodal Picard iteration with harmonic normal viscosity,
    the displacement-limited time step, post-Stokes steps, the heat step with shear heating and
    subgrid diffusion, RK4 advection and the channel recycling.  Returns (model, row-11 grid
    temperature after nsteps)."""
    from oracle import boundary as B
    from oracle.heat import HeatOracle
    from oracle.picard import OraclePicard
    model = eb.synthetic.couette_flow_viscous_heating()
    op = OraclePicard(model)
    p, g, m = op.model.params, model.grid, op.mic
    dt_ve = p["timestep"]
    for _ in range(nsteps):
        p["timestep"] = dt_ve
        m.get_marker_inside_flags()
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(1)
        op.picard_loop_nodes(1, 1e-3, 1)
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        p["timestep"] = B.timestep_displacement_limit(g, op.gr["vx1"], op.gr["vy1"], p["marker_cell_displ_max"], 0,
                                                      dt_ve)
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.update_subgrid_stress()
        m.apply_marker_stress_correction()
        ho = HeatOracle(op.model, grids=op.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            op.gr[k] = np.asfortranarray(ho.gr[k])
        m.subgrid_heat_diffusion_update()
        m.add_remaining_grid_change_to_marker_temperature()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        y, tk, _ = B.recycle_channel(m.mk["y"], m.mk["tk"], g.ymin, g.ymax, p["temperature_top"], p["temperature_top"])
        m.mk["y"][:] = y
        m.mk["tk"][:] = tk
    m.get_marker_inside_flags()
    m.initialize_bilinear_interpolation()
    m.interpolate_marker_heat_parameters_to_grid()
    return model, op.gr["tk1"][COUETTE_ROW - 1, :].copy()


VCOND_STEPS = 495    # output 100 at 0.5 Myr per output with 100 kyr steps: 49.5 Myr
VCOND_ROW = 11


def vcond_error(eb, model, row) -> float:
    """ChannelFlowVariableConductivityManager.get_test_results: row 11 of the grid temperature
    against the steady analytic profile built from its wall temperature, relative error in
    Celsius (largest over the nodes)."""
    g = model.grid
    ana = eb.synthetic.channel_flow_variable_conductivity_temperature(
        g.gridx_b, g.xmax - g.xmin, (g.ymax - g.ymin) - g.ystp_b[0], row[0], 3e7, 1e19, 8.0, 1.0)
    a, n = ana - 273.15, row - 273.15
    return float(np.max(np.abs(n - a) / np.abs(a)))


def vcond_oracle(eb, nsteps: int = VCOND_STEPS):
    """The variable-conductivity channel benchmark through the oracle: per step the rock
    properties (temperature-dependent conductivity), the pre-solver averages, one nodal Picard
    iteration, the post-Stokes steps and the heat step with shear heating (markers do not
    move).  Returns (model, row-11 grid temperature after nsteps)."""
    from oracle import boundary as B
    from oracle.heat import HeatOracle
    from oracle.picard import OraclePicard
    model = eb.synthetic.channel_flow_variable_conductivity()
    op = OraclePicard(model)
    p, m = op.model.params, op.mic
    rt = p["rock_tables"]

    def pre():
        m.get_marker_inside_flags()
        upd = B.rock_properties(m.mk, rt["mat_rho"], rt["mat_cp"], rt["mat_kt"], rt["density_model"],
                                rt["rhocp_model"], rt["conductivity_model"], p["temperature_top"], 1200.0)
        for k, v in upd.items():
            m.mk[k][:] = v
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
    for _ in range(nsteps):
        pre()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(0)
        op.picard_loop_nodes(1, 1e-3, 0)
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.update_subgrid_stress()
        m.apply_marker_stress_correction()
        ho = HeatOracle(op.model, grids=op.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            op.gr[k] = np.asfortranarray(ho.gr[k])
        m.subgrid_heat_diffusion_update()
        m.add_remaining_grid_change_to_marker_temperature()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
    pre()
    return model, op.gr["tk1"][VCOND_ROW - 1, :].copy()


SLAB_OUTPUTS = (80, 100, 120, 140, 160)


def elastic_slab_oracle(eb, outputs=SLAB_OUTPUTS):
    """The elastic-slab benchmark through the oracle (about 8 minutes on one core: 7950 steps with
    a direct Stokes solve each, so no CPU test runs it): gravity off after step 100, the step
    multiplied by 10 after step 250, one output per 50 steps.  Returns {output: largest relative
    change of a slab marker's distance from the origin}."""
    from oracle import boundary as B
    from oracle.picard import OraclePicard
    model = eb.synthetic.elastic_slab()
    op = OraclePicard(model)
    p, g, m = op.model.params, model.grid, op.mic
    W, H = g.xmax - g.xmin, g.ymax - g.ymin
    x0, y0 = m.mk["x"].copy(), m.mk["y"].copy()
    slab = (0.2 < y0 / H) & (y0 / H < 0.8) & (x0 / W < 0.8)
    d0 = np.hypot(x0[slab], y0[slab])
    dt, nskip, worst = p["timestep"], p["nskip_output"], {}
    for step in range(1, 1 + (max(outputs) - 1) * nskip + 1):
        out = (step - 1) // nskip + 1
        if (step - 1) % nskip == 0 and out in outputs:
            worst[out] = float(np.max(np.abs(np.hypot(m.mk["x"][slab], m.mk["y"][slab]) - d0) / d0))
            if out == max(outputs):
                break
        p["timestep"] = dt
        m.get_marker_inside_flags()
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(0)
        op.picard_loop_nodes(1, 1e-3, 0)
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        p["timestep"] = B.timestep_displacement_limit(g, op.gr["vx1"], op.gr["vy1"], p["marker_cell_displ_max"], 0, dt)
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.apply_marker_stress_correction()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        if step == p["nsteps_turn_off_gravity"]:
            p["gravity_y"] = 0.0
        if step == p["ntime_increase"]:
            dt = dt * p["time_increase_factor"]
    return worst


NST_OUTPUTS = (1, 10, 20, 30, 40, 50, 60, 70, 80, 100, 120, 140, 160, 180, 200, 220, 240)
NST_ROW = 11


def nst_error(eb, model, row_k, tmyr) -> float:
    """ChannelFlowNonSteadyTemperatureManager.get_test_results for one output: row 11 of the grid
    temperature (Celsius) against the transient analytic profile at the output's time; largest
    relative error."""
    g = model.grid
    ana = eb.synthetic.channel_flow_non_steady_temperature_profile(
        g.gridx_b, tmyr, g.xmax - g.xmin, g.ymax - g.ymin, g.ynum, NST_ROW, 727.0, 1227.0, 1e5, 1e19, 2.0, 3000.0,
        1000.0)
    num = row_k - 273.15
    return float(np.max(np.abs(num - ana) / np.abs(ana)))


def nst_oracle(eb):
    """The non-steady channel benchmark through the oracle, run as the reference's time loop runs
    it: the initial grid temperature interpolated back to the markers, then per step the
    pre-solver averages, one nodal Picard iteration, the displacement-limited step, the
    post-Stokes steps, the heat step, RK4 advection and the channel recycling (which shifts a
    recycled marker's temperature by T_top - T_bottom).  Returns (model, {output: (time in Myr,
    row-11 grid temperature)}) for the reference's outputs (one per 5 steps)."""
    from oracle import boundary as B
    from oracle.heat import HeatOracle
    from oracle.picard import OraclePicard
    model = eb.synthetic.channel_flow_non_steady_temperature()
    op = OraclePicard(model)
    p, g, m = op.model.params, model.grid, op.mic
    dt_ve, nskip = p["timestep"], p["nskip_output"]

    def pre():
        m.get_marker_inside_flags()
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
    pre()
    m.interpolate_temperature_to_markers()
    tsum, rows = 0.0, {}
    for step in range(1, 1 + (max(NST_OUTPUTS) - 1) * nskip + 1):
        p["timestep"] = dt_ve
        pre()
        out = (step - 1) // nskip + 1
        if (step - 1) % nskip == 0 and out in NST_OUTPUTS:
            rows[out] = (tsum / (1e6 * 365.25 * 24.0 * 3600.0), m.gr["tk1"][NST_ROW - 1, :].copy())
            if out == max(NST_OUTPUTS):
                break
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(0)
        op.picard_loop_nodes(1, 1e-3, 0)
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        p["timestep"] = B.timestep_displacement_limit(g, op.gr["vx1"], op.gr["vy1"], p["marker_cell_displ_max"], 0,
                                                      dt_ve)
        tsum += p["timestep"]
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.update_subgrid_stress()
        m.apply_marker_stress_correction()
        ho = HeatOracle(op.model, grids=op.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            op.gr[k] = np.asfortranarray(ho.gr[k])
        m.subgrid_heat_diffusion_update()
        m.add_remaining_grid_change_to_marker_temperature()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        y, tk, _ = B.recycle_channel(m.mk["y"], m.mk["tk"], g.ymin, g.ymax, p["temperature_top"],
                                     p["temperature_bottom"])
        m.mk["y"][:] = y
        m.mk["tk"][:] = tk
    return model, rows


def box_convection_oracle(eb, every: int = 1000):
    """The box-convection benchmark through the oracle (about 12.5 minutes on one core for the
    9900 steps, so no CPU test runs it): the initial grid temperature interpolated back to the
    markers, then per step the rock properties, the pre-solver averages, one nodal Picard
    iteration, the displacement-limited step, the post-Stokes steps, the heat step and RK4
    advection.  Returns {step: dimensionless RMS velocity} every `every` steps and at the last."""
    from oracle import boundary as B
    from oracle.heat import HeatOracle
    from oracle.picard import OraclePicard
    syn = eb.synthetic
    model = syn.box_convection()
    op = OraclePicard(model)
    p, g, m = op.model.params, model.grid, op.mic
    rt, dt_ve = p["rock_tables"], p["timestep"]
    m.get_marker_inside_flags()
    m.initialize_bilinear_interpolation()
    m.interpolate_marker_heat_parameters_to_grid()
    m.interpolate_temperature_to_markers()
    nsteps, out = 99 * p["nskip_output"], {}
    for step in range(1, nsteps + 1):
        p["timestep"] = dt_ve
        m.get_marker_inside_flags()
        upd = B.rock_properties(m.mk, rt["mat_rho"], rt["mat_cp"], rt["mat_kt"], rt["density_model"],
                                rt["rhocp_model"], rt["conductivity_model"], p["temperature_top"], 1200.0)
        for k, v in upd.items():
            m.mk[k][:] = v
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(0)
        op.picard_loop_nodes(1, 1e-3, 0)
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        p["timestep"] = B.timestep_displacement_limit(g, op.gr["vx1"], op.gr["vy1"], p["marker_cell_displ_max"], 0,
                                                      dt_ve)
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.apply_marker_stress_correction()
        ho = HeatOracle(op.model, grids=op.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            op.gr[k] = np.asfortranarray(ho.gr[k])
        m.subgrid_heat_diffusion_update()
        m.add_remaining_grid_change_to_marker_temperature()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        if step % every == 0 or step == nsteps:
            out[step] = syn.box_convection_vrms(g, op.gr["vx1"], op.gr["vy1"], 5.0, 1250.0, 4000.0)
    return out


KAUS10_SEED = 10


def kaus10_oracle(eb, nsteps: int | None = None, log=None):
    """The Kaus (2010) plasticity benchmark through the oracle (tens of minutes on the host's
    cores: a direct Stokes solve per nodal Picard iteration, so no CPU test runs it).  Per step,
    as TimeLoop.run_loop! does for this model: inside flags, the pre-solver averages and rheology,
    the nodal Picard loop (PlasticityLoopNodes.jl:36-92; up to nglobal iterations), the staggered
    velocity on basic nodes, the nodal viscoplastic viscosity back to the markers, the
    displacement-limited step, the post-Stokes steps with the subgrid stress diffusion, RK4
    advection, the strain update, and the ExtensionNoBottomInflow recycling of the markers that
    left the box.  The heat solve is left out: the temperature is uniform and stays so.  Stops at
    the reference's extensional-strain limit (v_full t / xsize >= 0.02) or after nsteps.
    log(step, Picard records, model time, pressure-grid strain-rate invariant) runs after each step.
    Returns (model, final pressure-grid strain-rate invariant, per-step Picard iteration counts)."""
    from oracle import boundary as B
    from oracle.picard import OraclePicard
    model = eb.synthetic.plasticity_benchmark_kaus10()
    op = OraclePicard(model)
    p, g, m = op.model.params, model.grid, op.mic
    W = g.xmax - g.xmin
    dt_ve, timesum, step, iters = p["timestep"], 0.0, 0, []
    while True:
        step += 1
        p["timestep"] = dt_ve
        m.get_marker_inside_flags()
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=False)
        m.interpolate_marker_stokes_parameters_to_grid()
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(1)
        hist = op.picard_loop_nodes(int(p["nglobal"]), p["tolerance_picard"], 1)
        iters.append(len(hist))
        op.so.interpolate_stag_velocity_to_basic_grid()
        m.calc_marker_viscoplastic_viscosity()
        p["timestep"] = B.timestep_displacement_limit(g, op.gr["vx1"], op.gr["vy1"], p["marker_cell_displ_max"], 0,
                                                      dt_ve)
        op.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        m.update_subgrid_stress()
        m.apply_marker_stress_correction()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        m.get_marker_inside_flags()
        out, _, _ = B.recycle_no_bottom_inflow(m.mk, 1, W, p["velocity_y_upper"], p["timestep"],
                                               p["temperature_top"], model.mats.mat_plastic, KAUS10_SEED, step)
        for k, v in out.items():
            m.mk[k][:] = v
        timesum += p["timestep"]
        if log is not None:
            log(step, hist, timesum, op.gr["eii"])
        if p["full_velocity_extension"] * timesum / W >= p["strain_limit"] or (nsteps and step >= nsteps):
            break
    return model, np.array(op.gr["eii"]), iters
