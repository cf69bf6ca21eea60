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


def solid_body_rotation_oracle(eb, nsteps: int = ROTATION_STEPS):
    """TimeLoop.run_loop!'s body for the benchmark (src/time_loop/TimeLoop.jl:181-194) through the
    oracle: inside flags, bilinear set-up and heat averages (the output's TempC is this grid
    temperature), the kinematic velocity (Kinematics.solid_body_rotation!) with its spin, the heat
    step (RHS, heat loop, grid change, subgrid diffusion, remaining change to the markers) and RK4
    advection.  Returns (model, row-11 grid temperature at step 1, at step nsteps + 1)."""
    from oracle.heat import HeatOracle
    from oracle.oracle import OracleMIC
    model = eb.synthetic.solid_body_rotation()
    g = model.grid
    mic = OracleMIC(model)
    # spin of the rigid rotation: 0.5 (dvy/dx - dvx/dy) = vrotation / (xsize / 2) everywhere
    omega = model.params["velocity_rotation"] / (0.5 * (g.xmax - g.xmin))
    mic.gr["esp"] = np.asfortranarray(np.full((g.ynum, g.xnum), omega))
    rows = []
    for step in range(1, nsteps + 2):
        mic.get_marker_inside_flags()
        mic.initialize_bilinear_interpolation()
        mic.interpolate_marker_heat_parameters_to_grid()
        if step in (1, nsteps + 1):
            rows.append(mic.gr["tk1"][Y_INDEX - 1, :].copy())
        if step == nsteps + 1:
            break
        ho = HeatOracle(model, grids=mic.gr)
        ho.heat_step()
        for k in ("dtk1", "tk2"):
            mic.gr[k] = np.asfortranarray(ho.gr[k])
        mic.subgrid_heat_diffusion_update()
        mic.add_remaining_grid_change_to_marker_temperature()
        mic.advect_markers_and_rotate_stress()
    return model, rows[0], rows[1]
