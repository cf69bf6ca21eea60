"""The Stokes oracle against analytic solutions and the reference's structure (CPU only).

No reference test pins the Stokes assembly or the direct solve (the reference
has no golden vectors for them), so the oracle is pinned here by solutions
the discrete equations must reproduce to rounding: a hydrostatic box (v = 0,
p = pressure_bc + rho g dy) and plane Couette flow (a linear vx profile), plus
the structural facts of StokesBuildManager's COO list.
"""
import numpy as np
import pytest

from stokes_cases import couette, marker_model, random_box


@pytest.fixture(scope="module")
def S_mod():
    from oracle.stokes import StokesOracle
    return StokesOracle


def test_hydrostatic_box(eb, S_mod):
    m = random_box(eb)
    o = S_mod(m)
    o.stokes_steps()
    S = o.solve_direct()
    assert o.residual(S) < 1e-12
    o.process_stokes_solution(S)
    g = m.grid
    v_scale = 3000.0 * 9.81 * (g.ymax - g.ymin) ** 2 / 1e21  # rho g H^2 / eta
    assert np.abs(o.gr["vx1"]).max() < 1e-10 * v_scale
    assert np.abs(o.gr["vy1"]).max() < 1e-10 * v_scale
    yc = g.gridy_vx[1:g.ynum]
    pr = 1e5 + 3000.0 * 9.81 * (yc - yc[0])
    assert np.abs(o.gr["pr1"] - pr[:, None]).max() < 1e-12 * pr.max()


def test_couette_flow(eb, S_mod):
    m = random_box(eb, xnum=19, ynum=23, seed=3)
    U = 1e-9
    vex = couette(m, U)
    o = S_mod(m)
    o.stokes_steps()
    S = o.solve_direct()
    o.process_stokes_solution(S)
    g = m.grid
    assert np.abs(o.gr["vx1"] - vex(g.gridy_vx)[:, None]).max() < 1e-12 * U
    assert np.abs(o.gr["vy1"]).max() < 1e-12 * U


def test_coo_structure(eb, S_mod):
    """Rows, columns and entry counts of StokesBuildManager.build_system_of_equations."""
    m = random_box(eb, xnum=9, ynum=7)
    o = S_mod(m)
    Li, Lj, Lv, R = o.stokes_steps()
    nx, ny = 8, 6
    N = 3 * nx * ny
    assert Li.min() >= 1 and Li.max() <= N and Lj.min() >= 1 and Lj.max() <= N
    # entries come row by row: cells in row-major (i outer) order, rows vx, vy, p of each cell
    cell = (Li - 1) // 3
    j, i = cell // ny, cell % ny
    key = i * nx + j
    assert np.all(np.diff(key) >= 0)
    # every momentum row has a diagonal entry; of the continuity rows (zero pressure block)
    # only the pressure-condition row of the upper-left cell has one
    diag = Li == Lj
    kind_d = (Li[diag] - 1) % 3
    assert len(np.unique(Li[diag][kind_d < 2])) == 2 * nx * ny
    assert list(Li[diag][kind_d == 2]) == [3]
    hs = 3 * ny
    allowed = {0: {0, -hs, hs, -3, 3, -2, -2 + hs, 1, 1 + hs, 2, 2 + hs},
               1: {0, -3, 3, -hs, hs, -1 - hs, -1, 2 - hs, 2, 1, 4},
               2: {0, -2 - hs, -2, -4, -1}}
    kind = (Li - 1) % 3
    for k, offs in allowed.items():
        assert set(np.unique(Lj[kind == k] - Li[kind == k])) <= offs
    # x-Stokes rows of the last column (vx on the right boundary) and y-Stokes rows of the
    # last row are identity rows with 2 pscale / (xstpavg + ystpavg)
    kb = 2.0 * o.pscale / (m.grid.xstpavg + m.grid.ystpavg)
    xrows = 3 * ((nx - 1) * ny + np.arange(ny)) + 1
    for r in xrows:
        sel = Li == r
        assert sel.sum() == 1 and Lv[sel][0] == kb
    # pressure_bc_mode 0: the upper-left cell's continuity row fixes the pressure
    sel = Li == 3
    assert sel.sum() == 1 and Lv[sel][0] == kb
    assert R[2] == 2.0 * m.params["pressure_bc"] / (m.grid.xstpavg + m.grid.ystpavg)


def test_process_solution_mapping(eb, S_mod):
    """reload_solu_vel! and apply_vel_bc! on a random solution vector."""
    m = random_box(eb, xnum=8, ynum=6)
    o = S_mod(m)
    o.stokes_steps()
    rng = np.random.default_rng(5)
    S = rng.normal(size=o.N)
    o.process_stokes_solution(S)
    X, Y = 8, 6
    ny = Y - 1
    vx1, vy1, pr1 = o.gr["vx1"], o.gr["vy1"], o.gr["pr1"]
    for j in range(1, X):
        for i in range(1, Y):
            c = (j - 1) * ny + i
            ivx = 3 * c - 2
            if j < X - 1 and 1 < i + 1 < Y + 1 and 1 < j + 1 < X:
                assert vx1[i, j] == S[ivx - 1]
            if i < Y - 1 and 1 < i + 1 < Y and 1 < j + 1 < X + 1:
                assert vy1[i, j] == S[ivx]
            assert pr1[i - 1, j - 1] == S[ivx + 1] * o.pscale
    G = o.gr
    # free-slip top for vx (ghost = interior) and zero vy on the top boundary
    assert np.array_equal(vx1[0, 1:-1], vx1[1, 1:-1])
    assert np.all(vy1[0, 1:-1] == G["btopy"][1:-1, 0])


def test_nonlinear_residual_matches_sparse_product(eb, S_mod):
    m = marker_model(eb, "rift_small")
    o = S_mod(m)
    o.stokes_steps()
    S_old = np.random.default_rng(2).normal(size=o.N) * 1e-10
    res = o.nonlinear_residual(S_old)
    ref = np.abs(o.matrix() @ S_old - o.coo[3])
    assert np.allclose(res, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_direct_solve_of_marker_model(eb, S_mod):
    """The rift's system (sticky air 1e18 over 1e20-1e24 rock) solves to rounding with SuperLU."""
    m = marker_model(eb, "rift_small")
    o = S_mod(m)
    o.stokes_steps()
    S = o.solve_direct()
    assert o.residual(S) < 1e-12


def test_solution_sensitivity_to_averaging_precision(eb):
    """How far the Stokes solution moves when its averaged input grids move by 1e-6 relative.

    The GPU's marker->grid averages agree with the oracle's within 1e-6 (FP32 weights and sums),
    so this sets how closely anything computed from a GPU velocity field can follow the oracle
    through a Picard loop or a time step (tests/test_gpu_picard.py, tests/test_gpu_rift_2p5M.py).
    On the weak-crust rift after one time step (1e18 Pa s sticky air over up to 1e26 Pa s rock),
    random perturbations of 1e-6 move the oracle's own direct solution by well over 1e-6 of
    max|v| (about 2-6e-5), and by less than the 1e-4 those tests allow."""
    import test_gpu_picard as tp
    from oracle.picard import OraclePicard
    from oracle.stokes import StokesOracle
    model = tp.weak_rift(eb, 0)
    op = OraclePicard(model)
    op.time_step(6, 1e-3)
    m = op.mic
    for st in ("get_marker_inside_flags", "initialize_bilinear_interpolation",
               "interpolate_marker_heat_parameters_to_grid", "update_marker_rheology"):
        getattr(m, st)()
    m.update_marker_viscoplastic_viscosity(True)
    m.interpolate_marker_stokes_parameters_to_grid()
    base = {k: v.copy(order="F") for k, v in op.gr.items()}

    def solve(gr):
        so = StokesOracle(model, gr)
        so.stokes_steps()
        return so.solve_direct()

    S0 = solve(base)
    rng = np.random.default_rng(0)
    moves = []
    for _ in range(2):
        g = {k: v.copy(order="F") for k, v in base.items()}
        for k in ("etas1", "etan1", "rho1", "rho1_vy", "mus1", "mun1", "sxy1", "sxx1"):
            g[k] = np.asfortranarray(g[k] * (1 + 1e-6 * rng.uniform(-1, 1, g[k].shape)))
        S = solve(g)
        moves.append(max(np.abs(S[c::3] - S0[c::3]).max() / np.abs(S0[c::3]).max() for c in (0, 1)))
    assert 5e-6 < max(moves) < 1e-4, moves


def test_oracle_rayleigh_taylor_matches_ramberg(eb):
    """The reference's Rayleigh-Taylor benchmark (Ramberg 1968) through the oracle: marker
    averages, assembly, a direct solve, the basic-node velocity (mean of the two vy nodes
    beside each basic node), and the crest velocity within the reference's 3.5 % limit of the
    analytic value (RayleighTaylorInstabilityManager.jl)."""
    from oracle.oracle import OracleMIC
    from oracle.stokes import StokesOracle
    from stokes_cases import bilinear_basic
    model = eb.synthetic.rayleigh_taylor()
    ref = OracleMIC(model)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_stokes_parameters_to_grid()
    model.grids.update({k: np.asfortranarray(v) for k, v in ref.gr.items()})
    o = StokesOracle(model)
    o.stokes_steps()
    S = o.solve_direct()
    o.process_stokes_solution(S)
    vyb = 0.5 * (o.gr["vy1"][:, :-1] + o.gr["vy1"][:, 1:])
    g = model.grid
    v = bilinear_basic(g, vyb, 0.5 * (g.xmax - g.xmin), 1500.0 - 10.0)
    va = eb.synthetic.ramberg_wave_velocity(1500.0, 1500.0, 3000.0, 2900.0, 1e13, 1e19, 10.0, 4000.0)
    assert abs(v - va) / abs(va) < 0.035, (v, va)


def channel_flow_oracle(eb, nsteps: int = 60):
    """The reference's non-Newtonian channel-flow benchmark through the oracle: per step the
    pre-solver averages and rheology, one nodal Picard iteration (direct solve), the
    displacement-limited time step (TimeLoop.jl:244), the post-Stokes steps, RK4 advection and
    the channel recycling (MarkerRecycle types/Channel.jl).  Returns (model, basic-node vy)."""
    from oracle.picard import OraclePicard
    from oracle import boundary as B
    model = eb.synthetic.channel_flow_non_newtonian()
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
        op.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(0)
        op.picard_loop_nodes(1, 1e-3, 0)
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
        y, tk, _ = B.recycle_channel(m.mk["y"], m.mk["tk"], g.ymin, g.ymax, p["temperature_top"], p["temperature_top"])
        m.mk["y"][:] = y
        m.mk["tk"][:] = tk
    return model, op.gr["vyb"].copy()


def channel_flow_error(eb, model, vyb) -> float:
    """The reference's check (ChannelFlowNonNewtonianManager.jl, Options.jl y_index = 11): the
    basic-node vy profile of row 11 against the analytic profile, largest relative error over the
    nodes where the analytic velocity is not zero."""
    g = model.grid
    ana = eb.synthetic.channel_flow_velocity(g.gridx_b, g.xmax - g.xmin, (g.ymax - g.ymin) - g.ystp_b[0], 1e9, 5e-20,
                                             3.0)
    nz = ana != 0.0
    return float(np.max(np.abs(vyb[10, nz] - ana[nz]) / np.abs(ana[nz])))


def test_oracle_channel_flow_non_newtonian_matches_the_power_law(eb):
    """Sixty steps as the reference runs the benchmark (Options.jl time_steps = [60]): the
    velocity profile within the reference's 1.1 % limit of the analytic power-law flow."""
    model, vyb = channel_flow_oracle(eb)
    err = channel_flow_error(eb, model, vyb)
    assert err < 0.011, err
