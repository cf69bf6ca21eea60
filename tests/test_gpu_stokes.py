"""GPU Stokes-continuity step against the oracle, through the C-ABI.

Inputs are the oracle's marker averages of small synthetic models (and
analytic boxes), uploaded as grid fields; every step is compared with the C
restatement of the reference:
  - viscoelastic terms and RHS grids: identical to rounding (1e-15 relative);
  - the assembled stencil: every coefficient equal to the reference's COO value
    (the assembly keeps the reference's operand order, no FMA contraction);
  - the operator product: equal to the COO sparse product within 1e-14 of the
    row scale;
  - the iterative solve: unscaled relative residual <= 1e-8 (the metric's
    tolerance) and velocities/pressures within 1e-6 of SuperLU's solution
    (relative to each field's maximum) when solved to 1e-11;
  - the unpacked grids vx1, vy1, pr1: equal to the oracle's unpacking of the
    GPU solution.
"""
import numpy as np
import pytest

from stokes_cases import STOKES_GRIDS, couette, marker_model, random_box

pytestmark = pytest.mark.gpu

BC = ("btopx", "bbottomx", "btopy", "bbottomy", "bleftx", "brightx", "blefty", "brighty")


def gpu_ctx(eb, model):
    mic = eb.MarkerInCell(0)
    mic.set_grid(model.grid)
    mic.set_params(model.params)
    mic.set_stokes_params(model.params)
    for k in STOKES_GRIDS + BC + ("eii_plastic_pressure",):
        mic.upload_grid(k, model.grids[k])
    return mic


def oracle_for(model):
    from oracle.stokes import StokesOracle
    o = StokesOracle(model)
    o.stokes_steps()
    return o


def stencil_from_coo(o, nx, ny):
    """The oracle's COO list folded into the 27-slot stencil (duplicates summed)."""
    Li, Lj, Lv, _ = o.coo
    hs = 3 * ny
    xo = [0, -hs, hs, -3, 3, -2, -2 + hs, 1, 1 + hs, 2, 2 + hs]
    yo = [0, -3, 3, -hs, hs, -1 - hs, -1, 2 - hs, 2, 1, 4]
    co = [0, -2 - hs, -2, -4, -1]
    st = np.zeros((27, nx, ny))
    cell = (Li - 1) // 3
    kind = (Li - 1) % 3
    j, i = cell // ny, cell % ny
    d = Lj - Li
    for k, (offs, base) in enumerate(((xo, 0), (yo, 11), (co, 22))):
        for s, off in enumerate(offs):
            m = (kind == k) & (d == off)
            np.add.at(st[base + s], (j[m], i[m]), Lv[m])
    return st


@pytest.mark.parametrize("case", ["box", "rift_small", "sinking_block"])
def test_build_steps_match_oracle(eb, case):
    model = random_box(eb) if case == "box" else marker_model(eb, case)
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    for k in ("etas0", "sxy0", "etan0", "sxx0", "RX1", "RY1"):
        got, want = mic.download_grid(k), o.gr[k]
        assert np.array_equal(got, want), f"{k} differs"
    got, want = mic.download_grid("RC1"), o.gr["RC1"]
    assert np.allclose(got, want, rtol=1e-15, atol=0)
    mic.build_system_of_equations()
    assert mic.pscale == o.pscale
    nx, ny = model.grid.xnum - 1, model.grid.ynum - 1
    st = mic.stokes_stencil()
    ref = stencil_from_coo(o, nx, ny)
    bad = np.argwhere(st != ref)
    assert bad.size == 0, f"{len(bad)} stencil coefficients differ, first at slot/j/i {bad[0]}"
    R = mic.download_stokes_vector("rhs")
    assert np.array_equal(R, o.coo[3])
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_operator_apply_matches_coo_product(eb, case):
    model = marker_model(eb, case)
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    K = o.matrix()
    rng = np.random.default_rng(7)
    for x in (rng.normal(size=o.N), np.abs(rng.normal(size=o.N))):
        y = mic.stokes_apply(x)
        ref = K @ x
        scale = abs(K) @ np.abs(x)
        assert np.all(np.abs(y - ref) <= 1e-14 * scale + 1e-300)
    mic.close()


def solve_case(eb, model, rtol):
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=rtol, max_iters=4000)
    S = mic.download_stokes_vector("solution")
    return o, mic, rep, S


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_solve_reaches_metric_tolerance(eb, case):
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-8)
    assert rep["status"] == 0
    assert rep["rel_residual"] <= 1e-8, rep
    assert o.residual(S) <= 1e-8 * 1.01
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_solution_matches_superlu(eb, case):
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-11)
    assert rep["status"] == 0, rep
    S_ref = o.solve_direct()
    for comp in range(3):
        a, b = S[comp::3], S_ref[comp::3]
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max(), (comp, np.abs(a - b).max() / np.abs(b).max())
    # unpacked grids equal the oracle's unpacking of the GPU solution
    o.process_stokes_solution(S)
    for k in ("vx1", "vy1", "pr1"):
        assert np.array_equal(mic.download_grid(k), o.gr[k]), k
    mic.close()


def test_couette_and_hydrostatic_on_gpu(eb):
    m = random_box(eb, xnum=33, ynum=25, seed=4)
    o, mic, rep, S = solve_case(eb, m, 1e-11)
    g = m.grid
    yc = g.gridy_vx[1:g.ynum]
    pr = 1e5 + 3000.0 * 9.81 * (yc - yc[0])
    assert np.abs(mic.download_grid("pr1") - pr[:, None]).max() < 1e-9 * pr.max()
    mic.close()
    m = random_box(eb, xnum=33, ynum=25, seed=6)
    U = 1e-9
    vex = couette(m, U)
    o, mic, rep, S = solve_case(eb, m, 1e-11)
    assert np.abs(mic.download_grid("vx1") - vex(m.grid.gridy_vx)[:, None]).max() < 1e-8 * U
    mic.close()


def test_nonlinear_residual_and_backup(eb):
    model = marker_model(eb, "rift_small")
    o, mic, rep, S = solve_case(eb, model, 1e-8)
    mic.backup_stokes_solution()
    assert np.array_equal(mic.download_stokes_vector("solution_old"), S)
    res = mic.stokes_nonlinear_residual()
    ref = o.nonlinear_residual(S)
    scale = abs(o.matrix()) @ np.abs(S) + np.abs(o.coo[3])
    assert np.all(np.abs(res - ref) <= 1e-14 * scale + 1e-300)
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_post_solve_grid_kernels_match_oracle(eb, case):
    """Grid strain rate/spin, viscoelastic stress forecast and change, basic-node velocity:
    identical to the oracle applied to the GPU's own solution."""
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-8)
    o.process_stokes_solution(S)
    mic.update_grid_strain_rate_and_spin()
    mic.forecast_viscoelastic_grid_stress()
    mic.calculate_deviatoric_grid_stress_change()
    mic.interpolate_stag_velocity_to_basic_grid()
    o.update_grid_strain_rate_and_spin()
    o.forecast_viscoelastic_grid_stress()
    o.interpolate_stag_velocity_to_basic_grid()
    for k in ("exx", "exy", "eii", "esp", "sxy2", "sxx2", "dsxy", "dsxx", "vxb", "vyb"):
        assert np.array_equal(mic.download_grid(k), o.gr[k]), k
    mic.close()
