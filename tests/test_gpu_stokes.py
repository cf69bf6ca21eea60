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


@pytest.mark.parametrize("stab,mode", [(1, 0), (0, 1), (1, 2)])
@pytest.mark.parametrize("case", ["box", "rift_small", "sinking_block"])
def test_build_steps_match_oracle(eb, case, stab, mode):
    model = random_box(eb) if case == "box" else marker_model(eb, case)
    model.params["iuse_interface_stabilization"] = stab
    model.params["pressure_bc_mode"] = mode
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
    # the COO export reproduces the reference's list entry for entry
    Li, Lj, Lv, R2 = mic.export_coo()
    for got, want in zip((Li, Lj, Lv, R2), o.coo):
        assert np.array_equal(got, want)
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


def solve_case(eb, model, rtol, method="fgmres", precision="mixed"):
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=rtol, max_iters=4000, method=method,
                                                            precision=precision)
    S = mic.download_stokes_vector("solution")
    return o, mic, rep, S


@pytest.mark.parametrize("method", ["fgmres", "bicgstab"])
@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_solve_reaches_metric_tolerance(eb, case, method):
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-8, method)
    assert rep["status"] == 0
    assert rep["rel_residual"] <= 1e-8, rep
    assert o.residual(S) <= 1e-8 * 1.01
    mic.close()


@pytest.mark.parametrize("method,precision", [("fgmres", "mixed"), ("bicgstab", "mixed"), ("fgmres", "fp64"),
                                              ("bicgstab", "fp64")])
@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_solution_matches_superlu(eb, case, method, precision):
    """Both the mixed method (FP32 V-cycle and stored directions) and the plain FP64 method."""
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-11, method, precision)
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
    mic.backup_stokes_arrays()
    assert np.array_equal(mic.download_stokes_vector("solution_old"), S)
    for k in ("vx1", "vy1", "pr1"):
        assert np.array_equal(mic.download_grid(k + "_old"), mic.download_grid(k))
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


def test_stokes_norms_match_numpy(eb):
    """StokesNorms.calculate_stokes_norms! solution-change norms between two Picard iterates."""
    model = marker_model(eb, "rift_small")
    o, mic, rep, S0 = solve_case(eb, model, 1e-6)
    mic.backup_stokes_arrays()
    old = {k: mic.download_grid(k) for k in ("vx1", "vy1", "pr1")}
    mic.solve_system(rtol=1e-10, use_initial_guess=True)
    mic.process_stokes_solution()
    mic.stokes_nonlinear_residual()
    S = mic.download_stokes_vector("solution")
    new = {k: mic.download_grid(k) for k in ("vx1", "vy1", "pr1")}
    res = mic.download_stokes_vector("resnl")
    got = mic.calculate_stokes_norms()

    def l2(v, v0):
        a = np.linalg.norm(np.abs(v0 - v)); n = np.linalg.norm(v)
        return a, (a / n if n != 0 else 1e38)

    def linf(v, v0):
        a = np.max(np.abs(v0 - v)); n = np.max(np.abs(v))
        return a, (a / n if n != 0 else 1e38)
    vxy = np.concatenate([new["vx1"].ravel(order="C"), new["vy1"].ravel(order="C")])
    vxy0 = np.concatenate([old["vx1"].ravel(order="C"), old["vy1"].ravel(order="C")])
    want = {}
    want["dsoluv1_abs_inf"], want["dsoluv1_rel_inf"] = linf(S, S0)
    want["dsoluv1_abs_L2"], want["dsoluv1_rel_L2"] = l2(S, S0)
    for k in ("vx1", "vy1", "pr1"):
        want[f"d{k}_abs_L2"], want[f"d{k}_rel_L2"] = l2(new[k], old[k])
    want["dvxy_abs_inf"], want["dvxy_rel_inf"] = linf(vxy, vxy0)
    want["dvxy_abs_L2"], want["dvxy_rel_L2"] = l2(vxy, vxy0)
    want["resnl_L2"] = np.linalg.norm(res)
    for k, v in want.items():
        assert abs(got[k] - v) <= 1e-12 * abs(v) + 1e-300, (k, got[k], v)
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_harmonic_normal_viscosity_matches_oracle(eb, case):
    """HarmonicAverage.normal_viscosity_from_harmonic_avg_shear_viscosity! on yielding cells."""
    model = marker_model(eb, case)
    rng = np.random.default_rng(3)
    X, Y = model.grid.xnum, model.grid.ynum
    # mark a random subset of nodes and cells as yielding
    model.grids["plastics"] = np.asfortranarray((rng.random((Y, X)) < 0.1).astype(float))
    model.grids["plasticn"] = np.asfortranarray((rng.random((Y - 1, X - 1)) < 0.1).astype(float))
    model.grids["plastic_yield"] = np.asfortranarray(np.zeros((Y, X)))
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    for k in ("plastics", "plasticn", "plastic_yield"):
        mic.upload_grid(k, model.grids[k])
    mic.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(1)
    o.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(1)
    assert np.array_equal(mic.download_grid("etan1"), o.gr["etan1"])
    assert not np.array_equal(o.gr["etan1"], model.grids["etan1"])  # the update did something
    mic.close()


def test_picard_loop_markers_runs_and_converges(eb):
    """The marker Picard loop on the GPU context: the first iteration equals a single Stokes step,
    the loop stops on the reference's criterion, and every solve meets the metric tolerance."""
    model = eb.synthetic.rift(101, 41, 4)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_stokes_parameters_to_grid()
    mic.update_marker_rheology()
    hist = mic.picard_loop_markers(nglobal=4, tolerance_picard=1e-3)
    assert 1 <= len(hist) <= 4
    for h in hist:
        assert h["status"] == 0 and h["rel_residual"] <= 1e-8
    assert hist[0]["dvxy_rel_L2"] == pytest.approx(1.0)  # compared with zero previous velocities
    if len(hist) < 4:
        assert hist[-1]["dvxy_rel_L2"] < 1e-3
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_nodal_plastic_yielding_matches_oracle(eb, case):
    """PlasticFailureNodes.update_nodes_for_plastic_yielding on the GPU's own solved state."""
    model = marker_model(eb, case)
    o, mic, rep, S = solve_case(eb, model, 1e-8)
    mic.update_grid_strain_rate_and_spin()
    mic.forecast_viscoelastic_grid_stress()
    # yield state and material strength from the same arrays on both sides
    X, Y = model.grid.xnum, model.grid.ynum
    rng = np.random.default_rng(11)
    G = {"plastic_yield": (rng.random((Y, X)) < 0.2).astype(float),
         "cohesion_grid": np.full((Y, X), 5e6), "fric_degrees_grid": rng.uniform(5.0, 30.0, (Y, X)),
         "eta_flow": mic.download_grid("etas1") * 10.0}
    for k, v in G.items():
        mic.upload_grid(k, np.asfortranarray(v))
    for k in ("etas1", "mus1", "sxy2", "sxx2", "pr1"):
        o.gr[k] = np.asfortranarray(mic.download_grid(k))
    for k, v in G.items():
        o.gr[k] = np.asfortranarray(v)
    n_gpu, e_gpu = mic.update_nodes_for_plastic_yielding()
    n_ref, e_ref = o.update_nodes_for_plastic_yielding()
    assert n_gpu == n_ref and n_ref > 0
    assert e_gpu == pytest.approx(e_ref, rel=1e-12)
    assert np.array_equal(mic.download_grid("plastic_yield_buffer"), o.gr["plastic_yield_buffer"])
    for k in ("etavp_buffer", "plastic_strain_rate_buffer"):
        a, b = mic.download_grid(k), o.gr[k]
        assert np.allclose(a, b, rtol=1e-13, atol=0), k
    yb = o.gr["plastic_yield_buffer"] > 0
    assert np.allclose(mic.download_grid("yield_error")[yb], o.gr["yield_error"][yb], rtol=1e-12, atol=1e-6)
    mic.apply_nodal_plastic_yielding()
    assert np.array_equal(mic.download_grid("etas1"), mic.download_grid("etavp_buffer"))
    eb_ = mic.download_grid("eii_plastic_basic")
    ep = (eb_[:-1, :-1] + eb_[:-1, 1:] + eb_[1:, :-1] + eb_[1:, 1:]) / 4.0
    assert np.allclose(mic.download_grid("eii_plastic_pressure"), ep, rtol=1e-15, atol=0)
    mic.close()


def test_circles_box_matches_superlu(eb):
    """The circles solver benchmark at 129 x 129 nodes: 20 inclusions of 1e18-1e27 Pa s, solved
    to 1e-10 (the benchmark's tolerance) and compared with SuperLU per unknown type."""
    from oracle.stokes import StokesOracle
    model = eb.synthetic.circles(129, 20)
    mic = gpu_ctx(eb, model)
    rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-10)
    assert rep["status"] == 0 and rep["rel_residual"] <= 1e-10, rep
    o = StokesOracle(model)
    o.stokes_steps()
    S, S_ref = mic.download_stokes_vector("solution"), o.solve_direct()
    assert o.residual(S) < 1e-9
    for k in range(3):
        err = np.max(np.abs(S[k::3] - S_ref[k::3])) / np.max(np.abs(S_ref[k::3]))
        assert err < 1e-6, (k, err)
    mic.close()


def test_mixed_and_fp64_methods_share_one_context(eb):
    """Switching the V-cycle precision rebuilds the hierarchy; both reach the tolerance and the
    FP64 V-cycle is no weaker a preconditioner than the FP32 one."""
    model = marker_model(eb, "rift_small")
    o, mic, rep32, S = solve_case(eb, model, 1e-8)
    rep64 = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-8, precision="fp64")
    rep32b = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-8, precision="mixed")
    for r in (rep32, rep64, rep32b):
        assert r["status"] == 0 and r["rel_residual"] <= 1e-8, r
    assert rep64["iterations"] <= rep32["iterations"] + 2
    assert rep32b["iterations"] == rep32["iterations"]
    mic.close()


@pytest.mark.parametrize("gs_relax", [1e3, 1e20])
@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_fp32_gram_schmidt_matches_superlu(eb, case, gs_relax):
    """The mixed method's FP32 Gram-Schmidt (projection on FP32 copies of the basis below
    gs_relax x the target): at 1e20 every iteration takes that form (a residual gap left by the
    FP32 products makes the method restart from its iterate), and the solution still meets 1e-11
    and equals SuperLU's to 1e-6; gs_relax < 0 switches it off."""
    model = marker_model(eb, case)
    o = oracle_for(model)
    mic = gpu_ctx(eb, model)
    rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-11, max_iters=4000, gs_relax=gs_relax)
    assert rep["status"] == 0 and rep["rel_residual"] <= 1e-11, rep
    assert rep["relaxed_iterations"] > 0
    if gs_relax > 1e6:
        assert rep["relaxed_iterations"] == rep["iterations"], rep
    S = mic.download_stokes_vector("solution")
    S_ref = o.solve_direct()
    for comp in range(3):
        a, b = S[comp::3], S_ref[comp::3]
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max(), (comp, np.abs(a - b).max() / np.abs(b).max())
    off = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-11, max_iters=4000, gs_relax=-1.0)
    assert off["status"] == 0 and off["relaxed_iterations"] == 0, off
    fp64 = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-11, max_iters=4000, precision="fp64",
                                                              gs_relax=1e20)
    assert fp64["status"] == 0 and fp64["relaxed_iterations"] == 0, fp64   # plain method: never FP32
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_double_float_arnoldi_step_matches_the_fp64_step(eb, case):
    """The mixed method's Arnoldi step on FP32 pairs (double-float operator product and
    Gram-Schmidt, FP32 preconditioner input and output), with the FP32 products disabled
    (gs_relax tiny): against the FP64 Arnoldi step with the same FP32 V-cycle (gs_relax < 0),
    the same number of FGMRES iterations to within one (the reductions sum in another order)
    and the same solution to 1e-9 of each field's maximum at rtol 1e-11."""
    model = marker_model(eb, case)
    mic = gpu_ctx(eb, model)
    out = {}
    for name, relax in (("split", 1e-30), ("fp64_step", -1.0)):
        rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-11, max_iters=4000, gs_relax=relax)
        assert rep["status"] == 0 and rep["rel_residual"] <= 1e-11 and rep["relaxed_iterations"] == 0, rep
        out[name] = (rep["iterations"], mic.download_stokes_vector("solution"))
    print(f"\n{case}: FGMRES iterations, double-float step {out['split'][0]}, FP64 step {out['fp64_step'][0]}")
    assert abs(out["split"][0] - out["fp64_step"][0]) <= 1, out
    a, b = out["split"][1], out["fp64_step"][1]
    for comp in range(3):
        x, y = a[comp::3], b[comp::3]
        assert np.abs(x - y).max() <= 1e-9 * np.abs(y).max(), (comp, np.abs(x - y).max() / np.abs(y).max())
    mic.close()


def test_warm_start_rescales_pressure_to_the_new_system(eb):
    """A solve that starts from the solution of an earlier system: the pressure unknowns are
    p / pscale, and pscale = 2 etan0[1,1] / (xstpavg + ystpavg) changes between systems, so the
    start is rescaled to the new pscale.  Ten times the viscosity of the upper-left cell alone moves
    pscale by ten and the solution only near that corner, so the warm start's residual is small:
    to a loose tolerance (1e-4) it must need far fewer iterations than a cold start (an unscaled
    start, every pressure unknown off by ten, would not), and to 1e-10 both must reach the same
    solution."""
    model = marker_model(eb, "rift_small")
    mic = gpu_ctx(eb, model)
    mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-10)
    p0 = mic.pscale
    etan1 = model.grids["etan1"].copy(order="F")
    etan1[0, 0] *= 10.0
    mic.upload_grid("etan1", etan1)
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    assert mic.pscale == pytest.approx(10.0 * p0, rel=1e-6)
    warm4 = mic.solve_system(rtol=1e-4, use_initial_guess=True)   # from the first system's solution
    warm = mic.solve_system(rtol=1e-10, use_initial_guess=True)   # ... continued to 1e-10
    S_warm = mic.download_stokes_vector("solution")
    cold4 = mic.solve_system(rtol=1e-4)
    cold = mic.solve_system(rtol=1e-10)
    S_cold = mic.download_stokes_vector("solution")
    print(f"\nto 1e-4: warm start {warm4['iterations']} iterations, cold start {cold4['iterations']}")
    assert warm4["iterations"] <= 0.5 * cold4["iterations"], (warm4["iterations"], cold4["iterations"])
    assert warm["rel_residual"] <= 1e-10 and cold["rel_residual"] <= 1e-10
    for comp in range(3):
        a, b = S_warm[comp::3], S_cold[comp::3]
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max(), comp
    mic.close()
