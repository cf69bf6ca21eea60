"""GPU heat step against the oracle, through the C-ABI.

  - RHS terms RT1, the assembled system (exported as the reference's COO list and R) and
    the residual grid: identical to the oracle (the kernels keep the Julia operand order,
    no FMA contraction);
  - the solve: tk2 within 1e-9 of SuperLU's solution relative to max|T|, and the reference's
    (unscaled) system solved to a relative residual below 1e-10;
  - the adaptive heat loop: the same number of passes and integrated time as the oracle's
    loop, tk2 and dtk1 within 1e-9 relative.
"""
import numpy as np
import pytest

from heat_cases import marker_heat_model, random_bcs, slab

pytestmark = pytest.mark.gpu

INPUTS = ("tk1", "kt1", "rhocp1", "hr1", "ha1", "rho1", "vx1", "vy1", "sxy2", "etas1", "sxx2", "etan1",
          "btopt", "bbottomt", "bleftt", "brightt")


def gpu_ctx(eb, model):
    mic = eb.MarkerInCell(0)
    mic.set_grid(model.grid)
    mic.set_params(model.params)
    mic.heat = eb.heat_params(model.params)
    for k in INPUTS:
        mic.upload_grid(k, model.grids[k])
    return mic


def case(eb, name):
    if name == "slab":
        return slab(eb, kt=(2.0, 6.0))
    if name == "slab_mixed_bc":
        return random_bcs(slab(eb, xnum=17, ynum=11))
    return marker_heat_model(eb, name)


CASES = ["slab", "slab_mixed_bc", "rift_small", "rift_medium"]


@pytest.mark.parametrize("name", CASES)
def test_assembly_matches_oracle(eb, name):
    from oracle.heat import HeatOracle
    m = case(eb, name)
    o = HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    coo = o.build_system_of_equations()
    mic = gpu_ctx(eb, m)
    mic.calculate_heat_rhs_terms()
    assert np.array_equal(mic.download_grid("RT1"), o.gr["RT1"])
    mic.initialize_old_temperature_array()
    mic.build_heat_system(o.timestep_heat)
    for got, want in zip(mic.export_heat_coo(), coo):
        assert np.array_equal(got, want)
    mic.close()


@pytest.mark.parametrize("name", CASES)
def test_solve_matches_superlu(eb, name):
    from oracle.heat import HeatOracle
    m = case(eb, name)
    o = HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    o.discretize_and_solve()
    mic = gpu_ctx(eb, m)
    mic.calculate_heat_rhs_terms()
    mic.initialize_old_temperature_array()
    mic.build_heat_system(o.timestep_heat)
    rep = mic.solve_heat_system()
    assert rep["status"] == 0 and rep["rel_residual"] < 1e-10, rep
    T = mic.download_grid("tk2")
    want = o.gr["tk2"]
    assert np.max(np.abs(T - want)) <= 1e-9 * np.max(np.abs(want)), rep
    # residual grid on the GPU solution: the same formula as the oracle's, bit for bit
    mic.heat_residuals(o.timestep_heat)
    o.gr["tk2"][...] = T
    o.compute_residuals_temp()
    assert np.array_equal(mic.download_grid("rest"), o.gr["rest"])
    mic.close()


@pytest.mark.parametrize("name", ["slab_source", "rift_small"])
def test_heat_loop_matches_oracle(eb, name):
    from oracle.heat import HeatOracle
    # inputs whose passes stay clear of max|tk2 - tk0| == max_temp_change (the branch of the
    # reference's loop; at a tie, rounding decides whether a pass solves twice)
    if name == "slab_source":
        m = slab(eb, dt=1e5 * 365.25 * 24 * 3600.0)
        depth = np.linspace(0.0, 1.0, 21)[:, None] * np.ones((1, 13))
        m.grids["hr1"] = np.asfortranarray(1e-4 * (1.0 + 2.0 * depth ** 2))
        m.params["max_temp_change"] = 10.0
    else:
        m = case(eb, name)
        m.params["max_temp_change"] = 2.0
    o = HeatOracle(m)
    o.heat_step()
    mic = gpu_ctx(eb, m)
    mic.calculate_heat_rhs_terms()
    mic.initialize_old_temperature_array()
    rep = mic.run_conductive_heat_solver_loop()
    mic.calculate_grid_temp_change()
    assert rep["substeps"] == o.substeps and rep["solves"] == o.solves, rep
    assert rep["timestep_sum"] == pytest.approx(m.params["timestep"], rel=1e-12)
    assert rep["max_rel_residual"] < 1e-10
    scale = np.max(np.abs(o.gr["tk2"]))
    assert np.max(np.abs(mic.download_grid("tk2") - o.gr["tk2"])) <= 1e-9 * scale
    assert np.max(np.abs(mic.download_grid("dtk1") - o.gr["dtk1"])) <= 1e-9 * scale
    mic.close()


def test_bad_inputs_fail_loudly(eb):
    m = slab(eb)
    mic = gpu_ctx(eb, m)
    with pytest.raises(RuntimeError):
        mic.solve_heat_system()          # nothing assembled yet
    with pytest.raises(RuntimeError):
        mic.build_heat_system(0.0)       # non-positive step
    mic.close()
