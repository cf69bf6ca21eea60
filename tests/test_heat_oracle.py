"""The heat oracle (C restatement of HeatRhs, HeatBuildManager, HeatResiduals and the heat
loop) against analytic solutions and structural properties of the reference's system."""
import numpy as np
import pytest

from heat_cases import YEAR, slab


@pytest.fixture(scope="module")
def H():
    from oracle import heat
    heat.build()
    return heat


def test_linear_geotherm_is_steady(eb, H):
    """Uniform conductivity, no sources: a linear profile between the Dirichlet values stays put."""
    m = slab(eb)
    o = H.HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    S = o.discretize_and_solve()
    assert o.residual(S) < 1e-13
    T0 = m.grids["tk1"]
    assert np.max(np.abs(o.gr["tk2"] - T0)) <= 1e-10 * np.max(T0)
    o.compute_residuals_temp()
    assert np.max(np.abs(o.gr["rest"])) <= 1e-12 * 2.5e6 * np.max(T0) / o.hp["timestep"]


def test_layered_slab_steady_state(eb, H):
    """Two conductivities, a long step: the discrete steady state carries the same flux across
    every row edge, so T follows the series sum of the edge resistances."""
    m = slab(eb, kt=(2.0, 6.0), dt=1e30)
    o = H.HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    o.discretize_and_solve()
    k = m.grids["kt1"][:, 3]
    dy = np.diff(m.grid.gridy_b)
    res = dy / ((k[:-1] + k[1:]) / 2.0)           # resistance of each row edge
    T = np.concatenate([[0.0], np.cumsum(res)]) / np.sum(res)
    T = 273.15 + (1573.15 - 273.15) * T
    for j in range(m.grid.xnum):
        np.testing.assert_allclose(o.gr["tk2"][:, j], T, rtol=1e-10)


def test_coo_structure(eb, H):
    m = slab(eb, xnum=9, ynum=7)
    o = H.HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    Li, Lj, Lv, R = o.build_system_of_equations()
    X, Y = 9, 7
    assert len(Li) == 5 * (X - 2) * (Y - 2) + 2 * (2 * (X - 2) + 2 * Y)
    assert np.all(np.diff(Li) >= 0)                  # rows in order (j outer, i inner)
    rhocp, dt = 2.5e6, o.hp["timestep"]
    A = o.matrix().toarray()
    for j in range(X):
        for i in range(Y):
            n = j * Y + i
            row = A[n]
            if i in (0, Y - 1) or j in (0, X - 1):
                assert row[n] == 1.0 and np.count_nonzero(row) <= 2
            else:                                    # conservation: the row sums to rhocp/dt
                assert abs(row.sum() - rhocp / dt) <= 1e-9 * row[n]


def test_rhs_terms(eb, H):
    rng = np.random.default_rng(3)
    m = slab(eb, xnum=8, ynum=6)
    X, Y = 8, 6
    G = m.grids
    for k in ("hr1", "ha1", "rho1", "sxy2", "etas1"):
        G[k] = np.asfortranarray(rng.uniform(0.5, 2.0, (Y, X)))
    for k in ("sxx2", "etan1"):
        G[k] = np.asfortranarray(rng.uniform(0.5, 2.0, (Y - 1, X - 1)))
    G["vx1"] = np.asfortranarray(rng.normal(0, 1, (Y + 1, X)))
    G["vy1"] = np.asfortranarray(rng.normal(0, 1, (Y, X + 1)))
    m.params.update(iuse_adiabatic_heating=1, iuse_shear_heating=1, gravity_x=0.3, gravity_y=9.81)
    o = H.HeatOracle(m)
    o.calculate_heat_rhs_terms()
    RT = G["hr1"].copy()
    for j in range(1, X - 1):
        for i in range(1, Y - 1):
            RT[i, j] += G["ha1"][i, j] * G["rho1"][i, j] * (
                0.3 * (G["vx1"][i, j] + G["vx1"][i + 1, j]) + 9.81 * (G["vy1"][i, j] + G["vy1"][i, j + 1])) / 2.0
            RT[i, j] += G["sxy2"][i, j] ** 2 / G["etas1"][i, j]
            RT[i, j] += (G["sxx2"][i - 1, j - 1] ** 2 / G["etan1"][i - 1, j - 1] + G["sxx2"][i, j - 1] ** 2 /
                         G["etan1"][i, j - 1] + G["sxx2"][i - 1, j] ** 2 / G["etan1"][i - 1, j] +
                         G["sxx2"][i, j] ** 2 / G["etan1"][i, j]) / 4.0
    np.testing.assert_array_equal(o.gr["RT1"], RT)


def test_heat_loop_substeps(eb, H):
    """A strong source makes the first pass exceed max_temp_change: the loop shortens its step
    and integrates exactly up to the main time step."""
    m = slab(eb, dt=1e5 * YEAR)
    m.grids["hr1"] = np.asfortranarray(np.full((21, 13), 1e-4))
    m.params["max_temp_change"] = 10.0
    o = H.HeatOracle(m)
    o.calculate_heat_rhs_terms()
    o.initialize_old_temperature_array()
    total = o.run_conductive_heat_solver_loop()
    assert o.substeps >= 2 and o.solves > o.substeps
    assert total == pytest.approx(m.params["timestep"], rel=1e-12)
    np.testing.assert_array_equal(o.gr["tk0"], o.gr["tk2"])
    o.calculate_grid_temp_change()
    np.testing.assert_array_equal(o.gr["dtk1"], o.gr["tk2"] - o.gr["tk1"])
