"""Inputs of the step-boundary tests: rock tables, sediment porosity and markers."""
import numpy as np


def rock_tables(nmat, seed=0):
    rng = np.random.default_rng(seed)
    mat_rho = np.column_stack([rng.uniform(1000.0, 3300.0, nmat), rng.uniform(1e-5, 4e-5, nmat),
                               rng.uniform(1e-12, 1e-11, nmat)])
    mat_cp = rng.uniform(750.0, 1250.0, nmat)
    k0 = rng.uniform(1.5, 5.0, nmat)
    k0[0] = 200.0  # above the SekiguchiWaples cut (20 W/m/K): kept as is
    mat_kt = np.column_stack([k0, rng.uniform(0.0, 500.0, nmat)])
    return mat_rho, mat_cp, mat_kt


def sediment(grid, seed=1):
    rng = np.random.default_rng(seed)
    tx = np.linspace(grid.xmin, grid.xmax, 57)
    ty = 12e3 + 2e3 * np.sin(tx / (grid.xmax - grid.xmin) * 6.0) + rng.uniform(-100.0, 100.0, tx.size)
    return {"matids": np.array([2, 3], np.int16), "topo_x": tx, "topo_y": ty, "conductivity_water": 0.6,
            "density_water": 1025.0, "heat_capacity_water": 4184.0}


def porosity_fields(M, seed=2):
    rng = np.random.default_rng(seed)
    return {"porosity_initial": rng.uniform(0.4, 0.65, M), "decay_depth": rng.uniform(1e3, 3e3, M),
            "max_burial_depth": rng.uniform(0.0, 2e3, M)}
