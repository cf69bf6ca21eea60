"""Inputs of the step-boundary tests: rock tables, sediment porosity and markers."""
import json
import pathlib

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


def rock_golden_markers():
    """Markers at the conditions of the reference's rock-property known answers
    (tests/golden/rock_props_reference.json): material 1 for the heat capacity (density
    exactly 1, so rho cp = cp), material 2 for the Liao14 and material 3 for the
    Sekiguchi-Waples conductivity; temperatures in kelvin with the reference's offset."""
    g = json.loads((pathlib.Path(__file__).parent / "golden" / "rock_props_reference.json").read_text())
    off = g["celsius_to_kelvin_offset"]
    W, L, S = g["waples"], g["liao14"], g["sekiguchi_waples"]
    T, P, mat = [], [], []
    for tc in W["temperatures_celsius"]:
        T.append(tc + off); P.append(0.0); mat.append(1)
    for d in L["depths_m"]:
        T.append(off + L["gradient_c_per_km"] * (d / 1000.0)); P.append(L["density"] * L["gravity"] * d); mat.append(2)
    for tc in S["temperatures_celsius"]:
        T.append(tc + off); P.append(0.0); mat.append(3)
    M = len(T)
    mk = {"x": np.zeros(M), "y": np.zeros(M), "pr": np.array(P), "tk": np.array(T), "rho": np.zeros(M),
          "rhocp": np.zeros(M), "kt": np.zeros(M), "ha": np.zeros(M), "inside": np.ones(M, np.int8),
          "matid": np.array(mat, np.int16)}
    mat_rho = np.array([[1.0, 0.0, 0.0]] * 3)
    mat_cp = np.array([W["heat_capacity_at_20celsius"], 1000.0, 1000.0])
    mat_kt = np.array([[1.0, 0.0], [L["k0"], L["a"]], [S["k0"], 0.0]])
    n = (len(W["expected_cp"]), len(L["expected_k"]), len(S["expected_k"]))
    return g, mk, (mat_rho, mat_cp, mat_kt), n
