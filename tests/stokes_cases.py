"""Shared inputs of the Stokes tests: analytic boxes and marker-averaged synthetic models."""
from __future__ import annotations

import numpy as np

F = np.asfortranarray


def random_box(eb, xnum=21, ynum=17, seed=0, eta=1e21, rho=3000.0):
    """Uniform viscosity and density on a non-uniform grid, free slip on every side."""
    syn = eb.synthetic
    rng = np.random.default_rng(seed)
    x = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, xnum - 1))]) * 10e3
    y = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, ynum - 1))]) * 10e3
    g = syn.staggered_grid(x, y)
    X, Y = xnum, ynum
    gr = {"etas1": F(np.full((Y, X), eta)), "mus1": F(np.full((Y, X), 1e10)), "sxy1": F(np.zeros((Y, X))),
          "etan1": F(np.full((Y - 1, X - 1), eta)), "mun1": F(np.full((Y - 1, X - 1), 1e10)),
          "sxx1": F(np.zeros((Y - 1, X - 1))), "rho1": F(np.full((Y, X), rho)),
          "rho1_vy": F(np.full((Y, X + 1), rho)), "dilatation_grid": F(np.zeros((Y - 1, X - 1)))}
    gr.update(syn.velocity_bcs(g))
    params = syn.default_params()
    params.update(syn.stokes_params())
    return syn.Model("box", g, None, params, {}, gr)


def couette(model, U=1e-9):
    """Turn a box into plane Couette flow: lid at y = ymin moving at U, no slip at the bottom,
    the exact linear profile prescribed on the sides, no gravity."""
    g = model.grid
    X, Y = g.xnum, g.ynum
    H = g.ymax - g.ymin
    vex = lambda yy: U * (g.ymax - yy) / H
    model.params["gravity_y"] = 0.0
    model.params["pressure_bc"] = 0.0
    G = model.grids
    G["btopx"] = F(np.column_stack([np.full(X, 2 * U), -np.ones(X)]))
    G["bbottomx"] = F(np.column_stack([np.zeros(X), -np.ones(X)]))
    G["bleftx"] = F(np.column_stack([vex(g.gridy_vx), np.zeros(Y + 1)]))
    G["brightx"] = F(np.column_stack([vex(g.gridy_vx), np.zeros(Y + 1)]))
    G["bbottomy"] = F(np.column_stack([np.zeros(X + 1), np.zeros(X + 1)]))
    return vex


STOKES_GRIDS = ("etas1", "etan1", "mus1", "mun1", "sxy1", "sxx1", "rho1", "rho1_vy", "dilatation_grid")


def marker_model(eb, name: str, **kw):
    """A synthetic model whose Stokes input grids are the oracle's marker averages."""
    from oracle.oracle import OracleMIC
    if name == "rift_small":
        model = eb.synthetic.rift(101, 41, 4, **kw)
    elif name == "sinking_block":
        model = eb.synthetic.sinking_block(**kw)
    elif name == "rift_medium":
        model = eb.synthetic.rift(201, 81, 4, **kw)
    else:
        raise KeyError(name)
    o = OracleMIC(model)
    o.get_marker_inside_flags()
    o.initialize_bilinear_interpolation()
    o.interpolate_marker_stokes_parameters_to_grid()
    grids = {k: np.asfortranarray(o.gr[k]) for k in STOKES_GRIDS}
    model.grids.update(grids)
    return model


def bilinear_basic(grid, field, x, y):
    """Bilinear value of a basic-grid field (ynum x xnum) at (x, y)."""
    j = int(np.clip(np.searchsorted(grid.gridx_b, x, side="right") - 1, 0, grid.xnum - 2))
    i = int(np.clip(np.searchsorted(grid.gridy_b, y, side="right") - 1, 0, grid.ynum - 2))
    dx = (x - grid.gridx_b[j]) / (grid.gridx_b[j + 1] - grid.gridx_b[j])
    dy = (y - grid.gridy_b[i]) / (grid.gridy_b[i + 1] - grid.gridy_b[i])
    return ((1 - dx) * (1 - dy) * field[i, j] + dx * (1 - dy) * field[i, j + 1] + (1 - dx) * dy * field[i + 1, j]
            + dx * dy * field[i + 1, j + 1])
