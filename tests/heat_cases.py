"""Shared inputs of the heat tests: analytic slabs and marker-averaged synthetic models."""
from __future__ import annotations

import numpy as np

F = np.asfortranarray
YEAR = 365.25 * 24 * 3600.0


def slab(eb, xnum=13, ynum=21, seed=0, kt=(2.5, 2.5), rhocp=2.5e6, T=(273.15, 1573.15), split=0.5, dt=1e4 * YEAR):
    """Conduction across a slab on a non-uniform grid: Dirichlet top and bottom, insulated sides,
    conductivity kt[0] above y = split*H and kt[1] below, no heat sources."""
    syn = eb.synthetic
    rng = np.random.default_rng(seed)
    x = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, xnum - 1))]) * 5e3
    y = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, ynum - 1))]) * 5e3
    g = syn.staggered_grid(x, y)
    X, Y = xnum, ynum
    H = y[-1] - y[0]
    Yb = np.repeat(y[:, None], X, axis=1)
    k = np.where(Yb < split * H, kt[0], kt[1])
    T0 = T[0] + (T[1] - T[0]) * (Yb - y[0]) / H
    gr = {"tk1": F(T0), "kt1": F(k), "rhocp1": F(np.full((Y, X), rhocp)), "hr1": F(np.zeros((Y, X))),
          "ha1": F(np.zeros((Y, X))), "rho1": F(np.full((Y, X), 3000.0)), "vx1": F(np.zeros((Y + 1, X))),
          "vy1": F(np.zeros((Y, X + 1))), "sxy2": F(np.zeros((Y, X))), "etas1": F(np.full((Y, X), 1e21)),
          "sxx2": F(np.zeros((Y - 1, X - 1))), "etan1": F(np.full((Y - 1, X - 1), 1e21)),
          "btopt": F(np.column_stack([np.full(X, T[0]), np.zeros(X)])),
          "bbottomt": F(np.column_stack([np.full(X, T[1]), np.zeros(X)])),
          "bleftt": F(np.column_stack([np.zeros(Y), np.ones(Y)])),
          "brightt": F(np.column_stack([np.zeros(Y), np.ones(Y)]))}
    params = syn.default_params(timestep=dt, max_temp_change=1e9, iuse_adiabatic_heating=0, iuse_shear_heating=0)
    params.update(syn.stokes_params())
    return syn.Model("slab", g, None, params, {}, gr)


def random_bcs(model, seed=1):
    """Mixed thermal BCs: random b1 and b2 in [0, 1] on every side."""
    rng = np.random.default_rng(seed)
    X, Y = model.grid.xnum, model.grid.ynum
    for name, n in (("btopt", X), ("bbottomt", X), ("bleftt", Y), ("brightt", Y)):
        model.grids[name] = F(np.column_stack([rng.uniform(200.0, 1500.0, n), rng.uniform(0.0, 1.0, n)]))
    return model


HEAT_GRIDS = ("tk1", "kt1", "rhocp1", "hr1", "ha1", "rho1", "etas1", "etan1")


def marker_heat_model(eb, name: str, **kw):
    """A synthetic rift whose heat and Stokes grids are the oracle's marker averages."""
    from oracle.oracle import OracleMIC
    sizes = {"rift_small": (101, 41), "rift_medium": (201, 81)}
    model = eb.synthetic.rift(*sizes[name], 4, **kw)
    o = OracleMIC(model)
    o.get_marker_inside_flags()
    o.initialize_bilinear_interpolation()
    o.interpolate_marker_heat_parameters_to_grid()
    o.interpolate_marker_stokes_parameters_to_grid()
    model.grids.update({k: F(o.gr[k]) for k in HEAT_GRIDS})
    model.params.update(max_temp_change=20.0, iuse_adiabatic_heating=1, iuse_shear_heating=1)
    return model
