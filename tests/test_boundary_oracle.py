"""The step-boundary oracle (rock properties, displacement-limited time step) against direct
numpy transcriptions of the reference's formulas."""
import numpy as np
import pytest

from boundary_cases import porosity_fields, rock_tables, sediment


@pytest.fixture(scope="module")
def B():
    from oracle import boundary
    boundary.build()
    return boundary


def markers(eb, M=3000, seed=5):
    rng = np.random.default_rng(seed)
    g = eb.synthetic.staggered_grid(np.linspace(0, 100e3, 11), np.linspace(0, 150e3, 16))
    mk = {"x": rng.uniform(-1e3, 101e3, M), "y": rng.uniform(0, 150e3, M), "matid": rng.integers(1, 5, M).astype(np.int16),
          "pr": rng.uniform(1e5, 4e9, M), "tk": rng.uniform(273.0, 1700.0, M), "inside": np.where(rng.random(M) < 0.95, 1, -1).astype(np.int8)}
    for k in ("rho", "rhocp", "kt", "ha"):
        mk[k] = rng.uniform(0, 1, M)
    mk.update(porosity_fields(M))
    return g, mk


def numpy_props(mk, mat_rho, mat_cp, mat_kt, dm, cm, km, Ttop, cpmax, sed=None):
    id_ = mk["matid"].astype(np.int64) - 1
    rs, a, b = mat_rho[id_, 0], mat_rho[id_, 1], mat_rho[id_, 2]
    T, P, y = mk["tk"], mk["pr"], mk["y"]
    rho = [rs * (1.0 - a * (T - 298.15)) * (1.0 + b * (P - 1e5)), rs * (1.0 - a * (T - Ttop)),
           rs * (1.0 - a * (T - 830.0))][dm]
    cp20 = mat_cp[id_]
    tc = T - 273.0
    cpw = np.minimum(cp20 * (0.953 + 2.29e-3 * tc - 2.835e-6 * tc ** 2 + 1.191e-9 * tc ** 3), cpmax)
    rhocp = rho * (cp20 if cm == 0 else cpw)
    k0, ka = mat_kt[id_, 0], mat_kt[id_, 1]
    k = [(k0 + ka / (T + 77.0)) * np.exp(0.00004 * P / 1e6), k0, k0 / (1.0 + ka * (T - Ttop) / Ttop),
         np.where(y > 110000.0, 39.25, k0), np.where(y > 110000.0, 0.1 * 2.25 * 1330.0 / 4.5, k0),
         np.where(k0 <= 20.0, 358.0 * (1.0227 * k0 - 1.882) * (1.0 / T - 0.00068) + 1.84, k0)][km]
    ha = a * T
    if sed is not None:
        ymud = np.interp(mk["x"], sed["topo_x"], sed["topo_y"])
        ysub = np.maximum(y - ymud, mk["max_burial_depth"])
        phi = mk["porosity_initial"] * np.exp(-(1.0 / mk["decay_depth"]) * ysub)
        s = np.isin(mk["matid"], sed["matids"])
        k = np.where(s, k * (1 - phi) + sed["conductivity_water"] * phi, k)
        rho = np.where(s, rho * (1 - phi) + sed["density_water"] * phi, rho)
        rhocp = np.where(s, rho * (cp20 * (1 - phi) + sed["heat_capacity_water"] * phi), rhocp)
    ins = mk["inside"] == 1
    return {n: np.where(ins, v, mk[n]) for n, v in (("rho", rho), ("rhocp", rhocp), ("kt", k), ("ha", ha))}


@pytest.mark.parametrize("dm,cm,km", [(d, c, k) for d in range(3) for c in range(2) for k in range(6)])
def test_rock_properties(eb, B, dm, cm, km):
    g, mk = markers(eb)
    tabs = rock_tables(4)
    got = B.rock_properties(mk, *tabs, dm, cm, km, 273.15, 1200.0)
    want = numpy_props(mk, *tabs, dm, cm, km, 273.15, 1200.0)
    for n in want:
        np.testing.assert_allclose(got[n], want[n], rtol=2e-15, atol=0, err_msg=n)


def test_rock_properties_porosity(eb, B):
    g, mk = markers(eb)
    tabs = rock_tables(4)
    sed = sediment(g)
    got = B.rock_properties(mk, *tabs, 0, 1, 0, 273.15, 1200.0, iuse_por=1, sed=sed)
    want = numpy_props(mk, *tabs, 0, 1, 0, 273.15, 1200.0, sed=sed)
    for n in want:
        np.testing.assert_allclose(got[n], want[n], rtol=1e-13, atol=0, err_msg=n)


@pytest.mark.parametrize("local", [0, 1])
def test_timestep_displacement_limit(eb, B, local):
    rng = np.random.default_rng(7)
    x = np.concatenate([[0.0], np.cumsum(rng.uniform(400.0, 1200.0, 30))])
    y = np.concatenate([[0.0], np.cumsum(rng.uniform(300.0, 900.0, 20))])
    g = eb.synthetic.staggered_grid(x, y)
    vx = rng.normal(0, 1e-9, (g.ynum + 1, g.xnum))
    vy = rng.normal(0, 1e-9, (g.ynum, g.xnum + 1))
    vx[3, 4] = 0.0
    dt_old, displ = 1e13, 0.4
    got = B.timestep_displacement_limit(g, vx, vy, displ, local, dt_old)
    if local == 0:
        want = min(dt_old, displ * g.xstpavg / np.abs(vx).max(), displ * g.ystpavg / np.abs(vy).max())
    else:
        xs, ys = g.xstp_b, g.ystp_b
        cx = np.concatenate([[xs[0]], np.minimum(xs[:-1], xs[1:]), [xs[-1]]])
        cy = np.concatenate([[ys[0]], np.minimum(ys[:-1], ys[1:]), [ys[-1]]])
        with np.errstate(divide="ignore"):
            lx = np.where(vx != 0, displ * cx[None, :] / np.abs(vx), np.inf)
            ly = np.where(vy != 0, displ * cy[:, None] / np.abs(vy), np.inf)
        want = min(dt_old, lx.min(), ly.min())
    assert got == want
