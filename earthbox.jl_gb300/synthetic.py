"""Seeded synthetic inputs for the marker-in-cell hot path.

No dataset is involved: every model below is generated from a seed with the
shapes, spacings, marker densities and value ranges of the three marker-path
configurations:

* ``sinking_block``  -- 101x101 basic nodes over 500x500 km, 4x4 markers per
  cell (160,000 markers); background 1e21 Pa s / 3200 kg/m^3, a centred
  100x100 km block of 1e27 Pa s / 3300 kg/m^3; dt = 10 kyr.
* ``rift``           -- 500x160 km with 10 km of sticky air (1e18 Pa s, 1 kg/m^3),
  upper crust 0-20 km (2700, wet quartzite), lower crust 20-35 km (2850,
  plagioclase/anorthite), mantle (3300, dry olivine), power-law creep,
  Drucker-Prager friction 30 deg -> 15 deg by strain 1.0, cohesion 10 MPa,
  initial plastic strain U(0, 0.5) in a central 50 km zone, linear geotherm
  0 C -> 1330 C at 120 km, +-1 cm/yr extension.  ``rift(801, 201, 4)`` is the
  2.56M-marker case; ``rift(2001, 801, 5)`` the 40M-marker case.

Flow-law constants are the values of the reference's material registry
(src/material_library/registries/lithospheric_deformation/lithospheric_deformation_eb1.yml).
Marker placement follows MarkersRandomized.initialize! (outer loop over x,
inner over y: markers of a cell sit in runs along y) with independent x and y
jitter drawn from a Philox stream (the reference draws one value for both and
does not seed it).  Grid-side inputs of the gathers and of the advection
(velocities, spin, strain rates, stresses, pressure) are smooth analytic
fields with the magnitudes of a rifting model.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import _abi

YEAR = 365.25 * 24.0 * 3600.0


@dataclasses.dataclass
class Grid:
    xnum: int
    ynum: int
    gridx_b: np.ndarray
    gridy_b: np.ndarray
    xstp_b: np.ndarray
    ystp_b: np.ndarray
    gridx_vy: np.ndarray
    xstp_vy: np.ndarray
    gridy_vx: np.ndarray
    ystp_vx: np.ndarray
    xmin: float
    xmax: float
    ymin: float
    ymax: float
    xstpavg: float
    ystpavg: float


@dataclasses.dataclass
class Materials:
    mat_mu: np.ndarray
    mat_hr: np.ndarray
    mat_flow_type: np.ndarray
    mat_flow: np.ndarray      # (nmat, 12), Fortran order
    mat_plastic: np.ndarray   # (nmat, 6), Fortran order
    mat_rho: np.ndarray

    @property
    def nmat(self) -> int:
        return len(self.mat_mu)


@dataclasses.dataclass
class Model:
    name: str
    grid: Grid
    mats: Materials
    params: dict
    markers: dict             # name -> 1-D array (dtype of _abi.MARKER_DTYPE)
    grids: dict               # name -> 2-D Fortran-order array

    @property
    def marknum(self) -> int:
        return len(self.markers["x"])

    def copy(self) -> "Model":
        return Model(self.name, self.grid, self.mats, dict(self.params),
                     {k: v.copy() for k, v in self.markers.items()},
                     {k: np.asfortranarray(v.copy()) for k, v in self.grids.items()})


def staggered_grid(x: np.ndarray, y: np.ndarray) -> Grid:
    """Basic coordinates -> staggered vx/vy coordinates and spacings
    (restating VyGridTools / VxGridTools in src/staggered_grid/utils)."""
    def stag(b):
        n = len(b)
        stp = np.diff(b)
        g = np.empty(n + 1)
        g[0] = b[0] - stp[0] / 2.0
        g[n] = b[n - 1] + stp[n - 2] / 2.0
        g[1:n] = (b[1:] + b[:-1]) / 2.0
        s = np.empty(n)
        s[0] = stp[0]
        s[n - 1] = stp[n - 2]
        s[1:n - 1] = (b[2:] - b[:-2]) / 2.0
        return g, s
    gxvy, sxvy = stag(x)
    gyvx, syvx = stag(y)
    return Grid(len(x), len(y), x, y, np.diff(x), np.diff(y), gxvy, sxvy, gyvx, syvx,
                float(x[0]), float(x[-1]), float(y[0]), float(y[-1]),
                float((x[-1] - x[0]) / (len(x) - 1)), float((y[-1] - y[0]) / (len(y) - 1)))


def default_params(**kw) -> dict:
    p = dict(timestep=1e4 * YEAR, ntimestep=1, temperature_top=273.15, viscosity_min=1e18, viscosity_max=1e26,
             powerlaw_stress_min=1e4, yield_stress_min=0.0, yield_stress_max=1e12, gas_constant=8.314,
             iuse_viscous_strain_soft=0, vsoftfac=1.0, iuse_fluid_pressure_for_yield=0, y_sealevel=10e3,
             itype_global=0, no_yielding_in_mobile_wall=0, matid_sticky_air=-1, matid_mobile_wall=-1,
             matid_plate_extension=-1, plastic_healing_rate=0.0, subgrid_diff_coef_stress=1.0,
             subgrid_diff_coef_temp=1.0, iuse_melt_damage=0, iuse_serpentinization=0, iuse_topo=0,
             matid_sticky_air_rho=-1, matid_sticky_water_rho=-1, runge_kutta_order=4)
    p.update(kw)
    return p


def _markers_xy(rng, grid: Grid, mpc: int):
    """MarkersRandomized layout: mxnum x mynum markers, x outer / y inner."""
    W, H = grid.xmax - grid.xmin, grid.ymax - grid.ymin
    mx, my = (grid.xnum - 1) * mpc, (grid.ynum - 1) * mpc
    mxstep, mystep = W / mx, H / my
    ix = np.repeat(np.arange(1, mx + 1, dtype=np.float64), my)
    iy = np.tile(np.arange(1, my + 1, dtype=np.float64), mx)
    rx = rng.random(mx * my)
    ry = rng.random(mx * my)
    x = grid.xmin + ix * mxstep - mxstep / 2.0 + (rx - 0.5) * mxstep
    y = grid.ymin + iy * mystep - mystep / 2.0 + (ry - 0.5) * mystep
    return x, y


def _fields_common(rng, n: int, markers: dict) -> None:
    markers["pfailure"] = (rng.random(n) < 0.1).astype(np.float32)
    markers["dilatation"] = np.zeros(n, np.float32)
    markers["meltfrac"] = np.zeros(n)
    markers["melt_damage"] = np.ones(n)
    markers["serp_hr"] = np.zeros(n)
    for k in ("vx", "vy", "spin", "subgrid_dt", "strain_rate_plastic"):
        markers[k] = np.zeros(n)


def _analytic_grids(grid: Grid, v0: float, eta_ref: float, rho_ref: float, T0: float, T1: float,
                    depth_T1: float, y_surface: float, g: float = 9.81) -> dict:
    """Smooth grid-side inputs of the gathers and of the advection."""
    X, Y = grid.xnum, grid.ynum
    W, H = grid.xmax - grid.xmin, grid.ymax - grid.ymin
    xb, yb = grid.gridx_b, grid.gridy_b
    xc = grid.gridx_vy[1:X]        # pressure-node x (cell centres)
    yc = grid.gridy_vx[1:Y]
    kx, ky = 2.0 * math.pi / W, math.pi / H
    A = 0.3 * v0                    # cellular perturbation amplitude

    def F(a):
        return np.asfortranarray(a)
    # stream function psi = A/kx sin(kx x) sin(ky y) + extension: vx = dpsi/dy, vy = -dpsi/dx
    def vx_at(x, y):
        return v0 * (2.0 * (x - grid.xmin) / W - 1.0) + A * ky / kx * np.sin(kx * x) * np.cos(ky * y)
    def vy_at(x, y):
        return -2.0 * v0 / W * (y - (grid.ymin + 0.5 * H)) - A * np.cos(kx * x) * np.sin(ky * y)
    Yvx, Xvx = np.meshgrid(grid.gridy_vx, xb, indexing="ij")
    Yvy, Xvy = np.meshgrid(yb, grid.gridx_vy, indexing="ij")
    Yb, Xb = np.meshgrid(yb, xb, indexing="ij")
    Yp, Xp = np.meshgrid(yc, xc, indexing="ij")
    out = {}
    out["vx1"] = F(vx_at(Xvx, Yvx))
    out["vy1"] = F(vy_at(Xvy, Yvy))
    # spin 0.5 (dvy/dx - dvx/dy) of the perturbation
    out["esp"] = F(0.5 * (A * kx * np.sin(kx * Xb) * np.sin(ky * Yb) + A * ky * ky / kx * np.sin(kx * Xb) * np.sin(ky * Yb)))
    exx_p = 2.0 * v0 / W + A * ky * np.cos(kx * Xp) * np.cos(ky * Yp)
    out["exx"] = F(exx_p)
    out["exy"] = F(0.5 * A * (-ky * ky / kx + kx) * np.sin(kx * Xb) * np.sin(ky * Yb))
    # deviatoric stress vanishes in the sticky layer (y < y_surface)
    out["sxx2"] = F(np.where(Yp < y_surface, 0.0, 2.0 * eta_ref * exx_p))
    out["sxy2"] = F(np.where(Yb < y_surface, 0.0, 2.0 * eta_ref * out["exy"]))
    out["dsxx"] = F(0.05 * out["sxx2"])
    out["dsxy"] = F(0.05 * out["sxy2"])
    depth_p = np.clip(Yp - y_surface, 0.0, None)
    out["pr1"] = F(rho_ref * g * depth_p + 1e5 * np.cos(kx * Xp))
    depth_b = np.clip(Yb - y_surface, 0.0, None)
    Tb = T0 + (T1 - T0) * np.clip(depth_b / depth_T1, 0.0, 1.0)
    out["tk2"] = F(Tb)
    out["dtk1"] = F(0.5 * np.sin(kx * Xb) * np.sin(ky * Yb))
    out["btopt"] = F(np.column_stack([np.full(X, T0), np.zeros(X)]))
    out["bbottomt"] = F(np.column_stack([np.full(X, Tb[-1, 0]), np.zeros(X)]))
    out["bleftt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    out["brightt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    # transport grids start from plausible values so that empty nodes keep a backup
    for name, val in (("rho1", rho_ref), ("etas1", eta_ref), ("eta_flow", eta_ref), ("mus1", 3e10), ("sxy1", 0.0),
                      ("plastics", 0.0), ("cohesion_grid", 1e7), ("fric_degrees_grid", 30.0), ("tk1", T0),
                      ("kt1", 2.5), ("rhocp1", 2.5e6), ("hr1", 1e-6), ("ha1", 0.0)):
        out[name] = F(np.full((Y, X), val))
    for name, val in (("etan1", eta_ref), ("mun1", 3e10), ("sxx1", 0.0), ("plasticn", 0.0), ("dilatation_grid", 0.0),
                      ("extractable_meltfrac_grid", 0.0)):
        out[name] = F(np.full((Y - 1, X - 1), val))
    out["rho1_vy"] = F(np.full((Y, X + 1), rho_ref))
    # stress grids of the subgrid-stress step: interpolated marker stress, smooth
    out["sxy1"] = F(out["sxy2"] * 0.9)
    out["sxx1"] = F(out["sxx2"] * 0.9)
    return out


def velocity_bcs(grid: Grid, v_ext: float = 0.0, free_slip_bottom: bool = True) -> dict:
    """Velocity boundary-condition coefficient arrays (the reference's vel_comp
    arrays): ghost = b[:, 0] + b[:, 1] * interior.  Free slip on top and on the
    sides for the tangential component; the sides move outwards at v_ext and the
    bottom brings in the balancing inflow (zero when v_ext = 0)."""
    X, Y = grid.xnum, grid.ynum
    W, H = grid.xmax - grid.xmin, grid.ymax - grid.ymin
    F = np.asfortranarray
    v_in = -2.0 * v_ext * H / W            # upward (y grows with depth)
    out = {}
    out["btopx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    out["btopy"] = F(np.column_stack([np.zeros(X + 1), np.zeros(X + 1)]))
    out["bbottomx"] = F(np.column_stack([np.zeros(X), np.ones(X) if free_slip_bottom else -np.ones(X)]))
    out["bbottomy"] = F(np.column_stack([np.full(X + 1, v_in), np.zeros(X + 1)]))
    out["bleftx"] = F(np.column_stack([np.full(Y + 1, -v_ext), np.zeros(Y + 1)]))
    out["brightx"] = F(np.column_stack([np.full(Y + 1, v_ext), np.zeros(Y + 1)]))
    out["blefty"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    out["brighty"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    out["eii_plastic_pressure"] = F(np.zeros((Y - 1, X - 1)))
    for name, shape in (("RX1", (Y + 1, X)), ("RY1", (Y, X + 1)), ("RC1", (Y - 1, X - 1))):
        out[name] = F(np.zeros(shape))
    return out


def stokes_params(**kw) -> dict:
    """Scalar Stokes parameters (gravity, interface stabilisation, pressure BC, internal velocity zone off)."""
    p = dict(gravity_x=0.0, gravity_y=9.81, iuse_interface_stabilization=1, pressure_bc_mode=0, pressure_bc=1e5,
             bintern_zone=np.array([-1, 0, 0, 0, -1, 0, 0, 0], np.int64), bintern_velocity=np.zeros(8))
    p.update(kw)
    return p


def sinking_block(xnum: int = 101, ynum: int = 101, mpc: int = 4, seed: int = 1) -> Model:
    rng = np.random.Generator(np.random.Philox(seed))
    W = H = 500e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    x, y = _markers_xy(rng, grid, mpc)
    n = len(x)
    block = (np.abs(x - W / 2) <= 50e3) & (np.abs(y - H / 2) <= 50e3)
    matid = np.where(block, 2, 1).astype(np.int16)
    mats = Materials(
        mat_mu=np.array([1e10, 1e10]), mat_hr=np.zeros(2), mat_flow_type=np.array([0, 0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((2, 12))), mat_plastic=np.asfortranarray(np.zeros((2, 6))),
        mat_rho=np.array([3200.0, 3300.0]))
    mats.mat_flow[:, 0] = [1e21, 1e27]
    m = {"x": x, "y": y, "matid": matid}
    m["rho"] = np.where(block, 3300.0, 3200.0)
    m["eta"] = np.where(block, 1e27, 1e21)
    m["eta_flow"] = m["eta"].copy()
    m["cohesion"] = np.zeros(n)
    m["fric"] = np.zeros(n)
    m["fric_ini"] = np.zeros(n)
    m["preexp"] = np.zeros(n)
    m["sxx"] = rng.normal(0.0, 1e5, n)
    m["sxy"] = rng.normal(0.0, 1e5, n)
    m["exx"] = rng.normal(0.0, 1e-15, n)
    m["exy"] = rng.normal(0.0, 1e-15, n)
    m["pr"] = 3200.0 * 9.81 * y
    m["sr_ratio"] = np.ones(n)
    m["gii"] = np.zeros(n)
    m["strain_plastic"] = np.zeros(n)
    m["tk"] = 273.15 + 1000.0 * y / H
    m["kt"] = np.full(n, 3.0)
    m["rhocp"] = m["rho"] * 1000.0
    m["ha"] = 3e-5 * m["tk"]
    _fields_common(rng, n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=1e-2 / YEAR, eta_ref=1e21, rho_ref=3200.0, T0=273.15, T1=1273.15,
                            depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    params = default_params(timestep=1e4 * YEAR, viscosity_min=1e18, viscosity_max=1e28, ntimestep=1)
    params.update(stokes_params())
    return Model("sinking_block", grid, mats, params, m, grids)


def rift(xnum: int = 801, ynum: int = 201, mpc: int = 4, seed: int = 2, width: float = 500e3) -> Model:
    rng = np.random.Generator(np.random.Philox(seed))
    W, H, air = width, 160e3, 10e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    x, y = _markers_xy(rng, grid, mpc)
    n = len(x)
    depth = y - air
    matid = np.full(n, 4, np.int16)
    matid[depth < 35e3] = 3
    matid[depth < 20e3] = 2
    matid[depth < 0.0] = 1
    # registry values (lithospheric_deformation_eb1.yml): air, wet quartzite, anorthite, dry olivine
    nmat = 4
    mat_flow = np.zeros((nmat, 12))
    mat_flow[0, 0] = 1e18
    mat_flow[1, [1, 2, 3, 4]] = [8.57e-4, 4.0, 223.0, 0.0]
    mat_flow[2, [1, 2, 3, 4]] = [3.57e3, 3.0, 345.0, 38.0]
    mat_flow[3, [1, 2, 3, 4]] = [6.51e5, 3.5, 530.0, 13.0]
    mat_flow[3, [5, 6, 7, 8]] = [2.5e7, 1.0, 2.0, 9100.0]
    mat_flow[3, [9, 10, 11]] = [1.04e-2, 375.0, 6.0]
    sin30, sin15 = math.sin(math.radians(30.0)), math.sin(math.radians(15.0))
    mat_plastic = np.zeros((nmat, 6))
    mat_plastic[1:, :] = [10e6, 10e6, sin30, sin15, 0.0, 1.0]
    mats = Materials(
        mat_mu=np.array([1e20, 3.6e10, 4.0e10, 6.6e10]), mat_hr=np.array([0.0, 1.8e-6, 0.5e-6, 0.0]),
        mat_flow_type=np.array([0, 1, 1, 1], np.int64), mat_flow=np.asfortranarray(mat_flow),
        mat_plastic=np.asfortranarray(mat_plastic), mat_rho=np.array([1.0, 2700.0, 2850.0, 3300.0]))
    rho_of = mats.mat_rho
    m = {"x": x, "y": y, "matid": matid}
    mi = matid.astype(np.int64) - 1
    m["rho"] = rho_of[mi].copy()
    T = 273.15 + 1330.0 * np.clip(depth / 120e3, 0.0, 1.0)
    m["tk"] = T
    rock = matid > 1
    m["fric_ini"] = np.where(rock, sin30, 0.0)
    m["strain_plastic"] = np.where(rock & (np.abs(x - W / 2) < 25e3), rng.uniform(0.0, 0.5, n), 0.0)
    m["cohesion"] = np.where(rock, 10e6, 0.0)
    m["fric"] = m["fric_ini"].copy()
    m["eta"] = np.where(rock, 10.0 ** rng.uniform(20.0, 24.0, n), 1e18)
    m["eta_flow"] = m["eta"] * np.where(rock, 10.0 ** rng.uniform(0.0, 0.5, n), 1.0)
    m["preexp"] = mat_flow[mi, 1].copy()
    m["sxx"] = np.where(rock, rng.normal(0.0, 5e6, n), 0.0)
    m["sxy"] = np.where(rock, rng.normal(0.0, 5e6, n), 0.0)
    v0 = 1e-2 / YEAR
    m["exx"] = 2.0 * v0 / W * (1.0 + 0.3 * rng.normal(0.0, 1.0, n))
    m["exy"] = 0.3 * 2.0 * v0 / W * rng.normal(0.0, 1.0, n)
    m["pr"] = np.where(rock, 2900.0 * 9.81 * np.clip(depth, 0.0, None), 0.0) + 1e5
    m["sr_ratio"] = rng.uniform(0.8, 1.2, n)
    m["gii"] = rng.uniform(0.0, 1.0, n)
    m["kt"] = np.where(rock, 2.5, 200.0)
    m["rhocp"] = m["rho"] * np.where(rock, 800.0, 100.0)
    m["ha"] = 3e-5 * T
    _fields_common(rng, n, m)
    grids = _analytic_grids(grid, v0=v0, eta_ref=1e22, rho_ref=2900.0, T0=273.15, T1=1603.15, depth_T1=120e3,
                            y_surface=air)
    grids.update(velocity_bcs(grid, v_ext=0.5 * v0))
    params = default_params(timestep=1e4 * YEAR, y_sealevel=air, matid_sticky_air=1)
    params.update(stokes_params())
    return Model(f"rift_{xnum}x{ynum}_{mpc}", grid, mats, params, m, grids)


def circles(n: int = 1025, ncircles: int = 200, seed: int = 4, width: float = 1000e3) -> Model:
    """Grid-only Stokes benchmark: a square n x n-node box (eta = 1e21, rho = 3300) with
    `ncircles` seeded circular inclusions, r ~ U(5, 20) km, log10 eta ~ U(18, 27) and
    density contrast ~ U(-100, 100) kg/m^3; free slip on every side, purely viscous
    (shear modulus 1e40).  Later circles overwrite earlier ones where they overlap.
    Viscosity and density are evaluated at each grid's own nodes (basic, pressure, vy)."""
    rng = np.random.Generator(np.random.Philox(seed))
    x = np.linspace(0.0, width, n)
    grid = staggered_grid(x, x.copy())
    X = Y = n
    cx = rng.uniform(0.0, width, ncircles)
    cy = rng.uniform(0.0, width, ncircles)
    r = rng.uniform(5e3, 20e3, ncircles)
    leta = rng.uniform(18.0, 27.0, ncircles)
    drho = rng.uniform(-100.0, 100.0, ncircles)

    def paint(xs, ys):
        Yg, Xg = np.meshgrid(ys, xs, indexing="ij")
        eta = np.full(Yg.shape, 1e21)
        rho = np.full(Yg.shape, 3300.0)
        for k in range(ncircles):
            inside = (Xg - cx[k]) ** 2 + (Yg - cy[k]) ** 2 <= r[k] ** 2
            eta[inside] = 10.0 ** leta[k]
            rho[inside] = 3300.0 + drho[k]
        return np.asfortranarray(eta), np.asfortranarray(rho)

    xb, yb = grid.gridx_b, grid.gridy_b
    xp, yp = grid.gridx_vy[1:X], grid.gridy_vx[1:Y]
    etas, rho = paint(xb, yb)
    etan, _ = paint(xp, yp)
    _, rho_vy = paint(grid.gridx_vy, yb)
    F = np.asfortranarray
    gr = {"etas1": etas, "etan1": etan, "rho1": rho, "rho1_vy": rho_vy,
          "mus1": F(np.full((Y, X), 1e40)), "mun1": F(np.full((Y - 1, X - 1), 1e40)),
          "sxy1": F(np.zeros((Y, X))), "sxx1": F(np.zeros((Y - 1, X - 1))),
          "dilatation_grid": F(np.zeros((Y - 1, X - 1)))}
    gr.update(velocity_bcs(grid))
    params = default_params()
    params.update(stokes_params())
    return Model(f"circles_{n}", grid, None, params, {}, gr)


def rayleigh_taylor(xnum: int = 51, ynum: int = 51, mpc: int = 5) -> Model:
    """The reference's Rayleigh-Taylor instability benchmark (Ramberg 1968), as configured in
    src/benchmarks/models/rayleigh_taylor_instability/{model,materials}.yml and the benchmark
    material library: an 8 x 3 km uniform grid, 5 x 5 markers per cell on a regular lattice, a
    dense weak layer (3000 kg/m^3, 1e13 Pa s) over a light viscous one (2900 kg/m^3, 1e19 Pa s)
    with the interface at 1500 m depth, shear modulus 1e20 Pa, a 100 kyr time step, no slip on
    top and bottom and free slip on the sides, pressure fixed at the upper-left cell, interface
    stabilisation off.  Material ids follow the marker's depth before the perturbation; every
    marker is then moved up by cos(2 pi (x - xsize/2) / lambda) A (markers/utils/RayleighTaylor.jl),
    lambda = 4 km, A = 10 m, so the interface peaks at x = xsize/2."""
    W, H, h1, lam, amp = 8000.0, 3000.0, 1500.0, 4000.0, 10.0
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y0 = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    matid = np.where(y0 >= h1, 2, 1).astype(np.int16)
    y = y0 - np.cos(2.0 * math.pi * (x - W / 2.0) / lam) * amp
    n = len(x)
    rho_l, eta_l = np.array([3000.0, 2900.0]), np.array([1e13, 1e19])
    mats = Materials(
        mat_mu=np.array([1e20, 1e20]), mat_hr=np.zeros(2), mat_flow_type=np.array([0, 0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((2, 12))), mat_plastic=np.asfortranarray(np.zeros((2, 6))),
        mat_rho=rho_l.copy())
    mats.mat_flow[:, 0] = eta_l
    k = matid - 1
    m = {"x": x, "y": y, "matid": matid, "rho": rho_l[k], "eta": eta_l[k], "eta_flow": eta_l[k].copy()}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    m["sr_ratio"] = np.ones(n)
    m["tk"] = np.full(n, 273.0)
    m["kt"] = np.full(n, 2e-6)
    m["rhocp"] = m["rho"] * 1000.0
    m["ha"] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e19, rho_ref=2900.0, T0=273.0, T1=273.0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid, 0.0, free_slip_bottom=False))
    grids["btopx"] = np.asfortranarray(np.column_stack([np.zeros(xnum), -np.ones(xnum)]))  # no slip on top
    params = default_params(timestep=1e5 * YEAR, viscosity_min=1e13, viscosity_max=1e25, ntimestep=1,
                            temperature_top=273.0)
    params.update(stokes_params(iuse_interface_stabilization=0, pressure_bc=0.0))
    return Model("rayleigh_taylor", grid, mats, params, m, grids)


def stress_buildup(xnum: int = 51, ynum: int = 51, mpc: int = 4) -> Model:
    """The reference's viscoelastic stress-buildup benchmark, as configured in
    src/benchmarks/models/viscoelastic_stress_buildup/{model,materials}.yml and the benchmark
    material library (Viscoelastic_Material): a 100 x 100 km uniform grid, 4 x 4 markers per
    cell on a regular lattice, one isoviscous material (1e21 Pa s, shear modulus 1e10 Pa,
    4000 kg/m^3), no gravity, a 10 yr time step, and pure shear at 1e-14 1/s
    (PureShearDeformationBC.jl with VelocityFromStrainRate.jl: full extension velocity
    strain rate x width, half of it out through each side and in through the top and the
    bottom, tangential components free).  The deviatoric stress builds up as a Maxwell body:
    sxx(t) = 2 eta edot (1 - exp(-mu t / eta))."""
    W = H = 100e3
    edot = 1e-14
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    eta, mu, rho = 1e21, 1e10, 4000.0
    mats = Materials(
        mat_mu=np.array([mu]), mat_hr=np.zeros(1), mat_flow_type=np.array([0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((1, 12))), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([rho]))
    mats.mat_flow[0, 0] = eta
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, rho), "eta": np.full(n, eta),
         "eta_flow": np.full(n, eta)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    m["sr_ratio"] = np.ones(n)
    m["tk"] = np.full(n, 273.0)
    m["kt"] = np.full(n, 2.0)
    m["rhocp"] = m["rho"] * 1000.0
    m["ha"] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=eta, rho_ref=rho, T0=273.0, T1=273.0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    v = edot * W
    F = np.asfortranarray
    grids["btopy"] = F(np.column_stack([np.full(xnum + 1, 0.5 * v), np.zeros(xnum + 1)]))
    grids["bbottomy"] = F(np.column_stack([np.full(xnum + 1, -0.5 * v), np.zeros(xnum + 1)]))
    grids["bleftx"] = F(np.column_stack([np.full(ynum + 1, -0.5 * v), np.zeros(ynum + 1)]))
    grids["brightx"] = F(np.column_stack([np.full(ynum + 1, 0.5 * v), np.zeros(ynum + 1)]))
    params = default_params(timestep=10.0 * YEAR, viscosity_min=1e18, viscosity_max=1e25, ntimestep=1,
                            temperature_top=273.0)
    params.update(stokes_params(iuse_interface_stabilization=0, pressure_bc=0.0, gravity_y=0.0))
    return Model("stress_buildup", grid, mats, params, m, grids)


def channel_flow_non_newtonian(xnum: int = 51, ynum: int = 21, mpc: int = 5) -> Model:
    """The reference's non-Newtonian channel-flow benchmark, as configured in
    src/benchmarks/models/channel_flow_non_newtonian/{model,materials}.yml and the benchmark
    material library (NonNewtonianMaterialChannelFlowBenchmark): a 10 x 10 km vertical channel on
    51 x 21 nodes with 5 x 5 markers per cell on a regular lattice, one dislocation-creep material
    (5e-20 1/s/MPa^n, n = 3, no activation energy or volume; 3200 kg/m^3; shear modulus 1e21 Pa),
    no gravity, the nodal plasticity loop with one Picard iteration per step, and a 100 kyr time
    step limited to half a cell of marker displacement.  VerticalChannelFlowNonNewtonianBC.jl:
    pressure 1e9 Pa on the top row of pressure cells and 0 on the bottom row (pressure condition
    mode 1), zero vertical gradients of vx and vy through the top and bottom (VerticalChannelBC.jl),
    no slip on both sides."""
    W = H = 10e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    mat_flow = np.zeros((1, 12))
    mat_flow[0, [1, 2, 3, 4]] = [5e-20, 3.0, 0.0, 0.0]
    mats = Materials(
        mat_mu=np.array([1e21]), mat_hr=np.zeros(1), mat_flow_type=np.array([1], np.int64),
        mat_flow=np.asfortranarray(mat_flow), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([3200.0]))
    T0 = 273.15
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, 3200.0), "eta": np.full(n, 1e21),
         "eta_flow": np.full(n, 1e21), "preexp": np.full(n, 5e-20), "sr_ratio": np.ones(n), "tk": np.full(n, T0),
         "kt": np.full(n, 3.0), "rhocp": np.full(n, 3200.0 * 3000.0), "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e21, rho_ref=3200.0, T0=T0, T1=T0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    grids["btopx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["btopy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bbottomy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bleftx"] = F(np.zeros((Y + 1, 2)))
    grids["brightx"] = F(np.zeros((Y + 1, 2)))
    grids["blefty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["brighty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    params = default_params(timestep=1e5 * YEAR, viscosity_min=1e18, viscosity_max=1e25, powerlaw_stress_min=1e4,
                            itype_global=1, temperature_top=T0, ntimestep=1)
    params.update(stokes_params(pressure_bc_mode=1, pressure_bc=1e9, gravity_y=0.0, iuse_interface_stabilization=0))
    params["marker_cell_displ_max"] = 0.5
    return Model("channel_flow_non_newtonian", grid, mats, params, m, grids)


def channel_flow_velocity(x: np.ndarray, width: float, ydim: float, top_pressure: float, pre_exponential_dc: float,
                          n: float) -> np.ndarray:
    """Analytic vertical velocity of pressure-driven power-law flow between no-slip walls, as the
    reference's benchmark evaluates it (post_processing/analytical/ChannelFlowNonNewtonianManager.jl):
    C1 = 2 A / (1e6)^n from the MPa-based pre-exponential factor A, dp/dy = -top_pressure / ydim and
    v(x) = C1 / (n + 1) (-dp/dy)^n ((W/2)^(n+1) - (x - W/2)^(n+1)) (m/s, positive downwards)."""
    c1 = pre_exponential_dc * 2.0 / (1e6 ** n)
    grad = -top_pressure / ydim
    return c1 / (n + 1.0) * (-grad) ** n * ((width / 2.0) ** (n + 1.0) - np.abs(x - width / 2.0) ** (n + 1.0))


def solid_body_rotation(xnum: int = 51, ynum: int = 51, mpc: int = 5) -> Model:
    """The reference's solid-body-rotation benchmark, as configured in
    src/benchmarks/models/solid_body_rotation/{model,materials}.yml and the benchmark material
    library (MaterialForSolidBodyRotation): a 50 x 50 km box on 51 x 51 nodes with 5 x 5 markers per
    cell on a regular lattice, one isoviscous material (1e19 Pa s, shear modulus 1e20 Pa, 3000 kg/m^3,
    1000 J/kg/K, conductivity 2e-6 W/m/K), 727 C everywhere but the temperature wave
    (TemperatureWave.jl: 1500 K where 0.4 <= x/xsize <= 0.6 and 0.1 <= y/ysize <= 0.3), the
    kinematic velocity of solid_body_rotation_velocity (3.1536 cm/yr at the box's half width),
    SolidBodyRotationBC.jl's thermal conditions (zero flux through the top and the bottom, 727 C on
    both sides), subgrid temperature diffusion on and subgrid stress diffusion off, and a
    55344.0275 yr time step: one rotation takes 90 steps."""
    W = H = 50e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    T0 = 727.0 + 273.15
    T = np.full(n, T0)
    T[(0.4 <= x / W) & (x / W <= 0.6) & (0.1 <= y / H) & (y / H <= 0.3)] = 1500.0
    mats = Materials(
        mat_mu=np.array([1e20]), mat_hr=np.zeros(1), mat_flow_type=np.array([0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((1, 12))), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([3000.0]))
    mats.mat_flow[0, 0] = 1e19
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, 3000.0), "eta": np.full(n, 1e19),
         "eta_flow": np.full(n, 1e19), "sr_ratio": np.ones(n), "tk": T, "kt": np.full(n, 2e-6),
         "rhocp": np.full(n, 3000.0 * 1000.0), "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e19, rho_ref=3000.0, T0=T0, T1=T0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    grids["btopt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bleftt"] = F(np.column_stack([np.full(Y, T0), np.zeros(Y)]))
    grids["brightt"] = F(np.column_stack([np.full(Y, T0), np.zeros(Y)]))
    vx1, vy1 = solid_body_rotation_velocity(grid, 3.1536e-2 / YEAR)
    grids["vx1"], grids["vy1"] = vx1, vy1
    params = default_params(timestep=55344.0275 * YEAR, viscosity_min=1e18, viscosity_max=1e25, temperature_top=T0,
                            subgrid_diff_coef_stress=0.0, subgrid_diff_coef_temp=1.0)
    params.update(stokes_params(gravity_y=0.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=20.0, iuse_adiabatic_heating=0, iuse_shear_heating=0, iuse_heat=1,
                  velocity_rotation=3.1536e-2 / YEAR)
    return Model("solid_body_rotation", grid, mats, params, m, grids)


def solid_body_rotation_velocity(grid: Grid, vrotation: float) -> tuple:
    """Kinematics.solid_body_rotation! (src/kinematics/Kinematics.jl): the staggered velocities
    of a rigid rotation about the box centre, vrotation at half the box width:
    vx1[i, j] = -vrotation ((i - 1.5) dy - ysize/2) / (xsize/2) and
    vy1[i, j] = vrotation ((j - 1.5) dx - xsize/2) / (xsize/2) (1-based i, j, mean spacings)."""
    X, Y = grid.xnum, grid.ynum
    W, H = grid.xmax - grid.xmin, grid.ymax - grid.ymin
    i = np.arange(1, Y + 2, dtype=np.float64)[:, None]
    j = np.arange(1, X + 1, dtype=np.float64)[None, :]
    dy = ((i - 1.0) - 0.5) * grid.ystpavg - H / 2.0
    vx1 = np.broadcast_to(-vrotation * (dy / (W / 2.0)), (Y + 1, X))
    i = np.arange(1, Y + 1, dtype=np.float64)[:, None]
    j = np.arange(1, X + 2, dtype=np.float64)[None, :]
    dx = (j - 1.0 - 0.5) * grid.xstpavg - W / 2.0
    vy1 = np.broadcast_to(vrotation * (dx / (W / 2.0)), (Y, X + 1))
    return np.asfortranarray(vx1), np.asfortranarray(vy1)


def couette_flow_viscous_heating(xnum: int = 51, ynum: int = 11, mpc: int = 5) -> Model:
    """The reference's Couette-flow viscous-heating benchmark, as configured in
    src/benchmarks/models/couette_flow_viscous_heating/{model,materials}.yml and the benchmark
    material library (TempDependentViscosityCouetteFlowBenchmark): a 30 x 12.5 km vertical shear
    zone on 51 x 11 nodes with 5 x 5 markers per cell on a regular lattice, the
    temperature-dependent Couette flow law (mat_flow_type 4: 1e15 Pa s, 150 kJ/mol about the left
    wall's 727 C), 3000 kg/m^3, 1000 J/kg/K, conductivity 2 W/m/K, shear heating on,
    VerticalCouetteFlowBC.jl: the open channel of VerticalChannelBC.jl with no pressure drop, no
    slip on the left wall, vy ghost = 6.3072 cm/yr - vy interior on the right wall
    (NoSlipBC.set_vy_for_no_slip_with_shear_at_right_boundary!), zero vertical temperature
    gradient through the top and the bottom, 727 C on the left wall and no heat flux through the
    right one; nodal plasticity loop with one Picard iteration, harmonic normal viscosity, and a
    5 Myr time step limited to five cells of marker displacement."""
    W, H = 30e3, 12.5e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    T0 = 727.0 + 273.15
    flow = np.zeros((1, 17))
    flow[0, 12], flow[0, 13] = 1e15, 150.0
    mats = Materials(
        mat_mu=np.array([1e20]), mat_hr=np.zeros(1), mat_flow_type=np.array([4], np.int64),
        mat_flow=np.asfortranarray(flow), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([3000.0]))
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, 3000.0), "eta": np.full(n, 1e21),
         "eta_flow": np.full(n, 1e21), "sr_ratio": np.ones(n), "tk": np.full(n, T0), "kt": np.full(n, 2.0),
         "rhocp": np.full(n, 3000.0 * 1000.0), "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e21, rho_ref=3000.0, T0=T0, T1=T0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    vshear = 6.3072e-2 / YEAR
    grids["btopx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["btopy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bbottomy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bleftx"] = F(np.zeros((Y + 1, 2)))
    grids["brightx"] = F(np.zeros((Y + 1, 2)))
    grids["blefty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["brighty"] = F(np.column_stack([np.full(Y, vshear), -np.ones(Y)]))
    grids["btopt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bleftt"] = F(np.column_stack([np.full(Y, T0), np.zeros(Y)]))
    grids["brightt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    params = default_params(timestep=5e6 * YEAR, viscosity_min=1e18, viscosity_max=1e25, temperature_top=T0,
                            itype_global=1, ntimestep=1, temperature_bottom=T0, temperature_left=T0)
    params.update(stokes_params(pressure_bc_mode=1, pressure_bc=0.0, gravity_y=0.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=10.0, iuse_adiabatic_heating=0, iuse_shear_heating=1, iuse_heat=1,
                  marker_cell_displ_max=5.0)
    return Model("couette_flow_viscous_heating", grid, mats, params, m, grids)


def couette_temperature_profile(t_left: float, t_right: float, width: float, activation_energy: float,
                                gas_constant: float = 8.314, npoints: int = 100) -> tuple:
    """Steady temperature across a Couette shear zone with the temperature-dependent viscosity,
    as the reference's benchmark evaluates it (post_processing/analytical/
    CouetteFlowViscousHeatingManager.jl, after Gerya 2010): phi1 = exp(Ea (T_right - T_left) /
    (R T_left^2)); the Brinkman number from the bisection on b in [1e-6, 10] with
    Br = b^2/2 (1 - tanh(b/2)^2) and phi1 = b^2 / (2 Br); then for phi from 1 to phi1 the
    position x(phi) and T = T_left + log(phi) R T_left^2 / Ea.  Returns (x m, T K)."""
    def br_of(b):
        return b ** 2.0 / 2.0 * (1.0 - ((math.exp(b) - 1.0) / (math.exp(b) + 1.0)) ** 2.0)

    def phi_of(b, br):
        return b ** 2.0 / 2.0 / br
    phi1 = math.exp(activation_energy * (t_right - t_left) / gas_constant / t_left ** 2)
    lo, hi = 1e-6, 10.0
    br, ph = 0.0, 0.0
    if phi_of(lo, br_of(lo)) - phi1 <= 0.0 <= phi_of(hi, br_of(hi)) - phi1:
        d = 1e6
        while abs(d) > 1e-6:
            b = (lo + hi) / 2.0
            br = br_of(b)
            ph = phi_of(b, br)
            d = ph - phi1
            if d <= 0.0:
                lo = b
            else:
                hi = b
    phi1 = ph
    xs, ts = np.zeros(npoints), np.zeros(npoints)
    dphi = (phi1 - 1.0) / (npoints - 1)
    for j in range(npoints):
        phi = 1.0 + j * dphi
        c = math.sqrt(2.0 * br * (phi1 - phi))
        bb = math.sqrt(2.0 * br * phi1)
        dd = math.sqrt(2.0 * br * (phi1 - 1.0))
        xs[j] = width * (1.0 / math.sqrt(2.0 * br * phi1)) * math.log((dd + bb) / (dd - bb) * ((c - bb) / (c + bb)))
        ts[j] = t_left + math.log(phi) * gas_constant * t_left ** 2.0 / activation_energy
    return xs, ts


def channel_flow_variable_conductivity(xnum: int = 51, ynum: int = 11, mpc: int = 5) -> Model:
    """The reference's variable-conductivity channel-flow benchmark, as configured in
    src/benchmarks/models/channel_flow_variable_conductivity/{model,materials}.yml and the
    benchmark material library (ConstantViscosityChannelVariableThermalConductivity): a 30 x 12.5 km
    vertical channel on 51 x 11 nodes with 5 x 5 markers per cell on a regular lattice that do not
    move (NoMotion), an isoviscous material (1e19 Pa s, 3000 kg/m^3, 1000 J/kg/K) with the
    temperature-dependent conductivity k = k0 / (1 + a (T - T_top) / T_top), k0 = 8 W/m/K, a = 1
    (rock-property conductivity model 2; params["rock_tables"] holds the tables), shear heating on,
    VerticalChannelFlowShearHeatingBC.jl: the open channel with 3e7 Pa on the top row of pressure
    cells, no slip on both walls, 25 C on both walls and zero vertical temperature gradient through
    the top and the bottom; nodal plasticity loop with one Picard iteration, 100 kyr steps."""
    W, H = 30e3, 12.5e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    T0 = 25.0 + 273.15
    mats = Materials(
        mat_mu=np.array([1e20]), mat_hr=np.zeros(1), mat_flow_type=np.array([0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((1, 12))), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([3000.0]))
    mats.mat_flow[0, 0] = 1e19
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, 3000.0), "eta": np.full(n, 1e19),
         "eta_flow": np.full(n, 1e19), "sr_ratio": np.ones(n), "tk": np.full(n, T0), "kt": np.full(n, 8.0),
         "rhocp": np.full(n, 3000.0 * 1000.0), "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e19, rho_ref=3000.0, T0=T0, T1=T0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    grids["btopx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["btopy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bbottomy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bleftx"] = F(np.zeros((Y + 1, 2)))
    grids["brightx"] = F(np.zeros((Y + 1, 2)))
    grids["blefty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["brighty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["btopt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomt"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bleftt"] = F(np.column_stack([np.full(Y, T0), np.zeros(Y)]))
    grids["brightt"] = F(np.column_stack([np.full(Y, T0), np.zeros(Y)]))
    params = default_params(timestep=1e5 * YEAR, viscosity_min=1e18, viscosity_max=1e25, temperature_top=T0,
                            itype_global=1, ntimestep=1, runge_kutta_order=0, temperature_bottom=T0)
    params.update(stokes_params(pressure_bc_mode=1, pressure_bc=3e7, gravity_y=0.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=10.0, iuse_adiabatic_heating=0, iuse_shear_heating=1, iuse_heat=1)
    params["rock_tables"] = {"mat_rho": np.array([[3000.0, 0.0, 0.0]]), "mat_cp": np.array([1000.0]),
                             "mat_kt": np.array([[8.0, 1.0]]), "density_model": 0, "rhocp_model": 0,
                             "conductivity_model": 2}
    return Model("channel_flow_variable_conductivity", grid, mats, params, m, grids)


def channel_flow_variable_conductivity_temperature(x: np.ndarray, width: float, height: float, t_wall: float,
                                                   top_pressure: float, viscosity: float, k0: float,
                                                   b: float) -> np.ndarray:
    """Steady temperature of shear-heated Poiseuille flow with k = k0 / (1 + b (T - T_wall) / T_wall),
    as the reference's benchmark evaluates it (post_processing/analytical/
    ChannelFlowVariableConductivityManager.jl, after Gerya 2010): dp/dy = -top_pressure / height,
    t1 = W^4 b / 192 / k0 / T_wall / eta (dp/dy)^2, T = T_wall / b (exp(t1 (1 - (2x/W - 1)^4)) + b - 1)."""
    grad = -top_pressure / height
    t1 = width ** 4.0 * b / 192.0 / k0 / t_wall / viscosity * grad ** 2.0
    return t_wall / b * (np.exp(t1 * (1.0 - (2.0 * x / width - 1.0) ** 4.0)) + b - 1.0)


def elastic_slab(xnum: int = 51, ynum: int = 51, mpc: int = 5) -> Model:
    """The reference's elastic-slab benchmark, as configured in
    src/benchmarks/models/elastic_slab/{model,materials}.yml and the benchmark material library:
    a 1000 x 1000 km box on 51 x 51 nodes with 5 x 5 markers per cell on a regular lattice; the
    slab 0.2 < y/ysize < 0.8, x/xsize < 0.8 (ElasticSlab.in_elastic_slab) of 4000 kg/m^3,
    1e27 Pa s, shear modulus 1e10 Pa, attached to the left wall, in a medium of 1 kg/m^3, 1e21 Pa s,
    1e20 Pa; both split into the reference's checkerboard of material ids 2-5
    (ElasticSlab.define_material, 20 x 20 squares).  ElasticSlabBC.jl: no slip on the left wall,
    free slip elsewhere, pressure fixed in the upper-left cell.  Gravity 10 m/s^2 for the first
    100 steps (GravityFuncs.turn_off_gravity!), 200 yr steps multiplied by 10 after step 250
    (TimeStepIncrease single increase), subgrid stress diffusion off, heat on with uniform 0 C."""
    W = H = 1000e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)

    def check(v, size):
        c = np.ceil(v / (size / 20.0)) + 1.0
        return c - np.ceil(c / 2.0) * 2.0
    matid = np.where(check(y, H) == check(x, W), 3, 2)
    slab = (0.2 < y / H) & (y / H < 0.8) & (x / W < 0.8)
    matid = np.where(slab, np.where(matid == 2, 4, 5), matid).astype(np.int16)
    # material ids 1-5 (id 1 unused, as in the reference's material model)
    eta = np.array([1e21, 1e21, 1e21, 1e27, 1e27])
    mu = np.array([1e20, 1e20, 1e20, 1e10, 1e10])
    rho = np.array([1.0, 1.0, 1.0, 4000.0, 4000.0])
    mats = Materials(
        mat_mu=mu, mat_hr=np.zeros(5), mat_flow_type=np.zeros(5, np.int64),
        mat_flow=np.asfortranarray(np.zeros((5, 12))), mat_plastic=np.asfortranarray(np.zeros((5, 6))), mat_rho=rho)
    mats.mat_flow[:, 0] = eta
    mi = matid.astype(np.int64) - 1
    T0 = 273.15
    m = {"x": x, "y": y, "matid": matid, "rho": rho[mi].copy(), "eta": eta[mi].copy(), "eta_flow": eta[mi].copy(),
         "sr_ratio": np.ones(n), "tk": np.full(n, T0), "kt": np.full(n, 3.0), "rhocp": rho[mi] * 1000.0,
         "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e21, rho_ref=1.0, T0=T0, T1=T0, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    grids["bleftx"] = F(np.zeros((Y + 1, 2)))
    grids["blefty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["bleftt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    grids["brightt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    params = default_params(timestep=200.0 * YEAR, viscosity_min=1e18, viscosity_max=1e27, temperature_top=T0,
                            itype_global=1, ntimestep=1, subgrid_diff_coef_stress=0.0, subgrid_diff_coef_temp=1.0,
                            temperature_bottom=T0)
    params.update(stokes_params(pressure_bc_mode=0, pressure_bc=0.0, gravity_y=10.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=20.0, iuse_adiabatic_heating=0, iuse_shear_heating=0, iuse_heat=1,
                  marker_cell_displ_max=0.3333, nsteps_turn_off_gravity=100, ntime_increase=250,
                  time_increase_factor=10.0, nskip_output=50)
    return Model("elastic_slab", grid, mats, params, m, grids)


def box_convection(mpc: int = 4) -> Model:
    """The reference's isoviscous box-convection benchmark, Blankenbach et al. (1989) case 1a, as
    configured in src/benchmarks/models/box_convection_isoviscous_1a/{model,materials}.yml and the
    benchmark material library (IsoviscousFluidBlankenbach89): a 1000 x 1000 km box on the
    reference's 51 x 51 grid refined along the sides (sides_with_highres/core/Initialization.jl:
    10 km cells, a 1.2407234 geometric transition, 30 km cells in the middle), 4 x 4 markers per
    (average) cell on a regular lattice, the Blankenbach flow law (1e23 Pa s, b = c = 0) and
    density rho0 (1 - alpha (T - T_top)) (4000 kg/m^3, 2.5e-5 1/K; rock-property density model 1,
    rhocp constant with 1250 J/kg/K, uniform conductivity 5 W/m/K: params["rock_tables"]),
    gravity 10 m/s^2, free slip on every side, 0 C at the top, 1000 C at the bottom, no heat flux
    through the sides, the BoxConvection initial temperature, and 0.5 Myr steps limited to half a
    cell of marker displacement: Ra = 1e4."""
    X = Y = 51
    W = H = 1000e3
    gy = np.zeros(Y)
    for i in range(2, 12):
        gy[i - 1] = gy[i - 2] + 10000.0
    for i in range(12, 17):
        gy[i - 1] = gy[i - 2] + 10000.0 * 1.2407234 ** float(i - 10)
    for i in range(17, 37):
        gy[i - 1] = gy[i - 2] + 30000.0
    for i in range(37, 42):
        gy[i - 1] = gy[i - 2] + 10000.0 * 1.2407234 ** float(41 - i)
    for i in range(42, Y + 1):
        gy[i - 1] = gy[i - 2] + 10000.0
    gy[Y - 1] = H
    gx = gy * W / H
    grid = staggered_grid(gx, gy)
    mx, my = (X - 1) * mpc, (Y - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    t_top, t_bot = 273.15, 1273.15
    xw, yw = x / W, y / H
    yw = np.where(yw > 0.5, 0.5 + 0.5 * (np.abs(yw - 0.5) / 0.5) ** 10, 0.5 - 0.5 * (np.abs(yw - 0.5) / 0.5) ** 10)
    T = (t_top + (t_bot - t_top) * yw ** (2.0 + xw) + t_bot + (t_top - t_bot) * (1.0 - yw) ** (3.0 - xw)) / 2.0
    flow = np.zeros((1, 17))
    flow[0, 14] = 1e23
    mats = Materials(
        mat_mu=np.array([1e28]), mat_hr=np.zeros(1), mat_flow_type=np.array([5], np.int64),
        mat_flow=np.asfortranarray(flow), mat_plastic=np.asfortranarray(np.zeros((1, 6))), mat_rho=np.array([4000.0]))
    rho = 4000.0 * (1.0 - 2.5e-5 * (T - t_top))
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": rho, "eta": np.full(n, 1e23),
         "eta_flow": np.full(n, 1e23), "sr_ratio": np.ones(n), "tk": T, "kt": np.full(n, 5.0),
         "rhocp": rho * 1250.0, "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e23, rho_ref=4000.0, T0=t_top, T1=t_bot, depth_T1=H, y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    grids["btopt"] = F(np.column_stack([np.full(X, t_top), np.zeros(X)]))
    grids["bbottomt"] = F(np.column_stack([np.full(X, t_bot), np.zeros(X)]))
    grids["bleftt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    grids["brightt"] = F(np.column_stack([np.zeros(Y), np.ones(Y)]))
    params = default_params(timestep=0.5e6 * YEAR, viscosity_min=1e18, viscosity_max=1e27, temperature_top=t_top,
                            temperature_bottom=t_bot, itype_global=1, ntimestep=1, subgrid_diff_coef_stress=0.0,
                            subgrid_diff_coef_temp=1.0)
    params.update(stokes_params(pressure_bc_mode=0, pressure_bc=0.0, gravity_y=10.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=20.0, iuse_adiabatic_heating=0, iuse_shear_heating=0, iuse_heat=1,
                  marker_cell_displ_max=0.5, nskip_output=100)
    params["rock_tables"] = {"mat_rho": np.array([[4000.0, 2.5e-5, 0.0]]), "mat_cp": np.array([1250.0]),
                             "mat_kt": np.array([[5.0, 0.0]]), "density_model": 1, "rhocp_model": 0,
                             "conductivity_model": 1}
    return Model("box_convection_isoviscous_1a", grid, mats, params, m, grids)


def box_convection_vrms(grid: Grid, vx1: np.ndarray, vy1: np.ndarray, conductivity: float, heat_capacity: float,
                        density: float) -> float:
    """BoxConvection.calculate_nondimensional_rms_velocity (post_processing/numerical/box_convection/
    BoxConvection.jl:66-88): the cell-weighted mean of (vx^2 at the cell's two vx nodes + vy^2 at
    its two vy nodes) / 2, its square root scaled by ysize / kappa."""
    xs, ys = grid.xstp_b, grid.ystp_b
    W, H = grid.xmax - grid.xmin, grid.ymax - grid.ymin
    a = (vx1[1:-1, :-1] ** 2 + vx1[1:-1, 1:] ** 2 + vy1[:-1, 1:-1] ** 2 + vy1[1:, 1:-1] ** 2) / 2.0
    v = float(np.sum(a * ys[:, None] * xs[None, :]))
    return math.sqrt(v / W / H) * H / (conductivity / heat_capacity / density)


def channel_flow_non_steady_temperature(xnum: int = 51, ynum: int = 11, mpc: int = 5) -> Model:
    """The reference's non-steady channel-temperature benchmark, as configured in
    src/benchmarks/models/channel_flow_non_steady_temperature/{model,materials}.yml and the
    benchmark material library (ConstantViscosityChannel): a 30 x 12.5 km vertical channel on
    51 x 11 nodes with 5 x 5 markers per cell on a regular lattice, an isoviscous material
    (1e19 Pa s, 3000 kg/m^3, 1000 J/kg/K, 2 W/m/K), the linear initial temperature from 727 C at
    the top to 1227 C at the bottom, VerticalChannelFlowIsoviscousBC.jl: the open channel with
    1e5 Pa on the top row of pressure cells, no slip on both walls, the initial linear profile held
    on both walls (TemperatureBC.set_variable_temperature_at_*_boundary!) and its gradient through
    the top and the bottom (ConstantGradientBC.jl); subgrid diffusion on, 1 Myr steps limited to a
    tenth of a cell of displacement, the channel recycling."""
    W, H = 30e3, 12.5e3
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    t_top, t_bot = 727.0 + 273.15, 1227.0 + 273.15
    T = t_top + (t_bot - t_top) * y / H
    mats = Materials(
        mat_mu=np.array([1e20]), mat_hr=np.zeros(1), mat_flow_type=np.array([0], np.int64),
        mat_flow=np.asfortranarray(np.zeros((1, 12))), mat_plastic=np.asfortranarray(np.zeros((1, 6))),
        mat_rho=np.array([3000.0]))
    mats.mat_flow[0, 0] = 1e19
    m = {"x": x, "y": y, "matid": np.ones(n, np.int16), "rho": np.full(n, 3000.0), "eta": np.full(n, 1e19),
         "eta_flow": np.full(n, 1e19), "sr_ratio": np.ones(n), "tk": T, "kt": np.full(n, 2.0),
         "rhocp": np.full(n, 3000.0 * 1000.0), "ha": np.zeros(n)}
    for f in ("cohesion", "fric", "fric_ini", "preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e19, rho_ref=3000.0, T0=t_top, T1=t_bot, depth_T1=H,
                            y_surface=0.0)
    grids.update(velocity_bcs(grid))
    F = np.asfortranarray
    X, Y = xnum, ynum
    ystp, dtdy = H / (Y - 1), (t_bot - t_top) / H
    grids["btopx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["bbottomx"] = F(np.column_stack([np.zeros(X), np.ones(X)]))
    grids["btopy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bbottomy"] = F(np.column_stack([np.zeros(X + 1), np.ones(X + 1)]))
    grids["bleftx"] = F(np.zeros((Y + 1, 2)))
    grids["brightx"] = F(np.zeros((Y + 1, 2)))
    grids["blefty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["brighty"] = F(np.column_stack([np.zeros(Y), -np.ones(Y)]))
    grids["btopt"] = F(np.column_stack([np.full(X, -ystp * dtdy), np.ones(X)]))
    grids["bbottomt"] = F(np.column_stack([np.full(X, ystp * dtdy), np.ones(X)]))
    wall = t_top + np.arange(Y) * ystp * dtdy
    grids["bleftt"] = F(np.column_stack([wall, np.zeros(Y)]))
    grids["brightt"] = F(np.column_stack([wall, np.zeros(Y)]))
    params = default_params(timestep=1e6 * YEAR, viscosity_min=1e18, viscosity_max=1e25, temperature_top=t_top,
                            temperature_bottom=t_bot, itype_global=1, ntimestep=1)
    params.update(stokes_params(pressure_bc_mode=1, pressure_bc=1e5, gravity_y=0.0, iuse_interface_stabilization=0))
    params.update(max_temp_change=10.0, iuse_adiabatic_heating=0, iuse_shear_heating=0, iuse_heat=1,
                  marker_cell_displ_max=0.1, nskip_output=5)
    return Model("channel_flow_non_steady_temperature", grid, mats, params, m, grids)


def channel_flow_non_steady_temperature_profile(x: np.ndarray, tmyr: float, width: float, ysize: float, ynum: int,
                                                y_index: int, t_top_c: float, t_bottom_c: float,
                                                top_pressure: float, viscosity: float, conductivity: float,
                                                density: float, heat_capacity: float) -> np.ndarray:
    """Temperature (C) across the channel at the row y_index after tmyr Myr, as the reference's
    benchmark evaluates it (post_processing/analytical/ChannelFlowNonSteadyTemperatureManager.jl,
    after Gerya 2010 with its 1/4 factor): T0 = T_top + y G at the row (Celsius + 273.0, the
    reference's conversion), dp/dy = -top_pressure / (ysize - dy), e = -dp/dy G / (4 eta), and
    100 terms m = 1..100 of F_m E_m sin(pi (2m' - 1) x / W) with m' = m - 1 (the reference's
    indexing), F_m = -8 e W^2 / (pi (2m' - 1))^3, E_m = W^2 (1 - exp(-kappa t (pi (2m' - 1))^2 / W^2))
    / (kappa (pi (2m' - 1))^2) and t = tmyr in 365-day years."""
    t_top, t_bot = t_top_c + 273.0, t_bottom_c + 273.0
    grad_t = (t_bot - t_top) / ysize
    y_test = (y_index - 1) * ysize / (ynum - 1)
    t0 = t_top + y_test * grad_t
    grad_p = -top_pressure / (ysize - ysize / (ynum - 1))
    tsec = tmyr * 1e6 * 365.0 * 24.0 * 60.0 * 60.0
    ep = -1.0 / 4.0 / viscosity * grad_p * grad_t
    kappa = conductivity / density / heat_capacity
    dT = np.zeros_like(np.asarray(x, dtype=np.float64))
    for mm in range(1, 101):
        mf = float(mm - 1)
        a = math.pi * (2.0 * mf - 1.0)
        emt = width * width * (1.0 - math.exp(-kappa * tsec / width / width * a ** 2.0)) / (kappa * a ** 2.0)
        fm = -8.0 * ep * width * width / a ** 3.0
        dT = dT + fm * emt * np.sin(a * np.asarray(x) / width)
    return t0 + dT - 273.0


def plasticity_benchmark_kaus10(xnum: int = 401, ynum: int = 101, mpc: int = 3) -> Model:
    """The reference's Kaus (2010) plasticity benchmark, as configured in
    src/benchmarks/models/plasticity_benchmark_kaus10/{model,materials}.yml and the benchmark
    material library (Plasticity_Benchmark_Kaus10): a 40 x 12 km box on 401 x 101 nodes with
    3 x 3 markers per cell on a regular lattice; 2 km of sticky air (1 kg/m^3, 1e19 Pa s, shear
    modulus 1e21 Pa) over a visco-elasto-plastic layer (1e25 Pa s, 5e10 Pa, cohesion 40 MPa
    softening to 5 MPa between plastic strains 0 and 0.1, friction angle 30 degrees), the
    layer split into the seven-layer model's material ids 3-8 (SevenLayerEarthModel2D, all of
    them CrustKaus10), with a weak notch of 1e20 Pa s at the bottom centre
    (WeakNotch.get_seed_limits_weak_notch with the model height as its base: 800 m wide,
    400 m high, material id 9).  Density: DensityLiao14 at the uniform 273 K,
    rho0 (1 - alpha (T - 298.15)).  ExtensionNoBottomInflowBC.jl: the sides move apart at half of
    the full extension velocity strain_rate_bc x xsize = 1e-15 1/s x 40 km
    (VelocityFromStrainRate.jl), the top lets in vyu = v_full ysize / xsize
    (ExtensionFreeSlipAlongBottom.calc_velocity!), free slip on the bottom, pressure 1e5 Pa in
    the upper-left cell; nodal plasticity loop (up to 100 iterations, tolerance 1e-3), 15 kyr
    viscoelastic steps with the 0.5-cell displacement limit, viscosity 1e19-1e25 Pa s, yield
    stress 20 MPa-1 GPa, gravity 10 m/s^2.  The reference stops at an extensional strain
    v_full t / xsize of 0.02 (Stopping.check_extensional_strain_stopping).  The heat solve is
    on in the reference but leaves the uniform temperature unchanged (equal top and bottom
    temperatures, no shear, adiabatic or radiogenic heating)."""
    W, H = 40000.0, 12000.0
    grid = staggered_grid(np.linspace(0.0, W, xnum), np.linspace(0.0, H, ynum))
    mx, my = (xnum - 1) * mpc, (ynum - 1) * mpc
    x = np.repeat((np.arange(mx) + 0.5) * (W / mx), my)
    y = np.tile((np.arange(my) + 0.5) * (H / my), mx)
    n = len(x)
    thick_air, thick_layer = 2000.0, 1666.67
    tops = thick_air + thick_layer * np.arange(1, 6)
    matid = np.where(y <= thick_air, 1, 3 + np.searchsorted(tops, y, side="left")).astype(np.int16)
    matid = np.minimum(matid, 8).astype(np.int16)
    w_seed, x_seed = 800.0, 20000.0
    notch = (H - w_seed / 2.0 <= y) & (y <= H) & (x_seed - w_seed / 2.0 <= x) & (x <= x_seed + w_seed / 2.0)
    matid[notch] = 9
    T0 = 273.0
    nmat = 9
    rock = np.zeros(nmat, bool)
    rock[2:8] = True
    rho_rock = 2700.0 * (1.0 - 3.0e-5 * (T0 - 298.15))
    rho = np.where(np.arange(nmat) >= 2, rho_rock, 1.0)
    eta = np.where(rock, 1e25, 1e19)
    eta[8] = 1e20
    mu = np.where(np.arange(nmat) >= 2, 5e10, 1e21)
    cp = np.where(np.arange(nmat) >= 2, 1200.0, 100.0)
    kt = np.where(np.arange(nmat) >= 2, 3.0, 20.0)
    sin30 = math.sin(math.radians(30.0))
    mat_plastic = np.zeros((nmat, 6))
    mat_plastic[rock, :] = [40e6, 5e6, sin30, sin30, 0.0, 0.1]
    mat_flow = np.zeros((nmat, 12))
    mat_flow[:, 0] = eta
    mats = Materials(mat_mu=mu, mat_hr=np.zeros(nmat), mat_flow_type=np.zeros(nmat, np.int64),
                     mat_flow=np.asfortranarray(mat_flow), mat_plastic=np.asfortranarray(mat_plastic), mat_rho=rho)
    mi = matid.astype(np.int64) - 1
    m = {"x": x, "y": y, "matid": matid, "rho": rho[mi].copy(), "eta": eta[mi].copy(), "eta_flow": eta[mi].copy(),
         "sr_ratio": np.ones(n), "tk": np.full(n, T0), "kt": kt[mi].copy(), "rhocp": rho[mi] * cp[mi],
         "ha": np.zeros(n)}
    m["cohesion"] = mat_plastic[mi, 0].copy()
    m["fric_ini"] = mat_plastic[mi, 2].copy()
    m["fric"] = m["fric_ini"].copy()
    for f in ("preexp", "sxx", "sxy", "exx", "exy", "pr", "gii", "strain_plastic"):
        m[f] = np.zeros(n)
    _fields_common(np.random.Generator(np.random.Philox(0)), n, m)
    m["pfailure"][:] = 0.0
    grids = _analytic_grids(grid, v0=0.0, eta_ref=1e25, rho_ref=rho_rock, T0=T0, T1=T0, depth_T1=H,
                            y_surface=thick_air)
    edot = 1e-15
    v_full = edot * W
    vyu = v_full * H / W
    grids.update(velocity_bcs(grid, v_ext=0.5 * v_full))
    F = np.asfortranarray
    grids["btopy"] = F(np.column_stack([np.full(xnum + 1, vyu), np.zeros(xnum + 1)]))
    grids["bbottomy"] = F(np.zeros((xnum + 1, 2)))
    params = default_params(timestep=15e3 * YEAR, viscosity_min=1e19, viscosity_max=1e25, yield_stress_min=2e7,
                            yield_stress_max=1e9, temperature_top=T0, temperature_bottom=T0, itype_global=1,
                            matid_sticky_air=1, subgrid_diff_coef_stress=1.0, subgrid_diff_coef_temp=1.0)
    params.update(stokes_params(pressure_bc_mode=0, pressure_bc=1e5, gravity_y=10.0, iuse_interface_stabilization=0))
    params.update(nglobal=100, tolerance_picard=1e-3, marker_cell_displ_max=0.5, strain_rate_bc=edot,
                  full_velocity_extension=v_full, velocity_y_upper=vyu, strain_limit=0.02, thick_air=thick_air,
                  w_seed=w_seed, x_seed=x_seed, friction_angle=30.0, dilation_angle=0.0)
    return Model("plasticity_benchmark_kaus10", grid, mats, params, m, grids)


def pressure_grid_value(grid: Grid, arr: np.ndarray, x: float, y: float) -> float:
    """GridToMarker.get_marker_value_from_pressure_grid_without_mapping_input
    (interpolation/utils/GridToMarker.jl:51-79 with MarkerGridMapping.upr_left_index_pressure and
    upr_left_dist_pressure, :311-350): the basic cell holding the point, the pressure node up and
    to the left of it (clamped to the interior cells), and bilinear weights from the staggered
    coordinates; arr is a (ynum-1, xnum-1) pressure-grid array."""
    def axis(b, stag, sstag, v, nn):
        i = int(np.clip(np.searchsorted(b, v, side="right") - 1, 0, nn - 2))
        p = i - 1 if v < stag[i + 1] else i
        p = min(max(p, 0), nn - 3)
        return p, (v - stag[p + 1]) / sstag[p + 1]
    yn, dy = axis(grid.gridy_b, grid.gridy_vx, grid.ystp_vx, y, grid.ynum)
    xn, dx = axis(grid.gridx_b, grid.gridx_vy, grid.xstp_vy, x, grid.xnum)
    return float((1.0 - dx) * (1.0 - dy) * arr[yn, xn] + (1.0 - dx) * dy * arr[yn + 1, xn]
                 + dx * (1.0 - dy) * arr[yn, xn + 1] + dx * dy * arr[yn + 1, xn + 1])


def kaus10_measurement_lines(grid: Grid, params: dict) -> tuple:
    """The sample points of the reference's shear-zone measurement
    (post_processing/numerical/PlasticityBenchmarkK10.jl:325-400): four vertical lines, at w_seed/4
    and w_seed/4 + 2 km outside the left and the right edge of the notch (left near, left far,
    right near, right far), each sampled at ynum x 10 points between the bottom of the sticky air
    and the top of the notch.  Returns (x of the four lines, y of the samples)."""
    H = grid.ymax
    w_seed, x_seed = params["w_seed"], params["x_seed"]
    xmin_n, xmax_n = x_seed - w_seed / 2.0, x_seed + w_seed / 2.0
    notch_thick = w_seed / 2.0
    y0 = params["thick_air"]
    npoints = grid.ynum * 10
    ys = y0 + (H - y0 - notch_thick) / (npoints - 1) * np.arange(npoints)
    xs = (xmin_n - w_seed / 4.0, xmin_n - (w_seed / 4.0 + 2000.0), xmax_n + w_seed / 4.0,
          xmax_n + (w_seed / 4.0 + 2000.0))
    return xs, ys


def kaus10_fault_dip(grid: Grid, eii: np.ndarray, params: dict) -> dict:
    """The reference's measurement of the shear-zone dip
    (post_processing/numerical/PlasticityBenchmarkK10.jl:200-245 and 325-450): on each of the
    lines of kaus10_measurement_lines the depth of the largest strain-rate invariant (the first
    of equal maxima) gives one end of a fault stick; each side's dip is atan(|dy| / |dx|) of its
    stick, and the mean of the two dips is compared with the target, the mean of the Coulomb
    (45 + phi/2) and Arthur (45 + (phi + psi)/4) angles.  Returns the dips (degrees), the target
    and the relative error."""
    xs, ys = kaus10_measurement_lines(grid, params)

    def ymax_at(xp):
        best, ybest = -1e32, -1e32
        for yp in ys:
            v = pressure_grid_value(grid, eii, xp, yp)
            if v > best:
                best, ybest = v, yp
        return ybest
    x1l, x2l, x1r, x2r = xs
    y1l, y2l, y1r, y2r = (ymax_at(x) for x in xs)
    th_l = math.degrees(math.atan(abs(y2l - y1l) / abs(x2l - x1l)))
    th_r = math.degrees(math.atan(abs(y2r - y1r) / abs(x2r - x1r)))
    phi, psi = params["friction_angle"], params["dilation_angle"]
    coulomb, arthur = 45.0 + phi / 2.0, 45.0 + (phi + psi) / 4.0
    target = (coulomb + arthur) / 2.0
    theta = (th_l + th_r) / 2.0
    return {"theta_left": th_l, "theta_right": th_r, "theta": theta, "target": target,
            "relative_error": abs(theta - target) / abs(target),
            "sticks": {"left": ((x1l, y1l), (x2l, y2l)), "right": ((x1r, y1r), (x2r, y2r))}}


def ramberg_wave_velocity(h1: float, h2: float, rho1: float, rho2: float, eta1: float, eta2: float, amp: float,
                          lam: float, g: float = 9.81) -> float:
    """Ramberg's (1968) analytical vertical velocity at the crest of a sinusoidal interface
    between a top layer (thickness h1, density rho1, viscosity eta1) and a bottom layer (h2, rho2,
    eta2) between no-slip walls, as the reference's benchmark evaluates it
    (post_processing/analytical/RayleighTaylorInstabilityManager.jl): the growth factor
    K = -d12 / (c11 j22 - d12 j21) and v = -K (rho1 - rho2) h2 g / (2 eta2) A."""
    t1, t2 = 2.0 * math.pi * h1 / lam, 2.0 * math.pi * h2 / lam
    r = eta1 / eta2
    den1 = math.cosh(2.0 * t1) - 1.0 - 2.0 * t1 ** 2
    den2 = math.cosh(2.0 * t2) - 1.0 - 2.0 * t2 ** 2
    c11 = r * 2.0 * t1 ** 2 / den1 - 2.0 * t2 ** 2 / den2
    d12 = r * (math.sinh(2.0 * t1) - 2.0 * t1) / den1 + (math.sinh(2.0 * t2) - 2.0 * t2) / den2
    j21 = r * t2 * (math.sinh(2.0 * t1) + 2.0 * t1) / den1 + t2 * (math.sinh(2.0 * t2) + 2.0 * t2) / den2
    j22 = r * 2.0 * t1 ** 2 * t2 / den1 - 2.0 * t2 ** 3 / den2
    K = -d12 / (c11 * j22 - d12 * j21)
    return -K * (rho1 - rho2) * h2 * g / 2.0 / eta2 * amp


def config(name: str, seed: int | None = None) -> Model:
    """Named workloads: sinking_block, rift_small, rift_2p5M, rift_40M, rift_40M_strip, circles_1025."""
    kw = {} if seed is None else {"seed": seed}
    if name == "sinking_block":
        return sinking_block(**kw)
    if name == "rift_small":
        return rift(101, 41, 4, **kw)
    if name == "rift_2p5M":
        return rift(801, 201, 4, **kw)
    if name == "rift_40M":
        return rift(2001, 801, 5, **kw)
    if name == "rift_40M_strip":
        return rift(101, 801, 5, width=25e3, **kw)
    if name == "circles_1025":
        return circles(1025, **kw)
    raise KeyError(name)


def marker_arrays_for_upload(model: Model) -> dict:
    """Marker arrays cast to the C-ABI host types."""
    out = {}
    for k, v in model.markers.items():
        out[k] = np.ascontiguousarray(v, dtype=_abi.MARKER_DTYPE[k])
    return out
