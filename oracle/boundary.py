"""CPU oracle (TEST INFRASTRUCTURE ONLY) for the step-boundary updates: the rock
properties of the markers (rock_properties/RockProperties.jl:99-125) and the
displacement-limited time step (time_step/update/Update.jl:16-219) and the marker recycling
of every model type (marker_recycle/types/{Extension,ExtensionNoBottomInflow,Channel,
ContractionViscoelastic,ExtensionInflowAndOutflowAlongSides,ContractionFractureZone}.jl),
restated in boundary_oracle.c.  Only tests/ use it."""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libboundary_oracle.so"
SRC = HERE / "boundary_oracle.c"
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def build(force: bool = False) -> pathlib.Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        BUILD.mkdir(exist_ok=True)
        tmp = BUILD / "libboundary_oracle.so.tmp"
        subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.o_timestep_displacement_limit.restype = C.c_double
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def timestep_displacement_limit(grid, vx1, vy1, displ: float, iuse_local: int, dt_old: float) -> float:
    vx = np.asfortranarray(vx1, dtype=np.float64)
    vy = np.asfortranarray(vy1, dtype=np.float64)
    xs = np.ascontiguousarray(grid.xstp_b, dtype=np.float64)
    ys = np.ascontiguousarray(grid.ystp_b, dtype=np.float64)
    return lib().o_timestep_displacement_limit(C.c_int64(grid.xnum), C.c_int64(grid.ynum), _p(vx), _p(vy), _p(xs),
                                               _p(ys), C.c_double(grid.xstpavg), C.c_double(grid.ystpavg),
                                               C.c_double(displ), C.c_int64(iuse_local), C.c_double(dt_old))


def rock_properties(mk: dict, mat_rho, mat_cp, mat_kt, density_model, rhocp_model, cond_model, temperature_top,
                    maximum_heat_capacity, iuse_por=0, sed=None) -> dict:
    """Returns updated copies of rho, rhocp, kt, ha (inside markers only, as the reference)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in ("rho", "rhocp", "kt", "ha")}
    rho_t = np.asfortranarray(mat_rho, dtype=np.float64)
    cp_t = np.ascontiguousarray(mat_cp, dtype=np.float64)
    kt_t = np.asfortranarray(mat_kt, dtype=np.float64)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    matid = np.ascontiguousarray(mk["matid"], dtype=np.int16)
    f = {k: np.ascontiguousarray(mk[k], dtype=np.float64) for k in ("x", "y", "pr", "tk")}
    if iuse_por == 1:
        por = [np.ascontiguousarray(mk[k], dtype=np.float64) for k in ("porosity_initial", "decay_depth",
                                                                         "max_burial_depth")]
        ids = np.ascontiguousarray(sed["matids"], dtype=np.int16)
        tx = np.ascontiguousarray(sed["topo_x"], dtype=np.float64)
        ty = np.ascontiguousarray(sed["topo_y"], dtype=np.float64)
        wk, wr, wc = sed["conductivity_water"], sed["density_water"], sed["heat_capacity_water"]
    else:
        por = [None, None, None]
        ids = tx = ty = None
        wk = wr = wc = 0.0
    lib().o_rock_properties(C.c_int64(M), _p(inside), _p(matid), _p(f["x"]), _p(f["y"]), _p(f["pr"]), _p(f["tk"]),
                            _p(out["rho"]), _p(out["rhocp"]), _p(out["kt"]), _p(out["ha"]), C.c_int64(len(cp_t)),
                            _p(rho_t), _p(cp_t), _p(kt_t), C.c_int64(density_model), C.c_int64(rhocp_model),
                            C.c_int64(cond_model), C.c_double(temperature_top), C.c_double(maximum_heat_capacity),
                            C.c_int64(iuse_por), _p(por[0]), _p(por[1]), _p(por[2]), _p(tx), _p(ty),
                            C.c_int64(0 if tx is None else len(tx)), _p(ids), C.c_int64(0 if ids is None else len(ids)),
                            C.c_double(wk), C.c_double(wr), C.c_double(wc))
    return out


RECYCLE_FIELDS = ("x", "y", "tk", "pr", "sxx", "sxy", "exx", "exy", "eta", "sr_ratio", "gii", "strain_plastic",
                  "strain_rate_plastic", "meltfrac", "fric_ini", "fric")


def fz_lithosphere_temperature(t_top, t_bottom, grad, asth, kappa, depth, age) -> float:
    """FractureZone.calc_lithosphere_temperature (the half-space cooling erf law) of the
    oracle's fracture-zone recycling."""
    f = lib().o_fz_lithosphere_temperature
    f.restype = C.c_double
    return f(*[C.c_double(v) for v in (t_top, t_bottom, grad, asth, kappa, depth, age)])


def philox4x32_10(ctr, key) -> tuple:
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    lib().o_philox4x32_10(c, C.c_uint32(key[0]), C.c_uint32(key[1]))
    return tuple(c)


def recycle_uniforms(seed: int, step: int, stream: int, j: int) -> tuple:
    u0, u1 = C.c_double(), C.c_double()
    lib().o_recycle_uniforms(C.c_uint64(seed), C.c_int64(step), C.c_uint32(stream), C.c_int64(j), C.byref(u0),
                             C.byref(u1))
    return u0.value, u1.value


def recycle_extension(mk: dict, matid_sticky_air, matid_sticky_water, matid_asthenosphere, xsize, ysize,
                      velocity_y_upper, velocity_y_lower, timestep, temperature_top, temperature_bottom, gridy_last,
                      mat_plastic, iuse_random_fric, delta_fric_coef, seed, step) -> tuple:
    """Returns (fields after recycling, 1-based indices, flags, n_air)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in RECYCLE_FIELDS}
    out["matid"] = np.array(mk["matid"], dtype=np.int16, copy=True)
    out["pfailure"] = np.array(mk["pfailure"], dtype=np.float32, copy=True)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    ptrs = (C.c_void_p * len(RECYCLE_FIELDS))(*[out[k].ctypes.data for k in RECYCLE_FIELDS])
    s = np.array([matid_sticky_air, matid_sticky_water, matid_asthenosphere], np.int16)
    d = np.array([xsize, ysize, velocity_y_upper, velocity_y_lower, timestep, temperature_top, temperature_bottom,
                  gridy_last, delta_fric_coef], np.float64)
    mp = np.asfortranarray(mat_plastic, dtype=np.float64)
    lst = np.zeros(max(M, 1), np.int64)
    fl = np.zeros(max(M, 1), np.int8)
    n_air = C.c_int64()
    lib().o_recycle_extension.restype = C.c_int64
    n = lib().o_recycle_extension(C.c_int64(M), _p(inside), _p(out["matid"]), ptrs, _p(out["pfailure"]), _p(s),
                                  _p(d), C.c_int64(mp.shape[0]), _p(mp), C.c_int64(iuse_random_fric),
                                  C.c_uint64(seed), C.c_int64(step), _p(lst), _p(fl), C.byref(n_air))
    return out, lst[:n].copy(), fl[:n].copy(), n_air.value


def recycle_contraction(mk: dict, matid_sticky_air, matid_sticky_water, matid_layers, matid_strong, xsize, ysize,
                        full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
                        temperature_top, layer_thickness, x_left_strong, x_right_strong, mat_plastic,
                        iuse_random_fric, delta_fric_coef, seed, step, asymmetric=0) -> tuple:
    """ContractionViscoelastic recycling; returns (fields, 1-based indices, flags, n_air)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in RECYCLE_FIELDS}
    out["matid"] = np.array(mk["matid"], dtype=np.int16, copy=True)
    out["pfailure"] = np.array(mk["pfailure"], dtype=np.float32, copy=True)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    ptrs = (C.c_void_p * len(RECYCLE_FIELDS))(*[out[k].ctypes.data for k in RECYCLE_FIELDS])
    ids = np.array([matid_sticky_air, matid_sticky_water, *matid_layers, *matid_strong], np.int16)
    assert len(ids) == 12 and len(layer_thickness) == 6
    d = np.array([xsize, ysize, full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
                  temperature_top, *layer_thickness, x_left_strong, x_right_strong, delta_fric_coef], np.float64)
    mp = np.asfortranarray(mat_plastic, dtype=np.float64)
    lst = np.zeros(max(M, 1), np.int64)
    fl = np.zeros(max(M, 1), np.int8)
    nx, ny = np.zeros(max(M, 1)), np.zeros(max(M, 1))
    n_air = C.c_int64()
    lib().o_recycle_contraction.restype = C.c_int64
    n = lib().o_recycle_contraction(C.c_int64(M), _p(inside), _p(out["matid"]), ptrs, _p(out["pfailure"]), _p(ids),
                                    _p(d), C.c_int64(int(asymmetric)), C.c_int64(mp.shape[0]), _p(mp),
                                    C.c_int64(iuse_random_fric), C.c_uint64(seed), C.c_int64(step), _p(lst), _p(fl),
                                    _p(nx), _p(ny), C.byref(n_air))
    return out, lst[:n].copy(), fl[:n].copy(), n_air.value


def recycle_side_inflow(mk: dict, matid_sticky_air, matid_sticky_water, matid_asthenosphere, xsize, ysize,
                        velocity_y_upper, timestep, temperature_top, temperature_bottom, sticky_thickness_left,
                        sticky_thickness_right, plate_thickness, smoothing_thickness, velocity_inflow_left,
                        velocity_inflow_right, adiabatic_gradient, mat_plastic, iuse_random_fric, delta_fric_coef,
                        seed, step) -> tuple:
    """ExtensionInflowAndOutflowAlongSides recycling; returns (fields, 1-based indices, flags, n_air)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in RECYCLE_FIELDS}
    out["matid"] = np.array(mk["matid"], dtype=np.int16, copy=True)
    out["pfailure"] = np.array(mk["pfailure"], dtype=np.float32, copy=True)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    ptrs = (C.c_void_p * len(RECYCLE_FIELDS))(*[out[k].ctypes.data for k in RECYCLE_FIELDS])
    ids = np.array([matid_sticky_air, matid_sticky_water, matid_asthenosphere], np.int16)
    d = np.array([xsize, ysize, velocity_y_upper, timestep, temperature_top, temperature_bottom,
                  sticky_thickness_left, sticky_thickness_right, plate_thickness, smoothing_thickness,
                  velocity_inflow_left, velocity_inflow_right, adiabatic_gradient, delta_fric_coef], np.float64)
    mp = np.asfortranarray(mat_plastic, dtype=np.float64)
    lst = np.zeros(max(M, 1), np.int64)
    fl = np.zeros(max(M, 1), np.int8)
    nx, ny = np.zeros(max(M, 1)), np.zeros(max(M, 1))
    n_air = C.c_int64()
    lib().o_recycle_side_inflow.restype = C.c_int64
    n = lib().o_recycle_side_inflow(C.c_int64(M), _p(inside), _p(out["matid"]), ptrs, _p(out["pfailure"]), _p(ids),
                                    _p(d), C.c_int64(mp.shape[0]), _p(mp), C.c_int64(iuse_random_fric),
                                    C.c_uint64(seed), C.c_int64(step), _p(lst), _p(fl), _p(nx), _p(ny),
                                    C.byref(n_air))
    return out, lst[:n].copy(), fl[:n].copy(), n_air.value


def recycle_fracture_zone(mk: dict, matid_sticky_air, matid_sticky_water, matid_fz, xsize, ysize,
                          full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
                          temperature_top, temperature_bottom, adiabatic_gradient, fz_thickness,
                          x_fracture_zone_start, x_fracture_zone_end, age_lithosphere_left, age_lithosphere_right,
                          thermal_lithosphere_depth_left, thermal_lithosphere_depth_right, thermal_diffusivity,
                          mat_plastic, iuse_random_fric, delta_fric_coef, seed, step, asymmetric=0) -> tuple:
    """ContractionFractureZone recycling; returns (fields, 1-based indices, flags, n_air)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in RECYCLE_FIELDS}
    out["matid"] = np.array(mk["matid"], dtype=np.int16, copy=True)
    out["pfailure"] = np.array(mk["pfailure"], dtype=np.float32, copy=True)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    ptrs = (C.c_void_p * len(RECYCLE_FIELDS))(*[out[k].ctypes.data for k in RECYCLE_FIELDS])
    ids = np.array([matid_sticky_air, matid_sticky_water, *matid_fz], np.int16)
    assert len(ids) == 9 and len(fz_thickness) == 7
    d = np.array([xsize, ysize, full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
                  temperature_top, temperature_bottom, adiabatic_gradient, *fz_thickness, x_fracture_zone_start,
                  x_fracture_zone_end, age_lithosphere_left, age_lithosphere_right, thermal_lithosphere_depth_left,
                  thermal_lithosphere_depth_right, thermal_diffusivity, delta_fric_coef], np.float64)
    assert len(d) == 24
    mp = np.asfortranarray(mat_plastic, dtype=np.float64)
    lst = np.zeros(max(M, 1), np.int64)
    fl = np.zeros(max(M, 1), np.int8)
    nx, ny = np.zeros(max(M, 1)), np.zeros(max(M, 1))
    n_air = C.c_int64()
    lib().o_recycle_fracture_zone.restype = C.c_int64
    n = lib().o_recycle_fracture_zone(C.c_int64(M), _p(inside), _p(out["matid"]), ptrs, _p(out["pfailure"]),
                                      _p(ids), _p(d), C.c_int64(int(asymmetric)), C.c_int64(mp.shape[0]), _p(mp),
                                      C.c_int64(iuse_random_fric), C.c_uint64(seed), C.c_int64(step), _p(lst),
                                      _p(fl), _p(nx), _p(ny), C.byref(n_air))
    return out, lst[:n].copy(), fl[:n].copy(), n_air.value


def recycle_no_bottom_inflow(mk: dict, matid_sticky_air, xsize, velocity_y_upper, timestep, temperature_top,
                             mat_plastic, seed, step) -> tuple:
    """ExtensionNoBottomInflow recycling; returns (fields, 1-based indices, flags)."""
    M = len(mk["x"])
    out = {k: np.array(mk[k], dtype=np.float64, copy=True) for k in RECYCLE_FIELDS}
    out["matid"] = np.array(mk["matid"], dtype=np.int16, copy=True)
    out["pfailure"] = np.array(mk["pfailure"], dtype=np.float32, copy=True)
    inside = np.ascontiguousarray(mk["inside"], dtype=np.int8)
    ptrs = (C.c_void_p * len(RECYCLE_FIELDS))(*[out[k].ctypes.data for k in RECYCLE_FIELDS])
    d = np.array([xsize, velocity_y_upper, timestep, temperature_top], np.float64)
    mp = np.asfortranarray(mat_plastic, dtype=np.float64)
    lst = np.zeros(max(M, 1), np.int64)
    fl = np.zeros(max(M, 1), np.int8)
    lib().o_recycle_no_bottom_inflow.restype = C.c_int64
    n = lib().o_recycle_no_bottom_inflow(C.c_int64(M), _p(inside), _p(out["matid"]), ptrs, _p(out["pfailure"]),
                                         C.c_int16(matid_sticky_air), _p(d), C.c_int64(mp.shape[0]), _p(mp),
                                         C.c_uint64(seed), C.c_int64(step), _p(lst), _p(fl))
    return out, lst[:n].copy(), fl[:n].copy()


def recycle_channel(y, tk, gridy_min, gridy_max, temperature_top, temperature_bottom) -> tuple:
    """Channel recycling; returns (y, tk, 1-based indices)."""
    y = np.array(y, dtype=np.float64, copy=True)
    tk = np.array(tk, dtype=np.float64, copy=True)
    lst = np.zeros(max(len(y), 1), np.int64)
    lib().o_recycle_channel.restype = C.c_int64
    n = lib().o_recycle_channel(C.c_int64(len(y)), _p(y), _p(tk), C.c_double(gridy_min), C.c_double(gridy_max),
                                C.c_double(temperature_top), C.c_double(temperature_bottom), _p(lst))
    return y, tk, lst[:n].copy()
