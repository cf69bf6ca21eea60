"""ctypes binding of include/ebgpu.h (the C-ABI of libebgpu.so).

This is the same binding a Julia host writes with ``ccall``; the field and
status enumerations mirror the header one to one.
"""
from __future__ import annotations

import ctypes as C
import pathlib

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libebgpu.so"

EB_OK, EB_NOT_CONVERGED, EB_NAN, EB_BAD_INPUT, EB_CUDA_ERROR, EB_NOT_READY = range(6)

MARKER_FIELDS = [
    "x", "y", "matid", "rho", "cohesion", "fric", "fric_ini", "eta", "eta_flow", "preexp",
    "sxx", "sxy", "exx", "exy", "pr", "sr_ratio", "gii", "strain_plastic", "strain_rate_plastic",
    "tk", "kt", "rhocp", "ha", "meltfrac", "melt_damage", "serp_hr", "pfailure", "dilatation",
    "vx", "vy", "spin", "subgrid_dt", "xn", "yn", "xn_vy", "yn_vy", "inside",
    "porosity_initial", "decay_depth", "max_burial_depth",
]
MARKER_ID = {n: i for i, n in enumerate(MARKER_FIELDS)}
MARKER_DTYPE = {n: "f8" for n in MARKER_FIELDS}
MARKER_DTYPE.update({"matid": "i2", "pfailure": "f4", "dilatation": "f4", "xn": "i4", "yn": "i4",
                     "xn_vy": "i4", "yn_vy": "i4", "inside": "i1"})

GRID_FIELDS = [
    # basic (ynum, xnum)
    "rho1", "rho0", "etas1", "etas0", "eta_flow", "eta_flow0", "mus1", "mus0", "sxy1", "sxy0",
    "plastics", "plastics0", "cohesion_grid", "cohesion_grid0", "fric_degrees_grid", "fric_degrees_grid0",
    "wtnodes", "wtetas", "tk1", "tk0", "tk2", "kt1", "kt0", "rhocp1", "rhocp0", "hr1", "hr0", "ha1", "ha0",
    "exy", "esp", "sxy2", "dsxy", "dsxyn", "dtk1", "dtkn", "plastic_yield",
    # pressure (ynum-1, xnum-1)
    "etan1", "etan0", "mun1", "mun0", "sxx1", "sxx0", "plasticn", "plasticn0", "dilatation_grid",
    "dilatation_grid0", "extractable_meltfrac_grid", "extractable_meltfrac_grid0", "wtetan", "exx",
    "sxx2", "dsxx", "dsxxn", "pr1",
    # vx / vy
    "vx1", "vy1", "rho1_vy", "rho0_vy", "wtnodes_vy",
    # thermal BC coefficients
    "btopt", "bbottomt", "bleftt", "brightt",
    # Stokes right-hand sides, plastic strain rate at pressure nodes
    "RX1", "RY1", "RC1", "eii_plastic_pressure",
    # velocity BC coefficients
    "btopx", "bbottomx", "btopy", "bbottomy", "bleftx", "brightx", "blefty", "brighty",
    # post-solve grids
    "eii", "vxb", "vyb",
    # previous Picard iterate
    "vx1_old", "vy1_old", "pr1_old",
    # nodal Picard variant (basic grid)
    "etavp_buffer", "plastic_yield_buffer", "plastic_strain_rate_buffer", "yield_error", "eii_plastic_basic",
    # heat step (basic grid)
    "RT1", "rest",
]
GRID_ID = {n: i for i, n in enumerate(GRID_FIELDS)}


def grid_shape(name: str, xnum: int, ynum: int) -> tuple[int, int]:
    i = GRID_ID[name]
    if i <= GRID_ID["plastic_yield"]:
        return (ynum, xnum)
    if i <= GRID_ID["pr1"]:
        return (ynum - 1, xnum - 1)
    if name == "vx1":
        return (ynum + 1, xnum)
    if i <= GRID_ID["wtnodes_vy"]:
        return (ynum, xnum + 1)
    if name in ("btopt", "bbottomt", "btopx", "bbottomx"):
        return (xnum, 2)
    if name in ("bleftt", "brightt", "blefty", "brighty"):
        return (ynum, 2)
    if name in ("btopy", "bbottomy"):
        return (xnum + 1, 2)
    if name in ("bleftx", "brightx"):
        return (ynum + 1, 2)
    if name == "RX1":
        return (ynum + 1, xnum)
    if name == "RY1":
        return (ynum, xnum + 1)
    if name in ("vxb", "vyb", "etavp_buffer", "plastic_yield_buffer", "plastic_strain_rate_buffer", "yield_error",
                "eii_plastic_basic", "RT1", "rest"):
        return (ynum, xnum)
    if name == "vx1_old":
        return (ynum + 1, xnum)
    if name == "vy1_old":
        return (ynum, xnum + 1)
    return (ynum - 1, xnum - 1)   # RC1, eii_plastic_pressure, eii


class GridDesc(C.Structure):
    _fields_ = [("xnum", C.c_int64), ("ynum", C.c_int64)] + [
        (n, C.c_void_p) for n in ("gridx_b", "gridy_b", "xstp_b", "ystp_b", "gridx_vy", "xstp_vy", "gridy_vx", "ystp_vx")
    ] + [(n, C.c_double) for n in ("xmin", "xmax", "ymin", "ymax", "xstpavg", "ystpavg")]


class MaterialDesc(C.Structure):
    _fields_ = [("nmat", C.c_int64)] + [
        (n, C.c_void_p) for n in ("mat_mu", "mat_hr", "mat_flow_type", "mat_flow", "mat_plastic", "mat_rho")
    ]


class Params(C.Structure):
    _fields_ = [
        ("timestep", C.c_double), ("ntimestep", C.c_int64), ("temperature_top", C.c_double),
        ("viscosity_min", C.c_double), ("viscosity_max", C.c_double), ("powerlaw_stress_min", C.c_double),
        ("yield_stress_min", C.c_double), ("yield_stress_max", C.c_double), ("gas_constant", C.c_double),
        ("iuse_viscous_strain_soft", C.c_int64), ("vsoftfac", C.c_double),
        ("iuse_fluid_pressure_for_yield", C.c_int64), ("y_sealevel", C.c_double),
        ("itype_global", C.c_int64), ("no_yielding_in_mobile_wall", C.c_int64),
        ("matid_sticky_air", C.c_int64), ("matid_mobile_wall", C.c_int64), ("matid_plate_extension", C.c_int64),
        ("plastic_healing_rate", C.c_double), ("subgrid_diff_coef_stress", C.c_double),
        ("subgrid_diff_coef_temp", C.c_double), ("iuse_melt_damage", C.c_int64),
        ("iuse_serpentinization", C.c_int64), ("iuse_topo", C.c_int64),
        ("matid_sticky_air_rho", C.c_int64), ("matid_sticky_water_rho", C.c_int64),
        ("runge_kutta_order", C.c_int64), ("temperature_bottom", C.c_double), ("temperature_left", C.c_double),
    ]


class StokesParams(C.Structure):
    _fields_ = [("gravity_x", C.c_double), ("gravity_y", C.c_double), ("iuse_interface_stabilization", C.c_int64),
                ("pressure_bc_mode", C.c_int64), ("pressure_bc", C.c_double),
                ("bintern_zone", C.c_int64 * 8), ("bintern_velocity", C.c_double * 8)]


class SolveOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("max_iters", C.c_int32), ("restart", C.c_int32), ("mg_sweeps", C.c_int32),
                ("use_initial_guess", C.c_int32), ("method", C.c_int32), ("learned", C.c_int32),
                ("precision", C.c_int32), ("gs_relax", C.c_double), ("fallback", C.c_int32),
                ("mg_inner", C.c_int32), ("mg_inner_tol", C.c_double), ("learned_warm", C.c_int32)]


class LearnedOpts(C.Structure):
    _fields_ = [("batch", C.c_int32), ("patch", C.c_int32), ("steps", C.c_int32), ("patches_per_sample", C.c_int32),
                ("mg_sweeps", C.c_int32), ("lr", C.c_double), ("seed", C.c_uint64)]


class LearnedReport(C.Structure):
    _fields_ = [("steps", C.c_int32), ("patch_h", C.c_int32), ("patch_w", C.c_int32), ("loss_first", C.c_double),
                ("loss_last", C.c_double), ("kappa", C.c_double), ("seconds", C.c_double)]


class StokesNorms(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dsoluv1_abs_inf", "dsoluv1_rel_inf", "dsoluv1_abs_L2", "dsoluv1_rel_L2", "dvx1_abs_L2", "dvx1_rel_L2",
        "dvy1_abs_L2", "dvy1_rel_L2", "dpr1_abs_L2", "dpr1_rel_L2", "dvxy_abs_inf", "dvxy_rel_inf", "dvxy_abs_L2",
        "dvxy_rel_L2", "resnl_L2")]


class MobileWall(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "timesum", "velocity_internal_x", "x_left_mobile_wall", "x_right_mobile_wall", "y_top_mobile_wall",
        "y_bottom_mobile_wall", "plate_extension_thickness", "plate_extension_width")] + [
        ("no_yielding_in_plate_extension", C.c_int64)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("levels", C.c_int32), ("rel_residual", C.c_double),
                ("rel_residual_scaled", C.c_double), ("seconds", C.c_double), ("reorthogonalisations", C.c_int32),
                ("relaxed_iterations", C.c_int32), ("fallback_used", C.c_int32), ("precision_used", C.c_int32),
                ("vcycles", C.c_int64)]


STOKES_VECTORS = {"solution": 0, "rhs": 1, "solution_old": 2, "resnl": 3}


class MarkerIO(C.Structure):
    _fields_ = [("n_in", C.c_int32), ("in_fields", C.POINTER(C.c_int32)), ("in_host", C.POINTER(C.c_void_p)),
                ("n_out", C.c_int32), ("out_fields", C.POINTER(C.c_int32)), ("out_host", C.POINTER(C.c_void_p))]


class RockDesc(C.Structure):
    _fields_ = [("nmat", C.c_int64), ("mat_rho", C.c_void_p), ("mat_cp", C.c_void_p), ("mat_kt", C.c_void_p)]


class SedimentDesc(C.Structure):
    _fields_ = [("nsed", C.c_int64), ("matids_sediments", C.c_void_p), ("ntopo", C.c_int64), ("topo_x", C.c_void_p),
                ("topo_y", C.c_void_p), ("conductivity_water", C.c_double), ("density_water", C.c_double),
                ("heat_capacity_water", C.c_double)]


class RockParams(C.Structure):
    _fields_ = [("density_model", C.c_int32), ("rhocp_model", C.c_int32), ("conductivity_model", C.c_int32),
                ("iuse_sed_porosity", C.c_int32), ("maximum_heat_capacity", C.c_double)]


class RecycleParams(C.Structure):
    _fields_ = [("recycle_type", C.c_int32), ("matid_sticky_air", C.c_int32), ("matid_sticky_water", C.c_int32),
                ("matid_asthenosphere", C.c_int32), ("xsize", C.c_double), ("ysize", C.c_double),
                ("velocity_y_upper", C.c_double), ("velocity_y_lower", C.c_double),
                ("temperature_bottom", C.c_double), ("iuse_random_fric", C.c_int32), ("delta_fric_coef", C.c_double),
                ("seed", C.c_uint64), ("counter", C.c_int64), ("asymmetric", C.c_int32),
                ("full_velocity_contraction", C.c_double), ("sticky_thickness_left", C.c_double),
                ("sticky_thickness_right", C.c_double), ("layer_thickness", C.c_double * 6),
                ("x_left_strong", C.c_double), ("x_right_strong", C.c_double), ("matid_layers", C.c_int32 * 7),
                ("matid_strong", C.c_int32 * 3), ("plate_thickness", C.c_double), ("smoothing_thickness", C.c_double),
                ("velocity_inflow_left", C.c_double), ("velocity_inflow_right", C.c_double),
                ("adiabatic_gradient", C.c_double), ("fz_thickness", C.c_double * 7),
                ("x_fracture_zone_start", C.c_double), ("x_fracture_zone_end", C.c_double),
                ("matid_fz", C.c_int32 * 7), ("age_lithosphere_left", C.c_double),
                ("age_lithosphere_right", C.c_double), ("thermal_lithosphere_depth_left", C.c_double),
                ("thermal_lithosphere_depth_right", C.c_double), ("thermal_diffusivity", C.c_double)]


class HeatParams(C.Structure):
    _fields_ = [("timestep", C.c_double), ("max_temp_change", C.c_double), ("gravity_x", C.c_double),
                ("gravity_y", C.c_double), ("iuse_adiabatic_heating", C.c_int32), ("iuse_shear_heating", C.c_int32)]


class HeatLoopReport(C.Structure):
    _fields_ = [("substeps", C.c_int32), ("solves", C.c_int32), ("iterations", C.c_int32), ("levels", C.c_int32),
                ("timestep_sum", C.c_double), ("timestep_heat", C.c_double), ("max_rel_residual", C.c_double),
                ("seconds", C.c_double)]


HEAT_ENTRY_POINTS = [
    "eb_calculate_heat_rhs_terms", "eb_initialize_old_temperature", "eb_build_heat_system", "eb_solve_heat_system",
    "eb_heat_residuals", "eb_run_conductive_heat_solver_loop", "eb_calculate_grid_temp_change",
    "eb_heat_export_coo", "eb_heat_rhs_download", "eb_heat_size",
]

STOKES_ENTRY_POINTS = [
    "eb_calc_viscoelastic_terms", "eb_viscoelastic_rhs", "eb_build_stokes_system", "eb_process_stokes_solution",
    "eb_stokes_nonlinear_residual", "eb_backup_stokes_arrays", "eb_update_grid_strain_rate_and_spin",
    "eb_forecast_viscoelastic_grid_stress", "eb_calculate_deviatoric_grid_stress_change",
    "eb_interpolate_stag_velocity_to_basic_grid", "eb_apply_nodal_plastic_yielding",
]

ENTRY_POINTS = [
    "eb_get_marker_inside_flags", "eb_initialize_bilinear_interpolation",
    "eb_interpolate_marker_stokes_parameters_to_grid", "eb_interpolate_marker_heat_parameters_to_grid",
    "eb_backup_and_clear_viscosity_transport_arrays", "eb_interpolate_viscosity_to_transport_arrays",
    "eb_interpolate_temperature_to_markers", "eb_update_marker_rheology", "eb_update_plastic_yielding",
    "eb_post_stokes_marker_gathers", "eb_update_subgrid_stress", "eb_apply_marker_stress_correction",
    "eb_subgrid_heat_diffusion_update", "eb_add_remaining_grid_change_to_marker_temperature",
    "eb_advect_markers_and_rotate_stress", "eb_update_marker_strain", "eb_correct_advect_and_update_strain",
    "eb_calc_marker_viscoplastic_viscosity", "eb_initialize_bilinear_interpolation_and_heat_scatter",
]
ALL_SYMBOLS = [
    "eb_create", "eb_destroy", "eb_last_error", "eb_set_grid", "eb_set_materials", "eb_set_params",
    "eb_resize_markers", "eb_marker_upload", "eb_marker_download", "eb_grid_upload", "eb_grid_download",
    "eb_marker_device_ptr", "eb_grid_device_ptr", "eb_stream", "eb_launch_count",
    "eb_update_marker_viscoplastic_viscosity", "eb_profile_enable", "eb_profile_count", "eb_profile_entry",
    "eb_set_stokes_params", "eb_solve_stokes_system", "eb_stokes_apply", "eb_stokes_vector_upload",
    "eb_stokes_vector_download", "eb_stokes_stencil_download", "eb_stokes_pscale", "eb_stokes_size",
    "eb_calculate_stokes_norms", "eb_interpolate_basic_viscoplastic_viscosity_to_pressure_grid",
    "eb_update_nodes_for_plastic_yielding", "eb_stokes_export_coo",
    "eb_marker_to_basic_grid_average_noalloc", "eb_marker_cycle_host", "eb_set_rock_tables",
    "eb_set_sediment_porosity", "eb_update_marker_rock_properties",
    "eb_update_model_time_step_using_displacement_limit", "eb_checkpoint_write", "eb_checkpoint_read",
    "eb_recycle_markers", "eb_recycled_markers", "eb_recycle_uniforms", "eb_nn_gemm_bf16", "eb_nn_conv2d_bf16",
    "eb_learned_init", "eb_learned_train", "eb_learned_params", "eb_learned_state", "eb_learned_forward",
    "eb_learned_loss_grad", "eb_learned_stats", "eb_update_marker_rheology_and_viscoplastic_viscosity",
] + ENTRY_POINTS + STOKES_ENTRY_POINTS + HEAT_ENTRY_POINTS

_lib = None


def load(path: pathlib.Path | str | None = None) -> C.CDLL:
    """Load libebgpu.so and declare its signatures.  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libebgpu.so not built ({p}); run earthbox_gb300.build.build()")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.eb_create.argtypes = [C.POINTER(vp), C.c_int]
    lib.eb_destroy.argtypes = [vp]
    lib.eb_last_error.argtypes = [vp]
    lib.eb_last_error.restype = C.c_char_p
    lib.eb_set_grid.argtypes = [vp, C.POINTER(GridDesc)]
    lib.eb_set_materials.argtypes = [vp, C.POINTER(MaterialDesc)]
    lib.eb_set_params.argtypes = [vp, C.POINTER(Params)]
    lib.eb_resize_markers.argtypes = [vp, C.c_int64]
    lib.eb_marker_upload.argtypes = [vp, C.c_int, vp]
    lib.eb_marker_download.argtypes = [vp, C.c_int, vp]
    lib.eb_grid_upload.argtypes = [vp, C.c_int, vp]
    lib.eb_grid_download.argtypes = [vp, C.c_int, vp]
    lib.eb_marker_device_ptr.argtypes = [vp, C.c_int, C.POINTER(vp)]
    lib.eb_grid_device_ptr.argtypes = [vp, C.c_int, C.POINTER(vp)]
    lib.eb_stream.argtypes = [vp]
    lib.eb_stream.restype = vp
    lib.eb_launch_count.argtypes = [vp]
    lib.eb_launch_count.restype = C.c_int64
    lib.eb_update_marker_viscoplastic_viscosity.argtypes = [vp, C.c_int]
    lib.eb_profile_enable.argtypes = [vp, C.c_int]
    lib.eb_profile_count.argtypes = [vp]
    lib.eb_profile_entry.argtypes = [vp, C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_int64)]
    for name in ENTRY_POINTS + STOKES_ENTRY_POINTS:
        getattr(lib, name).argtypes = [vp]
    lib.eb_set_stokes_params.argtypes = [vp, C.POINTER(StokesParams)]
    lib.eb_solve_stokes_system.argtypes = [vp, C.POINTER(SolveOpts), C.POINTER(SolveReport)]
    lib.eb_stokes_apply.argtypes = [vp, vp, vp]
    lib.eb_stokes_vector_upload.argtypes = [vp, C.c_int, vp]
    lib.eb_stokes_vector_download.argtypes = [vp, C.c_int, vp]
    lib.eb_stokes_stencil_download.argtypes = [vp, vp]
    lib.eb_calculate_stokes_norms.argtypes = [vp, C.POINTER(StokesNorms)]
    lib.eb_interpolate_basic_viscoplastic_viscosity_to_pressure_grid.argtypes = [vp, C.c_int]
    lib.eb_stokes_export_coo.argtypes = [vp, vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    lib.eb_update_nodes_for_plastic_yielding.argtypes = [vp, C.POINTER(MobileWall), C.POINTER(C.c_int64),
                                                         C.POINTER(C.c_double)]
    lib.eb_stokes_pscale.argtypes = [vp]
    lib.eb_stokes_pscale.restype = C.c_double
    lib.eb_stokes_size.argtypes = [vp]
    lib.eb_stokes_size.restype = C.c_int64
    lib.eb_marker_to_basic_grid_average_noalloc.argtypes = [vp, vp, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64,
                                                            vp, vp, vp, C.c_char_p, C.c_size_t]
    lib.eb_marker_cycle_host.argtypes = [vp, C.POINTER(MarkerIO)]
    lib.eb_recycle_markers.argtypes = [vp, C.POINTER(RecycleParams), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.eb_recycled_markers.argtypes = [vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    lib.eb_recycle_uniforms.argtypes = [C.c_uint64, C.c_int64, C.c_uint32, C.c_int64, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
    lib.eb_recycle_uniforms.restype = None
    lib.eb_nn_gemm_bf16.argtypes = [C.c_int64, C.c_int32, C.c_int64, vp, vp, vp, C.c_int32]
    lib.eb_nn_conv2d_bf16.argtypes = [C.c_int32] * 7 + [vp, vp, vp, C.c_int32, vp, vp]
    lib.eb_update_marker_rheology_and_viscoplastic_viscosity.argtypes = [vp, C.c_int]
    lib.eb_learned_init.argtypes = [vp, C.c_uint64]
    lib.eb_learned_train.argtypes = [vp, C.POINTER(LearnedOpts), C.POINTER(LearnedReport)]
    lib.eb_learned_params.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64), C.c_int32]
    lib.eb_learned_state.argtypes = [vp, vp, C.c_int32]
    lib.eb_learned_forward.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, vp]
    lib.eb_learned_loss_grad.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, vp, C.POINTER(C.c_double), vp]
    lib.eb_learned_stats.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
    lib.eb_checkpoint_write.argtypes = [vp, C.c_char_p]
    lib.eb_checkpoint_read.argtypes = [vp, C.c_char_p]
    lib.eb_set_rock_tables.argtypes = [vp, C.POINTER(RockDesc)]
    lib.eb_set_sediment_porosity.argtypes = [vp, C.POINTER(SedimentDesc)]
    lib.eb_update_marker_rock_properties.argtypes = [vp, C.POINTER(RockParams)]
    lib.eb_update_model_time_step_using_displacement_limit.argtypes = [vp, C.c_double, C.c_int32,
                                                                       C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    lib.eb_calculate_heat_rhs_terms.argtypes = [vp, C.POINTER(HeatParams)]
    lib.eb_initialize_old_temperature.argtypes = [vp]
    lib.eb_build_heat_system.argtypes = [vp, C.c_double]
    lib.eb_solve_heat_system.argtypes = [vp, C.POINTER(SolveOpts), C.POINTER(SolveReport)]
    lib.eb_heat_residuals.argtypes = [vp, C.c_double]
    lib.eb_run_conductive_heat_solver_loop.argtypes = [vp, C.POINTER(HeatParams), C.POINTER(SolveOpts),
                                                       C.POINTER(HeatLoopReport)]
    lib.eb_calculate_grid_temp_change.argtypes = [vp]
    lib.eb_heat_export_coo.argtypes = [vp, vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    lib.eb_heat_rhs_download.argtypes = [vp, vp]
    lib.eb_heat_size.argtypes = [vp]
    lib.eb_heat_size.restype = C.c_int64
    for name in ALL_SYMBOLS:
        if name not in ("eb_last_error", "eb_stream", "eb_launch_count", "eb_stokes_pscale", "eb_stokes_size",
                        "eb_heat_size", "eb_recycle_uniforms"):
            getattr(lib, name).restype = C.c_int
    if path is None:
        _lib = lib
    return lib
