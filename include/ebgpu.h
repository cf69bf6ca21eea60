/*
 * ebgpu.h -- C-ABI of the GB300 (sm_103a) marker-in-cell hot path for EarthBox.jl.
 *
 * One opaque context (eb_ctx) per GPU holds the marker SoA, the staggered grids and
 * the material tables device-resident.  The host (Julia through `ccall`, or any
 * C/C++/Python caller) uploads its arrays once, calls one entry point per
 * reference step, and copies fields back only when it needs them (output,
 * checkpoint).  Every entry point returns an int status (EB_OK on success) and
 * never aborts or traps; eb_last_error() gives the message of the last failure.
 *
 * Layout conventions are the reference's:
 *   - grid arrays are Julia column-major Matrix{Float64} of shape (rows, cols):
 *     element (i, j), 1-based, lives at offset (j-1)*rows + (i-1);
 *   - marker cell indices (marker_xn/yn, marker_xn_vy/yn_vy) are 1-based Int32;
 *   - marker_matid is Int16 (the reference's storage type) on the host and on
 *     the device; its upload checks 1 <= matid (<= nmat once materials are set);
 *   - material tables mat_flow (nmat x 17) and mat_plastic (nmat x 6) are
 *     column-major, indexed by the 1-based material id.
 * All calls are synchronous with respect to the host on return, on the
 * context's own CUDA stream.
 */
#ifndef EBGPU_H
#define EBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define EB_OK            0
#define EB_NOT_CONVERGED 1  /* iterative solve stopped before its tolerance     */
#define EB_NAN           2  /* NaN/Inf found in an input or a result            */
#define EB_BAD_INPUT     3  /* sizes, pointers or field ids out of range        */
#define EB_CUDA_ERROR    4  /* a CUDA runtime call failed (message in last_error)*/
#define EB_NOT_READY     5  /* a prerequisite step has not been run             */

typedef struct eb_ctx eb_ctx;

/* ---- grid geometry (reference: model.grids.arrays.*, model.grids.parameters.geometry) */
typedef struct eb_grid_desc {
  int64_t xnum, ynum;          /* basic-grid node counts                              */
  const double* gridx_b;       /* [xnum]    basic x coordinates                       */
  const double* gridy_b;       /* [ynum]    basic y coordinates                       */
  const double* xstp_b;        /* [xnum-1]  basic x spacings                          */
  const double* ystp_b;        /* [ynum-1]  basic y spacings                          */
  const double* gridx_vy;      /* [xnum+1]  vy-grid x coordinates                     */
  const double* xstp_vy;       /* [xnum]    vy-grid x spacings                        */
  const double* gridy_vx;      /* [ynum+1]  vx-grid y coordinates                     */
  const double* ystp_vx;       /* [ynum]    vx-grid y spacings                        */
  double xmin, xmax, ymin, ymax;  /* domain limits used by the inside test           */
  double xstpavg, ystpavg;        /* average spacings (subgrid thermal timescale)     */
} eb_grid_desc;

/* ---- material tables (reference: model.materials.arrays.*) ----------------- */
typedef struct eb_material_desc {
  int64_t nmat;
  const double*  mat_mu;        /* [nmat]      shear modulus (Pa)                     */
  const double*  mat_hr;        /* [nmat]      radiogenic heat production (W/m^3)     */
  /* mat_flow_type: the flow law of each material.  As in FlowViscosity.jl:21-44, the
   * largest value in the table selects the law of the whole model: -1 x-dependent
   * (Xdependent.jl), 0 isoviscous (Isoviscous.jl), 1 or 2 composite creep with the
   * materials of type 0 isoviscous (CompositeViscosity.jl), 4 the temperature-dependent
   * Couette-flow law (CouetteFlowBenchmark.jl: mat_flow columns 13-14), 5 the
   * Blankenbach (1989) convection law (Blankenback89.jl: columns 15-17).          */
  const int64_t* mat_flow_type; /* [nmat]                                            */
  const double*  mat_flow;      /* [nmat x 17] column-major flow-law table (the
                                 * reference's model.materials.arrays.mat_flow)       */
  const double*  mat_plastic;   /* [nmat x 6]  column-major plasticity table          */
  const double*  mat_rho;       /* [nmat]      first column of mat_rho (sticky flatten)*/
} eb_material_desc;

/* ---- scalar model parameters (reference parameter registry values) -------- */
typedef struct eb_params {
  double  timestep;                 /* s                                               */
  int64_t ntimestep;                /* current time-step counter                       */
  double  temperature_top;          /* K                                               */
  double  viscosity_min, viscosity_max;
  double  powerlaw_stress_min;      /* Pa                                              */
  double  yield_stress_min, yield_stress_max;
  double  gas_constant;             /* J/mol/K                                         */
  int64_t iuse_viscous_strain_soft; double vsoftfac;
  int64_t iuse_fluid_pressure_for_yield; double y_sealevel;
  int64_t itype_global;             /* 0 marker Picard loop, 1 nodal Picard loop       */
  int64_t no_yielding_in_mobile_wall;
  int64_t matid_sticky_air, matid_mobile_wall, matid_plate_extension; /* -1 = none   */
  double  plastic_healing_rate;     /* 1/s                                             */
  double  subgrid_diff_coef_stress, subgrid_diff_coef_temp;
  int64_t iuse_melt_damage;
  int64_t iuse_serpentinization;
  int64_t iuse_topo;                /* sticky-layer density flattening switch          */
  int64_t matid_sticky_air_rho, matid_sticky_water_rho; /* ids for flattening, -1 none */
  int64_t runge_kutta_order;        /* 1 or 4 (0 = markers do not move)                */
  double  temperature_bottom;       /* K (Blankenbach flow law, mat_flow_type 5)        */
  double  temperature_left;         /* K (Couette flow law, mat_flow_type 4)            */
} eb_params;

/* ---- marker fields ----------------------------------------------------------
 * Types on the host side of eb_marker_upload/download: F64 unless noted. */
enum eb_marker_field {
  EB_M_X = 0, EB_M_Y,                     /* marker_x, marker_y                        */
  EB_M_MATID,                             /* marker_matid       (Int16 on the host)    */
  EB_M_RHO, EB_M_COHESION, EB_M_FRIC, EB_M_FRIC_INI,
  EB_M_ETA, EB_M_ETA_FLOW, EB_M_PREEXP,
  EB_M_SXX, EB_M_SXY, EB_M_EXX, EB_M_EXY, EB_M_PR, EB_M_SR_RATIO,
  EB_M_GII, EB_M_STRAIN_PLASTIC, EB_M_STRAIN_RATE_PLASTIC,
  EB_M_TK, EB_M_KT, EB_M_RHOCP, EB_M_HA,
  EB_M_MELTFRAC,                          /* marker_extractable_meltfrac               */
  EB_M_MELT_DAMAGE, EB_M_SERP_HR,         /* melt damage factor, serpentinisation heat */
  EB_M_PFAILURE,                          /* Float32                                   */
  EB_M_DILATATION,                        /* Float32 marker_dilatation_angle           */
  EB_M_VX, EB_M_VY, EB_M_SPIN,            /* RK4 velocity/spin at the marker           */
  EB_M_SUBGRID_DT,                        /* marker_subgrid_temp_delta_buffer          */
  EB_M_XN, EB_M_YN, EB_M_XN_VY, EB_M_YN_VY, /* Int32, 1-based, download only          */
  EB_M_INSIDE,                            /* Int8 (+1 inside / -1 outside)             */
  EB_M_POROSITY_INITIAL, EB_M_DECAY_DEPTH, EB_M_MAX_BURIAL_DEPTH, /* sediment porosity (Athy's law) */
  EB_M_NFIELDS
};

/* ---- grid fields ------------------------------------------------------------
 * Shapes: B = basic (ynum, xnum); P = pressure (ynum-1, xnum-1);
 *         VX = (ynum+1, xnum); VY = (ynum, xnum+1);
 *         BCX = (xnum, 2) thermal top/bottom BC; BCY = (ynum, 2) left/right BC;
 *         velocity BC shapes are listed beside them below. */
enum eb_grid_field {
  /* basic grid */
  EB_G_RHO1 = 0, EB_G_RHO0, EB_G_ETAS1, EB_G_ETAS0, EB_G_ETA_FLOW, EB_G_ETA_FLOW0,
  EB_G_MUS1, EB_G_MUS0, EB_G_SXY1, EB_G_SXY0, EB_G_PLASTICS, EB_G_PLASTICS0,
  EB_G_COHESION, EB_G_COHESION0, EB_G_FRIC_DEG, EB_G_FRIC_DEG0,
  EB_G_WTNODES, EB_G_WTETAS,
  EB_G_TK1, EB_G_TK0, EB_G_TK2, EB_G_KT1, EB_G_KT0, EB_G_RHOCP1, EB_G_RHOCP0,
  EB_G_HR1, EB_G_HR0, EB_G_HA1, EB_G_HA0,
  EB_G_EXY, EB_G_ESP, EB_G_SXY2, EB_G_DSXY, EB_G_DSXYN, EB_G_DTK1, EB_G_DTKN,
  EB_G_PLASTIC_YIELD,
  /* pressure grid */
  EB_G_ETAN1, EB_G_ETAN0, EB_G_MUN1, EB_G_MUN0, EB_G_SXX1, EB_G_SXX0,
  EB_G_PLASTICN, EB_G_PLASTICN0, EB_G_DILAT, EB_G_DILAT0, EB_G_MELTFRAC, EB_G_MELTFRAC0,
  EB_G_WTETAN, EB_G_EXX, EB_G_SXX2, EB_G_DSXX, EB_G_DSXXN, EB_G_PR1,
  /* vx / vy grids */
  EB_G_VX1,
  EB_G_VY1, EB_G_RHO1_VY, EB_G_RHO0_VY, EB_G_WTNODES_VY,
  /* thermal boundary-condition coefficient arrays */
  EB_G_BTOPT, EB_G_BBOTTOMT, EB_G_BLEFTT, EB_G_BRIGHTT,
  /* Stokes right-hand sides RX1 (VX), RY1 (VY), RC1 (P); plastic strain rate (P) */
  EB_G_RX1, EB_G_RY1, EB_G_RC1, EB_G_EII_PLASTIC_PRESSURE,
  /* velocity boundary-condition coefficient arrays (ghost = b[:,1] + b[:,2] * interior):
   * btopx/bbottomx (xnum, 2), btopy/bbottomy (xnum+1, 2), bleftx/brightx (ynum+1, 2),
   * blefty/brighty (ynum, 2) */
  EB_G_BTOPX, EB_G_BBOTTOMX, EB_G_BTOPY, EB_G_BBOTTOMY,
  EB_G_BLEFTX, EB_G_BRIGHTX, EB_G_BLEFTY, EB_G_BRIGHTY,
  /* post-solve grids: strain-rate invariant eii (P), velocity at basic nodes vxb, vyb (B) */
  EB_G_EII, EB_G_VXB, EB_G_VYB,
  /* previous Picard iterate (SystemSolver.backup_stokes_arrays!): vx1_old (VX), vy1_old (VY), pr1_old (P) */
  EB_G_VX1_OLD, EB_G_VY1_OLD, EB_G_PR1_OLD,
  /* nodal Picard variant (all basic grid): etavp_buffer, plastic_yield_buffer,
   * plastic_strain_rate_buffer, yield_error, eii_plastic_basic */
  EB_G_ETAVP_BUFFER, EB_G_PLASTIC_YIELD_BUFFER, EB_G_PLASTIC_STRAIN_RATE_BUFFER, EB_G_YIELD_ERROR,
  EB_G_EII_PLASTIC_BASIC,
  /* heat step (basic grid): RHS terms RT1 (HeatRhs.jl), residuals rest (HeatResiduals.jl) */
  EB_G_RT1, EB_G_REST,
  EB_G_NFIELDS
};

/* ---- context ------------------------------------------------------------- */
int         eb_create(eb_ctx** out, int device);
int         eb_destroy(eb_ctx* ctx);
const char* eb_last_error(const eb_ctx* ctx);
int         eb_set_grid(eb_ctx* ctx, const eb_grid_desc* grid);
int         eb_set_materials(eb_ctx* ctx, const eb_material_desc* mats);
int         eb_set_params(eb_ctx* ctx, const eb_params* params);
int         eb_resize_markers(eb_ctx* ctx, int64_t marknum);
/* Copy one marker field between host memory and the device (count = marknum).  */
int         eb_marker_upload(eb_ctx* ctx, int field, const void* host);
int         eb_marker_download(eb_ctx* ctx, int field, void* host);
/* Copy one grid field (count = rows*cols of the field's shape).                */
int         eb_grid_upload(eb_ctx* ctx, int field, const double* host);
int         eb_grid_download(eb_ctx* ctx, int field, double* host);
/* Device pointer of a field (for callers that already hold device buffers).    */
int         eb_marker_device_ptr(eb_ctx* ctx, int field, void** dptr);
int         eb_grid_device_ptr(eb_ctx* ctx, int field, double** dptr);
/* The context's CUDA stream (cudaStream_t) for event timing by the caller.     */
void*       eb_stream(eb_ctx* ctx);
/* Number of kernels this context has launched since creation.                  */
int64_t     eb_launch_count(const eb_ctx* ctx);
/* Per-kernel timing with CUDA events on the context's stream.  Enabling (or
 * disabling) clears the counters; entries are kernels in name order, each with
 * its summed device time and launch count since the last enable.  No
 * counterpart in the reference (it times whole steps with @timeit_memit,
 * src/utils/PrintFuncs.jl:46-94).                                              */
int         eb_profile_enable(eb_ctx* ctx, int on);
int         eb_profile_count(const eb_ctx* ctx);
int         eb_profile_entry(const eb_ctx* ctx, int i, char* name, int name_len,
                             double* total_ms, int64_t* launches);

/* ---- hot-path entry points (one per reference step) -----------------------
 * Each mirrors the named reference function; inside flags are the context's
 * own (EB_M_INSIDE), set by eb_get_marker_inside_flags.                       */

/* GridFuncs.get_marker_inside_flags  (src/utils/GridFuncs.jl:54-80)            */
int eb_get_marker_inside_flags(eb_ctx* ctx);

/* InitializeInterpolation.initialize_bilinear_interpolation!
 *   (src/interpolation/initialize/InitializeInterpolation.jl:63-82):
 * upper-left indices on basic and vy grids (MarkerGridMapping.jl:78-173),
 * normalised distances and weights (recomputed on the fly, MarkerGridMapping.jl:185-265,
 * MarkerGridNodeWeights.jl:68-150), the cell-sorted marker list, and the
 * weight-sum denominators wtnodes/wtetas/wtetan/wtnodes_vy (BilinearDenominator.jl:34-157). */
int eb_initialize_bilinear_interpolation(eb_ctx* ctx);

/* eb_initialize_bilinear_interpolation followed by eb_interpolate_marker_heat_parameters_to_grid
 * (the order of MarkerInCell's marker cycle), with the weight denominators summed in the heat
 * scatter's walk of the cell lists instead of a walk of their own.  Every output (cell indices,
 * wtnodes/wtetas/wtetan/wtnodes_vy, the heat transport arrays and their backups) is
 * bit-identical to the two calls in sequence.  Needs the materials (as the heat scatter does). */
int eb_initialize_bilinear_interpolation_and_heat_scatter(eb_ctx* ctx);

/* MarkersToStokesArrays.interpolate_markers_to_transport_arrays!
 *   (src/interpolation/utils/MarkersToStokesArrays.jl:39-45): backup+clear
 * (BackupTransportArrays.jl:33-98), numerators (BilinearNumerator.jl:205-454),
 * averages (BilinearAverage.jl:57-178), sticky-layer flattening (FlattenDensity.jl:29-89). */
int eb_interpolate_marker_stokes_parameters_to_grid(eb_ctx* ctx);

/* MarkerToHeatArrays.interpolate_markers_to_transport_arrays!
 *   (src/interpolation/utils/MarkerToHeatArrays.jl:29-35): backup+clear,
 * numerators (BilinearNumerator.jl:31-141), averages (BilinearAverage.jl:10-50),
 * thermal BC rows (ApplyThermalBC.jl:20-44).                                     */
int eb_interpolate_marker_heat_parameters_to_grid(eb_ctx* ctx);

/* BackupTransportArrays.backup_and_clear_viscosity_transport_arrays!
 *   (src/interpolation/backup/BackupTransportArrays.jl:105-137)                  */
int eb_backup_and_clear_viscosity_transport_arrays(eb_ctx* ctx);

/* MarkersToStokesArrays.interpolate_viscosity_to_transport_arrays!
 *   (MarkersToStokesArrays.jl:60-64 -> BilinearNumerator.jl:470-533, BilinearAverage.jl:213-227) */
int eb_interpolate_viscosity_to_transport_arrays(eb_ctx* ctx);

/* GridTemperatureToMarkers.interpolate!  (GridTemperatureToMarkers.jl:18-45)     */
int eb_interpolate_temperature_to_markers(eb_ctx* ctx);

/* Rheology.update_marker_rheology!  (src/rheology/Rheology.jl:37-56):
 * FailureProperties.calculate_failure_properties_loop! (FailureProperties.jl:19-83) and
 * CompositeViscosity.update_marker_flow_viscosity! (CompositeViscosity.jl:133-284). */
int eb_update_marker_rheology(eb_ctx* ctx);

/* Rheology.update_marker_viscoplastic_viscosity!  (Rheology.jl:70-107):
 * ViscoplasticViscosity.jl:21-41, then (use_marker_plasticity != 0)
 * ViscoelasticForecast.update_plastic_yielding! (ViscoelasticForecast.jl:11-123). */
int eb_update_marker_viscoplastic_viscosity(eb_ctx* ctx, int use_marker_plasticity);

/* The two calls above as the time loop makes them (TimeLoop.jl:222-223), fused into one
 * marker pass: failure properties, flow viscosity, viscoplastic viscosity and (when
 * use_marker_plasticity != 0) yielding of each marker in turn.  Bit-identical to
 * eb_update_marker_rheology followed by eb_update_marker_viscoplastic_viscosity.        */
int eb_update_marker_rheology_and_viscoplastic_viscosity(eb_ctx* ctx, int use_marker_plasticity);

/* MarkerPlasticity.update_plastic_yielding! alone (Picard iterations >= 2,
 * PlasticityLoopMarkers.jl:52-57) -> ViscoelasticForecast.jl:11-123.            */
int eb_update_plastic_yielding(eb_ctx* ctx);

/* StokesContinuitySolver.execute_post_stokes_solver_steps! marker part
 * (StokesContinuitySolver.jl:286-290): MarkerStrainRate.jl:23-69,
 * MarkerStrainRateRatio.jl:191-271, MarkerPressure.jl:17-54, fused in one pass. */
int eb_post_stokes_marker_gathers(eb_ctx* ctx);

/* GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity!
 *   (src/rheology/plastic_failure/nodes/GridViscoplasticityToMarkers.jl:7-118), reached through
 * StokesContinuitySolver.interpolate_grid_viscoplastic_viscosity_to_markers! (StokesContinuitySolver.jl:256-266)
 * after the nodal Picard loop (itype_global = 1): plastic_yield and etas1 -> marker_eta, marker_pfailure.
 * Needs located markers (eb_initialize_bilinear_interpolation). */
int eb_calc_marker_viscoplastic_viscosity(eb_ctx* ctx);

/* SubGridStress.Update.update_subgrid_stress!  (subgrid_stress/update/Update.jl:69-87) */
int eb_update_subgrid_stress(eb_ctx* ctx);

/* StressCorrection.apply_marker_stress_correction_for_remaining_grid_stress!
 *   (subgrid_stress/stress_correction/StressCorrection.jl:35-82)                 */
int eb_apply_marker_stress_correction(eb_ctx* ctx);

/* SubgridDiffusion.subgrid_heat_diffusion_update! and
 * remove_subgrid_effects_from_grid_changes!  (heat_solver/subgrid_heat/SubgridDiffusion.jl:59-195) */
int eb_subgrid_heat_diffusion_update(eb_ctx* ctx);

/* MarkerTemperature.add_remaining_grid_change_to_marker_temperature!
 *   (heat_solver/marker_temperature/MarkerTemperature.jl:18-45)                  */
int eb_add_remaining_grid_change_to_marker_temperature(eb_ctx* ctx);

/* Advection.advect_markers_and_rotate_stress_tensor!  (src/advection/Advection.jl:109-114):
 * VelocityAndSpin.update_marker_velocity_and_spin_using_runge_kutta! (VelocityAndSpin.jl:45-129),
 * MarkersLocation.update! (MarkersLocation.jl:11-39), MarkersStressRotation.update!
 * (MarkersStressRotation.jl:15-75), fused into one pass over the markers.        */
int eb_advect_markers_and_rotate_stress(eb_ctx* ctx);

/* Advection.update_marker_strain!  (Advection.jl:169-178 -> MarkersStrain.jl:11-136) */
int eb_update_marker_strain(eb_ctx* ctx);

/* eb_apply_marker_stress_correction, eb_add_remaining_grid_change_to_marker_temperature,
 * eb_advect_markers_and_rotate_stress and eb_update_marker_strain in one pass over the
 * markers (each marker's fields read and written once), with the same results as the
 * four calls in that order.  Between eb_subgrid_heat_diffusion_update and the next time
 * step, the reference runs these four (StokesContinuitySolver.jl:365-381,
 * HeatSolver.jl:94-122, TimeLoop.jl:261); nothing it does in between reads or writes the
 * fields involved.                                                                  */
int eb_correct_advect_and_update_strain(eb_ctx* ctx);

/* ---- Stokes-continuity step --------------------------------------------------
 * The grid-side half of StokesContinuitySolver.solve_viscoelastic_stokes_continuity_equations!
 * (src/stokes_continuity_solver/StokesContinuitySolver.jl:68-110).  Inputs are
 * context grid fields (eb_grid_upload): etas1, mus1, sxy1, etan1, mun1, sxx1,
 * rho1, rho1_vy, dilatation_grid, eii_plastic_pressure and the eight velocity
 * BC arrays; outputs are etas0, sxy0, etan0, sxx0, RX1, RY1, RC1, vx1, vy1, pr1
 * and the solution vector S.
 * The system has N = 3 (xnum-1)(ynum-1) unknowns interleaved per basic cell
 * (vx, vy, p / pscale), cells column-major (GlobalIndices.jl:13-27), exactly
 * the reference's S.  It is kept on the device as a stored 27-coefficient
 * stencil per cell whose values are the reference's COO values (Li, Lj, Lv). */
typedef struct eb_stokes_params {
  double  gravity_x, gravity_y;          /* m/s^2 (model.gravity.parameters)                    */
  int64_t iuse_interface_stabilization;  /* 1: drho/dx, drho/dy g dt terms in the y-Stokes rows  */
  int64_t pressure_bc_mode;              /* 0 upper-left cell, 1 top/bottom rows, 2 left/right   */
  double  pressure_bc;                   /* Pa                                                   */
  int64_t bintern_zone[8];               /* internal prescribed-velocity zone, reference layout  */
  double  bintern_velocity[8];
} eb_stokes_params;

/* Options of the iterative solve that replaces the direct sparse solve. */
typedef struct eb_solve_opts {
  double  rtol;              /* stop when ||R - L S|| <= rtol ||R|| (the reference's assembled system; the
                                iteration runs on the W-scaled system and tightens its own target
                                until this holds); 0 -> 1e-8                                     */
  int32_t max_iters;         /* FGMRES iterations; 0 -> 3000                                          */
  int32_t restart;           /* Krylov basis size (FGMRES restarts after this many iterations); 0 -> 500,
                                the most allowed (Stokes; unused by the heat solve): restarting after
                                250 stalled on systems that converge within 550 unrestarted          */
  int32_t mg_sweeps;         /* red-black Gauss-Seidel sweeps before/after each coarse correction; 0 -> 3 */
  int32_t use_initial_guess; /* 1: start from the current device solution vector (a solution of an
                                earlier system has its pressure unknowns rescaled to this system's
                                pscale), 0: from zero                                                */
  int32_t method;            /* 0: FGMRES (long recurrence, robust); 1: BiCGStab (short recurrence, two
                                preconditioner applications per iteration)                           */
  int32_t learned;           /* 1: after each V-cycle, the learned stage (eb_learned_train) adds its
                                correction when that lowers the preconditioner residual (FGMRES only;
                                Stokes only)                                                        */
  int32_t precision;         /* 0: mixed (FP32 V-cycle, FP32 stored directions, FP64 FGMRES);
                                1: plain FP64 (V-cycle and directions in FP64; Stokes only)          */
  double  gs_relax;          /* mixed method only: once the FGMRES residual estimate is below
                                gs_relax x the target, Gram-Schmidt projects with FP32 products on
                                FP32 copies of the basis, before that with double-float products
                                (Dot2) on the basis split into FP32 hi + lo; 0 -> 1e3, negative ->
                                FP64 products throughout (Stokes only)                               */
  int32_t fallback;          /* mixed method only: 0 -> the plain FP64 method takes over whenever the
                                mixed method's FP64 residual fails to fall (an FGMRES cycle that does
                                not halve the true residual, the iteration limit reached, or NaN/Inf),
                                continuing from the mixed iterate (from zero after NaN/Inf) with
                                max_iters iterations of its own; negative -> no fallback (Stokes only) */
  int32_t mg_inner;          /* velocity stage of the preconditioner: 1 -> one V-cycle; k > 1 -> up to k
                                steps of GCR on the velocity block, each preconditioned by one V-cycle,
                                until the velocity residual falls below mg_inner_tol of its start
                                (at most 8); 0 -> 1 (Stokes only)                                    */
  double  mg_inner_tol;      /* 0 -> 0.1 */
  int32_t learned_warm;      /* with learned = 1 and use_initial_guess = 1: the learned stage also corrects
                                the initial guess, xhat += a NN(residual) when that lowers the residual
                                (the Picard warm start); Stokes only                                  */
} eb_solve_opts;

typedef struct eb_solve_report {
  int32_t iterations;        /* FGMRES iterations run                                   */
  int32_t levels;            /* multigrid levels of the velocity preconditioner         */
  double  rel_residual;      /* ||R - L S||_2 / ||R||_2 of the assembled (unscaled) system */
  double  rel_residual_scaled; /* the same for the diagonally scaled system             */
  double  seconds;           /* wall time of the solve                                  */
  int32_t reorthogonalisations; /* Gram-Schmidt second passes (severe cancellation only) */
  int32_t relaxed_iterations;   /* iterations whose Gram-Schmidt ran in FP32 (gs_relax)  */
  int32_t fallback_used;     /* 1: the mixed method's residual stopped falling and the plain FP64
                                method finished the solve (iterations and seconds cover both)  */
  int32_t precision_used;    /* method that produced S: 0 mixed, 1 plain FP64                  */
  int64_t vcycles;           /* V-cycles run (one per iteration, or the GCR steps of mg_inner) */
} eb_solve_report;

enum eb_stokes_vector {
  EB_SV_SOLUTION = 0,        /* S (soluv1)                                  */
  EB_SV_RHS,                 /* R (RHS)                                     */
  EB_SV_SOLUTION_OLD,        /* S of the previous Picard iteration (soluv1_old) */
  EB_SV_RESNL                /* |L S_old - R| (resnl)                       */
};

int eb_set_stokes_params(eb_ctx* ctx, const eb_stokes_params* p);

/* StokesViscoelasticTerms.calc_viscoelastic_terms!  (solver/rhs/StokesViscoelasticTerms.jl:26-125) */
int eb_calc_viscoelastic_terms(eb_ctx* ctx);

/* StokesContinuityRhs.viscoelastic_rhs!  (solver/rhs/StokesContinuityRhs.jl:30-190) */
int eb_viscoelastic_rhs(eb_ctx* ctx);

/* SystemSolver.initialize_solver! (solver/system_solver/SystemSolver.jl:99-115: vx1, vy1, pr1
 * zeroed, pscale = 2 etan0[1,1] / (xstpavg + ystpavg)) followed by
 * StokesBuildManager.build_system_of_equations (solver/build_system/StokesBuildManager.jl:661-712). */
int eb_build_stokes_system(eb_ctx* ctx);

/* Replaces SystemSolver.solve_system_optimized (SystemSolver.jl:67-91), whose direct
 * sparse solve (MUMPS, ParallelSolver.jl:52-126, or UMFPACK) becomes FGMRES in FP64,
 * preconditioned by a block-triangular split: FP32 geometric multigrid on the velocity
 * block and a viscosity-scaled diagonal on the pressure.  The mixed method falls back to the
 * plain FP64 method when its residual stops falling (opts->fallback).  EB_NOT_CONVERGED when
 * the tolerance is not met (S then holds the last iterate), EB_NAN on NaN/Inf in the
 * right-hand side or a solution that the fallback could not repair. */
int eb_solve_stokes_system(eb_ctx* ctx, const eb_solve_opts* opts, eb_solve_report* report);

/* SystemSolver.process_stokes_solution!  (SystemSolver.jl:141-271: reload_solu_vel!, apply_vel_bc!) */
int eb_process_stokes_solution(eb_ctx* ctx);

/* StokesResiduals.stokes_calc_nonlinear_system_residual_optimized!  (solver/residuals/StokesResiduals.jl:63-81):
 * resnl = |L S_old - R|, kept as EB_SV_RESNL. */
int eb_stokes_nonlinear_residual(eb_ctx* ctx);

/* SystemSolver.backup_stokes_arrays!  (SystemSolver.jl:306-318): S_old = S, vx1_old = vx1,
 * vy1_old = vy1, pr1_old = pr1 (vxy_old is vx1_old and vy1_old in row-major order). */
int eb_backup_stokes_arrays(eb_ctx* ctx);

/* StokesNorms.calculate_stokes_norms! (solver/norms/StokesNorms.jl:8-160) without the grid residual
 * arrays: the solution-change norms of calculate_solution_norms! (:64-120, MathTools.get_L2_norms /
 * get_inf_norms: abs = |v - v_old|, rel = abs / |v| or 1e38 when |v| = 0) and |resnl|_2. */
typedef struct eb_stokes_norms {
  double dsoluv1_abs_inf, dsoluv1_rel_inf, dsoluv1_abs_L2, dsoluv1_rel_L2;
  double dvx1_abs_L2, dvx1_rel_L2, dvy1_abs_L2, dvy1_rel_L2, dpr1_abs_L2, dpr1_rel_L2;
  double dvxy_abs_inf, dvxy_rel_inf, dvxy_abs_L2, dvxy_rel_L2;
  double resnl_L2;
} eb_stokes_norms;
int eb_calculate_stokes_norms(eb_ctx* ctx, eb_stokes_norms* out);

/* Post-solve grid kernels (src/stokes_continuity_solver/utils/):
 * GridStrainRate.update_grid_strain_rate_and_spin! (strain_rate/GridStrainRate.jl:6-182): exx, exy, eii, esp */
int eb_update_grid_strain_rate_and_spin(eb_ctx* ctx);
/* GridStress.forecast_viscoelastic_grid_stress! (GridStress.jl:30-126): sxy2, sxx2 */
int eb_forecast_viscoelastic_grid_stress(eb_ctx* ctx);
/* GridStress.calculate_deviatoric_grid_stress_change! (GridStress.jl:128-134): dsxy, dsxx */
int eb_calculate_deviatoric_grid_stress_change(eb_ctx* ctx);
/* Interpolation.interpolate_basic_viscoplastic_viscosity_to_pressure_grid! (src/interpolation/Interpolation.jl:97-108):
 * when iuse_harmonic (interp_options.iuse_harmonic_avg_normal_viscosity) is 1, yielding cells take
 * etan1 = harmonic mean of their corner etas1 (HarmonicAverage.jl:20-51); otherwise nothing happens. */
int eb_interpolate_basic_viscoplastic_viscosity_to_pressure_grid(eb_ctx* ctx, int iuse_harmonic);
/* StokesInterpolate.interpolate_stag_velocity_to_basic_grid! (StokesInterpolate.jl:16-33): vxb, vyb */
int eb_interpolate_stag_velocity_to_basic_grid(eb_ctx* ctx);

/* Nodal Picard variant (itype_global = 1). */
typedef struct eb_mobile_wall {
  double  timesum;                     /* model time (s): walls move with velocity_internal_x         */
  double  velocity_internal_x;
  double  x_left_mobile_wall, x_right_mobile_wall, y_top_mobile_wall, y_bottom_mobile_wall;
  double  plate_extension_thickness, plate_extension_width;
  int64_t no_yielding_in_plate_extension;
} eb_mobile_wall;

/* PlasticFailureNodes.update_nodes_for_plastic_yielding (rheology/plastic_failure/nodes/
 * PlasticFailureNodes.jl:24-184): Drucker-Prager yield on the basic grid from etas1, eta_flow, mus1,
 * cohesion_grid, fric_degrees_grid, plastic_yield, sxy2, sxx2, pr1.  Writes etavp_buffer,
 * plastic_yield_buffer, plastic_strain_rate_buffer and yield_error (at yielding nodes), and returns
 * nnode_yield and global_yield_error = sqrt(sum err^2 / nnode_yield).  `wall` may be NULL (no mobile
 * wall); eb_params.no_yielding_in_mobile_wall switches the wall test on. */
int eb_update_nodes_for_plastic_yielding(eb_ctx* ctx, const eb_mobile_wall* wall, int64_t* nnode_yield,
                                         double* global_yield_error);

/* The updates PlasticityLoopNodes.picard_loop makes when nnode_yield > 0
 * (plasticity_loop_nodes/PlasticityLoopNodes.jl:36-92, :128-152): etas1 = etavp_buffer,
 * plastic_yield = plastic_yield_buffer, eii_plastic_basic = plastic_strain_rate_buffer, and
 * eii_plastic_pressure = the 4-node average (PlasticStrainRateInterpolation.jl:13-40). */
int eb_apply_nodal_plastic_yielding(eb_ctx* ctx);

/* No counterpart in the reference (its COO product): y = L x for host vectors of N doubles. */
int eb_stokes_apply(eb_ctx* ctx, const double* x, double* y);

/* Copies of the N-vectors named by enum eb_stokes_vector (host arrays, interleaved layout).  An
 * uploaded solution is taken to be in the current system's pressure scale (its pressure unknowns
 * p / pscale of the last assembled system). */
int eb_stokes_vector_upload(eb_ctx* ctx, int which, const double* host);
int eb_stokes_vector_download(eb_ctx* ctx, int which, double* host);

/* The assembled system as the reference's COO list: Li, Lj 1-based (Int64), Lv (Float64), in
 * StokesBuildManager.build_system_of_equations' entry order (StokesBuildManager.jl:661-712), entry for
 * entry the reference's system_vectors (Li_out, Lj_out, Lv_out); with the RHS from
 * eb_stokes_vector_download(EB_SV_RHS) it is what parallel_direct_solver (ParallelSolver.jl:52) takes,
 * so MUMPS stays usable on a GPU-assembled system.  Host arrays of `capacity` entries; with Li, Lj or
 * Lv null only *nnz is set (size query). */
int eb_stokes_export_coo(eb_ctx* ctx, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity, int64_t* nnz);

/* The assembled coefficients: 27 slots x (xnum-1)(ynum-1) cells, slot-major, cells
 * column-major.  Slots 0-10: x-Stokes row (vx C, L, R, U, D; vy UL, UR, LL, LR; p L, R),
 * 11-21: y-Stokes row (vy C, U, D, L, R; vx UL, UR, LL, LR; p U, D), 22-26: continuity
 * row (p C; vx L, R; vy U, D).  Neighbours: L/R = cell column -/+ 1, U/D = row -/+ 1. */
int eb_stokes_stencil_download(eb_ctx* ctx, double* host);

double  eb_stokes_pscale(const eb_ctx* ctx);  /* pscale of the last eb_build_stokes_system */
int64_t eb_stokes_size(const eb_ctx* ctx);    /* N = 3 (xnum-1)(ynum-1), 0 before eb_set_grid */

/* ---- conductive heat step (src/heat_solver) --------------------------------
 * Grid fields read: tk1, kt1, rhocp1, hr1, ha1, rho1, vx1, vy1, sxy2, etas1, sxx2,
 * etan1 and the thermal BC arrays btopt, bbottomt (xnum, 2), bleftt, brightt (ynum, 2)
 * (tk[1,j] = btopt[j,1] + btopt[j,2] tk[2,j], and so on).  Written: RT1, tk0, tk2,
 * dtk1, rest.  The heat system has N = xnum*ynum unknowns, node (i, j) at
 * (j-1)*ynum + i (the reference's itk, HeatBuildManager.jl:55). */
typedef struct eb_heat_params {
  double  timestep;                /* main time step (s): the heat loop integrates over it      */
  double  max_temp_change;         /* K: larger grid changes shorten the heat-loop step        */
  double  gravity_x, gravity_y;    /* adiabatic heating term (HeatRhs.jl:28-47)                */
  int32_t iuse_adiabatic_heating;  /* 1: add alpha*T*rho*(g . v) to RT1                         */
  int32_t iuse_shear_heating;      /* 1: add sxy2^2/etas1 + <sxx2^2/etan1> to RT1               */
} eb_heat_params;

typedef struct eb_heat_loop_report {
  int32_t substeps;        /* passes of the heat loop                                      */
  int32_t solves;          /* heat solves (a pass that shortens its step solves twice)     */
  int32_t iterations;      /* conjugate-gradient iterations over all solves                */
  int32_t levels;          /* multigrid levels of the preconditioner                       */
  double  timestep_sum;    /* integrated heat time (s) = timestep on exit                  */
  double  timestep_heat;   /* heat-loop step after the last pass (s)                       */
  double  max_rel_residual;/* largest ||R - L T||_2 / ||R||_2 over the solves              */
  double  seconds;         /* wall time of the loop                                        */
} eb_heat_loop_report;

/* HeatSolver.calculate_heat_rhs_terms_grid! (heat_solver/HeatSolver.jl:139-150):
 * RT1 = hr1 (+ adiabatic, + shear heating terms, rhs/HeatRhs.jl:5-80).                */
int eb_calculate_heat_rhs_terms(eb_ctx* ctx, const eb_heat_params* hp);
/* HeatSolver.initialize_old_temperature_array! (HeatSolver.jl:199-204): tk0 = tk1.   */
int eb_initialize_old_temperature(eb_ctx* ctx);
/* HeatBuildManager.build_system_of_equations (solver/build_system/HeatBuildManager.jl:44-86)
 * for the heat-loop step timestep_heat: the 5-point system in the reference's coefficients
 * (bit-identical) from tk0, rhocp1, kt1, RT1 and the thermal BC arrays.                */
int eb_build_heat_system(eb_ctx* ctx, double timestep_heat);
/* The solve of SystemSolver.discretize_and_solve_conductive_heat_equation
 * (solver/SystemSolver.jl:32-66: MUMPS or UMFPACK) and reload_solu_temp (:85-110):
 * tk2 = L^-1 R.  The BC rows are folded into an area-scaled symmetric system on the
 * internal nodes, solved by flexible conjugate gradients with an FP32 multigrid
 * V-cycle; the BC rows then give the boundary values exactly.  opts: rtol (default
 * 1e-12, on the scaled internal system), max_iters, mg_sweeps (default 2),
 * use_initial_guess (1: start from tk0; default); restart and method are unused.
 * report->rel_residual is ||R - L tk2||_2 / ||R||_2 of the reference's system.        */
int eb_solve_heat_system(eb_ctx* ctx, const eb_solve_opts* opts, eb_solve_report* report);
/* HeatResiduals.compute_residuals_temp! (solver/residuals/HeatResiduals.jl:12-162):
 * rest from RT1, rhocp1, tk0, tk2, kt1 at the heat-loop step timestep_heat.           */
int eb_heat_residuals(eb_ctx* ctx, double timestep_heat);
/* HeatLoop.run_conductive_heat_solver_loop! (heat_loop/HeatLoop.jl:10-79): the
 * adaptive heat loop over hp->timestep, each pass building, solving and computing the
 * residuals, shortening its step to max_temp_change / max|tk2 - tk0| when the change
 * exceeds max_temp_change, then tk0 = tk2.  Leaves dtk1 = tk2 - tk0 of the last pass's
 * first solve, as the reference does.                                                 */
int eb_run_conductive_heat_solver_loop(eb_ctx* ctx, const eb_heat_params* hp, const eb_solve_opts* opts,
                                       eb_heat_loop_report* report);
/* HeatSolver.calculate_grid_temp_change! (HeatSolver.jl:211-216): dtk1 = tk2 - tk1.   */
int eb_calculate_grid_temp_change(eb_ctx* ctx);
/* The assembled heat system as the reference's COO list (1-based Li, Lj; Lv) in
 * HeatBuildManager's entry order, for parallel_direct_solver or UMFPACK on the host;
 * with Li, Lj or Lv null only *nnz is set.                                             */
int eb_heat_export_coo(eb_ctx* ctx, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity, int64_t* nnz);
/* The right-hand side R of the last eb_build_heat_system (N doubles).                 */
int eb_heat_rhs_download(eb_ctx* ctx, double* host);
int64_t eb_heat_size(const eb_ctx* ctx);      /* N = xnum*ynum, 0 before eb_set_grid */

/* ---- step boundary: rock properties and the time step ---------------------- */
/* Material tables of the rock-property models (model.materials.arrays.*). */
typedef struct eb_rock_desc {
  int64_t nmat;
  const double* mat_rho;   /* [nmat x 3] column-major: standard density, expansivity, compressibility */
  const double* mat_cp;    /* [nmat]     heat capacity (J/kg/K; at 20 C for the Waples model)         */
  const double* mat_kt;    /* [nmat x 2] column-major: reference conductivity, factor a              */
} eb_rock_desc;
int eb_set_rock_tables(eb_ctx* ctx, const eb_rock_desc* tables);

/* Sediment porosity (PorosityUpdate.jl): sediment material ids, the topography
 * (gridt rows 1 and 2: x and y of the sediment-water interface) and water properties. */
typedef struct eb_sediment_desc {
  int64_t nsed;
  const int16_t* matids_sediments;   /* materials.dicts.matid_types["Sediment"]             */
  int64_t ntopo;
  const double* topo_x;              /* gridt[1, :] (increasing)                            */
  const double* topo_y;              /* gridt[2, :]                                         */
  double conductivity_water, density_water, heat_capacity_water;
} eb_sediment_desc;
int eb_set_sediment_porosity(eb_ctx* ctx, const eb_sediment_desc* sed);

typedef struct eb_rock_params {
  int32_t density_model;       /* DensityModel options: 0 Liao14, 1 Blankenbach89, 2 Naliboff17          */
  int32_t rhocp_model;         /* RhoCpModel options: 0 Constant, 1 TemperatureDependentWaples           */
  int32_t conductivity_model;  /* ThermalConductivityModel options: 0 Liao14, 1 Uniform, 2 Temperature-
                                  Dependent, 3 Naliboff17, 4 Adiabatic, 5 SekiguchiWaples                 */
  int32_t iuse_sed_porosity;   /* 1: porosity correction of sediment markers (eb_set_sediment_porosity)  */
  double  maximum_heat_capacity;  /* J/kg/K cap of the Waples model                                    */
} eb_rock_params;
/* RockProperties.update_marker_rock_properties! (rock_properties/RockProperties.jl:99-125):
 * marker rho, rhocp, kt and ha of inside markers from matid, x, y, pr, tk (and the
 * porosity fields); temperature_top comes from eb_params.                            */
int eb_update_marker_rock_properties(eb_ctx* ctx, const eb_rock_params* p);

/* Update.update_model_time_step_using_displacement_limit (time_step/update/Update.jl:16-33):
 * the new main time step from vx1, vy1 (average spacings, or every staggered node when
 * iuse_local_adaptive_time_stepping == 1); *timestep is the old step on entry and the
 * new one on return, *timestep_update = (new != old).                                 */
int eb_update_model_time_step_using_displacement_limit(eb_ctx* ctx, double marker_cell_displ_max,
                                                       int32_t iuse_local_adaptive_time_stepping,
                                                       double* timestep, int32_t* timestep_update);

/* ---- marker recycling ------------------------------------------------------
 * MarkerRecycle.recycle_markers! for the extension models (boundary_conditions/marker_recycle/
 * types/Extension.jl:14-129 with utils/{InitializeMarkerRecycling,Coordinates,ResetMarkers,
 * PressureReset}.jl): the markers whose inside flag (eb_get_marker_inside_flags) is not +1,
 * in marker order, re-enter in the top band (sticky-air/water material) or the bottom band
 * (the rest) at uniformly random positions and have their properties reset (sticky air at
 * temperature_top; asthenosphere at temperature_bottom with the lithostatic reset pressure,
 * stress 1.96e6 Pa, strain rate 1e-14 1/s, viscosity 1e20 Pa s).  The uniforms come from
 * Philox-4x32-10 keyed by `seed`, counter (index, stream, `counter`): the reference uses
 * Julia's global generator, so positions match it in distribution, not value.  Fields the
 * context does not hold (serpentinisation, extracted melt, stratigraphic age) are reset by
 * the caller for the markers eb_recycled_markers lists.                            */
typedef struct eb_recycle_params {
  int32_t recycle_type;            /* 1: extension models (fixed boundaries, asymmetric, depth dependent)
                                      (types/Extension.jl:14-129); 2: extension without bottom inflow
                                      (types/ExtensionNoBottomInflow.jl:8-123: every outside marker
                                      re-enters in the top band as sticky air, one uniform for x and y,
                                      band vyu dt with its sign); 3: channel (types/Channel.jl:20-54:
                                      markers below gridy_b[ynum] move up by the grid height and
                                      their temperature by temperature_top - temperature_bottom; the
                                      inside flags are not used); 4: contraction, 5: extension with
                                      side inflow and outflow, 6: fracture-zone contraction (fields
                                      below)                                                        */
  int32_t matid_sticky_air, matid_sticky_water, matid_asthenosphere;  /* material ids                 */
  double  xsize, ysize;            /* model size (m); the domain starts at x = y = 0                    */
  double  velocity_y_upper, velocity_y_lower;  /* vyu, vyl (m/s): band widths |v dt|                   */
  double  temperature_bottom;      /* K (temperature_top comes from eb_params)                          */
  int32_t iuse_random_fric;        /* 1: fric_ini - delta_fric_coef for half of the subsurface markers  */
  double  delta_fric_coef;
  uint64_t seed;                   /* Philox key                                                        */
  int64_t counter;                 /* e.g. the time-step number: new numbers every call                 */
  /* recycle_type 4: contraction (ViscoelasticContraction -> types/ContractionViscoelastic.jl:20-134):
     outside sticky and subsurface markers re-enter at the two sides (ContractionRecycleLocations.jl),
     subsurface ones as the seven-layer / strong-zone material of their new position at pressure
     3300 * 9.81 * y and temperature 0                                                              */
  int32_t asymmetric;              /* 1: every marker enters at the right side (band |v| dt), 0: half at
                                      each side (band |v| dt / 2)                                   */
  double  full_velocity_contraction;  /* m/s                                                         */
  double  sticky_thickness_left, sticky_thickness_right;  /* StickyThickness.get_sticky_thickness (m) */
  double  layer_thickness[6];      /* thick_air, upper crust, lower crust, upper / middle / lower mantle
                                      lithosphere (LithosphericExtension.get_layer_thickness)       */
  double  x_left_strong, x_right_strong;  /* strong zones outside [x_left_strong, x_right_strong]     */
  int32_t matid_layers[7];         /* Atmosphere, UpperContinentalCrust, LowerContinentalCrust,
                                      Upper-, Middle-, LowerMantleLithosphere, Asthenosphere        */
  int32_t matid_strong[3];         /* Upper-, LowerContinentalCrustStrongZone, LithosphericMantleStrongZone */
  /* recycle_type 5: extension with side inflow and outflow
     (LithosphericExtensionInflowAndOutflowAlongSides -> types/ExtensionInflowAndOutflowAlongSides.jl):
     sticky markers as type 1, subsurface ones at the two sides below sticky + plate + smoothing
     (sticky_thickness_left/right above), as asthenosphere                                          */
  double  plate_thickness, smoothing_thickness;          /* OutflowGeometry.get_outflow_geometry (m) */
  double  velocity_inflow_left, velocity_inflow_right;   /* m/s                                      */
  double  adiabatic_gradient;      /* K/km: T = temperature_bottom - gradient (ysize - y) / 1000     */
  /* recycle_type 6: fracture-zone contraction (FractureZoneContractionFixedBoundaries[Asymmetric] ->
     types/ContractionFractureZone.jl): positions as type 4 (asymmetric, full_velocity_contraction,
     sticky_thickness_left/right); subsurface markers take the material and the temperature of the
     fracture-zone initial model (FractureZoneProperties.jl), pressure 3300 * 9.81 * y;
     adiabatic_gradient as above                                                                    */
  double  fz_thickness[7];         /* thick_air, sediment, basaltic crust, gabbroic crust, younger /
                                      older / weak lithosphere (FractureZone.define_geometry)       */
  double  x_fracture_zone_start, x_fracture_zone_end;
  int32_t matid_fz[7];             /* Atmosphere, SedimentaryBasin, BasalticOceanicCrust,
                                      GabbroicOceanicCrust, MantleLithosphere, WeakMantleLithosphere,
                                      Asthenosphere                                                 */
  double  age_lithosphere_left, age_lithosphere_right;   /* Myr                                      */
  double  thermal_lithosphere_depth_left, thermal_lithosphere_depth_right;  /* m                      */
  double  thermal_diffusivity;     /* m^2/s                                                          */
} eb_recycle_params;
int eb_recycle_markers(eb_ctx* ctx, const eb_recycle_params* p, int64_t* nrecycle_air, int64_t* nrecycle_subsurface);
/* The markers of the last eb_recycle_markers: 1-based indices and flags (0 sticky, 1 subsurface),
 * in marker order; with null arrays only *n is set.                                   */
int eb_recycled_markers(eb_ctx* ctx, int64_t* indices, int8_t* flags, int64_t capacity, int64_t* n);
/* The two uniforms of Philox-4x32-10 at (seed; j, stream, counter), as the recycling uses them. */
void eb_recycle_uniforms(uint64_t seed, int64_t counter, uint32_t stream, int64_t j, double* u0, double* u1);

/* ---- tensor-core building blocks of the learned preconditioner ----------------
 * Host-array entry points (temporary device buffers) for one BF16 GEMM / convolution on the
 * tcgen05 tensor cores with FP32 accumulation; BF16 values are passed as their uint16 bits.
 * eb_nn_gemm_bf16: D[M x N] (FP32, row-major) = A[M x K] . B[N x K]^T, K a multiple of 8;
 *   splits > 1 splits K across CTAs (partials summed on the host in split order).
 * eb_nn_conv2d_bf16: y[B,H,W,Cout] = conv(x[B,H,W,C], w[Cout][taps*C]) with zero padding,
 *   taps 9 (3x3, tap = 3(dy+1)+(dx+1)) or 1; flip 1 reads offset -d (input gradient);
 *   mode 0: FP32 output y32; 1: BF16 y16 = relu(acc + bias); 2: BF16 y16 = acc + bias. */
int eb_nn_gemm_bf16(int64_t M, int32_t N, int64_t K, const uint16_t* A, const uint16_t* B, float* D, int32_t splits);
int eb_nn_conv2d_bf16(int32_t B, int32_t H, int32_t W, int32_t C, int32_t Cout, int32_t taps, int32_t flip,
                      const uint16_t* x, const uint16_t* w, const float* bias, int32_t mode, float* y32,
                      uint16_t* y16);

/* ---- learned preconditioner stage --------------------------------------------
 * A BF16 convolutional U-Net (FP32 accumulation, tcgen05 tensor cores; 4 levels of 32, 64,
 * 128, 128 channels, 1.1M parameters) mapping (log10 viscosity, density, residual r / RMS(r))
 * on the Stokes cells to the correction e with A e = r of the diagonally scaled system.
 * eb_learned_train trains it on the GPU (forward, backward and Adam on the device) on pairs
 * generated from the current assembled system: e = z - P(A z) for z = P(noise), r = A e (P the
 * multigrid preconditioner), patches of patch x patch cells.  eb_solve_opts.learned = 1 then
 * applies z += a NN(v - A z) after each V-cycle inside FGMRES, a minimising |v - A z| (kept
 * when a > 0).                                                                             */
typedef struct eb_learned_opts {
  int32_t batch;             /* patches per optimizer step (1..16)                               */
  int32_t patch;             /* patch side in cells (multiple of 8; clipped to the grid)           */
  int32_t steps;             /* optimizer steps                                                   */
  int32_t patches_per_sample;/* optimizer steps per generated full-grid sample                     */
  int32_t mg_sweeps;         /* V-cycle sweeps of P (0 -> 3)                                       */
  double  lr;                /* Adam learning rate                                                 */
  uint64_t seed;             /* Philox noise and patch offsets                                     */
} eb_learned_opts;
typedef struct eb_learned_report {
  int32_t steps, patch_h, patch_w;
  double  loss_first, loss_last;  /* mean MSE of the first and of the last min(8, steps/2) steps */
  double  kappa;                  /* RMS(e) / RMS(r) scale of the output                          */
  double  seconds;
} eb_learned_report;
int eb_learned_init(eb_ctx* ctx, uint64_t seed);  /* He-normal weights                            */
int eb_learned_train(eb_ctx* ctx, const eb_learned_opts* opts, eb_learned_report* report);
/* FP32 parameters, per layer [cout][taps][cin] weights then [cout] biases; set 1 uploads.  */
int eb_learned_params(eb_ctx* ctx, float* params, int64_t capacity, int64_t* n, int32_t set);
/* state[6]: eta mean, eta 1/std, rho mean, rho 1/std, kappa, trained flag; set 1 uploads.   */
int eb_learned_state(eb_ctx* ctx, double* state, int32_t set);
/* Network on host arrays: x [B][H][W][8] FP32 (rounded to BF16), y [B][H][W][16] FP32.      */
int eb_learned_forward(eb_ctx* ctx, int32_t B, int32_t H, int32_t W, const float* x, float* y);
/* MSE loss against t [B][H][W][3] and the gradient of every parameter (layout as above).    */
int eb_learned_loss_grad(eb_ctx* ctx, int32_t B, int32_t H, int32_t W, const float* x, const float* t, double* loss,
                         float* grad);
/* Learned-stage corrections kept / rejected by FGMRES since the last call, their time, and the
 * mean fraction of the squared preconditioner residual they removed.                       */
int eb_learned_stats(eb_ctx* ctx, int64_t* accepted, int64_t* rejected, double* seconds, double* mean_removed);

/* ---- checkpoints -----------------------------------------------------------
 * No counterpart in the reference, whose backups (model_manager/backup/core/MakeBackup.jl:22)
 * and XDMF output (model_manager/xdmf/markers/core/TimeStep.jl) write the host arrays: those
 * arrays are eb_marker_download / eb_grid_download in the reference's layout, and a resumed
 * run uploads them again.  These two calls save and restore every field the context
 * holds in one file (a header with the grid size and marknum, then each field's bytes in
 * that same layout), so a GPU run can stop and resume without the host model.  Reading
 * needs eb_set_grid with the same grid (markers are resized to the file's marknum); the
 * next eb_initialize_bilinear_interpolation rebuilds the cell sort.  The file's headers
 * and sizes are all checked before anything changes: a truncated or mismatched file
 * returns EB_BAD_INPUT with the context untouched.  Fields the context holds that the file
 * does not are left as they were (a file written by eb_checkpoint_write holds them all). */
int eb_checkpoint_write(eb_ctx* ctx, const char* path);
int eb_checkpoint_read(eb_ctx* ctx, const char* path);

/* ---- one marker cycle from host arrays -------------------------------------
 * No single counterpart in the reference: the sequence of eb_get_marker_inside_flags,
 * eb_initialize_bilinear_interpolation, eb_interpolate_marker_heat_parameters_to_grid,
 * eb_interpolate_marker_stokes_parameters_to_grid, eb_post_stokes_marker_gathers,
 * eb_update_subgrid_stress, eb_apply_marker_stress_correction,
 * eb_subgrid_heat_diffusion_update, eb_add_remaining_grid_change_to_marker_temperature,
 * eb_advect_markers_and_rotate_stress and eb_update_marker_strain, with the caller's
 * host arrays copied in before the steps that read them and out as soon as the
 * last step writing each has finished.  The copies run on two copy streams beside
 * the steps (host memory should be pinned for them to overlap); the call returns
 * when everything has completed.  Fields and host types as for eb_marker_upload /
 * eb_marker_download; inputs cannot be cell indices or inside flags, outputs cannot
 * be marker_xn_vy/yn_vy.  marker_matid in the inputs is range-checked as on upload. */
typedef struct eb_marker_io {
  int32_t n_in;                 /* fields copied host -> device before their first use   */
  const int32_t* in_fields;     /* eb_marker_field ids                                   */
  const void* const* in_host;   /* host arrays (marknum elements each)                   */
  int32_t n_out;                /* fields copied device -> host after their last write   */
  const int32_t* out_fields;
  void* const* out_host;
} eb_marker_io;
int eb_marker_cycle_host(eb_ctx* ctx, const eb_marker_io* io);

/* ---- allocation-free entry point -------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (their device memory belongs to another allocator, or allocating is not
 * allowed where they run): the inclusive bilinear average of one marker field
 * on the basic grid (the operation of BilinearNumerator's inclusive update and
 * BilinearAverage.calc_bilinear_average_arithmetic!), computed without
 * allocating device memory.  All pointers are device pointers owned by the
 * caller: marker x, y and value (marknum doubles), gridx_b (xnum), gridy_b
 * (ynum); d_avg and d_wsum are (ynum, xnum) column-major grids, written on
 * return; nodes with a zero weight sum keep d_avg's previous value.
 * Working memory is one static 16 MiB device array that every GPU loading the
 * library holds until the process exits: marknum <= EB_NOALLOC_MAX_MARKERS and
 * (xnum-1)*(ynum-1) <= EB_NOALLOC_MAX_CELLS, else EB_BAD_INPUT with a message
 * in errbuf.  The first call on a device resolves the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  That address is kept for the life of the
 * process: after cudaDeviceReset on a device, this entry point must not be
 * called on it again.  Work is queued on `stream` (a cudaStream_t, 0 =
 * default) without synchronising.  All calls share the one array, so calls
 * that overlap on the GPU (different streams, or another host thread) race.
 * Cost is linear in marknum however the markers cluster: they are ordered by
 * (cell, marker index) with a stable radix sort, and each cell folds its own
 * markers in that order.  */
#define EB_NOALLOC_MAX_MARKERS 524288
#define EB_NOALLOC_MAX_CELLS   131072
int eb_marker_to_basic_grid_average_noalloc(
    const double* d_marker_x, const double* d_marker_y, const double* d_marker_value, int64_t marknum,
    const double* d_gridx_b, int64_t xnum, const double* d_gridy_b, int64_t ynum,
    double* d_avg, double* d_wsum, void* stream, char* errbuf, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* EBGPU_H */
