"""GB300 (sm_103a) marker-in-cell hot path for EarthBox.jl -- host-side mirror.

``MarkerInCell`` drives libebgpu.so through its C-ABI (include/ebgpu.h).  Its
methods carry the names of the EarthBox.jl functions they replace (the Julia
``!`` dropped), take no arguments beyond the model state the context already
holds, and raise ``EarthBoxGPUError`` with the library's message on any
non-zero status, like the reference raises a Julia error.

Typical use, one time step of the marker path::

    mic = MarkerInCell()
    mic.load_model(model)                       # grid, materials, params, markers, grids
    mic.get_marker_inside_flags()               # GridFuncs.get_marker_inside_flags
    mic.initialize_bilinear_interpolation()     # Interpolation.initialize_bilinear_interpolation!
    mic.interpolate_marker_heat_parameters_to_grid()
    mic.update_marker_rheology()
    mic.update_marker_viscoplastic_viscosity(use_marker_plasticity=True)
    mic.interpolate_marker_stokes_parameters_to_grid()
    ...                                         # Stokes solve (grid side)
    mic.post_stokes_marker_gathers()
    mic.update_subgrid_stress(); mic.apply_marker_stress_correction()
    mic.subgrid_heat_diffusion_update(); mic.add_remaining_grid_change_to_marker_temperature()
    mic.advect_markers_and_rotate_stress(); mic.update_marker_strain()
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from . import synthetic
from .build import build

__all__ = ["MarkerInCell", "EarthBoxGPUError", "build", "synthetic"]


class EarthBoxGPUError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[status {code}] {message}")
        self.code = code


def heat_params(params: dict) -> dict:
    """The heat-step scalars (reference parameter names) with this package's defaults."""
    return {"timestep": float(params["timestep"]), "max_temp_change": float(params.get("max_temp_change", 20.0)),
            "gravity_x": float(params.get("gravity_x", 0.0)), "gravity_y": float(params.get("gravity_y", 9.81)),
            "iuse_adiabatic_heating": int(params.get("iuse_adiabatic_heating", 1)),
            "iuse_shear_heating": int(params.get("iuse_shear_heating", 1)),
            "iuse_heat": int(params.get("iuse_heat", 1)),
            "subgrid_diff_coef_temp": float(params.get("subgrid_diff_coef_temp", 1.0))}


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class MarkerInCell:
    """One device context: marker SoA, staggered grids and material tables on one GPU."""

    def __init__(self, device: int = 0):
        self._lib = _abi.load()
        self._ctx = C.c_void_p()
        rc = self._lib.eb_create(C.byref(self._ctx), int(device))
        if rc != _abi.EB_OK:
            raise EarthBoxGPUError(rc, "eb_create failed (no CUDA device?)")
        self.xnum = self.ynum = 0
        self.marknum = 0

    # ------------------------------------------------------------ plumbing --
    def _check(self, rc: int) -> None:
        if rc != _abi.EB_OK:
            msg = self._lib.eb_last_error(self._ctx)
            raise EarthBoxGPUError(rc, msg.decode() if msg else "unknown error")

    def close(self) -> None:
        if self._ctx:
            self._lib.eb_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        """The context's cudaStream_t (as an integer) for event timing."""
        return int(self._lib.eb_stream(self._ctx) or 0)

    @property
    def launch_count(self) -> int:
        return int(self._lib.eb_launch_count(self._ctx))

    def profile_enable(self, on: bool = True) -> None:
        """Time every kernel with CUDA events on the context's stream (clears the counters)."""
        self._check(self._lib.eb_profile_enable(self._ctx, int(bool(on))))

    def profile(self) -> dict:
        """{kernel name: (total device ms, launches)} since the last profile_enable."""
        out = {}
        buf = C.create_string_buffer(128)
        for i in range(self._lib.eb_profile_count(self._ctx)):
            ms, n = C.c_double(), C.c_int64()
            self._check(self._lib.eb_profile_entry(self._ctx, i, buf, 128, C.byref(ms), C.byref(n)))
            out[buf.value.decode()] = (ms.value, n.value)
        return out

    # --------------------------------------------------------------- set-up --
    def set_grid(self, g: "synthetic.Grid") -> None:
        self._grid_keep = [np.ascontiguousarray(getattr(g, n), dtype=np.float64) for n in
                           ("gridx_b", "gridy_b", "xstp_b", "ystp_b", "gridx_vy", "xstp_vy", "gridy_vx", "ystp_vx")]
        d = _abi.GridDesc(g.xnum, g.ynum, *[_ptr(a) for a in self._grid_keep],
                          g.xmin, g.xmax, g.ymin, g.ymax, g.xstpavg, g.ystpavg)
        self._check(self._lib.eb_set_grid(self._ctx, C.byref(d)))
        self.xnum, self.ynum = int(g.xnum), int(g.ynum)

    def set_materials(self, m: "synthetic.Materials") -> None:
        """The material tables; mat_flow may hold the first 12 columns of the reference's
        nmat x 17 flow-law table (the composite-creep laws), the rest is then zero."""
        flow = np.zeros((len(m.mat_mu), 17))
        flow[:, :np.shape(m.mat_flow)[1]] = m.mat_flow
        keep = [np.ascontiguousarray(m.mat_mu, np.float64), np.ascontiguousarray(m.mat_hr, np.float64),
                np.ascontiguousarray(m.mat_flow_type, np.int64),
                np.asfortranarray(flow).ravel(order="F"),
                np.asfortranarray(m.mat_plastic, np.float64).ravel(order="F"),
                np.ascontiguousarray(m.mat_rho, np.float64)]
        d = _abi.MaterialDesc(len(keep[0]), *[_ptr(a) for a in keep])
        self._check(self._lib.eb_set_materials(self._ctx, C.byref(d)))

    def set_params(self, params: dict) -> None:
        p = _abi.Params()
        for name, _ in _abi.Params._fields_:
            if name in params:
                setattr(p, name, params[name])
        self._params = dict(params)
        self._check(self._lib.eb_set_params(self._ctx, C.byref(p)))

    def set_stokes_params(self, params: dict) -> None:
        """Gravity, interface stabilisation, pressure boundary condition and internal velocity zone."""
        p = _abi.StokesParams()
        p.gravity_x = float(params.get("gravity_x", 0.0))
        p.gravity_y = float(params.get("gravity_y", 9.81))
        p.iuse_interface_stabilization = int(params.get("iuse_interface_stabilization", 0))
        p.pressure_bc_mode = int(params.get("pressure_bc_mode", 0))
        p.pressure_bc = float(params.get("pressure_bc", 0.0))
        zone = np.asarray(params.get("bintern_zone", [-1, 0, 0, 0, -1, 0, 0, 0]), dtype=np.int64)
        vel = np.asarray(params.get("bintern_velocity", np.zeros(8)), dtype=np.float64)
        for k in range(8):
            p.bintern_zone[k] = int(zone[k])
            p.bintern_velocity[k] = float(vel[k])
        self._check(self._lib.eb_set_stokes_params(self._ctx, C.byref(p)))

    def resize_markers(self, marknum: int) -> None:
        self._check(self._lib.eb_resize_markers(self._ctx, int(marknum)))
        self.marknum = int(marknum)

    def upload_marker(self, name: str, values: np.ndarray) -> None:
        a = np.ascontiguousarray(values, dtype=_abi.MARKER_DTYPE[name])
        if a.shape != (self.marknum,):
            raise ValueError(f"{name}: expected {self.marknum} values, got {a.shape}")
        self._check(self._lib.eb_marker_upload(self._ctx, _abi.MARKER_ID[name], _ptr(a)))

    def download_marker(self, name: str) -> np.ndarray:
        a = np.empty(self.marknum, dtype=_abi.MARKER_DTYPE[name])
        self._check(self._lib.eb_marker_download(self._ctx, _abi.MARKER_ID[name], _ptr(a)))
        return a

    def upload_grid(self, name: str, values: np.ndarray) -> None:
        shape = _abi.grid_shape(name, self.xnum, self.ynum)
        a = np.asfortranarray(values, dtype=np.float64)
        if a.shape != shape:
            raise ValueError(f"{name}: expected shape {shape}, got {a.shape}")
        self._check(self._lib.eb_grid_upload(self._ctx, _abi.GRID_ID[name], _ptr(a)))

    def download_grid(self, name: str) -> np.ndarray:
        a = np.empty(_abi.grid_shape(name, self.xnum, self.ynum), dtype=np.float64, order="F")
        self._check(self._lib.eb_grid_download(self._ctx, _abi.GRID_ID[name], _ptr(a)))
        return a

    def marker_device_ptr(self, name: str) -> int:
        p = C.c_void_p()
        self._check(self._lib.eb_marker_device_ptr(self._ctx, _abi.MARKER_ID[name], C.byref(p)))
        return int(p.value or 0)

    def grid_device_ptr(self, name: str) -> int:
        p = C.c_void_p()
        self._check(self._lib.eb_grid_device_ptr(self._ctx, _abi.GRID_ID[name], C.byref(p)))
        return int(p.value or 0)

    def load_model(self, model: "synthetic.Model", grids: bool = True) -> None:
        """Upload a whole model: grid geometry, materials, parameters, markers and grid fields."""
        self.set_grid(model.grid)
        self.set_materials(model.mats)
        self.set_params(model.params)
        if "gravity_y" in model.params:
            self.set_stokes_params(model.params)
        self.heat = heat_params(model.params)
        self.resize_markers(model.marknum)
        for k, v in model.markers.items():
            if k in ("xn", "yn", "xn_vy", "yn_vy"):
                continue
            self.upload_marker(k, v)
        if grids:
            for k, v in model.grids.items():
                self.upload_grid(k, v)

    # --------------------------------------------------- hot-path steps ---
    def _call(self, name: str) -> None:
        self._check(getattr(self._lib, name)(self._ctx))

    def get_marker_inside_flags(self) -> None:
        """GridFuncs.get_marker_inside_flags (src/utils/GridFuncs.jl:54-80)."""
        self._call("eb_get_marker_inside_flags")

    def initialize_bilinear_interpolation(self) -> None:
        """InitializeInterpolation.initialize_bilinear_interpolation! (InitializeInterpolation.jl:63-82)."""
        self._call("eb_initialize_bilinear_interpolation")

    def interpolate_marker_stokes_parameters_to_grid(self) -> None:
        """MarkersToStokesArrays.interpolate_markers_to_transport_arrays! (MarkersToStokesArrays.jl:39-45)."""
        self._call("eb_interpolate_marker_stokes_parameters_to_grid")

    def interpolate_marker_heat_parameters_to_grid(self) -> None:
        """MarkerToHeatArrays.interpolate_markers_to_transport_arrays! (MarkerToHeatArrays.jl:29-35)."""
        self._call("eb_interpolate_marker_heat_parameters_to_grid")

    def backup_and_clear_viscosity_transport_arrays(self) -> None:
        """BackupTransportArrays.backup_and_clear_viscosity_transport_arrays! (BackupTransportArrays.jl:105-137)."""
        self._call("eb_backup_and_clear_viscosity_transport_arrays")

    def interpolate_viscosity_to_transport_arrays(self) -> None:
        """MarkersToStokesArrays.interpolate_viscosity_to_transport_arrays! (MarkersToStokesArrays.jl:60-64)."""
        self._call("eb_interpolate_viscosity_to_transport_arrays")

    def interpolate_temperature_to_markers(self) -> None:
        """GridTemperatureToMarkers.interpolate! (GridTemperatureToMarkers.jl:18-45)."""
        self._call("eb_interpolate_temperature_to_markers")

    def update_marker_rheology(self) -> None:
        """Rheology.update_marker_rheology! (src/rheology/Rheology.jl:37-56)."""
        self._call("eb_update_marker_rheology")

    def update_marker_viscoplastic_viscosity(self, use_marker_plasticity: bool = True) -> None:
        """Rheology.update_marker_viscoplastic_viscosity! (Rheology.jl:70-107)."""
        self._check(self._lib.eb_update_marker_viscoplastic_viscosity(self._ctx, int(bool(use_marker_plasticity))))

    def update_marker_rheology_and_viscoplastic_viscosity(self, use_marker_plasticity: bool = True) -> None:
        """Rheology.update_marker_rheology! then update_marker_viscoplastic_viscosity!
        (TimeLoop.jl:222-223) as one fused marker pass (same results as the two calls)."""
        self._check(self._lib.eb_update_marker_rheology_and_viscoplastic_viscosity(
            self._ctx, int(bool(use_marker_plasticity))))

    def update_plastic_yielding(self) -> None:
        """MarkerPlasticity.update_plastic_yielding! (ViscoelasticForecast.jl:11-123)."""
        self._call("eb_update_plastic_yielding")

    def calc_marker_viscoplastic_viscosity(self) -> None:
        """GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity!
        (src/rheology/plastic_failure/nodes/GridViscoplasticityToMarkers.jl:7-118): the nodal
        Picard variant's grid viscoplastic viscosity back to the markers (eta, pfailure)."""
        self._call("eb_calc_marker_viscoplastic_viscosity")

    def post_stokes_marker_gathers(self) -> None:
        """Marker part of StokesContinuitySolver.execute_post_stokes_solver_steps! (StokesContinuitySolver.jl:283-290)."""
        self._call("eb_post_stokes_marker_gathers")

    def update_subgrid_stress(self) -> None:
        """SubGridStress.Update.update_subgrid_stress! (subgrid_stress/update/Update.jl:69-87)."""
        self._call("eb_update_subgrid_stress")

    def apply_marker_stress_correction(self) -> None:
        """StressCorrection.apply_marker_stress_correction_for_remaining_grid_stress! (StressCorrection.jl:35-82)."""
        self._call("eb_apply_marker_stress_correction")

    def subgrid_heat_diffusion_update(self) -> None:
        """SubgridDiffusion.subgrid_heat_diffusion_update! + remove_subgrid_effects_from_grid_changes!."""
        self._call("eb_subgrid_heat_diffusion_update")

    def add_remaining_grid_change_to_marker_temperature(self) -> None:
        """MarkerTemperature.add_remaining_grid_change_to_marker_temperature! (MarkerTemperature.jl:18-45)."""
        self._call("eb_add_remaining_grid_change_to_marker_temperature")

    def advect_markers_and_rotate_stress(self) -> None:
        """Advection.advect_markers_and_rotate_stress_tensor! (src/advection/Advection.jl:109-114)."""
        self._call("eb_advect_markers_and_rotate_stress")

    def update_marker_strain(self) -> None:
        """Advection.update_marker_strain! (Advection.jl:169-178)."""
        self._call("eb_update_marker_strain")

    # -------------------------------------------- Stokes-continuity step ---
    def calc_viscoelastic_terms(self) -> None:
        """StokesViscoelasticTerms.calc_viscoelastic_terms! (StokesViscoelasticTerms.jl:26-125)."""
        self._call("eb_calc_viscoelastic_terms")

    def viscoelastic_rhs(self) -> None:
        """StokesContinuityRhs.viscoelastic_rhs! (StokesContinuityRhs.jl:30-190)."""
        self._call("eb_viscoelastic_rhs")

    def build_system_of_equations(self) -> None:
        """SystemSolver.initialize_solver! + StokesBuildManager.build_system_of_equations
        (SystemSolver.jl:99-115, StokesBuildManager.jl:661-712), kept on the device."""
        self._call("eb_build_stokes_system")

    def solve_system(self, rtol: float = 1e-8, max_iters: int = 0, restart: int = 0, mg_sweeps: int = 0,
                     use_initial_guess: bool = False, method: str = "fgmres", check: bool = True,
                     learned: bool = False, precision: str = "mixed", gs_relax: float = 0.0,
                     fallback: bool = True, mg_inner: int = 0, mg_inner_tol: float = 0.0,
                     learned_warm: bool = False) -> dict:
        """The Stokes solve (replaces SystemSolver.solve_system_optimized, SystemSolver.jl:67-91);
        method "fgmres" or "bicgstab"; learned: add the trained network's stage after each V-cycle;
        precision "mixed" (FP32 V-cycle and stored directions, the Arnoldi step on double-float
        FP32 pairs) or "fp64" (the plain method); gs_relax (mixed only): FP32 Gram-Schmidt
        products below gs_relax x the target (0: 1e3; <0: the FP64 Arnoldi step throughout);
        fallback (mixed only): the plain method takes over when the mixed residual stops falling;
        mg_inner: the velocity stage's GCR steps (1: a single V-cycle), mg_inner_tol its stopping
        residual reduction; learned_warm (with learned and use_initial_guess): the learned stage
        also corrects the initial guess."""
        o = _abi.SolveOpts(rtol, max_iters, restart, mg_sweeps, int(use_initial_guess),
                           {"fgmres": 0, "bicgstab": 1}[method], int(learned), {"mixed": 0, "fp64": 1}[precision],
                           gs_relax, 0 if fallback else -1, mg_inner, mg_inner_tol, int(learned_warm))
        r = _abi.SolveReport()
        rc = self._lib.eb_solve_stokes_system(self._ctx, C.byref(o), C.byref(r))
        rep = {"status": rc, "iterations": r.iterations, "levels": r.levels, "rel_residual": r.rel_residual,
               "rel_residual_scaled": r.rel_residual_scaled, "seconds": r.seconds,
               "reorthogonalisations": r.reorthogonalisations, "relaxed_iterations": r.relaxed_iterations,
               "fallback_used": r.fallback_used, "precision_used": ("mixed", "fp64")[r.precision_used],
               "vcycles": r.vcycles}
        if check:
            self._check(rc)
        return rep

    def process_stokes_solution(self) -> None:
        """SystemSolver.process_stokes_solution! (SystemSolver.jl:141-271)."""
        self._call("eb_process_stokes_solution")

    def stokes_nonlinear_residual(self) -> np.ndarray:
        """StokesResiduals.stokes_calc_nonlinear_system_residual_optimized! (StokesResiduals.jl:63-81)."""
        self._call("eb_stokes_nonlinear_residual")
        return self.download_stokes_vector("resnl")

    def backup_stokes_arrays(self) -> None:
        """SystemSolver.backup_stokes_arrays! (SystemSolver.jl:306-318): S, vx1, vy1, pr1 -> *_old."""
        self._call("eb_backup_stokes_arrays")

    def calculate_stokes_norms(self) -> dict:
        """StokesNorms.calculate_stokes_norms! solution-change norms and |resnl|_2 (StokesNorms.jl:8-160)."""
        n = _abi.StokesNorms()
        self._check(self._lib.eb_calculate_stokes_norms(self._ctx, C.byref(n)))
        return {k: getattr(n, k) for k, _ in _abi.StokesNorms._fields_}

    @property
    def stokes_size(self) -> int:
        return int(self._lib.eb_stokes_size(self._ctx))

    @property
    def pscale(self) -> float:
        return float(self._lib.eb_stokes_pscale(self._ctx))

    def stokes_apply(self, x: np.ndarray) -> np.ndarray:
        """y = L x with the assembled operator (interleaved N-vectors)."""
        a = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.stokes_size)
        self._check(self._lib.eb_stokes_apply(self._ctx, _ptr(a), _ptr(y)))
        return y

    def download_stokes_vector(self, name: str) -> np.ndarray:
        y = np.empty(self.stokes_size)
        self._check(self._lib.eb_stokes_vector_download(self._ctx, _abi.STOKES_VECTORS[name], _ptr(y)))
        return y

    def upload_stokes_vector(self, name: str, values: np.ndarray) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64)
        if a.shape != (self.stokes_size,):
            raise ValueError(f"expected {self.stokes_size} values")
        self._check(self._lib.eb_stokes_vector_upload(self._ctx, _abi.STOKES_VECTORS[name], _ptr(a)))

    def export_coo(self) -> tuple:
        """The assembled system as the reference's (Li, Lj, Lv, R): 1-based COO in
        StokesBuildManager's entry order, for a direct solver on the host."""
        n = C.c_int64()
        self._check(self._lib.eb_stokes_export_coo(self._ctx, None, None, None, 0, C.byref(n)))
        Li = np.empty(n.value, np.int64)
        Lj = np.empty(n.value, np.int64)
        Lv = np.empty(n.value, np.float64)
        self._check(self._lib.eb_stokes_export_coo(self._ctx, _ptr(Li), _ptr(Lj), _ptr(Lv), n.value, C.byref(n)))
        return Li, Lj, Lv, self.download_stokes_vector("rhs")

    def stokes_stencil(self) -> np.ndarray:
        """The assembled coefficients as a (27, xnum-1, ynum-1) array indexed [slot, j, i]."""
        nx, ny = self.xnum - 1, self.ynum - 1
        a = np.empty(27 * nx * ny)
        self._check(self._lib.eb_stokes_stencil_download(self._ctx, _ptr(a)))
        return a.reshape(27, nx, ny)

    def update_grid_strain_rate_and_spin(self) -> None:
        """GridStrainRate.update_grid_strain_rate_and_spin! (GridStrainRate.jl:6-182): exx, exy, eii, esp."""
        self._call("eb_update_grid_strain_rate_and_spin")

    def forecast_viscoelastic_grid_stress(self) -> None:
        """GridStress.forecast_viscoelastic_grid_stress! (GridStress.jl:30-126): sxy2, sxx2."""
        self._call("eb_forecast_viscoelastic_grid_stress")

    def calculate_deviatoric_grid_stress_change(self) -> None:
        """GridStress.calculate_deviatoric_grid_stress_change! (GridStress.jl:128-134): dsxy, dsxx."""
        self._call("eb_calculate_deviatoric_grid_stress_change")

    def interpolate_stag_velocity_to_basic_grid(self) -> None:
        """StokesInterpolate.interpolate_stag_velocity_to_basic_grid! (StokesInterpolate.jl:16-33): vxb, vyb."""
        self._call("eb_interpolate_stag_velocity_to_basic_grid")

    def interpolate_basic_viscoplastic_viscosity_to_pressure_grid(self, iuse_harmonic: int = 1) -> None:
        """Interpolation.interpolate_basic_viscoplastic_viscosity_to_pressure_grid! (Interpolation.jl:97-108)."""
        self._check(self._lib.eb_interpolate_basic_viscoplastic_viscosity_to_pressure_grid(self._ctx, int(iuse_harmonic)))

    def update_nodes_for_plastic_yielding(self, wall: dict | None = None) -> tuple:
        """PlasticFailureNodes.update_nodes_for_plastic_yielding (PlasticFailureNodes.jl:24-184).
        `wall` holds the mobile-wall geometry (eb_mobile_wall fields) or None.
        Returns (nnode_yield, global_yield_error)."""
        n, e = C.c_int64(), C.c_double()
        wp = None
        if wall is not None:
            wp = _abi.MobileWall(**{k: wall.get(k, 0) for k, _ in _abi.MobileWall._fields_})
        self._check(self._lib.eb_update_nodes_for_plastic_yielding(self._ctx, C.byref(wp) if wp else None,
                                                                   C.byref(n), C.byref(e)))
        return int(n.value), float(e.value)

    def apply_nodal_plastic_yielding(self) -> None:
        """The etas1 / plastic_yield / plastic strain-rate updates of PlasticityLoopNodes.picard_loop."""
        self._call("eb_apply_nodal_plastic_yielding")

    @staticmethod
    def _warm_kw(solve_kw: dict, warm: bool) -> dict:
        """Solve options starting from the current solution vector when `warm` (an explicit
        use_initial_guess in solve_kw wins)."""
        kw = dict(solve_kw)
        if warm:
            kw.setdefault("use_initial_guess", True)
        return kw

    def picard_loop_nodes(self, nglobal: int, tolerance_picard: float, iuse_harmonic: int = 1,
                          wall: dict | None = None, warm_start: bool = True, warm_first: bool = False,
                          **solve_kw) -> list:
        """PlasticityLoopNodes.picard_loop (plasticity_loop_nodes/PlasticityLoopNodes.jl:36-92): solve,
        process, nodal yield, apply it when nodes yield; stop when no node yields, at nglobal, or when
        the yield error or dvxy_rel_L2 drops below the tolerance (check_stop_global_loop_nodes).
        warm_start: each solve after the first starts from the previous iterate (the reference's
        direct solve needs no start; the iterative one reaches the same residual tolerance in fewer
        iterations); warm_first: the first one too (from the solution the context holds)."""
        history = []
        for iglobal in range(1, nglobal + 1):
            if iglobal > 1:
                self.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
            rep = self.solve_viscoelastic_stokes_continuity_equations(
                **self._warm_kw(solve_kw, warm_start and (iglobal > 1 or warm_first)))
            norms = self.stokes_solution_processing()
            nnode, gerr = self.update_nodes_for_plastic_yielding(wall)
            if nnode > 0:
                self.apply_nodal_plastic_yielding()
            history.append({"iglobal": iglobal, "nnode_yield": nnode, "global_yield_error": gerr, **rep, **norms})
            if (nnode == 0 or iglobal == nglobal or gerr < tolerance_picard
                    or norms["dvxy_rel_L2"] < tolerance_picard):
                break
        return history

    def solve_viscoelastic_stokes_continuity_equations(self, **solve_kw) -> dict:
        """StokesContinuitySolver.solve_viscoelastic_stokes_continuity_equations!
        (StokesContinuitySolver.jl:68-90): build steps, solve, unpack, and the nonlinear
        residual |L S_old - R| of calculate_residuals_optimized!."""
        self.calc_viscoelastic_terms()
        self.viscoelastic_rhs()
        self.build_system_of_equations()
        rep = self.solve_system(**solve_kw)
        self.process_stokes_solution()
        self._call("eb_stokes_nonlinear_residual")
        return rep

    def stokes_solution_processing(self) -> dict:
        """StokesContinuitySolver.stokes_solution_processing! (StokesContinuitySolver.jl:113-136):
        grid strain rate and spin, the post-Stokes grid and marker steps
        (execute_post_stokes_solver_steps!: stress forecast and change, marker strain rate,
        strain-rate ratio and pressure), the Stokes norms, and the backup of S, vx1, vy1, pr1.
        Returns the norms."""
        self.update_grid_strain_rate_and_spin()
        self.forecast_viscoelastic_grid_stress()
        self.calculate_deviatoric_grid_stress_change()
        self.post_stokes_marker_gathers()
        norms = self.calculate_stokes_norms()
        self.backup_stokes_arrays()
        return norms

    def picard_loop_markers(self, nglobal: int, tolerance_picard: float, iuse_harmonic: int = 1,
                            warm_start: bool = True, warm_first: bool = False, **solve_kw) -> list:
        """PlasticityLoopMarkers.picard_loop (global_plasticity_loop/plasticity_loop/
        plasticity_loop_markers/PlasticityLoopMarkers.jl:36-73): from the second iteration on,
        re-yield the markers and re-average the viscosity; solve; process; stop at nglobal or when
        dvxy_rel_L2 < tolerance_picard (LoopTermination.check_stop_global_loop_markers).
        warm_start / warm_first as in picard_loop_nodes.
        Returns one record per iteration (solve report and norms)."""
        history = []
        for iglobal in range(1, nglobal + 1):
            if iglobal > 1:
                self.backup_and_clear_viscosity_transport_arrays()
                self.update_plastic_yielding()
                self.interpolate_viscosity_to_transport_arrays()
                self.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
            rep = self.solve_viscoelastic_stokes_continuity_equations(
                **self._warm_kw(solve_kw, warm_start and (iglobal > 1 or warm_first)))
            norms = self.stokes_solution_processing()
            history.append({"iglobal": iglobal, **rep, **norms})
            if iglobal == nglobal or norms["dvxy_rel_L2"] < tolerance_picard:
                break
        return history

    def time_step(self, nglobal: int = 5, tolerance_picard: float = 1e-3, iuse_harmonic: int = 1,
                  heat: bool = False, warm_start: bool = True, marker_cell_displ_max: float | None = None,
                  **solve_kw) -> dict:
        """One pass of TimeLoop.run_loop!'s body (src/time_loop/TimeLoop.jl:181-194) restricted to the
        hot path, with a fixed time step:
          execute_pre_solver_steps! (:203-230): initialize_bilinear_interpolation! and the
            heat-parameter averages (one walk of the cell lists), update_marker_rheology! + update_marker_viscoplastic_viscosity! (marker
            plasticity when itype_global == 0; one fused pass), the Stokes-parameter averages and the
            harmonic normal viscosity;
          execute_stokes_continuity_solver_steps! (:232-248): the Picard loop of itype_global (markers
            or nodes), the staggered velocity on basic nodes, the nodal variant's grid viscoplastic
            viscosity back to the markers, the post-Stokes grid and marker steps, and
            update_marker_stress_for_grid_and_subgrid_changes! (StokesContinuitySolver.jl:365-381);
          execute_heat_solver_steps! (:250-259) when `heat`;
          execute_advection_steps! (:261-273): RK4 advection with stress rotation, strain update;
          and the inside flags of the moved markers.
        warm_start: every Stokes solve starts from the latest solution (the previous Picard iterate,
        or the previous time step's solution for the first solve of a step).
        marker_cell_displ_max: when given, the step runs as the reference's time loop does with a
        displacement limit: it starts from the viscoelastic time step (params "timestep_viscoelastic",
        else the time step the parameters were set with; TimeLoop.update_model_time_step!, :138) and,
        after the Picard loop, TimeStep.adjust_time_step_using_displacement_limit! (:244) shortens it
        so that no marker moves more than that fraction of a cell; the post-Stokes steps and the
        advection then use the shortened step.
        Returns {"picard": per-iteration records, "heat": heat-loop report or None, "timestep": s}."""
        p = getattr(self, "_params", {})
        nodes = int(p.get("itype_global", 0)) == 1
        if marker_cell_displ_max is not None:
            if "timestep_viscoelastic" not in p:
                p["timestep_viscoelastic"] = float(p["timestep"])
            if p["timestep"] != p["timestep_viscoelastic"]:
                p["timestep"] = float(p["timestep_viscoelastic"])
                self.set_params(p)
        self.get_marker_inside_flags()
        self.initialize_bilinear_interpolation_and_heat_scatter()
        self.update_marker_rheology_and_viscoplastic_viscosity(use_marker_plasticity=not nodes)
        self.interpolate_marker_stokes_parameters_to_grid()
        self.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
        loop = self.picard_loop_nodes if nodes else self.picard_loop_markers
        hist = loop(nglobal, tolerance_picard, iuse_harmonic, warm_start=warm_start,
                    warm_first=warm_start and getattr(self, "_solved", False), **solve_kw)
        self._solved = True
        self.interpolate_stag_velocity_to_basic_grid()
        if nodes:
            self.calc_marker_viscoplastic_viscosity()
        if marker_cell_displ_max is not None:
            dt, updated = self.update_model_time_step_using_displacement_limit(p["timestep"], marker_cell_displ_max)
            if updated:
                p["timestep"] = float(dt)
                self.set_params(p)
        self.forecast_viscoelastic_grid_stress()
        self.calculate_deviatoric_grid_stress_change()
        self.post_stokes_marker_gathers()
        if float(p.get("subgrid_diff_coef_stress", 1.0)) > 0:
            self.update_subgrid_stress()
        self.apply_marker_stress_correction()
        if heat and getattr(self, "heat", None) is not None:
            self.heat = dict(self.heat, timestep=float(p.get("timestep", self.heat["timestep"])))
        hrep = self.update_marker_temp_for_grid_and_subgrid_changes() if heat else None
        self.advect_markers_and_rotate_stress()
        self.update_marker_strain()
        self.get_marker_inside_flags()
        return {"picard": hist, "heat": hrep, "timestep": float(p.get("timestep", 0.0))}

    # ------------------------------------------- learned preconditioner stage --
    def learned_init(self, seed: int = 0) -> None:
        """He-normal initial weights of the U-Net stage."""
        self._check(self._lib.eb_learned_init(self._ctx, seed))

    def learned_train(self, steps: int, batch: int = 4, patch: int = 512, patches_per_sample: int = 4,
                      lr: float = 1e-3, seed: int = 0, mg_sweeps: int = 0) -> dict:
        """Train the stage on the GPU on correction pairs of the current assembled system."""
        o = _abi.LearnedOpts(batch, patch, steps, patches_per_sample, mg_sweeps, lr, seed)
        r = _abi.LearnedReport()
        self._check(self._lib.eb_learned_train(self._ctx, C.byref(o), C.byref(r)))
        return {k: getattr(r, k) for k, _ in _abi.LearnedReport._fields_}

    def learned_params(self, params: np.ndarray | None = None) -> np.ndarray:
        """FP32 parameters (per layer [cout][taps][cin] weights, then [cout] biases); with an
        array, upload it instead."""
        n = C.c_int64()
        self._check(self._lib.eb_learned_params(self._ctx, None, 0, C.byref(n), 0))
        if params is not None:
            p = np.ascontiguousarray(params, dtype=np.float32)
            assert p.size == n.value
            self._check(self._lib.eb_learned_params(self._ctx, _ptr(p), p.size, C.byref(n), 1))
            return p
        out = np.zeros(n.value, np.float32)
        self._check(self._lib.eb_learned_params(self._ctx, _ptr(out), out.size, C.byref(n), 0))
        return out

    def learned_state(self, state: np.ndarray | None = None) -> np.ndarray:
        """(eta mean, eta 1/std, rho mean, rho 1/std, kappa, trained) of the stage."""
        st = np.zeros(6) if state is None else np.ascontiguousarray(state, dtype=np.float64)
        self._check(self._lib.eb_learned_state(self._ctx, _ptr(st), 0 if state is None else 1))
        return st

    def learned_forward(self, x: np.ndarray) -> np.ndarray:
        """The network on x [B][H][W][8] (FP32, rounded to BF16) -> [B][H][W][16] FP32."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        B, H, W, _ = x.shape
        y = np.zeros((B, H, W, 16), np.float32)
        self._check(self._lib.eb_learned_forward(self._ctx, B, H, W, _ptr(x), _ptr(y)))
        return y

    def learned_loss_grad(self, x: np.ndarray, t: np.ndarray) -> tuple:
        """(MSE loss against t [B][H][W][3], gradient of every parameter)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        B, H, W, _ = x.shape
        n = C.c_int64()
        self._check(self._lib.eb_learned_params(self._ctx, None, 0, C.byref(n), 0))
        g = np.zeros(n.value, np.float32)
        loss = C.c_double()
        self._check(self._lib.eb_learned_loss_grad(self._ctx, B, H, W, _ptr(x), _ptr(t), C.byref(loss), _ptr(g)))
        return loss.value, g

    def learned_stats(self) -> dict:
        """Stage applications since the last call: kept, rejected, seconds and the mean fraction of
        the squared preconditioner residual removed."""
        a, r, s, m = C.c_int64(), C.c_int64(), C.c_double(), C.c_double()
        self._check(self._lib.eb_learned_stats(self._ctx, C.byref(a), C.byref(r), C.byref(s), C.byref(m)))
        return {"accepted": a.value, "rejected": r.value, "seconds": s.value, "mean_removed": m.value}

    # ----------------------------------------------------- marker recycling --
    def recycle_markers(self, matid_sticky_air: int, matid_sticky_water: int, matid_asthenosphere: int,
                        xsize: float, ysize: float, velocity_y_upper: float, velocity_y_lower: float,
                        temperature_bottom: float, seed: int, counter: int, iuse_random_fric: int = 0,
                        delta_fric_coef: float = 0.0, recycle_type: int = 1, contraction: dict | None = None,
                        side_inflow: dict | None = None, fracture_zone: dict | None = None) -> tuple:
        """MarkerRecycle.recycle_markers!: recycle_type 1 extension models (types/Extension.jl:14-129),
        2 extension without bottom inflow (types/ExtensionNoBottomInflow.jl), 3 channel
        (types/Channel.jl), 4 contraction (types/ContractionViscoelastic.jl; `contraction` holds
        asymmetric, full_velocity_contraction, sticky_thickness_left/right, layer_thickness (6),
        x_left_strong, x_right_strong, matid_layers (7), matid_strong (3)), 5 extension with side
        inflow and outflow (types/ExtensionInflowAndOutflowAlongSides.jl; `side_inflow` holds
        sticky_thickness_left/right, plate_thickness, smoothing_thickness, velocity_inflow_left/right,
        adiabatic_gradient), 6 fracture-zone contraction (types/ContractionFractureZone.jl; the
        `contraction` position fields plus `fracture_zone`: fz_thickness (7), x_fracture_zone_start/end,
        matid_fz (7), age_lithosphere_left/right (Myr), thermal_lithosphere_depth_left/right,
        thermal_diffusivity, adiabatic_gradient); returns (nrecycle_air, nrecycle_subsurface)."""
        p = _abi.RecycleParams(recycle_type, matid_sticky_air, matid_sticky_water, matid_asthenosphere, xsize, ysize,
                               velocity_y_upper, velocity_y_lower, temperature_bottom, iuse_random_fric,
                               delta_fric_coef, seed, counter)
        for group in (contraction, side_inflow, fracture_zone):
            for name, v in (group or {}).items():
                if name in ("layer_thickness", "matid_layers", "matid_strong", "fz_thickness", "matid_fz"):
                    getattr(p, name)[:] = list(v)
                else:
                    setattr(p, name, int(v) if name == "asymmetric" else v)
        na, ns = C.c_int64(), C.c_int64()
        self._check(self._lib.eb_recycle_markers(self._ctx, C.byref(p), C.byref(na), C.byref(ns)))
        return na.value, ns.value

    def recycled_markers(self) -> tuple:
        """(1-based indices, flags: 0 sticky / 1 subsurface) of the last recycle_markers."""
        n = C.c_int64()
        self._check(self._lib.eb_recycled_markers(self._ctx, None, None, 0, C.byref(n)))
        idx = np.zeros(n.value, np.int64)
        fl = np.zeros(n.value, np.int8)
        if n.value:
            self._check(self._lib.eb_recycled_markers(self._ctx, _ptr(idx), _ptr(fl), n.value, C.byref(n)))
        return idx, fl

    # --------------------------------------------------------- checkpoints --
    def checkpoint_write(self, path) -> None:
        """Every field the context holds, in one file (eb_checkpoint_write)."""
        self._check(self._lib.eb_checkpoint_write(self._ctx, str(path).encode()))

    def checkpoint_read(self, path) -> None:
        """Restore the fields of eb_checkpoint_write (same grid; markers resized to the file's count)."""
        self._check(self._lib.eb_checkpoint_read(self._ctx, str(path).encode()))
        import struct
        with open(path, "rb") as fh:
            self.marknum = struct.unpack("<8x4q", fh.read(40))[3]

    # ------------------------------------------------------- step boundary --
    def set_rock_tables(self, mat_rho: np.ndarray, mat_cp: np.ndarray, mat_kt: np.ndarray) -> None:
        """Material tables of the rock-property models: mat_rho (nmat, 3), mat_cp (nmat),
        mat_kt (nmat, 2) (model.materials.arrays)."""
        rho = np.asfortranarray(mat_rho, dtype=np.float64)
        cp = np.ascontiguousarray(mat_cp, dtype=np.float64)
        kt = np.asfortranarray(mat_kt, dtype=np.float64)
        n = cp.shape[0]
        if rho.shape != (n, 3) or kt.shape != (n, 2):
            raise ValueError("mat_rho must be (nmat, 3) and mat_kt (nmat, 2)")
        d = _abi.RockDesc(n, rho.ctypes.data, cp.ctypes.data, kt.ctypes.data)
        self._check(self._lib.eb_set_rock_tables(self._ctx, C.byref(d)))

    def set_sediment_porosity(self, matids_sediments, topo_x, topo_y, conductivity_water: float,
                              density_water: float, heat_capacity_water: float) -> None:
        """Inputs of the sediment porosity correction (PorosityUpdate.jl)."""
        ids = np.ascontiguousarray(matids_sediments, dtype=np.int16)
        tx = np.ascontiguousarray(topo_x, dtype=np.float64)
        ty = np.ascontiguousarray(topo_y, dtype=np.float64)
        d = _abi.SedimentDesc(len(ids), ids.ctypes.data if len(ids) else None, len(tx), tx.ctypes.data,
                              ty.ctypes.data, conductivity_water, density_water, heat_capacity_water)
        self._check(self._lib.eb_set_sediment_porosity(self._ctx, C.byref(d)))

    def update_marker_rock_properties(self, density_model: int = 0, rhocp_model: int = 0,
                                      conductivity_model: int = 0, iuse_sed_porosity: int = 0,
                                      maximum_heat_capacity: float = 1200.0) -> None:
        """RockProperties.update_marker_rock_properties! (rock_properties/RockProperties.jl:99-125)."""
        p = _abi.RockParams(density_model, rhocp_model, conductivity_model, iuse_sed_porosity,
                            maximum_heat_capacity)
        self._check(self._lib.eb_update_marker_rock_properties(self._ctx, C.byref(p)))

    def update_model_time_step_using_displacement_limit(self, timestep: float, marker_cell_displ_max: float,
                                                        iuse_local_adaptive_time_stepping: int = 0) -> tuple:
        """Update.update_model_time_step_using_displacement_limit (time_step/update/Update.jl:16-33):
        returns (new time step, updated?)."""
        dt = C.c_double(timestep)
        upd = C.c_int32()
        self._check(self._lib.eb_update_model_time_step_using_displacement_limit(
            self._ctx, marker_cell_displ_max, iuse_local_adaptive_time_stepping, C.byref(dt), C.byref(upd)))
        return dt.value, bool(upd.value)

    # ---------------------------------------------------------- heat step --
    def _heat(self, params: dict | None) -> "_abi.HeatParams":
        hp = heat_params(params) if params is not None else getattr(self, "heat", None)
        if hp is None:
            raise ValueError("heat parameters: pass params or call load_model first")
        return _abi.HeatParams(hp["timestep"], hp["max_temp_change"], hp["gravity_x"], hp["gravity_y"],
                               hp["iuse_adiabatic_heating"], hp["iuse_shear_heating"])

    def calculate_heat_rhs_terms(self, params: dict | None = None) -> None:
        """HeatSolver.calculate_heat_rhs_terms_grid! (heat_solver/HeatSolver.jl:139-150): RT1."""
        hp = self._heat(params)
        self._check(self._lib.eb_calculate_heat_rhs_terms(self._ctx, C.byref(hp)))

    def initialize_old_temperature_array(self) -> None:
        """HeatSolver.initialize_old_temperature_array! (HeatSolver.jl:199-204): tk0 = tk1."""
        self._call("eb_initialize_old_temperature")

    def build_heat_system(self, timestep_heat: float) -> None:
        """HeatBuildManager.build_system_of_equations (HeatBuildManager.jl:44-86)."""
        self._check(self._lib.eb_build_heat_system(self._ctx, C.c_double(timestep_heat)))

    def solve_heat_system(self, rtol: float = 0.0, max_iters: int = 0, mg_sweeps: int = 0,
                          use_initial_guess: bool = True, check: bool = True) -> dict:
        """The solve of SystemSolver.discretize_and_solve_conductive_heat_equation
        (heat_solver/solver/SystemSolver.jl:32-66) and reload_solu_temp: tk2."""
        o = _abi.SolveOpts(rtol, max_iters, 0, mg_sweeps, int(use_initial_guess), 0, 0, 0)
        r = _abi.SolveReport()
        rc = self._lib.eb_solve_heat_system(self._ctx, C.byref(o), C.byref(r))
        if check:
            self._check(rc)
        return {"status": rc, "iterations": r.iterations, "levels": r.levels, "rel_residual": r.rel_residual,
                "rel_residual_scaled": r.rel_residual_scaled, "seconds": r.seconds}

    def heat_residuals(self, timestep_heat: float) -> None:
        """HeatResiduals.compute_residuals_temp! (HeatResiduals.jl:12-162): rest."""
        self._check(self._lib.eb_heat_residuals(self._ctx, C.c_double(timestep_heat)))

    def run_conductive_heat_solver_loop(self, params: dict | None = None, rtol: float = 0.0, max_iters: int = 0,
                                        mg_sweeps: int = 0) -> dict:
        """HeatLoop.run_conductive_heat_solver_loop! (heat_loop/HeatLoop.jl:10-79)."""
        hp = self._heat(params)
        o = _abi.SolveOpts(rtol, max_iters, 0, mg_sweeps, 1, 0, 0, 0)
        r = _abi.HeatLoopReport()
        self._check(self._lib.eb_run_conductive_heat_solver_loop(self._ctx, C.byref(hp), C.byref(o), C.byref(r)))
        return {k: getattr(r, k) for k, _ in _abi.HeatLoopReport._fields_}

    def calculate_grid_temp_change(self) -> None:
        """HeatSolver.calculate_grid_temp_change! (HeatSolver.jl:211-216): dtk1 = tk2 - tk1."""
        self._call("eb_calculate_grid_temp_change")

    def export_heat_coo(self) -> tuple:
        """The assembled heat system as the reference's (Li, Lj, Lv, R) in HeatBuildManager's order."""
        n = C.c_int64()
        self._check(self._lib.eb_heat_export_coo(self._ctx, None, None, None, 0, C.byref(n)))
        Li = np.empty(n.value, np.int64)
        Lj = np.empty(n.value, np.int64)
        Lv = np.empty(n.value, np.float64)
        self._check(self._lib.eb_heat_export_coo(self._ctx, _ptr(Li), _ptr(Lj), _ptr(Lv), n.value, C.byref(n)))
        R = np.empty(int(self._lib.eb_heat_size(self._ctx)), np.float64)
        self._check(self._lib.eb_heat_rhs_download(self._ctx, _ptr(R)))
        return Li, Lj, Lv, R

    def update_marker_temp_for_grid_and_subgrid_changes(self, params: dict | None = None,
                                                        **solve_kw) -> dict | None:
        """HeatSolver.update_marker_temp_for_grid_and_subgrid_changes! (HeatSolver.jl:94-122): RHS
        terms, tk0 = tk1, the heat loop, dtk1 = tk2 - tk1, the subgrid diffusion (when its
        coefficient is positive) and the remaining change added to the marker temperature.
        Runs only when timestep > 0, max_temp_change > 0 and iuse_heat == 1 (use_heat_solver)."""
        p = params if params is not None else {}
        hp = heat_params(p) if params is not None else getattr(self, "heat", None)
        if hp is None or not (hp["timestep"] > 0 and hp["max_temp_change"] > 0 and hp["iuse_heat"] == 1):
            return None
        self.calculate_heat_rhs_terms(params)
        self.initialize_old_temperature_array()
        rep = self.run_conductive_heat_solver_loop(params, **solve_kw)
        self.calculate_grid_temp_change()
        if hp["subgrid_diff_coef_temp"] > 0:
            self.subgrid_heat_diffusion_update()
        self.add_remaining_grid_change_to_marker_temperature()
        return rep

    # ----------------------------------------------------- step sequences --
    def marker_cycle_host(self, inputs: dict, outputs: dict) -> None:
        """The marker cycle from host arrays (eb_marker_cycle_host): `inputs` maps field names to
        host arrays copied in before the steps that read them, `outputs` maps field names to host
        arrays filled as soon as the last step writing each has finished.  Arrays must have the
        field's dtype and marknum elements; pinned host memory lets the copies overlap the steps."""
        def check(name, a):
            want = np.dtype(_abi.MARKER_DTYPE[name])
            if a.dtype != want or a.shape != (self.marknum,) or not a.flags.c_contiguous:
                raise ValueError(f"{name}: need a contiguous {want} array of {self.marknum} markers")
        for k, a in inputs.items():
            check(k, a)
        for k, a in outputs.items():
            check(k, a)
        fin = (C.c_int32 * len(inputs))(*[_abi.MARKER_ID[k] for k in inputs])
        hin = (C.c_void_p * len(inputs))(*[a.ctypes.data for a in inputs.values()])
        fout = (C.c_int32 * len(outputs))(*[_abi.MARKER_ID[k] for k in outputs])
        hout = (C.c_void_p * len(outputs))(*[a.ctypes.data for a in outputs.values()])
        io = _abi.MarkerIO(len(inputs), fin, hin, len(outputs), fout, hout)
        self._check(self._lib.eb_marker_cycle_host(self._ctx, C.byref(io)))

    def correct_advect_and_update_strain(self) -> None:
        """Stress correction, remaining temperature change, RK4 advection with stress rotation
        and the strain update in one marker pass (eb_correct_advect_and_update_strain)."""
        self._call("eb_correct_advect_and_update_strain")

    def initialize_bilinear_interpolation_and_heat_scatter(self) -> None:
        """The bilinear set-up followed by the heat scatter, with the weight denominators summed in
        the heat scatter's walk of the cell lists (same results as the two calls in sequence)."""
        self._call("eb_initialize_bilinear_interpolation_and_heat_scatter")

    def marker_cycle(self, fused: bool = True) -> None:
        """The marker-in-cell transfer + RK4 sequence of one time step (no Stokes/heat solve):
        locate, heat and Stokes scatters, post-Stokes gathers, subgrid stress and temperature,
        stress and temperature corrections, RK4 advection and the strain update.  With
        fused=True the bilinear set-up shares the heat scatter's cell walk and the last four
        steps run as one pass (same results)."""
        self.get_marker_inside_flags()
        if fused:
            self.initialize_bilinear_interpolation_and_heat_scatter()
        else:
            self.initialize_bilinear_interpolation()
            self.interpolate_marker_heat_parameters_to_grid()
        self.interpolate_marker_stokes_parameters_to_grid()
        self.post_stokes_marker_gathers()
        self.update_subgrid_stress()
        if fused:
            self.subgrid_heat_diffusion_update()
            self.correct_advect_and_update_strain()
            return
        self.apply_marker_stress_correction()
        self.subgrid_heat_diffusion_update()
        self.add_remaining_grid_change_to_marker_temperature()
        self.advect_markers_and_rotate_stress()
        self.update_marker_strain()
