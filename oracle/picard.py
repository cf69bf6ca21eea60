"""CPU oracle (TEST INFRASTRUCTURE ONLY) of the Picard plasticity loops and the Stokes step.

``OraclePicard`` couples the marker oracle (``OracleMIC``, mic_oracle.c) and the Stokes oracle
(``StokesOracle``, stokes_oracle.c) over one shared set of grids, the way the reference's
ModelData holds them, and runs the reference's Picard drivers with the direct solve standing in
for MUMPS/UMFPACK.  Only tests/ may use it.

  picard_loop_markers   PlasticityLoopMarkers.picard_loop
                        (global_plasticity_loop/plasticity_loop/plasticity_loop_markers/
                        PlasticityLoopMarkers.jl:36-73) with LoopTermination.check_stop_global_loop_markers
                        (global_plasticity_loop/utils/LoopTermination.jl:3-14)
  picard_loop_nodes     PlasticityLoopNodes.picard_loop (plasticity_loop_nodes/PlasticityLoopNodes.jl:36-92)
                        with check_stop_global_loop_nodes (LoopTermination.jl:16-31) and the grid updates
                        of PlasticityLoopNodes.jl:119-137 and PlasticStrainRateInterpolation.jl:18-40
  stokes step           StokesContinuitySolver.solve_viscoelastic_stokes_continuity_equations!
                        (StokesContinuitySolver.jl:68-90) and stokes_solution_processing! (:113-136)
  norms                 StokesNorms.calculate_solution_norms! (solver/norms/StokesNorms.jl:64-120)
"""
from __future__ import annotations

import numpy as np

from .oracle import OracleMIC
from .stokes import StokesOracle


def _l2(v, v0):
    a = float(np.linalg.norm(np.abs(v0 - v)))
    n = float(np.linalg.norm(v))
    return a, (a / n if n != 0 else 1e38)


def _linf(v, v0):
    a = float(np.max(np.abs(v0 - v)))
    n = float(np.max(np.abs(v)))
    return a, (a / n if n != 0 else 1e38)


class OraclePicard:
    """One model's markers and grids, stepped through the reference's Picard drivers."""

    def __init__(self, model):
        self.mic = OracleMIC(model)
        self.model = self.mic.model
        self.gr = self.mic.gr
        self.so = StokesOracle(self.model)
        self.so.gr = self.gr           # one set of grids, as ModelData holds them
        X, Y = self.model.grid.xnum, self.model.grid.ynum
        self.N = 3 * (X - 1) * (Y - 1)
        self.S = np.zeros(self.N)
        self.S_old = np.zeros(self.N)
        self.old = {"vx1": np.zeros((Y + 1, X), order="F"), "vy1": np.zeros((Y, X + 1), order="F"),
                    "pr1": np.zeros((Y - 1, X - 1), order="F")}
        self.resnl = np.zeros(self.N)

    # StokesContinuitySolver.solve_viscoelastic_stokes_continuity_equations! (StokesContinuitySolver.jl:68-90)
    def solve_viscoelastic_stokes_continuity_equations(self) -> float:
        so = self.so
        so.stokes_steps()
        self.S = so.solve_direct()
        so.process_stokes_solution(self.S)
        self.resnl = so.nonlinear_residual(self.S_old)
        return so.residual(self.S)

    def calculate_stokes_norms(self) -> dict:
        """StokesNorms.calculate_solution_norms! and the nonlinear residual's L2 norm."""
        new = {k: self.gr[k] for k in ("vx1", "vy1", "pr1")}
        out = {}
        out["dsoluv1_abs_inf"], out["dsoluv1_rel_inf"] = _linf(self.S, self.S_old)
        out["dsoluv1_abs_L2"], out["dsoluv1_rel_L2"] = _l2(self.S, self.S_old)
        for k in ("vx1", "vy1", "pr1"):
            out[f"d{k}_abs_L2"], out[f"d{k}_rel_L2"] = _l2(new[k], self.old[k])
        vxy = np.concatenate([new["vx1"].ravel(order="C"), new["vy1"].ravel(order="C")])
        vxy0 = np.concatenate([self.old["vx1"].ravel(order="C"), self.old["vy1"].ravel(order="C")])
        out["dvxy_abs_inf"], out["dvxy_rel_inf"] = _linf(vxy, vxy0)
        out["dvxy_abs_L2"], out["dvxy_rel_L2"] = _l2(vxy, vxy0)
        out["resnl_L2"] = float(np.linalg.norm(self.resnl))
        return out

    # StokesContinuitySolver.stokes_solution_processing! (StokesContinuitySolver.jl:113-136)
    def stokes_solution_processing(self) -> dict:
        self.so.update_grid_strain_rate_and_spin()
        self.so.forecast_viscoelastic_grid_stress()
        self.mic.post_stokes_marker_gathers()
        norms = self.calculate_stokes_norms()
        # SystemSolver.backup_stokes_arrays! (SystemSolver.jl:306-318)
        self.S_old = self.S.copy()
        self.old = {k: self.gr[k].copy(order="F") for k in ("vx1", "vy1", "pr1")}
        return norms

    def picard_loop_markers(self, nglobal: int, tolerance_picard: float, iuse_harmonic: int = 1) -> list:
        history = []
        for iglobal in range(1, nglobal + 1):
            if iglobal > 1:
                self.mic.backup_and_clear_viscosity_transport_arrays()
                self.mic.update_plastic_yielding()
                self.mic.interpolate_viscosity_to_transport_arrays()
                self.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
            res = self.solve_viscoelastic_stokes_continuity_equations()
            norms = self.stokes_solution_processing()
            history.append({"iglobal": iglobal, "rel_residual": res, **norms})
            if iglobal == nglobal or norms["dvxy_rel_L2"] < tolerance_picard:
                break
        return history

    def time_step(self, nglobal: int = 5, tolerance_picard: float = 1e-3, iuse_harmonic: int = 1) -> dict:
        """TimeLoop.run_loop!'s body (src/time_loop/TimeLoop.jl:181-194) restricted to the hot path with
        a fixed time step and no heat solve: the pre-solver averages and rheology (:203-230), the
        Picard loop and the post-Stokes steps (:232-248, StokesContinuitySolver.jl:365-381), the
        advection steps (:261-273) and the inside flags of the moved markers."""
        m, p = self.mic, self.model.params
        nodes = int(p.get("itype_global", 0)) == 1
        m.get_marker_inside_flags()
        m.initialize_bilinear_interpolation()
        m.interpolate_marker_heat_parameters_to_grid()
        m.update_marker_rheology()
        m.update_marker_viscoplastic_viscosity(use_marker_plasticity=not nodes)
        m.interpolate_marker_stokes_parameters_to_grid()
        self.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
        loop = self.picard_loop_nodes if nodes else self.picard_loop_markers
        hist = loop(nglobal, tolerance_picard, iuse_harmonic)
        self.so.interpolate_stag_velocity_to_basic_grid()
        if nodes:
            m.calc_marker_viscoplastic_viscosity()
        self.so.forecast_viscoelastic_grid_stress()
        m.post_stokes_marker_gathers()
        if float(p.get("subgrid_diff_coef_stress", 1.0)) > 0:
            m.update_subgrid_stress()
        m.apply_marker_stress_correction()
        m.advect_markers_and_rotate_stress()
        m.update_marker_strain()
        m.get_marker_inside_flags()
        return {"picard": hist}

    def apply_nodal_plastic_yielding(self):
        """PlasticityLoopNodes.jl:119-137: etas1, plastic_yield and eii_plastic_basic from the
        nodal update; PlasticStrainRateInterpolation.interpolate_at_pressure_nodes!."""
        G = self.gr
        G["etas1"][:] = G["etavp_buffer"]
        G["plastic_yield"][:] = G["plastic_yield_buffer"]
        eb = G["plastic_strain_rate_buffer"]
        G["eii_plastic_basic"][:] = eb
        G["eii_plastic_pressure"][:] = (eb[:-1, :-1] + eb[:-1, 1:] + eb[1:, :-1] + eb[1:, 1:]) / 4.0

    def picard_loop_nodes(self, nglobal: int, tolerance_picard: float, iuse_harmonic: int = 1) -> list:
        history = []
        for iglobal in range(1, nglobal + 1):
            if iglobal > 1:
                self.so.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(iuse_harmonic)
            res = self.solve_viscoelastic_stokes_continuity_equations()
            norms = self.stokes_solution_processing()
            nnode, gerr = self.so.update_nodes_for_plastic_yielding()
            if nnode > 0:
                self.apply_nodal_plastic_yielding()
            history.append({"iglobal": iglobal, "nnode_yield": nnode, "global_yield_error": gerr,
                            "rel_residual": res, **norms})
            if (nnode == 0 or iglobal == nglobal or gerr < tolerance_picard
                    or norms["dvxy_rel_L2"] < tolerance_picard):
                break
        return history
