"""CPU oracle (TEST INFRASTRUCTURE ONLY) for the marker-in-cell hot path.

``OracleMIC`` runs the C restatement in mic_oracle.c on host copies of a
model, step by step, with the same method names as the GPU host mirror.  It
keeps the reference's intermediate marker arrays (marker_dx/dy, the nine
weight arrays) exactly as the reference stores them.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libmic_oracle.so"
SRC = HERE / "mic_oracle.c"
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-fopenmp"]


def build(force: bool = False) -> pathlib.Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        BUILD.mkdir(exist_ok=True)
        tmp = BUILD / "libmic_oracle.so.tmp"
        subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.o_index_of_left_node.restype = C.c_int32
        _lib.o_index_of_left_node.argtypes = [C.c_double, C.c_void_p, C.c_int64]
        _lib.o_scatter_stokes.restype = C.c_int64
    return _lib


def threads() -> int:
    """Host threads the oracle's threaded loops use (OMP_NUM_THREADS or all cores)."""
    return int(lib().o_threads())


def P(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def I(v) -> C.c_int64:
    return C.c_int64(int(v))


def D(v) -> C.c_double:
    return C.c_double(float(v))


class OracleMIC:
    """Host copy of a model plus the reference's per-step functions."""

    def __init__(self, model):
        m = model.copy()
        self.model = m
        self.g = m.grid
        self.mats = m.mats
        self.p = m.params
        self.mk = {k: np.ascontiguousarray(v) for k, v in m.markers.items()}
        self.gr = m.grids
        self.M = m.marknum
        X, Y = self.g.xnum, self.g.ynum
        for name, shape in self._grid_shapes().items():
            if name not in self.gr:
                self.gr[name] = np.zeros(shape, order="F")
        self.mk.setdefault("inside", np.zeros(self.M, np.int8))
        for k in ("xn", "yn", "xn_vy", "yn_vy"):
            self.mk.setdefault(k, np.zeros(self.M, np.int32))
        for k in ("dx", "dy", "dx_vy", "dy_vy", "wUL", "wLL", "wUR", "wLR", "wC", "wULvy", "wLLvy", "wURvy", "wLRvy"):
            self.mk[k] = np.zeros(self.M)
        self._gx = [np.ascontiguousarray(getattr(self.g, n), dtype=np.float64) for n in
                    ("gridx_b", "gridy_b", "xstp_b", "ystp_b", "gridx_vy", "xstp_vy", "gridy_vx", "ystp_vx")]
        flow = np.zeros((self.mats.mat_flow.shape[0], 17))  # the reference's nmat x 17 table
        flow[:, :self.mats.mat_flow.shape[1]] = self.mats.mat_flow
        self.mat_flow = np.asfortranarray(flow).ravel(order="F").copy()
        self.flow_option = int(np.max(self.mats.mat_flow_type))
        self.mat_plastic = np.asfortranarray(self.mats.mat_plastic).ravel(order="F").copy()
        self.mat_mu = np.ascontiguousarray(self.mats.mat_mu, np.float64)
        self.mat_hr = np.ascontiguousarray(self.mats.mat_hr, np.float64)
        self.mat_ft = np.ascontiguousarray(self.mats.mat_flow_type, np.int64)
        self.iters = np.zeros(self.M, np.int32)

    def _grid_shapes(self):
        import importlib
        import sys
        abi = sys.modules.get("earthbox_gb300._abi")
        if abi is None:
            abi = importlib.import_module("earthbox_gb300._abi")
        return {n: abi.grid_shape(n, self.g.xnum, self.g.ynum) for n in abi.GRID_FIELDS}

    # ------------------------------------------------------------- steps ---
    def get_marker_inside_flags(self):
        g = self.g
        lib().o_inside_flags(I(self.M), P(self.mk["x"]), P(self.mk["y"]), D(g.xmin), D(g.xmax), D(g.ymin),
                             D(g.ymax), P(self.mk["inside"]))

    def initialize_bilinear_interpolation(self):
        k, g = self.mk, self.g
        gx, gy, sx, sy, gxvy, sxvy, _, _ = self._gx
        lib().o_locate_and_weights(I(self.M), P(k["inside"]), P(k["x"]), P(k["y"]), I(g.xnum), I(g.ynum),
                                   P(gx), P(gy), P(sx), P(sy), P(gxvy), P(sxvy), P(k["xn"]), P(k["yn"]),
                                   P(k["xn_vy"]), P(k["yn_vy"]), P(k["dx"]), P(k["dy"]), P(k["dx_vy"]),
                                   P(k["dy_vy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]), P(k["wC"]),
                                   P(k["wULvy"]), P(k["wLLvy"]), P(k["wURvy"]), P(k["wLRvy"]))
        gr = self.gr
        lib().o_denominators(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]),
                             P(k["xn_vy"]), P(k["yn_vy"]), P(k["dx"]), P(k["dy"]), P(k["wUL"]), P(k["wLL"]),
                             P(k["wUR"]), P(k["wLR"]), P(k["wC"]), P(k["wULvy"]), P(k["wLLvy"]), P(k["wURvy"]),
                             P(k["wLRvy"]), P(gr["wtnodes"]), P(gr["wtetas"]), P(gr["wtetan"]), P(gr["wtnodes_vy"]))

    def interpolate_marker_stokes_parameters_to_grid(self):
        k, g, gr, p = self.mk, self.g, self.gr, self.p
        names = ["rho1", "rho0", "rho1_vy", "rho0_vy", "etas1", "etas0", "eta_flow", "eta_flow0", "mus1", "mus0",
                 "sxy1", "sxy0", "plastics", "plastics0", "cohesion_grid", "cohesion_grid0", "fric_degrees_grid",
                 "fric_degrees_grid0", "etan1", "etan0", "mun1", "mun0", "sxx1", "sxx0", "plasticn", "plasticn0",
                 "dilatation_grid", "dilatation_grid0", "extractable_meltfrac_grid", "extractable_meltfrac_grid0"]
        ptrs = (C.c_void_p * len(names))(*[gr[n].ctypes.data for n in names])
        rho = self.mats.mat_rho

        def mrho(i):
            return float(rho[i - 1]) if 1 <= i <= len(rho) else -1.0
        air = mrho(p["matid_sticky_air_rho"]) if p["iuse_topo"] == 1 else -1.0
        water = mrho(p["matid_sticky_water_rho"]) if p["iuse_topo"] == 1 else -1.0
        rc = lib().o_scatter_stokes(
            I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]), P(k["xn_vy"]), P(k["yn_vy"]),
            P(k["dx"]), P(k["dy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]), P(k["wC"]), P(k["wULvy"]),
            P(k["wLLvy"]), P(k["wURvy"]), P(k["wLRvy"]), P(gr["wtnodes"]), P(gr["wtetas"]), P(gr["wtetan"]),
            P(gr["wtnodes_vy"]), P(k["matid"]), P(self.mat_mu), P(k["rho"]), P(k["cohesion"]), P(k["fric"]),
            P(k["eta"]), P(k["eta_flow"]), P(k["sxx"]), P(k["sxy"]), P(k["pfailure"]), P(k["dilatation"]),
            P(k["meltfrac"]), ptrs, I(p["iuse_topo"]), P(self._gx[1]), P(gr["hr1"]), D(p["y_sealevel"]), D(air),
            D(water))
        if rc:
            raise RuntimeError(f"Shear modulus for marker material is zero (marker {rc})")

    def interpolate_marker_heat_parameters_to_grid(self):
        k, g, gr, p = self.mk, self.g, self.gr, self.p
        lib().o_scatter_heat(
            I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]), P(k["wUL"]), P(k["wLL"]),
            P(k["wUR"]), P(k["wLR"]), P(gr["wtnodes"]), P(k["matid"]), P(self.mat_hr), P(k["tk"]), P(k["kt"]),
            P(k["rhocp"]), P(k["ha"]), P(k["serp_hr"]), I(p["iuse_serpentinization"]), P(gr["tk1"]), P(gr["tk0"]),
            P(gr["tk2"]), P(gr["kt1"]), P(gr["kt0"]), P(gr["rhocp1"]), P(gr["rhocp0"]), P(gr["hr1"]), P(gr["hr0"]),
            P(gr["ha1"]), P(gr["ha0"]), P(gr["btopt"]), P(gr["bbottomt"]), P(gr["bleftt"]), P(gr["brightt"]))

    def backup_and_clear_viscosity_transport_arrays(self):
        gr, g = self.gr, self.g
        lib().o_backup_clear_viscosity(I(g.xnum), I(g.ynum), P(gr["etas1"]), P(gr["etas0"]), P(gr["etan1"]),
                                       P(gr["etan0"]))

    def interpolate_viscosity_to_transport_arrays(self):
        k, g, gr = self.mk, self.g, self.gr
        lib().o_scatter_viscosity(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]),
                                  P(k["dx"]), P(k["dy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]),
                                  P(k["wC"]), P(gr["wtetas"]), P(gr["wtetan"]), P(k["eta"]), P(gr["etas1"]),
                                  P(gr["etas0"]), P(gr["etan1"]), P(gr["etan0"]))

    def interpolate_temperature_to_markers(self):
        k = self.mk
        lib().o_temperature_to_markers(I(self.M), P(k["inside"]), I(self.g.ynum), P(k["xn"]), P(k["yn"]),
                                       P(k["dx"]), P(k["dy"]), P(self.gr["tk1"]), P(k["tk"]))

    def post_stokes_marker_gathers(self):
        k, g, gr = self.mk, self.g, self.gr
        lib().o_post_stokes_gathers(
            I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["x"]), P(k["y"]), P(k["xn"]), P(k["yn"]),
            P(k["dx"]), P(k["dy"]), P(self._gx[6]), P(self._gx[7]), P(self._gx[4]), P(self._gx[5]), P(gr["exx"]),
            P(gr["exy"]), P(gr["sxx2"]), P(gr["sxy2"]), P(gr["dsxx"]), P(gr["dsxy"]), P(gr["pr1"]), P(k["matid"]),
            P(self.mat_mu), P(k["eta"]), D(self.p["timestep"]), P(k["exx"]), P(k["exy"]), P(k["sr_ratio"]),
            P(k["pr"]))

    def update_subgrid_stress(self):
        if not self.p["subgrid_diff_coef_stress"] > 0:
            return
        k, g, gr = self.mk, self.g, self.gr
        lib().o_subgrid_stress(
            I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["x"]), P(k["y"]), P(k["xn"]), P(k["yn"]),
            P(k["dx"]), P(k["dy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]), P(k["wC"]), P(self._gx[6]),
            P(self._gx[7]), P(self._gx[4]), P(self._gx[5]), P(k["matid"]), P(self.mat_mu), P(k["eta"]),
            D(self.p["timestep"]), D(self.p["subgrid_diff_coef_stress"]), P(gr["sxy1"]), P(gr["sxx1"]),
            P(k["sxy"]), P(k["sxx"]), P(gr["dsxyn"]), P(gr["dsxxn"]), P(gr["wtetas"]), P(gr["wtetan"]),
            P(gr["dsxy"]), P(gr["dsxx"]))

    def excl_cent_average(self, v_excl, v_cent):
        """Weighted averages of per-marker values with the exclusive (basic grid) and central
        (pressure grid) weights of the current marker positions (test-side error scales)."""
        k, g = self.mk, self.g
        ve = np.ascontiguousarray(v_excl, dtype=np.float64)
        vc = np.ascontiguousarray(v_cent, dtype=np.float64)
        ae = np.zeros((g.ynum, g.xnum), order="F")
        ac = np.zeros((g.ynum - 1, g.xnum - 1), order="F")
        lib().o_excl_cent_average(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]),
                                  P(k["dx"]), P(k["dy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]),
                                  P(k["wC"]), P(ve), P(vc), P(ae), P(ac))
        return ae, ac

    def apply_marker_stress_correction(self):
        k, g, gr = self.mk, self.g, self.gr
        lib().o_stress_correction(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["x"]), P(k["y"]),
                                  P(k["xn"]), P(k["yn"]), P(k["dx"]), P(k["dy"]), P(self._gx[6]), P(self._gx[7]),
                                  P(self._gx[4]), P(self._gx[5]), P(gr["dsxy"]), P(gr["dsxx"]), P(k["sxy"]),
                                  P(k["sxx"]))

    def subgrid_heat_diffusion_update(self):
        k, g, gr = self.mk, self.g, self.gr
        lib().o_subgrid_heat(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(k["xn"]), P(k["yn"]), P(k["dx"]),
                             P(k["dy"]), P(k["wUL"]), P(k["wLL"]), P(k["wUR"]), P(k["wLR"]), D(g.xstpavg),
                             D(g.ystpavg), D(self.p["timestep"]), D(self.p["subgrid_diff_coef_temp"]), P(gr["tk1"]),
                             P(gr["kt1"]), P(gr["rhocp1"]), P(k["tk"]), P(k["subgrid_dt"]), P(gr["dtkn"]),
                             P(gr["wtnodes"]), P(gr["dtk1"]))

    def add_remaining_grid_change_to_marker_temperature(self):
        k = self.mk
        lib().o_add_remaining_dt(I(self.M), P(k["inside"]), I(self.g.ynum), P(k["xn"]), P(k["yn"]), P(k["dx"]),
                                 P(k["dy"]), P(self.gr["dtk1"]), P(k["tk"]))

    def advect_markers_and_rotate_stress(self):
        k, g, gr = self.mk, self.g, self.gr
        gx, gy, sx, sy, gxvy, sxvy, gyvx, syvx = self._gx
        lib().o_advect(I(self.M), P(k["inside"]), I(g.xnum), I(g.ynum), P(gx), P(gy), P(sx), P(sy), P(gxvy), P(sxvy),
                       P(gyvx), P(syvx), P(gr["vx1"]), P(gr["vy1"]), P(gr["esp"]), D(self.p["timestep"]),
                       I(self.p["runge_kutta_order"]), P(k["xn"]), P(k["yn"]), P(k["x"]), P(k["y"]), P(k["vx"]),
                       P(k["vy"]), P(k["spin"]), P(k["sxx"]), P(k["sxy"]))

    def update_marker_strain(self):
        k = self.mk
        lib().o_update_strain(I(self.M), P(k["inside"]), D(self.p["timestep"]), D(self.p["plastic_healing_rate"]),
                              P(k["exx"]), P(k["exy"]), P(k["gii"]), P(k["sxx"]), P(k["sxy"]), P(k["eta"]),
                              P(k["eta_flow"]), P(k["pfailure"]), P(k["strain_plastic"]),
                              P(k["strain_rate_plastic"]))

    def update_marker_rheology(self):
        k, p = self.mk, self.p
        lib().o_failure_properties(I(self.M), P(k["inside"]), P(k["matid"]), I(self.mats.nmat), P(self.mat_plastic),
                                   P(k["strain_plastic"]), P(k["fric_ini"]), I(p["iuse_melt_damage"]),
                                   P(k["melt_damage"]), P(k["cohesion"]), P(k["fric"]))
        if self.flow_option in (-1, 0, 4, 5):
            g = self.g
            lib().o_flow_viscosity_other(
                I(self.M), P(k["inside"]), P(k["matid"]), I(self.mats.nmat), I(self.flow_option), P(self.mat_flow),
                D(p["temperature_top"]), D(p.get("temperature_bottom", 0.0)), D(p.get("temperature_left", 0.0)),
                D(p["gas_constant"]), D(g.ymax - g.ymin), D(p["viscosity_max"]), P(k["x"]), P(k["y"]), P(k["tk"]),
                P(k["eta_flow"]), P(k["preexp"]))
            return
        lib().o_composite_viscosity(
            I(self.M), P(k["inside"]), P(k["matid"]), I(self.mats.nmat), P(self.mat_ft), P(self.mat_flow),
            P(self.mat_plastic), P(self.mat_mu), D(p["timestep"]), D(p["temperature_top"]), D(p["viscosity_min"]),
            D(p["viscosity_max"]), D(p["powerlaw_stress_min"]), D(p["gas_constant"]), I(p["iuse_viscous_strain_soft"]),
            D(p["vsoftfac"]), P(k["sxx"]), P(k["sxy"]), P(k["exx"]), P(k["exy"]), P(k["tk"]), P(k["pr"]), P(k["gii"]),
            P(k["sr_ratio"]), P(k["eta_flow"]), P(k["preexp"]), P(self.iters))

    def update_marker_viscoplastic_viscosity(self, use_marker_plasticity=True):
        k, p = self.mk, self.p
        lib().o_viscoplastic_viscosity(I(self.M), P(k["inside"]), I(p["ntimestep"]), I(p["itype_global"]),
                                       P(k["eta_flow"]), P(k["eta"]))
        if use_marker_plasticity:
            self.update_plastic_yielding()

    def update_plastic_yielding(self):
        k, p = self.mk, self.p
        lib().o_plastic_yielding(
            I(self.M), P(k["inside"]), I(p["ntimestep"]), D(p["timestep"]), I(p["iuse_fluid_pressure_for_yield"]),
            D(p["y_sealevel"]), D(p["viscosity_min"]), D(p["viscosity_max"]), D(p["yield_stress_min"]),
            D(p["yield_stress_max"]), I(p["no_yielding_in_mobile_wall"]), I(p["matid_sticky_air"]),
            I(p["matid_mobile_wall"]), I(p["matid_plate_extension"]), P(k["y"]), P(k["matid"]), P(self.mat_mu),
            P(k["cohesion"]), P(k["fric"]), P(k["exx"]), P(k["exy"]), P(k["sr_ratio"]), P(k["pr"]), P(k["sxx"]),
            P(k["sxy"]), P(k["eta"]), P(k["pfailure"]))

    def calc_marker_viscoplastic_viscosity(self):
        """GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity! (plastic_yield, etas1 -> eta)."""
        k, gr = self.mk, self.gr
        lib().o_marker_viscoplastic_viscosity_from_grid(
            I(self.M), P(k["inside"]), I(self.g.ynum), P(k["xn"]), P(k["yn"]), P(k["dx"]), P(k["dy"]),
            P(np.asfortranarray(gr["plastic_yield"])), P(np.asfortranarray(gr["etas1"])), P(k["eta_flow"]),
            P(k["eta"]), P(k["pfailure"]))

    def marker_cycle(self):
        self.get_marker_inside_flags()
        self.initialize_bilinear_interpolation()
        self.interpolate_marker_heat_parameters_to_grid()
        self.interpolate_marker_stokes_parameters_to_grid()
        self.post_stokes_marker_gathers()
        self.update_subgrid_stress()
        self.apply_marker_stress_correction()
        self.subgrid_heat_diffusion_update()
        self.add_remaining_grid_change_to_marker_temperature()
        self.advect_markers_and_rotate_stress()
        self.update_marker_strain()
