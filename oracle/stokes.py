"""CPU oracle (TEST INFRASTRUCTURE ONLY) for the Stokes-continuity step.

``StokesOracle`` runs the C restatement in stokes_oracle.c on host copies of
a model's grids, with the reference's step names: viscoelastic terms, RHS
grids, solver initialisation (pscale), the COO system in the reference's entry
order, a direct solve (scipy's SuperLU, standing in for the reference's
UMFPACK / MUMPS call), and the unpacking of the solution into vx1, vy1, pr1.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libstokes_oracle.so"
SRC = HERE / "stokes_oracle.c"
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def build(force: bool = False) -> pathlib.Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        BUILD.mkdir(exist_ok=True)
        tmp = BUILD / "libstokes_oracle.so.tmp"
        subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.o_build_system.restype = C.c_int64
    return _lib


class StokesIn(C.Structure):
    _fields_ = [("xnum", C.c_int64), ("ynum", C.c_int64), ("xstpavg", C.c_double), ("ystpavg", C.c_double)] + [
        (n, C.c_void_p) for n in ("xstp", "ystp", "xstpc", "ystpc", "btopx", "bbottomx", "btopy", "bbottomy",
                                  "bleftx", "brightx", "blefty", "brighty", "bintern_zone", "bintern_velocity")
    ] + [("pressure_bc_mode", C.c_int64), ("pressure_bc", C.c_double), ("timestep", C.c_double),
         ("gravity_y", C.c_double), ("iuse_interface_stabilization", C.c_int64), ("pscale", C.c_double)] + [
        (n, C.c_void_p) for n in ("etan", "etas", "rho1_vy", "RX", "RY", "RC")]


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _f(a) -> np.ndarray:
    return np.asfortranarray(np.array(a, dtype=np.float64, copy=True))


BC_NAMES = ("btopx", "bbottomx", "btopy", "bbottomy", "bleftx", "brightx", "blefty", "brighty")


class StokesOracle:
    """Host copies of the Stokes inputs of one model, stepped like the reference."""

    def __init__(self, model, grids: dict | None = None):
        g = model.grid
        self.model = model
        self.xnum, self.ynum = g.xnum, g.ynum
        self.p = model.params
        src = dict(model.grids)
        if grids:
            src.update(grids)
        self.gr = {k: _f(v) for k, v in src.items()}
        X, Y = self.xnum, self.ynum
        for name, shape in (("etas0", (Y, X)), ("sxy0", (Y, X)), ("etan0", (Y - 1, X - 1)), ("sxx0", (Y - 1, X - 1)),
                            ("RX1", (Y + 1, X)), ("RY1", (Y, X + 1)), ("RC1", (Y - 1, X - 1))):
            self.gr.setdefault(name, np.zeros(shape, order="F"))
        self.spacing = {k: np.ascontiguousarray(getattr(g, k), dtype=np.float64)
                        for k in ("xstp_b", "ystp_b", "xstp_vy", "ystp_vx")}
        self.pscale = None
        self.coo = None

    # StokesViscoelasticTerms.calc_viscoelastic_terms! (StokesViscoelasticTerms.jl:26-125)
    def calc_viscoelastic_terms(self):
        G = self.gr
        lib().o_viscoelastic_terms(C.c_int64(self.xnum), C.c_int64(self.ynum), C.c_double(self.p["timestep"]),
                                   _p(G["etas1"]), _p(G["mus1"]), _p(G["sxy1"]), _p(G["etan1"]), _p(G["mun1"]),
                                   _p(G["sxx1"]), _p(G["etas0"]), _p(G["sxy0"]), _p(G["etan0"]), _p(G["sxx0"]))

    # StokesContinuityRhs.viscoelastic_rhs! (StokesContinuityRhs.jl:30-190)
    def viscoelastic_rhs(self):
        G, S = self.gr, self.spacing
        lib().o_viscoelastic_rhs(C.c_int64(self.xnum), C.c_int64(self.ynum), C.c_double(self.p["gravity_x"]),
                                 C.c_double(self.p["gravity_y"]), C.c_int64(self.p["iuse_interface_stabilization"]),
                                 _p(S["xstp_b"]), _p(S["ystp_b"]), _p(S["xstp_vy"]), _p(S["ystp_vx"]),
                                 _p(G["rho1"]), _p(G["rho1_vy"]), _p(G["sxx0"]), _p(G["sxy0"]),
                                 _p(G["dilatation_grid"]), _p(G["eii_plastic_pressure"]),
                                 _p(G["RX1"]), _p(G["RY1"]), _p(G["RC1"]))

    # SystemSolver.initialize_solver! / pressure_scaling_coeff (SystemSolver.jl:99-115)
    def initialize_solver(self):
        g = self.model.grid
        self.pscale = 2.0 * self.gr["etan0"][0, 0] / (g.xstpavg + g.ystpavg)
        X, Y = self.xnum, self.ynum
        self.gr["vx1"] = np.zeros((Y + 1, X), order="F")
        self.gr["vy1"] = np.zeros((Y, X + 1), order="F")
        self.gr["pr1"] = np.zeros((Y - 1, X - 1), order="F")

    def _struct(self) -> StokesIn:
        g, G, S, p = self.model.grid, self.gr, self.spacing, self.p
        self._keep = [np.ascontiguousarray(p["bintern_zone"], dtype=np.int64),
                      np.ascontiguousarray(p["bintern_velocity"], dtype=np.float64)]
        s = StokesIn(xnum=self.xnum, ynum=self.ynum, xstpavg=g.xstpavg, ystpavg=g.ystpavg,
                     xstp=_p(S["xstp_b"]), ystp=_p(S["ystp_b"]), xstpc=_p(S["xstp_vy"]), ystpc=_p(S["ystp_vx"]),
                     bintern_zone=_p(self._keep[0]), bintern_velocity=_p(self._keep[1]),
                     pressure_bc_mode=int(p["pressure_bc_mode"]), pressure_bc=float(p["pressure_bc"]),
                     timestep=float(p["timestep"]), gravity_y=float(p["gravity_y"]),
                     iuse_interface_stabilization=int(p["iuse_interface_stabilization"]), pscale=self.pscale,
                     etan=_p(G["etan0"]), etas=_p(G["etas0"]), rho1_vy=_p(G["rho1_vy"]),
                     RX=_p(G["RX1"]), RY=_p(G["RY1"]), RC=_p(G["RC1"]))
        for n in BC_NAMES:
            setattr(s, n, _p(G[n]))
        return s

    @property
    def N(self) -> int:
        return 3 * (self.xnum - 1) * (self.ynum - 1)

    # StokesBuildManager.build_system_of_equations (StokesBuildManager.jl:661-712)
    def build_system_of_equations(self):
        ncell = (self.xnum - 1) * (self.ynum - 1)
        cap = 26 * ncell
        Li = np.zeros(cap, np.int64)
        Lj = np.zeros(cap, np.int64)
        Lv = np.zeros(cap, np.float64)
        R = np.zeros(self.N, np.float64)
        s = self._struct()
        n = lib().o_build_system(C.byref(s), _p(Li), _p(Lj), _p(Lv), _p(R))
        self.coo = (Li[:n].copy(), Lj[:n].copy(), Lv[:n].copy(), R)
        return self.coo

    def matrix(self):
        """sparse(Li, Lj, Lv, N, N): duplicate entries summed, as Julia's sparse does."""
        import scipy.sparse as sp
        Li, Lj, Lv, _ = self.coo
        return sp.csr_matrix((Lv, (Li - 1, Lj - 1)), shape=(self.N, self.N))

    def stokes_steps(self):
        """stokes_solver_build_steps (StokesContinuitySolver.jl:97-110) without the solve."""
        self.calc_viscoelastic_terms()
        self.viscoelastic_rhs()
        self.initialize_solver()
        return self.build_system_of_equations()

    def solve_direct(self) -> np.ndarray:
        """The direct solve (SystemSolver.jl:67-91 uses UMFPACK or MUMPS; SuperLU here)."""
        import scipy.sparse.linalg as spla
        return spla.spsolve(self.matrix().tocsc(), self.coo[3])

    def residual(self, S: np.ndarray) -> float:
        """||L S - R||_2 / ||R||_2 of the assembled system."""
        R = self.coo[3]
        return float(np.linalg.norm(self.matrix() @ S - R) / np.linalg.norm(R))

    # SystemSolver.process_stokes_solution! (SystemSolver.jl:141-271)
    def process_stokes_solution(self, S: np.ndarray):
        G = self.gr
        S = np.ascontiguousarray(S, dtype=np.float64)
        lib().o_process_stokes_solution(C.c_int64(self.xnum), C.c_int64(self.ynum), C.c_double(self.pscale), _p(S),
                                        *[_p(G[n]) for n in BC_NAMES], _p(G["vx1"]), _p(G["vy1"]), _p(G["pr1"]))

    # StokesResiduals.stokes_calc_nonlinear_system_residual_optimized! (StokesResiduals.jl:63-81)
    def nonlinear_residual(self, S_old: np.ndarray) -> np.ndarray:
        Li, Lj, Lv, R = self.coo
        work = np.zeros(self.N)
        resnl = np.zeros(self.N)
        x = np.ascontiguousarray(S_old, dtype=np.float64)
        lib().o_coo_residual(C.c_int64(len(Li)), _p(Li), _p(Lj), _p(Lv), _p(x), _p(R), C.c_int64(self.N),
                             _p(work), _p(resnl))
        return resnl

    # ---- post-solve grid kernels ------------------------------------------------
    def update_grid_strain_rate_and_spin(self):
        """GridStrainRate.update_grid_strain_rate_and_spin! (utils/strain_rate/GridStrainRate.jl:6-182)."""
        G, S = self.gr, self.spacing
        X, Y = self.xnum, self.ynum
        for k, sh in (("exx", (Y - 1, X - 1)), ("exy", (Y, X)), ("eii", (Y - 1, X - 1)), ("esp", (Y, X))):
            G[k] = np.zeros(sh, order="F")
        lib().o_grid_strain_rate_and_spin(C.c_int64(X), C.c_int64(Y), _p(S["xstp_b"]), _p(S["ystp_b"]),
                                          _p(S["xstp_vy"]), _p(S["ystp_vx"]), _p(G["vx1"]), _p(G["vy1"]),
                                          _p(G["exx"]), _p(G["exy"]), _p(G["eii"]), _p(G["esp"]))

    def forecast_viscoelastic_grid_stress(self):
        """GridStress.forecast_viscoelastic_grid_stress! and calculate_deviatoric_grid_stress_change!
        (utils/GridStress.jl:30-134)."""
        G = self.gr
        X, Y = self.xnum, self.ynum
        for k, sh in (("sxy2", (Y, X)), ("sxx2", (Y - 1, X - 1)), ("dsxy", (Y, X)), ("dsxx", (Y - 1, X - 1))):
            G[k] = np.zeros(sh, order="F")
        lib().o_forecast_grid_stress(C.c_int64(X), C.c_int64(Y), C.c_double(self.p["timestep"]), _p(G["etas1"]),
                                     _p(G["mus1"]), _p(G["exy"]), _p(G["sxy1"]), _p(G["etan1"]), _p(G["mun1"]),
                                     _p(G["exx"]), _p(G["sxx1"]), _p(G["sxy2"]), _p(G["sxx2"]), _p(G["dsxy"]),
                                     _p(G["dsxx"]))

    def interpolate_stag_velocity_to_basic_grid(self):
        """StokesInterpolate.interpolate_stag_velocity_to_basic_grid! (utils/StokesInterpolate.jl:16-33)."""
        G = self.gr
        X, Y = self.xnum, self.ynum
        G["vxb"] = np.zeros((Y, X), order="F")
        G["vyb"] = np.zeros((Y, X), order="F")
        lib().o_stag_velocity_to_basic(C.c_int64(X), C.c_int64(Y), _p(G["vx1"]), _p(G["vy1"]), _p(G["vxb"]),
                                       _p(G["vyb"]))

    def interpolate_basic_viscoplastic_viscosity_to_pressure_grid(self, iuse_harmonic: int = 1):
        """Interpolation.interpolate_basic_viscoplastic_viscosity_to_pressure_grid! (Interpolation.jl:97-108)."""
        if iuse_harmonic != 1:
            return
        G = self.gr
        lib().o_harmonic_normal_viscosity(C.c_int64(self.xnum), C.c_int64(self.ynum), _p(G["etas1"]),
                                          _p(G["plastics"]), _p(G["plasticn"]), _p(G["plastic_yield"]),
                                          _p(G["etan1"]))

    def update_nodes_for_plastic_yielding(self, wall: dict | None = None):
        """PlasticFailureNodes.update_nodes_for_plastic_yielding (PlasticFailureNodes.jl:24-184).
        Returns (nnode_yield, global_yield_error); fills etavp_buffer, plastic_yield_buffer,
        plastic_strain_rate_buffer and yield_error."""
        G, g, p = self.gr, self.model.grid, self.p
        X, Y = self.xnum, self.ynum
        for k in ("etavp_buffer", "plastic_yield_buffer", "plastic_strain_rate_buffer"):
            G[k] = np.zeros((Y, X), order="F")
        G.setdefault("yield_error", np.zeros((Y, X), order="F"))
        w = wall or {}

        class Q(C.Structure):
            _fields_ = [(n, C.c_int64) for n in ("ntimestep", "iuse_fluid", "no_wall", "no_plate")] + [
                (n, C.c_double) for n in ("timestep", "timesum", "vmin", "vmax", "y_sealevel", "vix", "xl", "xr",
                                          "yt", "yb", "pthick", "pwidth")]
        q = Q(ntimestep=int(p["ntimestep"]), iuse_fluid=int(p["iuse_fluid_pressure_for_yield"]),
              no_wall=int(p["no_yielding_in_mobile_wall"]) if wall else 0,
              no_plate=int(w.get("no_yielding_in_plate_extension", 0)), timestep=p["timestep"],
              timesum=w.get("timesum", 0.0), vmin=p["viscosity_min"], vmax=p["viscosity_max"],
              y_sealevel=p["y_sealevel"], vix=w.get("velocity_internal_x", 0.0), xl=w.get("x_left_mobile_wall", 0.0),
              xr=w.get("x_right_mobile_wall", 0.0), yt=w.get("y_top_mobile_wall", 0.0),
              yb=w.get("y_bottom_mobile_wall", 0.0), pthick=w.get("plate_extension_thickness", 0.0),
              pwidth=w.get("plate_extension_width", 0.0))
        gx = np.ascontiguousarray(g.gridx_b, dtype=np.float64)
        gy = np.ascontiguousarray(g.gridy_b, dtype=np.float64)
        gerr = C.c_double()
        f = lib().o_nodal_plastic_yielding
        f.restype = C.c_int64
        n = f(C.byref(q), C.c_int64(X), C.c_int64(Y), _p(gx), _p(gy), _p(G["plastic_yield"]), _p(G["etas1"]),
              _p(G["eta_flow"]), _p(G["mus1"]), _p(G["cohesion_grid"]), _p(G["fric_degrees_grid"]), _p(G["sxy2"]),
              _p(G["sxx2"]), _p(G["pr1"]), _p(G["yield_error"]), _p(G["etavp_buffer"]),
              _p(G["plastic_strain_rate_buffer"]), _p(G["plastic_yield_buffer"]), C.byref(gerr))
        return int(n), gerr.value
