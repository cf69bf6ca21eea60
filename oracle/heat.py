"""CPU oracle (TEST INFRASTRUCTURE ONLY) for the conductive heat step.

``HeatOracle`` runs the C restatement in heat_oracle.c on host copies of a
model's grids, with the reference's step names: the heat RHS terms
(HeatRhs.jl), tk0 <- tk1, the adaptive heat loop (HeatLoop.jl:10-79) around
the COO assembly (HeatBuildManager.jl:44-86) and a direct solve (scipy's
SuperLU standing in for the reference's UMFPACK / MUMPS call,
heat_solver/solver/SystemSolver.jl:32-66), the residual grid
(HeatResiduals.jl:12-162) and dtk1 = tk2 - tk1 (HeatSolver.jl:211-216).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libheat_oracle.so"
SRC = HERE / "heat_oracle.c"
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]

HEAT_GRIDS = ("tk1", "kt1", "rhocp1", "hr1", "ha1", "rho1", "vx1", "vy1", "sxy2", "etas1", "sxx2", "etan1",
              "btopt", "bbottomt", "bleftt", "brightt")


def build(force: bool = False) -> pathlib.Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        BUILD.mkdir(exist_ok=True)
        tmp = BUILD / "libheat_oracle.so.tmp"
        subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.o_heat_build.restype = C.c_int64
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _f(a) -> np.ndarray:
    return np.asfortranarray(np.array(a, dtype=np.float64, copy=True))


def heat_params(params: dict) -> dict:
    """The heat-step scalars with the reference's names and the build's defaults."""
    return {"timestep": float(params["timestep"]), "max_temp_change": float(params.get("max_temp_change", 20.0)),
            "gravity_x": float(params.get("gravity_x", 0.0)), "gravity_y": float(params.get("gravity_y", 9.81)),
            "iuse_adiabatic_heating": int(params.get("iuse_adiabatic_heating", 1)),
            "iuse_shear_heating": int(params.get("iuse_shear_heating", 1))}


class HeatOracle:
    """Host copies of the heat inputs of one model, stepped like the reference."""

    def __init__(self, model, grids: dict | None = None):
        g = model.grid
        self.model = model
        self.xnum, self.ynum = g.xnum, g.ynum
        self.hp = heat_params(model.params)
        src = dict(model.grids)
        if grids:
            src.update(grids)
        self.gr = {k: _f(src[k]) for k in HEAT_GRIDS}
        shape = (self.ynum, self.xnum)
        for k in ("RT1", "tk0", "tk2", "dtk1", "rest"):
            self.gr[k] = np.zeros(shape, order="F")
        self.gx = np.ascontiguousarray(g.gridx_b, dtype=np.float64)
        self.gy = np.ascontiguousarray(g.gridy_b, dtype=np.float64)
        self.xstp = np.ascontiguousarray(g.xstp_b, dtype=np.float64)
        self.ystp = np.ascontiguousarray(g.ystp_b, dtype=np.float64)
        self.coo = None
        self.timestep_heat = self.hp["timestep"]
        self.solves = 0
        self.substeps = 0

    @property
    def N(self) -> int:
        return self.xnum * self.ynum

    # HeatSolver.calculate_heat_rhs_terms_grid! (HeatSolver.jl:139-150) -> HeatRhs.jl:5-80
    def calculate_heat_rhs_terms(self):
        G, hp = self.gr, self.hp
        lib().o_heat_rhs_terms(C.c_int64(self.xnum), C.c_int64(self.ynum), _p(G["hr1"]), _p(G["ha1"]), _p(G["rho1"]),
                               _p(G["vx1"]), _p(G["vy1"]), _p(G["sxy2"]), _p(G["etas1"]), _p(G["sxx2"]),
                               _p(G["etan1"]), C.c_double(hp["gravity_x"]), C.c_double(hp["gravity_y"]),
                               C.c_int64(hp["iuse_adiabatic_heating"]), C.c_int64(hp["iuse_shear_heating"]),
                               _p(G["RT1"]))

    # HeatSolver.initialize_old_temperature_array! (HeatSolver.jl:199-204)
    def initialize_old_temperature_array(self):
        self.gr["tk0"][...] = self.gr["tk1"]

    # HeatBuildManager.build_system_of_equations (HeatBuildManager.jl:44-86)
    def build_system_of_equations(self, dt: float | None = None):
        G = self.gr
        dt = self.timestep_heat if dt is None else dt
        cap = 5 * self.N
        Li = np.zeros(cap, np.int64)
        Lj = np.zeros(cap, np.int64)
        Lv = np.zeros(cap)
        R = np.zeros(self.N)
        nnz = lib().o_heat_build(C.c_int64(self.xnum), C.c_int64(self.ynum), _p(self.gx), _p(self.gy), _p(self.xstp),
                                 _p(self.ystp), _p(G["tk0"]), _p(G["rhocp1"]), _p(G["kt1"]), _p(G["RT1"]),
                                 _p(G["btopt"]), _p(G["bbottomt"]), _p(G["bleftt"]), _p(G["brightt"]),
                                 C.c_double(dt), _p(Li), _p(Lj), _p(Lv), _p(R))
        self.coo = (Li[:nnz], Lj[:nnz], Lv[:nnz], R)
        return self.coo

    def matrix(self):
        import scipy.sparse as sp
        Li, Lj, Lv, _ = self.coo
        return sp.csr_matrix((Lv, (Li - 1, Lj - 1)), shape=(self.N, self.N))

    # SystemSolver.discretize_and_solve_conductive_heat_equation (SystemSolver.jl:32-66) + reload_solu_temp
    def discretize_and_solve(self, dt: float | None = None):
        import scipy.sparse.linalg as spla
        self.build_system_of_equations(dt)
        S = spla.spsolve(self.matrix().tocsc(), self.coo[3])
        self.gr["tk2"][...] = S.reshape((self.ynum, self.xnum), order="F")
        self.solves += 1
        return S

    def residual(self, S) -> float:
        R = self.coo[3]
        return float(np.linalg.norm(R - self.matrix() @ S) / np.linalg.norm(R))

    # HeatResiduals.compute_residuals_temp! (HeatResiduals.jl:12-17)
    def compute_residuals_temp(self, dt: float | None = None):
        G = self.gr
        dt = self.timestep_heat if dt is None else dt
        lib().o_heat_residuals(C.c_int64(self.xnum), C.c_int64(self.ynum), _p(self.gx), _p(self.gy), _p(self.xstp),
                               _p(self.ystp), _p(G["RT1"]), _p(G["rhocp1"]), _p(G["tk0"]), _p(G["tk2"]),
                               _p(G["kt1"]), C.c_double(dt), _p(G["rest"]))

    # HeatLoop.run_conductive_heat_solver_loop! (HeatLoop.jl:10-79)
    def run_conductive_heat_solver_loop(self):
        G = self.gr
        limit = self.hp["max_temp_change"]
        timestep_start = self.hp["timestep"]
        timestep_loop = timestep_start
        self.timestep_heat = timestep_loop
        timestep_sum = 0.0
        while timestep_sum < timestep_start:
            self.discretize_and_solve()
            self.compute_residuals_temp()
            G["dtk1"][...] = G["tk2"] - G["tk0"]
            dtkmax = float(np.max(np.abs(G["dtk1"])))
            if dtkmax > limit:
                timestep_loop = timestep_loop * limit / dtkmax
                self.timestep_heat = timestep_loop
                self.discretize_and_solve()
                self.compute_residuals_temp()
            timestep_sum = timestep_sum + timestep_loop
            timestep_loop = min(timestep_loop, timestep_start - timestep_sum)
            self.timestep_heat = timestep_loop
            G["tk0"][...] = G["tk2"]
            self.substeps += 1
        return timestep_sum

    # HeatSolver.calculate_grid_temp_change! (HeatSolver.jl:211-216)
    def calculate_grid_temp_change(self):
        self.gr["dtk1"][...] = self.gr["tk2"] - self.gr["tk1"]

    # the grid part of HeatSolver.update_marker_temp_for_grid_and_subgrid_changes! (HeatSolver.jl:94-122)
    def heat_step(self):
        self.calculate_heat_rhs_terms()
        self.initialize_old_temperature_array()
        self.run_conductive_heat_solver_loop()
        self.calculate_grid_temp_change()
