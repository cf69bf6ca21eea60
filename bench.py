"""Benchmark of the marker-in-cell hot path on one GB300 (markers/s, MIC transfer + RK4).

A step is one marker cycle of the 40M-marker rifting model (2001x801 basic
nodes, 25 markers per cell): inside flags, cell location and the cell-sorted
marker list, heat and Stokes marker->grid averaging, post-Stokes marker
gathers, subgrid stress and temperature diffusion, the stress and temperature
corrections, fused RK4 advection with stress rotation, and the strain update.
Every field is larger than L2 (40M x 8 B = 320 MB), so no L2 flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

Prints one JSON line.  ``value`` is markers/s with the model resident in HBM;
``e2e`` is the same metric through the C-ABI with host buffers: each step
uploads the marker state from pinned host memory and downloads the updated
state.  ``--impl reference`` times the CPU restatement of the reference (the
EarthBox.jl functions in plain C, OpenMP across the loops the reference runs
with Threads.@threads, serial scatters as in the reference) on a bounded strip
of the same model.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
from __graft_entry__ import load_oracle, load_package  # noqa: E402

METRIC = "markers/s (MIC transfer+RK4)"
UNIT = "markers/s"

# Bytes per marker each kernel must move (reads + writes of marker arrays), and
# grid bytes per call; the dominant-kernel roofline uses these.
ALGO_BYTES_PER_MARKER = {
    "k_cells<stokes>": 4 + 4 + 8 + 1 + 4 + 8 * 8 + 4 + 4,   # perm, xn, fx/fy, flags, matid, 8 f64, 2 f32
    "k_cells<heat>": 4 + 8 + 1 + 4 + 5 * 8,
    "k_cells<denominators>": 4 + 4 + 8 + 1,
    "k_cells<subgrid_stress>": 4 + 8 + 8 + 1 + 4 + 8 + 2 * 16,
    "k_cells<subgrid_heat>": 4 + 8 + 8 + 1 + 16 + 8,
    "k_advect": 8 + 8 + 1 + 16 + 16 + 24 + 32,             # xn/yn, fx/fy, flags, rw x/y, w vx/vy/spin, rw sxx/sxy
    "k_post_stokes": 8 + 8 + 1 + 4 + 8 + 4 * 8,
    "k_locate_count": 16 + 1 + 8 + 8 + 1 + 4,               # x,y, inside, w xn/yn, fx/fy, flags, count atomics
    # flags, xn/yn, fx/fy, rw sxx/sxy/tk/x/y/gii, w vx/vy/spin, r exx/exy/pfailure; plastic markers
    # (pfailure == 1) also read eta/eta_flow, rw strain_plastic, w strain_rate_plastic (+40 B)
    "k_tail": 1 + 8 + 8 + 6 * 16 + 24 + 16 + 4,
}
TAIL_PLASTIC_BYTES = 8 + 8 + 16 + 8


def algo_bytes_per_marker(kernel: str, model) -> float | None:
    """Algorithmic bytes per marker of `kernel` on this workload."""
    bpm = ALGO_BYTES_PER_MARKER.get(kernel)
    if bpm is not None and kernel == "k_tail":
        bpm += TAIL_PLASTIC_BYTES * float(np.mean(model.markers["pfailure"] == 1.0))
    return bpm

# DRAM bytes per marker (dram__bytes_read.sum + dram__bytes_write.sum) from one
# `ncu --set full` capture of each kernel on the 2.56M-marker rift (801x201
# nodes, 16 markers per cell); reads scale with the marker count,
# writes that still sit in L2 at that size make these a lower bound.
NCU_DRAM_BYTES_PER_MARKER = {
    "k_cells<stokes>": 101.2,
    "k_cells<subgrid_stress>": 57.3,
    "k_advect": 83.1,
    "k_post_stokes": 44.5,
    "k_tail": 167.9,
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="rift_40M")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-stokes", action="store_true")
    ap.add_argument("--no-heat", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-rheology", action="store_true")
    ap.add_argument("--learned-steps", type=int, default=200)
    ap.add_argument("--circles", action="store_true",
                    help="also time the circles_1025 Stokes benchmark (200 inclusions, 1e-10)")
    ap.add_argument("--stokes-method", default="fgmres", choices=["fgmres", "bicgstab"])
    ap.add_argument("--stokes-only", action="store_true",
                    help="after the warm-up marker cycles run ONE mixed Stokes step and print its line "
                         "(a small launch list for ncu; not the bench line)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def peaks_bf16() -> float:
    """Measured dense BF16 tensor throughput (TFLOP/s, burst), else the fallback figure."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text()).get("bf16_tflops", 1900.0))
    return 1900.0


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


E2E_IN = ["x", "y", "matid", "rho", "cohesion", "fric", "eta", "eta_flow", "sxx", "sxy", "pfailure", "dilatation",
          "meltfrac", "tk", "kt", "rhocp", "ha", "serp_hr", "gii", "strain_plastic"]
E2E_OUT = ["x", "y", "sxx", "sxy", "tk", "exx", "exy", "pr", "sr_ratio", "gii", "strain_plastic",
           "strain_rate_plastic"]


def cpu_baseline(eb, oracle, steps: int = 2):
    """The reference's algorithms (C restatement, OpenMP where the reference threads) on a strip
    of the 40M-marker model: 101x801 nodes at the same spacing, 25 markers per cell (2M markers)."""
    model = eb.synthetic.rift(101, 801, 5, width=25e3)
    ref = oracle.OracleMIC(model)
    ref.marker_cycle()  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        ref.marker_cycle()
    dt = (time.perf_counter() - t0) / steps
    return {"value": model.marknum / dt, "unit": UNIT, "cores": oracle.threads(), "kind": "port",
            "sample": f"{model.marknum} markers (101x801-node strip of the 2001x801 model, same spacing), "
                      f"{steps} marker cycles after one warm-up; {dt:.3f} s per cycle"}


STOKES_METRIC = "Stokes s/solve @1e-8 resid"
STOKES_GRIDS = ("etas1", "etan1", "mus1", "mun1", "sxy1", "sxx1", "rho1", "rho1_vy", "dilatation_grid",
                "eii_plastic_pressure", "btopx", "bbottomx", "btopy", "bbottomy", "bleftx", "brightx", "blefty",
                "brighty")


def unet_flops_per_pixel() -> float:
    """Forward FLOPs of the learned stage's U-Net per full-resolution pixel (2 per multiply-add
    of each convolution, pixels of level l = 1 / 4^l of the full resolution)."""
    layers = [(8, 32, 9, 0), (32, 32, 9, 0), (32, 64, 9, 1), (64, 64, 9, 1), (64, 128, 9, 2), (128, 128, 9, 2),
              (128, 128, 9, 3), (128, 128, 9, 3), (256, 128, 9, 2), (128, 128, 9, 2), (192, 64, 9, 1),
              (64, 64, 9, 1), (96, 32, 9, 0), (32, 32, 9, 0), (32, 16, 1, 0)]
    return sum(2.0 * t * ci * co / 4 ** lv for ci, co, t, lv in layers)


def stokes_gpu(mic, reps: int = 2, method: str = "fgmres", rtol: float = 1e-8, learned: bool = False,
               precision: str = "mixed", gs_relax: float = 0.0):
    """The Stokes step on the grids the context holds: build steps, solve to 1e-8, unpack.
    One warm-up (level set-up, graph capture), then `reps` timed steps (wall clock: the
    FGMRES loop is host-driven)."""
    import torch

    def one():
        mic.calc_viscoelastic_terms()
        mic.viscoelastic_rhs()
        mic.build_system_of_equations()
        rep = mic.solve_system(rtol=rtol, check=False, method=method, learned=learned, precision=precision,
                               gs_relax=gs_relax)
        mic.process_stokes_solution()
        return rep

    one()
    torch.cuda.synchronize()
    mic.profile_enable(True)
    t0 = time.perf_counter()
    reps_out = [one() for _ in range(reps)]
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    prof = mic.profile()
    mic.profile_enable(False)
    return dt, reps_out[-1], prof


def link_bandwidth(device: int, nbytes: int = 1 << 30) -> dict:
    """Host<->device copy rate of one large pinned buffer (best of 3, CUDA events), the
    denominator of the e2e copies."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{device}")
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = None
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) * 1e-3
            best = t if best is None else min(best, t)
        out[name] = round(nbytes / best / 1e9, 1)
    return out


def heat_gpu(mic, reps: int = 2):
    """The grid part of the heat step (HeatSolver.update_marker_temp_for_grid_and_subgrid_changes!
    up to dtk1): RHS terms, tk0 = tk1, the adaptive heat loop, dtk1 = tk2 - tk1.  One warm-up
    (level set-up, graph capture), then `reps` timed steps (wall clock: the loop is host-driven)."""
    import torch

    def one():
        mic.calculate_heat_rhs_terms()
        mic.initialize_old_temperature_array()
        rep = mic.run_conductive_heat_solver_loop()
        mic.calculate_grid_temp_change()
        return rep

    one()
    torch.cuda.synchronize()
    mic.profile_enable(True)
    t0 = time.perf_counter()
    reps_out = [one() for _ in range(reps)]
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    prof = mic.profile()
    mic.profile_enable(False)
    return dt, reps_out[-1], prof


def heat_cpu_sample(eb, oracle_mod, strip):
    """The oracle's heat step (assembly + scipy SuperLU standing in for UMFPACK/MUMPS) on the
    101x801 strip, inputs from the oracle's marker averages."""
    from oracle.heat import HeatOracle, HEAT_GRIDS
    ref = oracle_mod.OracleMIC(strip)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_heat_parameters_to_grid()
    ref.interpolate_marker_stokes_parameters_to_grid()
    ho = HeatOracle(strip, {k: ref.gr[k] for k in HEAT_GRIDS if k in ref.gr})
    t0 = time.perf_counter()
    ho.heat_step()
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/step", "cores": 1, "kind": "port",
            "sample": f"101x801-node strip, N={ho.N} unknowns, {ho.solves} solve(s): oracle assembly + scipy "
                      f"SuperLU per heat-loop pass"}


def stokes_cpu_sample(eb, oracle_mod):
    """SuperLU (scipy) on the oracle's assembly of the 101x801 strip, standing in for the
    reference's UMFPACK/MUMPS call; inputs are the oracle's marker averages."""
    from oracle.stokes import StokesOracle
    import scipy.sparse.linalg as spla
    model = eb.synthetic.rift(101, 801, 5, width=25e3)
    ref = oracle_mod.OracleMIC(model)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_stokes_parameters_to_grid()
    so = StokesOracle(model, {k: ref.gr[k] for k in STOKES_GRIDS if k in ref.gr})
    t0 = time.perf_counter()
    so.stokes_steps()
    K = so.matrix().tocsc()
    S = spla.spsolve(K, so.coo[3])
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/solve", "cores": 1, "kind": "port",
            "sample": f"101x801-node strip, N={so.N} unknowns: oracle assembly + scipy SuperLU "
                      f"(relative residual {so.residual(S):.1e})"}, model


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    eb = load_package()
    oracle = load_oracle()
    model = eb.synthetic.rift(101, 801, 5, width=25e3)
    ref = oracle.OracleMIC(model)
    for _ in range(args.warmup):
        ref.marker_cycle()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ref.marker_cycle()
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = model.marknum / dt
    sample = (f"{model.marknum} markers per step (101x801-node strip of the 2001x801, 25 markers/cell model, "
              f"same spacing); {dt:.3f} s per marker cycle")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "sample": "rift strip 101x801 nodes, 2.0M markers"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    eb = load_package()
    eb.build()
    t_gen = time.perf_counter()
    model = eb.synthetic.config(args.workload, seed=100 + rank)   # each replica its own seeded model
    t_gen = time.perf_counter() - t_gen
    mic = eb.MarkerInCell(local)
    mic.load_model(model)
    stream = torch.cuda.ExternalStream(mic.stream, device=local)
    M = model.marknum

    def step():
        mic.marker_cycle()

    for _ in range(max(args.warmup, 3)):
        step()
    if args.stokes_only:
        # one Stokes step (terms, RHS, assembly, mixed FGMRES + MG solve, unpacking), no warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mic.calc_viscoelastic_terms()
        mic.viscoelastic_rhs()
        mic.build_system_of_equations()
        rep = mic.solve_system(rtol=1e-8, check=True, method=args.stokes_method)
        mic.process_stokes_solution()
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"metric": "one Stokes step (profiling run)", "value": time.perf_counter() - t0,
                              "unit": "s", "workload": args.workload, "iterations": rep["iterations"],
                              "fp32_gram_schmidt_iterations": rep["relaxed_iterations"],
                              "rel_residual": rep["rel_residual"]}))
        mic.close()
        return
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = mic.launch_count
    mic.profile_enable(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    prof = mic.profile()
    mic.profile_enable(False)
    launches = mic.launch_count - launches0
    ms_t = torch.tensor([ms], device=f"cuda:{local}")
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = M * world / (ms * 1e-3)

    # dominant kernel: live per-kernel CUDA-event times on the library's stream
    kern = {k: (t / n, n) for k, (t, n) in prof.items()}
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = kern[dom]
    peak, peak_kind = peaks()
    bpm = algo_bytes_per_marker(dom, model)
    roofline = None
    if bpm is not None:
        achieved = bpm * M / (dom_ms * 1e-3) / 1e9
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                    "bytes_per_marker": bpm, "launch_ms": dom_ms}
        ncu_bpm = NCU_DRAM_BYTES_PER_MARKER.get(dom)
        if ncu_bpm is not None:
            roofline["traffic"] = ncu_bpm * M / 1e9
            roofline["traffic_unit"] = "GB per launch (ncu DRAM bytes per marker on 2.56M markers x markers)"

    # e2e: host buffers through the C-ABI, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        pinned_in = {k: torch.from_numpy(np.ascontiguousarray(model.markers[k])).pin_memory().numpy() for k in E2E_IN}
        pinned_out = {k: torch.empty(M, dtype={"f8": torch.float64, "f4": torch.float32}[
            eb._abi.MARKER_DTYPE[k]]).pin_memory().numpy() for k in E2E_OUT}
        h2d = sum(a.nbytes for a in pinned_in.values())
        d2h = sum(a.nbytes for a in pinned_out.values())
        reps = max(2, min(args.steps, 5))
        # one call per step with host arrays (eb_marker_cycle_host): the copies overlap the steps
        mic.marker_cycle_host(pinned_in, pinned_out)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            mic.marker_cycle_host(pinned_in, pinned_out)
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / reps
        # the same through the per-field upload/download calls and the eleven step calls
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            for k, a in pinned_in.items():
                mic.upload_marker(k, a)
            step()
            for k, a in pinned_out.items():
                mic._check(mic._lib.eb_marker_download(mic._ctx, eb._abi.MARKER_ID[k], a.ctypes.data))
        torch.cuda.synchronize()
        ts = (time.perf_counter() - t0) / reps
        link = link_bandwidth(local)
        e2e = {"value": M * world / te, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": te * 1e3, "call": "eb_marker_cycle_host (pinned host arrays in and out)",
               "link": link,
               "copy_bound_ms": round(max(h2d / link["h2d_gbs"], d2h / link["d2h_gbs"]) / 1e6, 2),
               "sequential": {"value": M * world / ts, "ms_per_step": ts * 1e3,
                              "call": "eb_marker_upload x20, 11 step calls, eb_marker_download x12"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(eb, load_oracle())
        except Exception as exc:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    # Stokes step of the same model: the marker cycle left the averaged grids on the device
    stokes = None
    if not args.no_stokes:
        alt = {}
        for meth in ("fgmres", "bicgstab"):
            if meth != args.stokes_method:
                a_dt, a_rep, _ = stokes_gpu(mic, reps=1, method=meth)
                alt[meth] = {"value": a_dt, "iterations": a_rep["iterations"], "status": a_rep["status"],
                             "rel_residual": a_rep["rel_residual"]}
        s_dt, s_rep, s_prof = stokes_gpu(mic, reps=2, method=args.stokes_method)
        s_kern = {k: (t / n, n) for k, (t, n) in s_prof.items()}
        stokes = {"metric": STOKES_METRIC, "value": s_dt, "unit": "s/solve", "higher_is_better": False,
                  "workload": f"{args.workload}: {model.grid.xnum}x{model.grid.ynum} nodes, "
                              f"N={3 * (model.grid.xnum - 1) * (model.grid.ynum - 1)} unknowns",
                  "includes": f"viscoelastic terms, RHS, assembly, {args.stokes_method}+MG solve, unpacking",
                  "method": args.stokes_method, "other_methods": alt,
                  "iterations": s_rep["iterations"], "levels": s_rep["levels"],
                  "rel_residual": s_rep["rel_residual"], "rel_residual_scaled": s_rep["rel_residual_scaled"],
                  "status": s_rep["status"], "solve_s": s_rep["seconds"],
                  "reorthogonalisations": s_rep["reorthogonalisations"],
                  "fp32_gram_schmidt_iterations": s_rep["relaxed_iterations"],
                  "kernels_ms": {k: round(v[0] * v[1], 3) for k, v in
                                 sorted(s_kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])[:12]}}
        # the plain method on the same system: FP64 V-cycle and FP64 stored directions
        p_dt, p_rep, _ = stokes_gpu(mic, reps=2, method=args.stokes_method, precision="fp64")
        stokes["plain_fp64"] = {"value": p_dt, "unit": "s/solve", "iterations": p_rep["iterations"],
                                "rel_residual": p_rep["rel_residual"], "status": p_rep["status"],
                                "mixed_speedup": p_dt / s_dt}
        # the mixed method with its Gram-Schmidt kept in FP64 throughout (gs_relax < 0)
        g_dt, g_rep, _ = stokes_gpu(mic, reps=2, method=args.stokes_method, gs_relax=-1.0)
        stokes["mixed_fp64_gram_schmidt"] = {"value": g_dt, "unit": "s/solve", "iterations": g_rep["iterations"],
                                             "rel_residual": g_rep["rel_residual"], "status": g_rep["status"]}
        # roofline of the Krylov-basis products (the solve's dominant kernels): per FGMRES
        # iteration k of a cycle, k_mdot reads the k+2 basis vectors and k_maxpy k+1 of them
        # plus the new direction (read and written); vectors are N doubles.  The last
        # `relaxed` iterations run the FP32 forms on N-float copies: k_mdot32 reads k+2 of
        # them, k_maxpy32 k+1 plus the FP64 direction (read, written) and its FP32 copy.
        n_unk = 3 * (model.grid.xnum - 1) * (model.grid.ynum - 1)
        its, m = s_rep["iterations"], 250
        ks = [k for c0 in range(0, its, m) for k in range(min(m, its - c0))] if args.stokes_method == "fgmres" else []
        n_rel = s_rep["relaxed_iterations"]
        ks64, ks32 = ks[:len(ks) - n_rel], ks[len(ks) - n_rel:]
        vbytes = n_unk * 8.0
        bytes_dot = sum(k + 2 for k in ks64) * vbytes
        bytes_axpy = sum(k + 3 for k in ks64) * vbytes
        bytes_dot32 = sum(k + 2 for k in ks32) * n_unk * 4.0
        bytes_axpy32 = sum((k + 1) * 4.0 + 20.0 for k in ks32) * n_unk
        peak, peak_kind = peaks()
        rl = {}
        nc_cells = n_unk // 3
        # operator product: 27 coefficients, x and the scaling w read, y written (FP64 per cell)
        bytes_apply = nc_cells * (27 + 3 + 3 + 3) * 8.0 * s_kern.get("k_apply64", (0, 0))[1] / 2
        for kname, b in (("k_mdot", bytes_dot), ("k_maxpy", bytes_axpy), ("k_mdot32", bytes_dot32),
                         ("k_maxpy32", bytes_axpy32), ("k_apply64", bytes_apply)):
            if kname in s_kern and b > 0:
                t = s_kern[kname][0] * s_kern[kname][1] / 2 * 1e-3  # seconds per solve (2 timed solves)
                rl[kname] = {"achieved": b / t / 1e9, "bytes_per_solve": b, "s_per_solve": t}
        if rl:
            dom_k = max(rl, key=lambda k: rl[k]["s_per_solve"])
            stokes["roofline"] = {"bound": "hbm", "kernel": dom_k, "achieved": rl[dom_k]["achieved"], "peak": peak,
                                  "unit": "GB/s", "frac": rl[dom_k]["achieved"] / peak, "peak_kind": peak_kind,
                                  "traffic": None, "kernels": rl}
        if rank == 0 and world == 1 and not args.no_cpu:
            try:
                s_cpu, strip = stokes_cpu_sample(eb, load_oracle())
                # the GPU on the same strip: marker averages from the GPU scatter, then the Stokes step
                smic = eb.MarkerInCell(local)
                smic.load_model(strip)
                smic.get_marker_inside_flags()
                smic.initialize_bilinear_interpolation()
                smic.interpolate_marker_stokes_parameters_to_grid()
                g_dt, g_rep, _ = stokes_gpu(smic, reps=2)
                smic.close()
                stokes["cpu_baseline"] = s_cpu
                stokes["gpu_same_sample"] = {"value": g_dt, "unit": "s/solve", "iterations": g_rep["iterations"],
                                             "rel_residual": g_rep["rel_residual"]}
            except Exception as exc:
                stokes["cpu_baseline"] = {"value": None, "sample": f"failed: {exc}"}

    # learned + MG against plain MG on the same system: the U-Net stage trained on the GPU on
    # patches of this system (its own forward, backward and Adam kernels), then the solve with
    # the stage after every V-cycle
    learned = None
    if stokes is not None and not args.no_learned:
        try:
            mic.learned_init(17)
            patch, batch = 512, 4
            tr = mic.learned_train(steps=args.learned_steps, batch=batch, patch=patch, patches_per_sample=4,
                                   lr=1e-3, seed=23)
            px = batch * tr["patch_h"] * tr["patch_w"]
            train_flops = 3.0 * unet_flops_per_pixel() * px * args.learned_steps
            mic.learned_stats()
            l_dt, l_rep, l_prof = stokes_gpu(mic, reps=2, method="fgmres", learned=True)
            st = mic.learned_stats()
            calls = st["accepted"] + st["rejected"]
            nc_cells = (model.grid.xnum - 1) * (model.grid.ynum - 1)
            infer_px = ((model.grid.xnum - 1 + 7) // 8 * 8) * ((model.grid.ynum - 1 + 7) // 8 * 8)
            l_kern = {k: (t / n, n) for k, (t, n) in l_prof.items()}
            gemm_ms = sum(v[0] * v[1] for k, v in l_kern.items() if k.startswith("k_gemm_bf16")) / 2
            infer_flops = unet_flops_per_pixel() * infer_px * calls / 3  # 3 solves counted (warm-up + 2)
            learned = {"metric": "Stokes s/solve @1e-8 resid, learned+MG", "value": l_dt, "unit": "s/solve",
                       "plain_mg_value": stokes["value"], "higher_is_better": False,
                       "iterations": l_rep["iterations"], "plain_mg_iterations": stokes["iterations"],
                       "rel_residual": l_rep["rel_residual"], "status": l_rep["status"],
                       "stage": {"kept": st["accepted"], "rejected": st["rejected"],
                                 "mean_removed_fraction": st["mean_removed"], "seconds_total": st["seconds"]},
                       "training": {**tr, "tflops": train_flops / tr["seconds"] / 1e12,
                                    "flops_per_step": train_flops / args.learned_steps},
                       "network": "BF16 U-Net 32-64-128-128, 1.1M parameters, FP32 accumulation (tcgen05)",
                       "inference": {"pixels": infer_px, "cells": nc_cells,
                                     "gemm_ms_per_solve": gemm_ms,
                                     "tensor_tflops": (infer_flops / (gemm_ms * 1e-3) / 1e12) if gemm_ms > 0 else None,
                                     "peak_bf16_tflops": peaks_bf16()},
                       "kernels_ms": {k: round(v[0] * v[1], 3) for k, v in
                                      sorted(l_kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])[:10]}}
        except Exception as exc:
            learned = {"value": None, "error": str(exc)}

    # the circles solver benchmark: 1025 x 1025 nodes, 200 inclusions (1e18-1e27 Pa s), to 1e-10
    stokes_circles = None
    if not args.no_stokes and args.circles:
        cm = eb.synthetic.config("circles_1025")
        cmic = eb.MarkerInCell(local)
        cmic.set_grid(cm.grid)
        cmic.set_params(cm.params)
        cmic.set_stokes_params(cm.params)
        for k, v in cm.grids.items():
            cmic.upload_grid(k, v)
        c_dt, c_rep, c_prof = stokes_gpu(cmic, reps=2, rtol=1e-10)
        cmic.close()
        c_kern = {k: (t / n, n) for k, (t, n) in c_prof.items()}
        stokes_circles = {"metric": "Stokes s/solve @1e-10 resid", "value": c_dt, "unit": "s/solve",
                          "higher_is_better": False,
                          "workload": "circles_1025: 1025x1025 nodes, N=3145728 unknowns, 200 circles, "
                                      "log10 eta U(18, 27), free slip",
                          "iterations": c_rep["iterations"], "levels": c_rep["levels"],
                          "rel_residual": c_rep["rel_residual"], "rel_residual_scaled": c_rep["rel_residual_scaled"],
                          "status": c_rep["status"],
                          "kernels_ms": {k: round(v[0] * v[1], 3) for k, v in
                                         sorted(c_kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])[:8]}}

    # heat step of the same model (grids from the marker cycle and the Stokes step)
    heat = None
    if not args.no_heat:
        h_dt, h_rep, h_prof = heat_gpu(mic, reps=2)
        h_kern = {k: (t / n, n) for k, (t, n) in h_prof.items()}
        n_nodes = model.grid.xnum * model.grid.ynum
        heat = {"metric": "heat s/step", "value": h_dt, "unit": "s/step", "higher_is_better": False,
                "workload": f"{args.workload}: {model.grid.xnum}x{model.grid.ynum} nodes, N={n_nodes} unknowns",
                "includes": "RHS terms, tk0 = tk1, adaptive heat loop (assembly, MG-CG solve to 1e-12, residuals), "
                            "dtk1",
                **{k: h_rep[k] for k in ("substeps", "solves", "iterations", "levels", "max_rel_residual")},
                "kernels_ms": {k: round(v[0] * v[1], 3) for k, v in
                               sorted(h_kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])[:10]}}
        # roofline of the FP64 operator product (d, cx, cy, x read; y written per internal node)
        if "k_heat_apply" in h_kern:
            t_apply, n_apply = h_kern["k_heat_apply"]
            nq = (model.grid.xnum - 2) * (model.grid.ynum - 2)
            peak, peak_kind = peaks()
            ach = nq * 5 * 8.0 / (t_apply * 1e-3) / 1e9
            heat["roofline"] = {"bound": "hbm", "kernel": "k_heat_apply", "achieved": ach, "peak": peak,
                                "unit": "GB/s", "frac": ach / peak, "peak_kind": peak_kind, "traffic": None,
                                "bytes_per_node": 40, "launch_ms": t_apply}
        if rank == 0 and world == 1 and not args.no_cpu:
            try:
                strip = eb.synthetic.rift(101, 801, 5, width=25e3)
                h_cpu = heat_cpu_sample(eb, load_oracle(), strip)
                smic = eb.MarkerInCell(local)
                smic.load_model(strip)
                smic.get_marker_inside_flags()
                smic.initialize_bilinear_interpolation()
                smic.interpolate_marker_heat_parameters_to_grid()
                smic.interpolate_marker_stokes_parameters_to_grid()
                g_dt, g_rep, _ = heat_gpu(smic, reps=2)
                smic.close()
                heat["cpu_baseline"] = h_cpu
                heat["gpu_same_sample"] = {"value": g_dt, "unit": "s/step", "solves": g_rep["solves"],
                                           "iterations": g_rep["iterations"]}
            except Exception as exc:
                heat["cpu_baseline"] = {"value": None, "sample": f"failed: {exc}"}

    # one whole time step, measured: marker cycle, Stokes step, heat step back to back
    timestep = None
    if not args.no_stokes and not args.no_heat:
        # two whole time steps; in each, the assembled Stokes system is also solved by the
        # plain FP64 method (outside the step's time) so both methods see the same systems
        import torch
        t_step = t_mixed = t_plain = 0.0
        its_m, its_p = [], []
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mic.update_marker_rheology_and_viscoplastic_viscosity(True)
            step()
            mic.calc_viscoelastic_terms()
            mic.viscoelastic_rhs()
            mic.build_system_of_equations()
            rep = mic.solve_system(rtol=1e-8, check=False, method=args.stokes_method)
            mic.process_stokes_solution()
            mic.calculate_heat_rhs_terms()
            mic.initialize_old_temperature_array()
            mic.run_conductive_heat_solver_loop()
            mic.calculate_grid_temp_change()
            torch.cuda.synchronize()
            t_step += time.perf_counter() - t0
            t_mixed += rep["seconds"]
            its_m.append(rep["iterations"])
            rep64 = mic.solve_system(rtol=1e-8, check=False, method=args.stokes_method, precision="fp64")
            t_plain += rep64["seconds"]
            its_p.append(rep64["iterations"])
        plain = (t_step - t_mixed + t_plain) / 2
        timestep = {"metric": "per-timestep wall time", "value": t_step / 2, "unit": "s/step",
                    "higher_is_better": False,
                    "includes": "marker rheology (failure, flow viscosity, viscoplastic, yield; one fused pass), "
                                "marker cycle (transfer + RK4), Stokes step (solve to 1e-8), heat step",
                    "stokes_solve_s": t_mixed / 2, "stokes_iterations": its_m,
                    "plain_fp64_mg_step": plain, "plain_fp64_solve_s": t_plain / 2, "plain_fp64_iterations": its_p,
                    "speedup_vs_plain_fp64": plain / (t_step / 2)}

    # the per-marker rheology of TimeLoop.jl:222-223 (failure properties, composite-creep
    # flow viscosity by bisection, viscoplastic viscosity, Drucker-Prager yielding) as one
    # fused pass, against the two reference calls
    rheology = None
    if not args.no_rheology:
        import torch
        for _ in range(2):
            mic.update_marker_rheology_and_viscoplastic_viscosity(True)
        torch.cuda.synchronize()
        mic.profile_enable(True)
        for _ in range(3):
            mic.update_marker_rheology_and_viscoplastic_viscosity(True)
        pf = mic.profile()
        for _ in range(3):
            mic.update_marker_rheology()
            mic.update_marker_viscoplastic_viscosity(True)
        pt = mic.profile()
        mic.profile_enable(False)
        t_f = pf["k_rheology"][0] / pf["k_rheology"][1]
        t_two = sum(pt[k][0] - pf.get(k, (0.0, 0))[0] for k in ("k_failure", "k_flow_viscosity", "k_viscoplastic",
                                                                "k_yield") if k in pt) / 3
        # reads inside, matid, strain_plastic, fric_ini, sxx, sxy, exx, exy, gii, pr, sr_ratio, tk,
        # pfailure; writes cohesion, fric, eta_flow, preexp, eta, pfailure (yielding markers also
        # rewrite sxx, sxy)
        bpm = 1 + 2 + 10 * 8 + 4 + 5 * 8 + 4
        peak, peak_kind = peaks()
        rheology = {"metric": "markers/s (rheology: failure, flow viscosity, viscoplastic, yield)",
                    "value": M / (t_f * 1e-3), "unit": "markers/s", "ms": t_f, "two_calls_ms": t_two,
                    "bytes_per_marker": bpm,
                    "roofline": {"bound": "fp64", "hbm_achieved": bpm * M / (t_f * 1e-3) / 1e9, "hbm_peak": peak,
                                 "hbm_frac": bpm * M / (t_f * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                                 "note": "FP64 arithmetic bound: up to 20 bisection steps of exp/pow per marker"}}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64 storage, f32 weights/sums", "data": "synthetic",
                "config": {"workload": args.workload, "markers": M, "xnum": model.grid.xnum, "ynum": model.grid.ynum,
                           "markers_per_cell": 25 if args.workload == "rift_40M" else None,
                           "l2": "inputs larger than L2 (each marker field 320 MB)", "parallelism": "replicas"},
                "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), "stokes": stokes, "stokes_learned": learned, "stokes_circles": stokes_circles,
                "heat": heat,
                "timestep": timestep, "rheology": rheology,
                "kernels_ms": {k: round(v[0], 4) for k, v in sorted(kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])},
                "generate_s": round(t_gen, 2)}
        print(json.dumps(line))
    mic.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
