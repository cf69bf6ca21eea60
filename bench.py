"""Benchmark of the marker-in-cell hot path on one GB300 (markers/s, MIC transfer + RK4).

A step is one marker cycle of the 40M-marker rifting model (2001x801 basic nodes, 25 markers per
cell): inside flags, cell location and the cell-sorted marker list, heat and Stokes marker->grid
averaging, post-Stokes marker gathers, subgrid stress and temperature diffusion, the stress and
temperature corrections, fused RK4 advection with stress rotation, and the strain update.  Every
marker field is larger than L2 (40M x 8 B = 320 MB), so no L2 flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

Prints one JSON line.  ``value`` is markers/s with the model resident in HBM; ``e2e`` is the same
metric through the C-ABI with host buffers (each step uploads the marker state from pinned host
memory and downloads the updated state).  Further legs, each on a freshly loaded model so that no
leg depends on --steps or on the legs before it:
  rheology   the fused per-marker rheology pass (failure, flow viscosity, yield) at 40M markers;
  stokes     the Stokes step of the 40M model: mixed method, plain FP64 method and the learned
             stage, s/solve to 1e-8 with every solution's error against an FP64 solve to 1e-12;
  timestep   whole hot-path time steps of the 40M model (rheology, averages, Picard loop with
             Stokes solves, post-Stokes steps, heat step, advection), mixed against plain FP64;
  config2    five time steps of the 2.56M-marker rift (Picard loop), mixed against plain FP64;
  heat       the heat step of the 40M model.
``--impl reference`` times the oracle (the reference's algorithms restated in C: OpenMP on the loops
the reference threads, serial marker->grid loops as in the reference) on the same 40M model.
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

# Bytes per marker each kernel must move (reads + writes of marker arrays); the dominant-kernel
# roofline uses these.
ALGO_BYTES_PER_MARKER = {
    "k_cells<stokes>": 4 + 4 + 8 + 1 + 4 + 8 * 8 + 4 + 4,   # perm, xn, fx/fy, flags, matid, 8 f64, 2 f32
    "k_cells<heat>": 4 + 8 + 1 + 4 + 5 * 8,
    "k_cells<denominators>": 4 + 4 + 8 + 1,
    "k_cells<heat+denominators>": 4 + 4 + 8 + 1 + 4 + 5 * 8,
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
# reads inside, matid, strain_plastic, fric_ini, sxx, sxy, exx, exy, gii, pr, sr_ratio, tk, pfailure;
# writes cohesion, fric, eta_flow, preexp, eta, pfailure
RHEOLOGY_BYTES_PER_MARKER = 1 + 2 + 10 * 8 + 4 + 5 * 8 + 4

# DRAM bytes per marker (dram__bytes_read.sum + dram__bytes_write.sum) from one `ncu --set full`
# capture of each kernel on the 2.56M-marker rift (801x201 nodes, 16 markers per cell); reads
# scale with the marker count, writes that still sit in L2 at that size make these a lower bound.
NCU_DRAM_BYTES_PER_MARKER = {
    "k_cells<stokes>": 101.2,
    "k_cells<subgrid_stress>": 57.3,
    "k_advect": 83.1,
    "k_post_stokes": 44.5,
    "k_tail": 167.9,
}


def algo_bytes_per_marker(kernel: str, model) -> float | None:
    """Algorithmic bytes per marker of `kernel` on this workload."""
    bpm = ALGO_BYTES_PER_MARKER.get(kernel)
    if bpm is not None and kernel == "k_tail":
        bpm += TAIL_PLASTIC_BYTES * float(np.mean(model.markers["pfailure"] == 1.0))
    return bpm


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
    ap.add_argument("--no-timestep", action="store_true")
    ap.add_argument("--no-config2", action="store_true")
    ap.add_argument("--timesteps", type=int, default=3, help="time steps of the 40M timestep leg per method")
    ap.add_argument("--learned-steps", type=int, default=200)
    ap.add_argument("--circles", action="store_true",
                    help="give the circles_1025 Stokes leg (200 inclusions, 1e-10) the full iteration budget "
                         "and the fallback (default: 1500 iterations)")
    ap.add_argument("--no-circles", action="store_true")
    ap.add_argument("--rheology-only", action="store_true",
                    help="run one time step of the workload, then three fused rheology passes, and print their "
                         "time (a small case for ncu; not the bench line)")
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


def r3(v):
    """Three significant digits (keeps the JSON line short)."""
    if v is None or isinstance(v, (bool, str)):
        return v
    if isinstance(v, (list, tuple)):
        return [r3(x) for x in v]
    if isinstance(v, dict):
        return {k: r3(x) for k, x in v.items()}
    if isinstance(v, (int, np.integer)):
        return int(v)
    v = float(v)
    return float(f"{v:.3g}") if np.isfinite(v) else None


class _Nvml:
    """Read-only NVML queries through ctypes: SM clock, its maximum and the active clock-event
    reasons of one device.  Nothing here changes a setting."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit_v2 failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise OSError("nvmlDeviceGetHandleByIndex_v2 failed")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        c = self.c
        clk, mx, rs = c.c_uint(), c.c_uint(), c.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, c.byref(clk)) != 0:
            return None
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, self.SM, c.byref(mx))
        self.reasons_fn(self.h, c.byref(rs))
        return float(clk.value), float(mx.value), {nm for bit, nm in self.REASONS.items() if rs.value & bit}


class Clocks:
    """SM clock and throttle-reason samples taken during the timed region: NVML polled every
    10 ms from a host thread (the timed regions last a fraction of a second), else nvidia-smi at
    its 200 ms period."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.thread = None
        self.samples = []
        self.source = None

    def __enter__(self):
        import threading
        try:
            nv = _Nvml(self.index)
            self.stop = threading.Event()

            def poll():
                while True:
                    s = nv.sample()
                    if s is not None:
                        self.samples.append(s)
                    if self.stop.wait(0.01):
                        break
            self.source = "nvml"
            self.thread = threading.Thread(target=poll, daemon=True)
            self.thread.start()
            return self
        except (OSError, AttributeError):
            pass
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi"
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.thread is not None:
            self.stop.set()
            self.thread.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for ln in out.splitlines():
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) < 7:
                    continue
                try:
                    sm, mx = float(parts[0]), float(parts[1])
                except ValueError:
                    continue
                self.samples.append((sm, mx, {nm for nm, v in zip(names, parts[3:7])
                                              if v.lower().startswith("active")}))

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        reasons = set().union(*(r for _, _, r in self.samples))
        return {"sm_mhz": float(np.median([s for s, _, _ in self.samples])), "sm_max_mhz": self.samples[-1][1],
                "sm_min_mhz": min(s for s, _, _ in self.samples), "reasons": sorted(reasons),
                "samples": len(self.samples), "source": self.source}


E2E_IN = ["x", "y", "matid", "rho", "cohesion", "fric", "eta", "eta_flow", "sxx", "sxy", "pfailure", "dilatation",
          "meltfrac", "tk", "kt", "rhocp", "ha", "serp_hr", "gii", "strain_plastic"]
E2E_OUT = ["x", "y", "sxx", "sxy", "tk", "exx", "exy", "pr", "sr_ratio", "gii", "strain_plastic",
           "strain_rate_plastic"]


def oracle_marker_cycles(oracle, model, warmup: int, steps: int) -> float:
    """Seconds per marker cycle of the oracle on `model` (OpenMP where the reference threads)."""
    ref = oracle.OracleMIC(model)
    for _ in range(warmup):
        ref.marker_cycle()
    t0 = time.perf_counter()
    for _ in range(steps):
        ref.marker_cycle()
    return (time.perf_counter() - t0) / max(steps, 1)


def cpu_baseline(oracle, model, steps: int = 2):
    """The reference's algorithms (C restatement, OpenMP where the reference threads) on the same
    40M-marker model: `steps` marker cycles after one warm-up."""
    dt = oracle_marker_cycles(oracle, model, 1, steps)
    return {"value": model.marknum / dt, "unit": UNIT, "cores": oracle.threads(), "kind": "port",
            "sample": f"{model.marknum} markers (the whole {model.grid.xnum}x{model.grid.ynum} model), {steps} "
                      f"marker cycles after one warm-up; {dt:.2f} s per cycle"}


def unet_flops_per_pixel() -> float:
    """Forward FLOPs of the learned stage's U-Net per full-resolution pixel (2 per multiply-add
    of each convolution, pixels of level l = 1 / 4^l of the full resolution)."""
    layers = [(8, 32, 9, 0), (32, 32, 9, 0), (32, 64, 9, 1), (64, 64, 9, 1), (64, 128, 9, 2), (128, 128, 9, 2),
              (128, 128, 9, 3), (128, 128, 9, 3), (256, 128, 9, 2), (128, 128, 9, 2), (192, 64, 9, 1),
              (64, 64, 9, 1), (96, 32, 9, 0), (32, 32, 9, 0), (32, 16, 1, 0)]
    return sum(2.0 * t * ci * co / 4 ** lv for ci, co, t, lv in layers)


def link_bandwidth(device: int, nbytes: int = 1 << 30) -> dict:
    """Host<->device copy rate of one large pinned buffer (best of 3, CUDA events)."""
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


def fresh_context(eb, model, local):
    mic = eb.MarkerInCell(local)
    mic.load_model(model)
    return mic


def stokes_state(eb, model, local):
    """A fresh context holding the model's first Stokes system: inside flags, locate, rheology
    (one fused pass), heat and Stokes averages, viscoelastic terms, RHS and assembly."""
    mic = fresh_context(eb, model, local)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_heat_parameters_to_grid()
    mic.update_marker_rheology_and_viscoplastic_viscosity(True)
    mic.interpolate_marker_stokes_parameters_to_grid()
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    return mic


def solution_error(S, S_ref) -> dict:
    """max |S - S_ref| per unknown kind, relative to max |S_ref| of that kind."""
    out = {}
    for k, name in enumerate(("vx", "vy", "p")):
        a, b = S[k::3], S_ref[k::3]
        out[name] = float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
    return out


def timed_solves(mic, reps: int, S_ref=None, **kw):
    """`reps` solves of the context's assembled system from zero (one untimed warm-up: level
    set-up, graph capture); wall seconds per solve, last report and the solution's error."""
    import torch
    mic.solve_system(rtol=1e-8, check=False, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        rep = mic.solve_system(rtol=1e-8, check=False, **kw)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    err = solution_error(mic.download_stokes_vector("solution"), S_ref) if S_ref is not None else None
    return dt, rep, err


def stokes_leg(eb, model, local, args, rank, world):
    """The Stokes solve of the 40M model's first system: mixed, plain FP64 and (optionally)
    learned+mixed, each against an FP64 solve of the same system to 1e-12."""
    import torch
    mic = stokes_state(eb, model, local)
    n_unk = mic.stokes_size
    ref = mic.solve_system(rtol=1e-12, precision="fp64", check=False)
    S_ref = mic.download_stokes_vector("solution")
    mic.profile_enable(True)
    m_dt, m_rep, m_err = timed_solves(mic, 2, S_ref)
    prof = mic.profile()
    mic.profile_enable(False)
    p_dt, p_rep, p_err = timed_solves(mic, 2, S_ref, precision="fp64")
    out = {"metric": "Stokes s/solve @1e-8 resid", "unit": "s/solve", "higher_is_better": False,
           "workload": f"{args.workload} first system: {model.grid.xnum}x{model.grid.ynum} nodes, N={n_unk}",
           "reference_solve": {"rtol": 1e-12, "rel_residual": ref["rel_residual"], "iterations": ref["iterations"]},
           "mixed": {"value": m_dt, "iterations": m_rep["iterations"], "rel_residual": m_rep["rel_residual"],
                     "status": m_rep["status"], "fallback_used": m_rep["fallback_used"],
                     "fp32_gram_schmidt_iterations": m_rep["relaxed_iterations"], "error_vs_fp64": m_err},
           "plain_fp64": {"value": p_dt, "iterations": p_rep["iterations"], "rel_residual": p_rep["rel_residual"],
                          "status": p_rep["status"], "error_vs_fp64": p_err},
           "mixed_speedup": p_dt / m_dt}
    # Krylov-basis product roofline of the mixed solve (its HBM-bound kernels)
    kern = {k: (t / n, n) for k, (t, n) in prof.items()}
    its, m = m_rep["iterations"], 500   # FGMRES restart length (the solver default)
    ks = [k for c0 in range(0, its, m) for k in range(min(m, its - c0))]
    n_rel = m_rep["relaxed_iterations"]
    ks64, ks32 = ks[:len(ks) - n_rel], ks[len(ks) - n_rel:]
    rl = {}
    # the mixed method's Arnoldi step: double-float pairs (8 bytes per element and vector); below
    # the FP32 threshold the products read the FP32 hi parts; k_apply64 remains for the
    # residuals of each cycle
    nc = n_unk // 3
    n_df = kern.get("k_apply_df", (0, 0))[1] / 3
    for kname, b in (("k_mdot_df", sum(k + 2 for k in ks64) * n_unk * 8.0),
                     ("k_maxpy_df", sum((k + 1) * 8.0 + 16.0 for k in ks64) * n_unk),
                     ("k_mdot32", sum(k + 2 for k in ks32) * n_unk * 4.0),
                     ("k_maxpy32", sum((k + 1) * 4.0 + 16.0 for k in ks32) * n_unk),
                     ("k_apply_df", nc * (27 * 8.0 + 12 + 24 + 24) * n_df),
                     ("k_apply64", nc * 36 * 8.0 * kern.get("k_apply64", (0, 0))[1] / 3)):
        if kname in kern and b > 0:
            t = kern[kname][0] * kern[kname][1] / 3 * 1e-3   # 3 mixed solves were profiled
            rl[kname] = {"GBps": b / t / 1e9, "ms_per_solve": t * 1e3}
    peak, peak_kind = peaks()
    if rl:
        dom = max(rl, key=lambda k: rl[k]["ms_per_solve"])
        out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": rl[dom]["GBps"], "peak": peak, "unit": "GB/s",
                           "frac": rl[dom]["GBps"] / peak, "peak_kind": peak_kind,
                           "kernels": {k: {"GBps": v["GBps"], "ms": v["ms_per_solve"]} for k, v in rl.items()}}
    vc = prof.get("vcycle_graph") or prof.get("vcycle")
    if vc:
        out["mixed"]["vcycle_ms_per_solve"] = vc[0] / 3
    # the learned stage, trained on the GPU on this system (own forward/backward/Adam kernels)
    if not args.no_learned:
        try:
            mic.learned_init(17)
            tr = mic.learned_train(steps=args.learned_steps, batch=4, patch=512, patches_per_sample=4, lr=1e-3,
                                   seed=23)
            px = 4 * tr["patch_h"] * tr["patch_w"]
            train_flops = 3.0 * unet_flops_per_pixel() * px * args.learned_steps
            mic.learned_stats()
            l_dt, l_rep, l_err = timed_solves(mic, 2, S_ref, learned=True)
            st = mic.learned_stats()
            out["learned"] = {"value": l_dt, "iterations": l_rep["iterations"], "rel_residual": l_rep["rel_residual"],
                              "error_vs_fp64": l_err, "stage_kept": st["accepted"], "stage_rejected": st["rejected"],
                              "mean_removed_fraction": st["mean_removed"],
                              "training_s": tr["seconds"], "training_tflops": train_flops / tr["seconds"] / 1e12,
                              "peak_bf16_tflops": peaks_bf16()}
        except Exception as exc:  # reported, not required
            out["learned"] = {"value": None, "error": str(exc)[:200]}
    mic.close()
    torch.cuda.synchronize()
    return out


def run_time_steps(eb, model, local, nsteps: int, precision: str, heat: bool, nglobal: int = 5,
                   learned_steps: int = 0):
    """`nsteps` hot-path time steps (MarkerInCell.time_step, every solve warm-started) of a fresh
    context, wall-timed.  With learned_steps > 0 the learned stage is first trained (untimed) on the
    model's first Stokes system and then used inside FGMRES and as the warm start of every solve."""
    import torch
    mic = fresh_context(eb, model, local) if not learned_steps else stokes_state(eb, model, local)
    extra, train = {}, None
    if learned_steps:
        mic.learned_init(17)
        train = mic.learned_train(steps=learned_steps, batch=4, patch=512, patches_per_sample=4, lr=1e-3, seed=23)
        extra = {"learned": True, "learned_warm": True}
        mic.learned_stats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    recs = []
    for _ in range(nsteps):
        recs.append(mic.time_step(nglobal, 1e-3, heat=heat, rtol=1e-8, precision=precision, check=False, **extra))
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / nsteps
    st = mic.learned_stats() if learned_steps else None
    mic.close()
    pic = [r["picard"] for r in recs]
    if learned_steps:
        return {"s_per_step": dt, "picard_iterations": [len(p) for p in pic],
                "fgmres_iterations": [[h["iterations"] for h in p] for p in pic],
                "solve_s": sum(h["seconds"] for p in pic for h in p) / nsteps,
                "status_ok": all(h["status"] == 0 for p in pic for h in p),
                "training_s": train["seconds"], "stage_kept": st["accepted"], "stage_rejected": st["rejected"]}
    return {"s_per_step": dt, "picard_iterations": [len(p) for p in pic],
            "fgmres_iterations": [[h["iterations"] for h in p] for p in pic],
            "solve_s": sum(h["seconds"] for p in pic for h in p) / nsteps,
            "fallbacks": sum(h["fallback_used"] for p in pic for h in p),
            "worst_rel_residual": max(h["rel_residual"] for p in pic for h in p),
            "status_ok": all(h["status"] == 0 for p in pic for h in p)}


def timestep_leg(eb, model, local, nsteps: int, heat: bool, workload: str, learned_steps: int = 0):
    """Whole hot-path time steps, the mixed method against the plain FP64 method, each on a
    freshly loaded copy of the model (one untimed warm-up step per method first)."""
    out = {"metric": "per-timestep wall time", "unit": "s/step", "higher_is_better": False, "workload": workload,
           "steps": nsteps,
           "includes": "rheology (one fused pass), marker->grid averages, Picard loop (nglobal 5, tol 1e-3) of "
                       "warm-started Stokes solves to 1e-8, post-Stokes grid/marker steps, subgrid stress"
                       + (", heat step" if heat else "") + ", RK4 advection, strain"}
    for prec in ("mixed", "fp64"):   # the context keeps its own copy of the model: `model` is not changed
        run_time_steps(eb, model, local, 1, prec, heat)          # warm-up (set-up, graph capture)
        out["mixed" if prec == "mixed" else "plain_fp64"] = run_time_steps(eb, model, local, nsteps, prec, heat)
    out["speedup_vs_plain_fp64"] = out["plain_fp64"]["s_per_step"] / out["mixed"]["s_per_step"]
    if learned_steps:
        try:
            ml = run_time_steps(eb, model, local, nsteps, "mixed", heat, learned_steps=learned_steps)
            ml["speedup_vs_plain_fp64"] = out["plain_fp64"]["s_per_step"] / ml["s_per_step"]
            out["mixed_learned"] = ml
        except Exception as exc:  # reported, not required
            out["mixed_learned"] = {"s_per_step": None, "error": str(exc)[:200]}
    return out


def heat_leg(eb, model, local):
    """The grid part of the heat step on the 40M model's averages: RHS terms, tk0 = tk1, the adaptive
    heat loop, dtk1.  One warm-up (set-up, graph capture), then two timed steps."""
    import torch
    mic = fresh_context(eb, model, local)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_heat_parameters_to_grid()
    mic.interpolate_marker_stokes_parameters_to_grid()

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
    for _ in range(2):
        rep = one()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / 2
    prof = mic.profile()
    mic.close()
    out = {"metric": "heat s/step", "value": dt, "unit": "s/step", "higher_is_better": False,
           **{k: rep[k] for k in ("substeps", "solves", "iterations", "max_rel_residual")}}
    if "k_heat_apply" in prof:
        t_apply = prof["k_heat_apply"][0] / prof["k_heat_apply"][1]
        nq = (model.grid.xnum - 2) * (model.grid.ynum - 2)
        peak, peak_kind = peaks()
        ach = nq * 5 * 8.0 / (t_apply * 1e-3) / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": "k_heat_apply", "achieved": ach, "peak": peak, "unit": "GB/s",
                           "frac": ach / peak, "peak_kind": peak_kind}
    return out


def rheology_leg(mic, model):
    """The fused rheology pass (TimeLoop.jl:222-223 as one marker pass) against the two calls."""
    import torch
    M = model.marknum
    for _ in range(2):
        mic.update_marker_rheology_and_viscoplastic_viscosity(True)
    torch.cuda.synchronize()
    mic.profile_enable(True)
    for _ in range(3):
        mic.update_marker_rheology_and_viscoplastic_viscosity(True)
    pf = mic.profile()
    mic.profile_enable(False)
    name = max((k for k in pf if k.startswith("k_rheology")), key=lambda k: pf[k][0])
    t_f = sum(v[0] for k, v in pf.items() if k.startswith("k_rheology")) / 3
    peak, peak_kind = peaks()
    ach = RHEOLOGY_BYTES_PER_MARKER * M / (t_f * 1e-3) / 1e9
    return {"metric": "markers/s (rheology: failure, flow viscosity, viscoplastic, yield)", "value": M / (t_f * 1e-3),
            "unit": "markers/s", "ms": t_f, "kernel": name, "bytes_per_marker": RHEOLOGY_BYTES_PER_MARKER,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "frac": ach / peak, "peak_kind": peak_kind}}


def stokes_cpu_baseline(eb, oracle_mod):
    """scipy's SuperLU (one core) on the oracle's assembly of the 2.56M-marker rift's first system
    (N = 480k), standing in for the reference's UMFPACK/MUMPS call, with the GPU on the same system."""
    from oracle.stokes import StokesOracle
    import scipy.sparse.linalg as spla
    model = eb.synthetic.config("rift_2p5M")
    ref = oracle_mod.OracleMIC(model)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_heat_parameters_to_grid()
    ref.update_marker_rheology()
    ref.update_marker_viscoplastic_viscosity(True)
    ref.interpolate_marker_stokes_parameters_to_grid()
    so = StokesOracle(model, dict(ref.gr))
    t0 = time.perf_counter()
    so.stokes_steps()
    S = spla.spsolve(so.matrix().tocsc(), so.coo[3])
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/solve", "cores": 1, "kind": "port",
            "sample": f"rift_2p5M first system, N={so.N}: oracle assembly + scipy SuperLU "
                      f"(relative residual {so.residual(S):.1e})"}, model


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    eb = load_package()
    oracle = load_oracle()
    model = eb.synthetic.config(args.workload)
    dt = oracle_marker_cycles(oracle, model, args.warmup, args.steps)
    value = model.marknum / dt
    sample = (f"{model.marknum} markers per step (the whole {model.grid.xnum}x{model.grid.ynum} model, "
              f"25 markers per cell); {dt:.2f} s per marker cycle")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "markers": model.marknum, "xnum": model.grid.xnum,
                       "ynum": model.grid.ynum},
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
    mic = fresh_context(eb, model, local)
    stream = torch.cuda.ExternalStream(mic.stream, device=local)
    M = model.marknum

    def step():
        mic.marker_cycle()

    if args.rheology_only:
        # markers with the strain rates and pressures of a real solution, then the fused pass
        mic.time_step(3, 1e-3, rtol=1e-8)
        torch.cuda.synchronize()
        mic.profile_enable(True)
        for _ in range(3):
            mic.update_marker_rheology_and_viscoplastic_viscosity(True)
        pr = mic.profile()
        if rank == 0:
            ms = pr["k_rheology"][0] / pr["k_rheology"][1]
            print(json.dumps({"metric": "fused rheology pass (profiling run)", "value": ms, "unit": "ms",
                              "workload": args.workload, "markers": M}))
        mic.close()
        return
    for _ in range(max(args.warmup, 3)):
        step()
    if args.stokes_only:
        # one Stokes step (terms, RHS, assembly, mixed FGMRES + MG solve, unpacking), no warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mic.calc_viscoelastic_terms()
        mic.viscoelastic_rhs()
        mic.build_system_of_equations()
        rep = mic.solve_system(rtol=1e-8, check=True)
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
    dom_ms = kern[dom][0]
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
    cycle_gbs = sum(algo_bytes_per_marker(k, model) * M * n for k, (t, n) in prof.items()
                    if algo_bytes_per_marker(k, model) is not None) / args.steps / (ms * 1e-3) / 1e9

    # e2e: host buffers through the C-ABI, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        pinned_in = {k: torch.from_numpy(np.ascontiguousarray(model.markers[k])).pin_memory().numpy() for k in E2E_IN}
        pinned_out = {k: torch.empty(M, dtype={"f8": torch.float64, "f4": torch.float32}[
            eb._abi.MARKER_DTYPE[k]]).pin_memory().numpy() for k in E2E_OUT}
        h2d = sum(a.nbytes for a in pinned_in.values())
        d2h = sum(a.nbytes for a in pinned_out.values())
        reps = max(2, min(args.steps, 5))
        mic.marker_cycle_host(pinned_in, pinned_out)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            mic.marker_cycle_host(pinned_in, pinned_out)
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / reps
        link = link_bandwidth(local)
        e2e = {"value": M * world / te, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": te * 1e3, "call": "eb_marker_cycle_host (pinned host arrays in and out)",
               "link_gbs": link, "copy_bound_ms": round(max(h2d / link["h2d_gbs"], d2h / link["d2h_gbs"]) / 1e6, 2)}

    rheology = None if args.no_rheology else rheology_leg(mic, model)
    mic.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(load_oracle(), model)
        except Exception as exc:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    stokes = None
    if not args.no_stokes:
        stokes = stokes_leg(eb, model, local, args, rank, world)
        if rank == 0 and world == 1 and not args.no_cpu:
            try:
                s_cpu, m2 = stokes_cpu_baseline(eb, load_oracle())
                smic = stokes_state(eb, m2, local)
                g_dt, g_rep, _ = timed_solves(smic, 2)
                smic.close()
                stokes["cpu_baseline"] = s_cpu
                stokes["gpu_same_system"] = {"value": g_dt, "unit": "s/solve", "iterations": g_rep["iterations"]}
            except Exception as exc:
                stokes["cpu_baseline"] = {"value": None, "sample": f"failed: {str(exc)[:200]}"}

    timestep = None
    if not args.no_stokes and not args.no_timestep:
        timestep = timestep_leg(eb, model, local, args.timesteps, heat=not args.no_heat,
                                workload=f"{args.workload} (time steps 1-{args.timesteps} from the initial state)",
                                learned_steps=0 if args.no_learned else args.learned_steps)
    config2 = None
    if not args.no_stokes and not args.no_config2:
        m2 = eb.synthetic.config("rift_2p5M", seed=100 + rank)
        config2 = timestep_leg(eb, m2, local, 5, heat=False,
                               workload="rift_2p5M: 801x201 nodes, 2.56M markers, 5 time steps")

    heat = None if args.no_heat else heat_leg(eb, model, local)

    # the circles box at 1025^2 (200 inclusions, contrasts up to 1e9): the velocity multigrid
    # stalls there, so the default leg is bounded (1500 FGMRES iterations, no fallback) and
    # reports the residual reached; --circles gives it the full budget and the fallback
    circles = None
    if not args.no_stokes and not args.no_circles:
        cm = eb.synthetic.config("circles_1025")
        cmic = eb.MarkerInCell(local)
        cmic.set_grid(cm.grid)
        cmic.set_params(cm.params)
        cmic.set_stokes_params(cm.params)
        for k, v in cm.grids.items():
            cmic.upload_grid(k, v)
        cmic.calc_viscoelastic_terms()
        cmic.viscoelastic_rhs()
        cmic.build_system_of_equations()
        t0 = time.perf_counter()
        kw = {} if args.circles else {"max_iters": 1500, "fallback": False}
        c_rep = cmic.solve_system(rtol=1e-10, check=False, **kw)
        cmic.close()
        circles = {"metric": "Stokes s/solve @1e-10 resid", "value": time.perf_counter() - t0, "unit": "s/solve",
                   "workload": "circles_1025: 1025x1025 nodes, 200 circles, log10 eta U(18, 27), free slip",
                   "budget": "full (3000 iterations, fallback)" if args.circles else "1500 iterations, no fallback",
                   "converged": c_rep["status"] == 0,
                   **{k: c_rep[k] for k in ("iterations", "rel_residual", "status", "fallback_used")}}

    if rank == 0:
        top = sorted(kern.items(), key=lambda kv: -kv[1][0] * kv[1][1])[:8]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64 storage, f32 weights/sums", "data": "synthetic",
                "config": {"workload": args.workload, "markers": M, "xnum": model.grid.xnum, "ynum": model.grid.ynum,
                           "markers_per_cell": 25 if args.workload == "rift_40M" else None,
                           "l2": (f"inputs larger than L2 (each marker field {M * 8 / 1e6:.0f} MB)" if M * 8 > 129e6
                                  else f"marker fields ({M * 8 / 1e6:.0f} MB each) fit in L2: a profiling case"),
                           "parallelism": "replicas"},
                "gpu_launches": launches, "roofline": r3(roofline), "cycle_GBps": r3(cycle_gbs),
                "cpu_baseline": cpu, "e2e": r3(e2e), "clocks": clk.summary(),
                "kernels_ms": {k: r3(v[0]) for k, v in top},
                "rheology": r3(rheology), "stokes": r3(stokes), "timestep": r3(timestep), "config2": r3(config2),
                "heat": r3(heat), "circles": r3(circles), "generate_s": round(t_gen, 1)}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
