"""Writes tests/golden/kaus10_oracle_9steps.npz, the oracle's record of the first nine time steps of
the Kaus (2010) plasticity benchmark (synthetic.plasticity_benchmark_kaus10: 401 x 101 basic
nodes, 40 x 12 km, 3 x 3 markers per cell, nodal Picard loop with up to 100 iterations) as
benchmark_cases.kaus10_oracle runs them (SuperLU for every Stokes solve).  The reference's
post-processing reads output 10, written before step 10's solve, so it sees the strain-rate
invariant of step 9.  Stored:
  iters                      Picard iterations of each step
  nnode_<s>                  yielding nodes of every Picard iteration of step s
  dips                       per step, the left, right and mean shear-zone dip (degrees) of
                             synthetic.kaus10_fault_dip
  lines                      after step 9, the strain-rate invariant sampled as the dip
                             measurement samples it: four vertical lines (left near, left far,
                             right near, right far) of ynum x 10 points
Run from the repository root (about fifteen minutes on eight cores):
    python tests/golden/make_kaus10_oracle.py
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

STEPS = 9
OUT = pathlib.Path(__file__).resolve().parent / "kaus10_oracle_9steps.npz"


def line_samples(syn, grid, eii, params) -> np.ndarray:
    """The strain-rate invariant on the four measurement lines of synthetic.kaus10_fault_dip."""
    xs, ys = syn.kaus10_measurement_lines(grid, params)
    return np.array([[syn.pressure_grid_value(grid, eii, x, y) for y in ys] for x in xs])


def main():
    from __graft_entry__ import load_oracle, load_package
    eb = load_package()
    load_oracle()
    import benchmark_cases as bc
    syn = eb.synthetic
    model = syn.plasticity_benchmark_kaus10()
    out, dips = {}, []

    def log(step, hist, timesum, eii):
        out[f"nnode_{step}"] = np.array([h["nnode_yield"] for h in hist], np.int64)
        r = syn.kaus10_fault_dip(model.grid, eii, model.params)
        dips.append((r["theta_left"], r["theta_right"], r["theta"]))
        print(f"step {step}: {len(hist)} Picard iterations, dip {r['theta']:.3f}", flush=True)
        if step == STEPS:
            out["lines"] = line_samples(syn, model.grid, eii, model.params)
    _, _, iters = bc.kaus10_oracle(eb, nsteps=STEPS, log=log)
    out["iters"] = np.array(iters, np.int64)
    out["dips"] = np.array(dips)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
