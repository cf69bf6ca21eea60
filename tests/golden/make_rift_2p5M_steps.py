"""Writes tests/golden/rift_2p5M_5steps.npz, the oracle's record of five hot-path time steps of the
2.56M-marker rift (801 x 201 basic nodes, 500 x 160 km, 16 markers per cell; the three-layer
lithosphere under 10 km of sticky air, cohesion 10 MPa, friction 30 -> 15 degrees by strain 1).

Each step is OraclePicard.time_step (TimeLoop.run_loop!'s body restricted to the hot path) with the
marker-based Picard loop (nglobal 5, tolerance 1e-3) and SuperLU for every Stokes solve.  Stored:
  picard_dvxy_<s>            dvxy_rel_L2 of every Picard iteration of step s
  vmax                       max |v| of the step's velocity grids
  vx1_<s>, vy1_<s>           the velocity grids, every 8th node in each direction
  sample                     4096 seeded marker indices
  <field>_<s>                the sampled markers' values after step s (inside, xn, yn, x, y, sxx,
                             sxy, eta, pfailure, exx, exy, pr, gii, strain_plastic)
  sum_<field>, abssum_<field>  per step, the sum and the sum of magnitudes of a field over the
                             markers inside the grid (all markers, not only the sample)
Run from the repository root (about five minutes on eight cores):
    python tests/golden/make_rift_2p5M_steps.py
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

STEPS, NGLOBAL, TOL = 5, 5, 1e-3
SAMPLED = ("inside", "xn", "yn", "x", "y", "sxx", "sxy", "eta", "pfailure", "exx", "exy", "pr", "gii",
           "strain_plastic")
SUMMED = ("x", "y", "sxx", "sxy", "eta", "exx", "exy", "pr", "gii", "strain_plastic", "pfailure")
OUT = pathlib.Path(__file__).resolve().parent / "rift_2p5M_5steps.npz"


def main():
    from __graft_entry__ import load_oracle, load_package
    eb = load_package()
    load_oracle()
    from oracle.picard import OraclePicard
    model = eb.synthetic.config("rift_2p5M")
    op = OraclePicard(model)
    sample = np.sort(np.random.Generator(np.random.Philox(77)).choice(model.marknum, 4096, replace=False))
    rec = {"sample": sample, "vmax": np.zeros(STEPS)}
    for f in SUMMED:
        rec[f"sum_{f}"] = np.zeros(STEPS)
        rec[f"abssum_{f}"] = np.zeros(STEPS)
    for s in range(STEPS):
        hist = op.time_step(NGLOBAL, TOL)["picard"]
        rec[f"picard_dvxy_{s}"] = np.array([h["dvxy_rel_L2"] for h in hist])
        mk = op.mic.mk
        inside = mk["inside"] == 1
        rec["vmax"][s] = max(np.abs(op.gr["vx1"]).max(), np.abs(op.gr["vy1"]).max())
        rec[f"vx1_{s}"] = np.asfortranarray(op.gr["vx1"][::8, ::8])
        rec[f"vy1_{s}"] = np.asfortranarray(op.gr["vy1"][::8, ::8])
        for f in SAMPLED:
            rec[f"{f}_{s}"] = mk[f][sample].copy()
        for f in SUMMED:
            v = mk[f][inside].astype(np.float64)
            rec[f"sum_{f}"][s] = v.sum()
            rec[f"abssum_{f}"][s] = np.abs(v).sum()
        print(f"step {s}: {len(hist)} Picard iterations, dvxy {rec[f'picard_dvxy_{s}']}", flush=True)
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
