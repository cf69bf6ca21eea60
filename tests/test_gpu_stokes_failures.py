"""Failure handling of the Stokes solve, injected on the host (no GPU fault is involved).

The reference's solve path retries and then raises (ParallelSolver.jl:75-123, the MUMPS retry
loop; SolverConfig.jl:20-77 for the configuration).  Here the solve entry point returns a status
instead and never traps:
  * a NaN in the right-hand side returns EB_NAN before any iteration, and the context stays
    usable for the next solve;
  * the mixed method falls back to the plain FP64 method whenever its FP64 residual fails to
    fall; an iteration limit that the mixed method cannot meet hands the solve to the plain
    method, which then either finishes it (EB_OK, precision_used "fp64") or reports
    EB_NOT_CONVERGED itself;
  * a learned stage that returns garbage (NaN parameters) is rejected at every application,
    and the solve still meets the tolerance with the multigrid alone.
"""
import numpy as np
import pytest

from stokes_cases import marker_model
from test_gpu_stokes import gpu_ctx

pytestmark = pytest.mark.gpu

EB_OK, EB_NOT_CONVERGED, EB_NAN = 0, 1, 2


def built(eb, case="rift_small"):
    mic = gpu_ctx(eb, marker_model(eb, case))
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    return mic


def test_nan_rhs_returns_eb_nan_and_context_recovers(eb):
    mic = built(eb)
    R = mic.download_stokes_vector("rhs")
    bad = R.copy()
    bad[17] = np.nan
    mic.upload_stokes_vector("rhs", bad)
    rep = mic.solve_system(rtol=1e-8, check=False)
    assert rep["status"] == EB_NAN, rep
    assert rep["fallback_used"] == 0  # no method can repair a NaN input
    mic.upload_stokes_vector("rhs", R)
    rep = mic.solve_system(rtol=1e-8, check=False)
    assert rep["status"] == EB_OK and rep["rel_residual"] <= 1e-8, rep
    mic.close()


def test_iteration_limit_hands_over_to_the_plain_method(eb):
    mic = built(eb)
    rep = mic.solve_system(rtol=1e-8, max_iters=1, check=False)
    assert rep["status"] == EB_NOT_CONVERGED, rep
    assert rep["fallback_used"] == 1 and rep["precision_used"] == "fp64", rep
    assert rep["iterations"] == 2, rep  # one mixed, then one plain iteration
    off = mic.solve_system(rtol=1e-8, max_iters=1, check=False, fallback=False)
    assert off["status"] == EB_NOT_CONVERGED and off["fallback_used"] == 0 and off["iterations"] == 1, off
    mic.close()


@pytest.mark.parametrize("case", ["rift_small", "sinking_block"])
def test_fallback_finishes_a_solve_the_mixed_method_cannot(eb, case):
    mic = built(eb, case)
    full = mic.solve_system(rtol=1e-10, fallback=False)
    n = full["iterations"]
    assert n > 8
    # the largest budget (in steps of 4) that the mixed method alone does not meet
    budget = next(k for k in range(n - 4, 0, -4)
                  if mic.solve_system(rtol=1e-10, max_iters=k, check=False, fallback=False)["status"]
                  == EB_NOT_CONVERGED)
    rep = mic.solve_system(rtol=1e-10, max_iters=budget, check=False)
    assert rep["status"] == EB_OK, rep
    assert rep["fallback_used"] == 1 and rep["precision_used"] == "fp64", rep
    assert rep["rel_residual"] <= 1e-10 and rep["iterations"] > budget, rep
    S = mic.download_stokes_vector("solution")
    mic.solve_system(rtol=1e-10, precision="fp64")
    S64 = mic.download_stokes_vector("solution")
    for comp in range(3):
        a, b = S[comp::3], S64[comp::3]
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max(), comp
    mic.close()


def test_garbage_learned_stage_is_rejected(eb):
    from test_gpu_learned import stokes_system
    mic = stokes_system(eb)
    mic.learned_init(2)
    mic.learned_train(steps=4, batch=1, patch=32, patches_per_sample=4, lr=1e-3, seed=3)
    p = mic.learned_params()
    mic.learned_params(np.full_like(p, np.nan))
    mic.learned_stats()
    rep = mic.solve_system(rtol=1e-8, learned=True, check=False)
    st = mic.learned_stats()
    assert rep["status"] == EB_OK and rep["rel_residual"] <= 1e-8, rep
    assert st["accepted"] == 0 and st["rejected"] == rep["iterations"], st
    mic.close()
