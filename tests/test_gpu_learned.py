"""The learned preconditioner stage on the GPU, through the C-ABI:
  * forward pass and the gradient of every parameter against the numpy oracle with the same
    BF16 rounding points (oracle/unet.py; its own backward is pinned by finite differences).
    The tensor cores sum in FP32 where the oracle sums in FP64; a rounding that lands on the
    other side of a BF16 step changes one stored value by 2^-8 relative and can flip a ReLU
    mask downstream.  Bounds: 1e-2 relative on the outputs and the loss; for each layer's
    gradient, half of what BF16 storage itself moves it (oracle with against oracle without
    BF16 rounding: 1-19 % here, deepest layers largest) plus 1 %;
  * training on the GPU lowers the loss, and FGMRES with the stage still meets the Stokes
    tolerance (the stage's corrections are kept only where they lower the preconditioner
    residual); the test prints what the stage gains or loses in iterations and time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_params(mic, rng):
    from oracle import unet
    p = mic.learned_params()
    for _, ws, bs in unet.layer_slices():
        p[bs] = rng.normal(0.0, 0.05, bs.stop - bs.start)
    return mic.learned_params(p)


def test_forward_and_gradients_match_oracle(eb):
    from oracle import unet
    rng = np.random.default_rng(11)
    mic = eb.MarkerInCell(0)
    mic.learned_init(7)
    params = random_params(mic, rng)
    x = rng.normal(size=(2, 16, 24, 8)).astype(np.float32)
    t = rng.normal(size=(2, 16, 24, 3)).astype(np.float32)
    y = mic.learned_forward(x)
    net = unet.UNet(params, bf16=True)
    yo = net.forward(x)
    assert np.max(np.abs(y - yo)) <= 1e-2 * np.max(np.abs(yo))
    loss, g = mic.learned_loss_grad(x, t)
    lo, go = net.loss_grad(x, t)
    _, g64 = unet.UNet(params, bf16=False).loss_grad(x, t)
    assert abs(loss - lo) <= 1e-2 * abs(lo)
    for name, ws, bs in unet.layer_slices():
        for sl in (ws, bs):
            ref = go[sl]
            if np.linalg.norm(ref) == 0:
                assert np.linalg.norm(g[sl]) == 0, name
                continue
            noise = np.linalg.norm(go[sl] - g64[sl])
            err = np.linalg.norm(g[sl] - ref)
            assert err <= 0.5 * noise + 1e-2 * np.linalg.norm(ref), (name, sl, err / np.linalg.norm(ref),
                                                                     noise / np.linalg.norm(ref))
    mic.close()


def stokes_system(eb, name="rift_small"):
    model = eb.synthetic.config(name)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.marker_cycle()
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    return mic


def test_learned_stage_requires_training(eb):
    mic = stokes_system(eb)
    rep = mic.solve_system(rtol=1e-8, learned=True, check=False)
    assert rep["status"] == 5  # EB_NOT_READY
    mic.close()


def test_training_lowers_loss_and_solve_still_converges(eb):
    mic = stokes_system(eb)
    plain = mic.solve_system(rtol=1e-8)
    mic.learned_init(1)
    rep = mic.learned_train(steps=60, batch=2, patch=32, patches_per_sample=4, lr=1e-3, seed=5)
    assert rep["loss_last"] < rep["loss_first"], rep
    st = mic.learned_state()
    assert st[5] == 1.0 and st[4] > 0
    learned = mic.solve_system(rtol=1e-8, learned=True)
    stats = mic.learned_stats()
    assert learned["rel_residual"] <= 1e-8
    assert stats["accepted"] + stats["rejected"] == learned["iterations"]
    print(f"\nlearned stage on rift_small: FGMRES {plain['iterations']} -> {learned['iterations']} iterations, "
          f"{plain['seconds']:.3f} -> {learned['seconds']:.3f} s, corrections kept {stats['accepted']} of "
          f"{stats['accepted'] + stats['rejected']}; training {rep}")
    mic.close()


def test_learned_warm_start_of_a_picard_iteration(eb):
    """The learned stage as a Picard warm start: the second Picard iteration's solve starts from the
    first one's solution, corrected by the network where that lowers the residual (the stage's own
    step and acceptance test).  The solve must meet the tolerance either way; the test records the
    iterations with and without the corrected start (on this model the network gains nothing)."""
    mic = stokes_system(eb)
    mic.learned_init(4)
    mic.learned_train(steps=40, batch=2, patch=32, patches_per_sample=4, lr=1e-3, seed=9)
    mic.solve_system(rtol=1e-8)
    S1 = mic.download_stokes_vector("solution")
    # the second Picard iteration's system: markers re-yielded, viscosity re-averaged
    mic.backup_and_clear_viscosity_transport_arrays()
    mic.update_plastic_yielding()
    mic.interpolate_viscosity_to_transport_arrays()
    mic.interpolate_basic_viscoplastic_viscosity_to_pressure_grid(1)
    mic.calc_viscoelastic_terms()
    mic.viscoelastic_rhs()
    mic.build_system_of_equations()
    out = {}
    for warm in (False, True):
        mic.upload_stokes_vector("solution", S1)
        mic.learned_stats()
        rep = mic.solve_system(rtol=1e-8, use_initial_guess=True, learned=True, learned_warm=warm)
        st = mic.learned_stats()
        assert rep["status"] == 0 and rep["rel_residual"] <= 1e-8, rep
        assert st["accepted"] + st["rejected"] == rep["iterations"] + (1 if warm else 0), (st, rep)
        out[warm] = rep["iterations"]
    cold = mic.solve_system(rtol=1e-8, learned=True)["iterations"]
    print(f"\nsecond Picard solve: {cold} iterations cold, {out[False]} from the previous solution, "
          f"{out[True]} from the previous solution corrected by the network")
    mic.close()
