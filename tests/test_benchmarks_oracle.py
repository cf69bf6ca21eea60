"""The reference's heat-path benchmarks through the oracle.

Solid-body rotation (src/benchmarks/models/solid_body_rotation, post_processing/analytical/
SolidBodyRotationManager.jl): three rotations of a hot square in a kinematic velocity field, the
grid temperature profile of row 11 back on its initial profile after each within the reference's
2 % limit.

Couette viscous heating (src/benchmarks/models/couette_flow_viscous_heating): a shear zone with a
temperature-dependent viscosity heating itself, against the steady analytic profile.

Variable-conductivity channel (src/benchmarks/models/channel_flow_variable_conductivity):
shear-heated Poiseuille flow with a temperature-dependent conductivity, against the steady
analytic profile.

Non-steady channel temperature (src/benchmarks/models/channel_flow_non_steady_temperature):
advection of a vertical temperature gradient by Poiseuille flow with conduction to the walls,
against the transient analytic profile at every output.

Kaus (2010) plasticity (src/benchmarks/models/plasticity_benchmark_kaus10): the first two steps
of the nodal Picard loop against the oracle's own nine-step record, which the GPU test reads."""
from benchmark_cases import rotation_check, solid_body_rotation_oracle


def test_oracle_solid_body_rotation_returns_the_temperature_wave(eb):
    """Outputs 91, 181 and 271 (one, two and three rotations) against output 1."""
    model, rows = solid_body_rotation_oracle(eb)
    assert rows[1].max() > 1400.0  # the profile crosses the hot square
    for step in (91, 181, 271):
        err = rotation_check(model, rows[1], rows[step])
        assert err < 0.02, (step, err)


def test_oracle_couette_flow_matches_the_steady_viscous_heating_profile(eb):
    """The reference's Couette viscous-heating benchmark (models/couette_flow_viscous_heating,
    CouetteFlowViscousHeatingManager.jl): after 99 steps (output 100) the temperature across the
    shear zone within the reference's 0.3 % of the steady analytic profile."""
    from benchmark_cases import couette_error, couette_oracle
    model, row = couette_oracle(eb)
    assert row[-1] > row[0] + 100.0  # the shear zone heated up
    err = couette_error(eb, model, row)
    assert err < 0.003, err


def test_oracle_variable_conductivity_channel_matches_the_steady_profile(eb):
    """The reference's variable-conductivity channel benchmark
    (models/channel_flow_variable_conductivity, ChannelFlowVariableConductivityManager.jl):
    after 495 steps (output 100) the shear-heated temperature across the channel within the
    reference's 2.2 % (Celsius) of the steady analytic profile."""
    from benchmark_cases import vcond_error, vcond_oracle
    model, row = vcond_oracle(eb)
    assert row.max() > 1000.0  # the channel centre heated from 298 K
    err = vcond_error(eb, model, row)
    assert err < 0.022, err


def test_oracle_non_steady_channel_temperature_follows_the_transient_solution(eb):
    """The reference's non-steady channel-temperature benchmark
    (models/channel_flow_non_steady_temperature, ChannelFlowNonSteadyTemperatureManager.jl):
    every output from 1 to 240 (one per 5 steps) within the reference's 0.7 % (Celsius) of the
    transient analytic profile."""
    from benchmark_cases import nst_error, nst_oracle
    model, rows = nst_oracle(eb)
    assert rows[240][1].min() < 1000.0  # the channel cooled from its initial 1227 C
    for out, (tmyr, row) in rows.items():
        err = nst_error(eb, model, row, tmyr)
        assert err < 0.007, (out, tmyr, err)


def test_oracle_kaus10_first_steps_reproduce_its_record(eb):
    """The Kaus (2010) benchmark's first two steps through the oracle (about ten seconds) give the
    Picard iterations and yielding-node counts recorded in tests/golden/kaus10_oracle_9steps.npz,
    the record the GPU test compares its nine steps against."""
    import pathlib

    import numpy as np

    from benchmark_cases import kaus10_oracle
    g = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "kaus10_oracle_9steps.npz")
    counts = []
    _, eii, iters = kaus10_oracle(eb, nsteps=2, log=lambda s, h, t, e: counts.append([r["nnode_yield"] for r in h]))
    assert iters == g["iters"][:2].tolist()
    for s, c in enumerate(counts, start=1):
        assert c == g[f"nnode_{s}"].tolist(), (s, c)
    assert np.all(np.isfinite(eii)) and eii.max() > 0.0
