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
against the transient analytic profile at every output."""
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
