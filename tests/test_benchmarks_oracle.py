"""The reference's heat-path benchmarks through the oracle.

Solid-body rotation (src/benchmarks/models/solid_body_rotation, post_processing/analytical/
SolidBodyRotationManager.jl): one rotation of a hot square in a kinematic velocity field, the
grid temperature profile of row 11 back on its initial profile within the reference's 2 % limit.

Couette viscous heating (src/benchmarks/models/couette_flow_viscous_heating): a shear zone with a
temperature-dependent viscosity heating itself, against the steady analytic profile."""
from benchmark_cases import rotation_check, solid_body_rotation_oracle


def test_oracle_solid_body_rotation_returns_the_temperature_wave(eb):
    model, t0, t1 = solid_body_rotation_oracle(eb)
    assert t0.max() > 1400.0  # the profile crosses the hot square
    err = rotation_check(model, t0, t1)
    assert err < 0.02, err


def test_oracle_couette_flow_matches_the_steady_viscous_heating_profile(eb):
    """The reference's Couette viscous-heating benchmark (models/couette_flow_viscous_heating,
    CouetteFlowViscousHeatingManager.jl): after 99 steps (output 100) the temperature across the
    shear zone within the reference's 0.3 % of the steady analytic profile."""
    from benchmark_cases import couette_error, couette_oracle
    model, row = couette_oracle(eb)
    assert row[-1] > row[0] + 100.0  # the shear zone heated up
    err = couette_error(eb, model, row)
    assert err < 0.003, err
