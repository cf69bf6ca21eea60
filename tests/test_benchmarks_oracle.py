"""The reference's solid-body-rotation benchmark (src/benchmarks/models/solid_body_rotation,
post_processing/analytical/SolidBodyRotationManager.jl) through the oracle: one rotation of a
hot square in a kinematic velocity field, the grid temperature profile of row 11 back on its
initial profile within the reference's 2 % limit."""
from benchmark_cases import rotation_check, solid_body_rotation_oracle


def test_oracle_solid_body_rotation_returns_the_temperature_wave(eb):
    model, t0, t1 = solid_body_rotation_oracle(eb)
    assert t0.max() > 1400.0  # the profile crosses the hot square
    err = rotation_check(model, t0, t1)
    assert err < 0.02, err
