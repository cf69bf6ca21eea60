"""The reference's own analytic benchmarks through the GPU path.

Rayleigh-Taylor instability (Ramberg 1968), as the reference runs and checks it
(src/benchmarks/models/rayleigh_taylor_instability, post_processing/analytical/
RayleighTaylorInstabilityManager.jl): markers of two layers with a sinusoidal interface are
averaged to the grid, the Stokes system is assembled and solved, the velocity is moved to the
basic nodes, and its vertical component at the interface crest (x = xsize/2, y = h1 - A,
bilinear on the basic grid) must agree with Ramberg's analytic crest velocity within the
reference's relative error limit of 3.5 %."""
import pytest

from stokes_cases import bilinear_basic

pytestmark = pytest.mark.gpu

RELATIVE_ERROR_LIMIT = 0.035


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_rayleigh_taylor_crest_velocity_matches_ramberg(eb, precision):
    syn = eb.synthetic
    model = syn.rayleigh_taylor()
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_stokes_parameters_to_grid()
    rep = mic.solve_viscoelastic_stokes_continuity_equations(rtol=1e-10, precision=precision)
    assert rep["status"] == 0, rep
    mic.interpolate_stag_velocity_to_basic_grid()
    vyb = mic.download_grid("vyb")
    g = model.grid
    W = g.xmax - g.xmin
    h1, amp, lam = 1500.0, 10.0, 4000.0
    v_num = bilinear_basic(g, vyb, W / 2.0, h1 - amp)
    v_ana = syn.ramberg_wave_velocity(h1, (g.ymax - g.ymin) - h1, 3000.0, 2900.0, 1e13, 1e19, amp, lam)
    err = abs(v_num - v_ana) / abs(v_ana)
    print(f"\nRayleigh-Taylor crest velocity ({precision}): GPU {v_num:.5e} m/s, Ramberg {v_ana:.5e} m/s, "
          f"relative error {100 * err:.2f} % (limit {100 * RELATIVE_ERROR_LIMIT:.1f} %)")
    assert err < RELATIVE_ERROR_LIMIT, (v_num, v_ana, err)
    mic.close()
