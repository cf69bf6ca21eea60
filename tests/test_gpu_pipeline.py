"""eb_marker_cycle_host (one marker cycle from host arrays, copies overlapped with the
steps) against the same cycle run entry point by entry point: identical results, since
the same kernels run on the same data; bad inputs rejected before any step runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IN = ["x", "y", "matid", "rho", "cohesion", "fric", "eta", "eta_flow", "sxx", "sxy", "pfailure", "dilatation",
      "meltfrac", "tk", "kt", "rhocp", "ha", "serp_hr", "gii", "strain_plastic"]
OUT = ["x", "y", "sxx", "sxy", "tk", "exx", "exy", "pr", "sr_ratio", "gii", "strain_plastic", "strain_rate_plastic",
       "xn", "yn", "inside", "subgrid_dt", "eta"]


@pytest.mark.parametrize("name", ["rift_small", "sinking_block"])
def test_cycle_from_host_matches_entry_points(eb, name):
    model = eb.synthetic.config(name)
    ref = eb.MarkerInCell(0)
    ref.load_model(model)
    ref.marker_cycle()
    want = {k: ref.download_marker(k) for k in OUT}
    ref.close()
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    # the context starts from different marker values: the call must replace them
    mic.upload_marker("tk", np.zeros(model.marknum))
    dt = eb._abi.MARKER_DTYPE
    inputs = {k: np.ascontiguousarray(model.markers[k], dtype=dt[k]) for k in IN}
    outputs = {k: np.zeros(model.marknum, dtype=dt[k]) for k in OUT}
    mic.marker_cycle_host(inputs, outputs)
    for k in OUT:
        assert np.array_equal(outputs[k], want[k]), k
    # a second call from the outputs continues the evolution like a second cycle
    mic.close()


def test_cycle_from_host_rejects_bad_matid(eb):
    model = eb.synthetic.config("rift_small")
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    bad = model.markers["matid"].astype(np.int16).copy()
    bad[7] = 0
    x0 = mic.download_marker("x")
    with pytest.raises(RuntimeError):
        mic.marker_cycle_host({"x": model.markers["x"], "matid": bad}, {"x": np.zeros(model.marknum)})
    # no step ran: a valid call afterwards works
    mic.marker_cycle_host({"matid": model.markers["matid"].astype(np.int16)}, {"x": np.zeros(model.marknum)})
    assert x0.shape == (model.marknum,)
    mic.close()


@pytest.mark.parametrize("name", ["rift_small", "sinking_block"])
def test_fused_tail_matches_the_four_calls(eb, name):
    """eb_correct_advect_and_update_strain against stress correction, remaining temperature
    change, advection and strain update called one by one: identical marker fields."""
    model = eb.synthetic.config(name)
    outs = []
    for fused in (False, True):
        mic = eb.MarkerInCell(0)
        mic.load_model(model)
        mic.marker_cycle(fused=fused)
        outs.append({k: mic.download_marker(k) for k in ("x", "y", "sxx", "sxy", "tk", "gii", "strain_plastic",
                                                         "strain_rate_plastic", "vx", "vy", "spin")})
        mic.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("plasticity", [True, False])
def test_fused_rheology_equals_the_two_calls(eb, plasticity):
    """eb_update_marker_rheology_and_viscoplastic_viscosity gives, bit for bit, what
    eb_update_marker_rheology followed by eb_update_marker_viscoplastic_viscosity gives."""
    model = eb.synthetic.config("rift_small")
    out = {}
    for fused in (False, True):
        mic = eb.MarkerInCell(0)
        mic.load_model(model)
        mic.marker_cycle()
        if fused:
            mic.update_marker_rheology_and_viscoplastic_viscosity(plasticity)
        else:
            mic.update_marker_rheology()
            mic.update_marker_viscoplastic_viscosity(plasticity)
        out[fused] = {k: mic.download_marker(k) for k in ("cohesion", "fric", "eta_flow", "preexp", "eta", "sxx",
                                                          "sxy", "pfailure")}
        mic.close()
    for k in out[False]:
        assert np.array_equal(out[False][k], out[True][k]), k
    if plasticity:
        assert np.any(out[True]["pfailure"] == 1.0)


def _on_lines(eb):
    """sinking_block with markers exactly on basic and staggered grid lines (two or four exclusive
    quadrants at once), on the domain edges and outside it."""
    model = eb.synthetic.config("sinking_block")
    g = model.grid
    rng = np.random.default_rng(11)
    xs = np.concatenate([g.gridx_b, g.gridx_vy[1:-1], np.nextafter(g.gridx_b, np.inf)[:-1]])
    ys = np.concatenate([g.gridy_b, g.gridy_vx[1:-1], np.nextafter(g.gridy_b, np.inf)[:-1]])
    n = model.marknum
    x, y = model.markers["x"].copy(), model.markers["y"].copy()
    pick = rng.random(n) < 0.3
    x[pick] = rng.choice(xs, int(pick.sum()))
    y[pick] = rng.choice(ys, int(pick.sum()))
    x[:4] = [g.xmin, g.xmax, g.xmin - 1.0, g.xmax + 1e-9]
    y[:4] = [g.ymin, g.ymax, g.ymax, g.ymin]
    model.markers["x"], model.markers["y"] = x, y
    return model


@pytest.mark.parametrize("name", ["rift_small", "sinking_block", "on_lines"])
def test_bilinear_setup_and_heat_scatter_equal_the_two_calls(eb, name):
    """eb_initialize_bilinear_interpolation_and_heat_scatter (denominators summed in the heat
    fold) gives, bit for bit, what eb_initialize_bilinear_interpolation followed by
    eb_interpolate_marker_heat_parameters_to_grid gives: cell indices, the four weight sums and
    the heat transport arrays with their backups."""
    model = _on_lines(eb) if name == "on_lines" else eb.synthetic.config(name)
    grids = ("wtnodes", "wtetas", "wtetan", "wtnodes_vy", "tk1", "kt1", "rhocp1", "hr1", "ha1",
             "tk0", "kt0", "rhocp0", "hr0", "ha0")
    out = {}
    for fused in (False, True):
        mic = eb.MarkerInCell(0)
        mic.load_model(model)
        mic.get_marker_inside_flags()
        if fused:
            mic.initialize_bilinear_interpolation_and_heat_scatter()
        else:
            mic.initialize_bilinear_interpolation()
            mic.interpolate_marker_heat_parameters_to_grid()
        out[fused] = {k: mic.download_grid(k) for k in grids}
        out[fused].update({k: mic.download_marker(k) for k in ("xn", "yn", "inside")})
        mic.close()
    for k in out[False]:
        assert np.array_equal(out[False][k], out[True][k]), k
    assert np.any(out[True]["wtetas"] != out[True]["wtnodes"])  # exclusive and inclusive sums differ
    if name == "on_lines":
        assert np.any(out[True]["inside"] != 1)  # some markers outside the domain
