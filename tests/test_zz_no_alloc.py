"""The allocation-free entry point, called through the C-ABI, against the CPU oracle.

eb_marker_to_basic_grid_average_noalloc is for callers that cannot call
cudaMalloc (their device memory comes from someone else's allocator, or
allocating is not allowed where they run).  It takes device pointers for all
inputs and outputs and works in a fixed 16 MiB static device array, which
keeps the previous call's contents.  Each case hands it device buffers and
compares the density average and the weight sums with the oracle's inclusive
average (BilinearNumerator + BilinearAverage: rho1, wtnodes), within the parity
tolerance (1e-6 relative); nodes without markers must keep the caller's value.
Cases: two calls in a row on the sinking block; markers outside the grid, on
grid lines and on the domain edges, a cell holding 40 % of all markers, and a
band of empty cells; a call with no markers; a smaller grid and fewer markers
after a larger call.  The context entry point is checked against the same
average as well.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _entry(eb):
    from earthbox_gb300 import _abi
    lib = _abi.load()
    fn = lib.eb_marker_to_basic_grid_average_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    fn.restype = C.c_int
    return fn


def oracle_average(oracle, model):
    """The oracle's inclusive density average and weight sums (empty nodes keep model rho1)."""
    ref = oracle.OracleMIC(model)
    ref.get_marker_inside_flags()
    ref.initialize_bilinear_interpolation()
    ref.interpolate_marker_stokes_parameters_to_grid()
    return ref.gr["rho1"], ref.gr["wtnodes"]


def noalloc_average(eb, model, avg0=None, marknum=None):
    import torch
    fn = _entry(eb)
    dev = torch.device("cuda:0")
    n = model.marknum if marknum is None else marknum
    x = torch.tensor(model.markers["x"][:max(n, 1)], device=dev)
    y = torch.tensor(model.markers["y"][:max(n, 1)], device=dev)
    rho = torch.tensor(model.markers["rho"][:max(n, 1)], device=dev)
    gx = torch.tensor(model.grid.gridx_b, device=dev)
    gy = torch.tensor(model.grid.gridy_b, device=dev)
    X, Y = model.grid.xnum, model.grid.ynum
    start = model.grids["rho1"] if avg0 is None else avg0
    avg = torch.tensor(np.asfortranarray(start).ravel(order="F"), device=dev)
    wsum = torch.full((X * Y,), -1.0, dtype=torch.float64, device=dev)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev)
    rc = fn(x.data_ptr(), y.data_ptr(), rho.data_ptr(), n, gx.data_ptr(), X, gy.data_ptr(), Y, avg.data_ptr(),
            wsum.data_ptr(), C.c_void_p(stream.cuda_stream), err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return avg.cpu().numpy().reshape((Y, X), order="F"), wsum.cpu().numpy().reshape((Y, X), order="F")


def assert_matches(got, want, what):
    g, w = got
    a, b = want
    assert np.array_equal(w == 0, b == 0), f"{what}: empty nodes differ"
    assert np.all(np.abs(w - b) <= RTOL * np.abs(b)), f"{what}: weight sums differ"
    assert np.all(np.abs(g - a) <= RTOL * np.abs(a)), f"{what}: density average differs"


def edge_case_model(eb):
    """Sinking-block markers moved onto grid lines, staggered lines and the domain edges, some
    outside the grid, 40 % of them into one cell, and none left in a band of cells (x in
    (150, 200) km), whose inner nodes then keep the caller's value."""
    model = eb.synthetic.config("sinking_block")
    g = model.grid
    rng = np.random.default_rng(7)
    n = model.marknum
    x, y = model.markers["x"].copy(), model.markers["y"].copy()
    k = n // 5
    xs = np.concatenate([g.gridx_b, g.gridx_vy[1:-1], np.nextafter(g.gridx_b, -np.inf)[1:],
                         np.nextafter(g.gridx_b, np.inf)[:-1]])
    ys = np.concatenate([g.gridy_b, g.gridy_vx[1:-1], np.nextafter(g.gridy_b, np.inf)[:-1]])
    x[:k], y[:k] = rng.choice(xs, k), rng.choice(ys, k)
    x[:6] = [g.xmin, g.xmax, g.xmin, g.xmax, g.xmin - 1.0, g.xmax + 1e-9]
    y[:6] = [g.ymin, g.ymax, g.ymax, g.ymin, g.ymin, g.ymax]
    cl = slice(k, k + int(0.4 * n))
    m = cl.stop - cl.start
    x[cl] = g.gridx_b[10] + rng.random(m) * (g.gridx_b[11] - g.gridx_b[10])
    y[cl] = g.gridy_b[20] + rng.random(m) * (g.gridy_b[21] - g.gridy_b[20])
    band = (x > 150e3) & (x < 200e3)
    x[band] = -1e9
    model.markers["x"], model.markers["y"] = x, y
    return model


def test_noalloc_average_two_calls_in_a_row(eb, oracle):
    eb.build()
    model = eb.synthetic.config("sinking_block")
    want = oracle_average(oracle, model)
    for call in range(2):
        assert_matches(noalloc_average(eb, model), want, f"call {call}")
    # the context entry point computes the same average
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_stokes_parameters_to_grid()
    assert_matches((mic.download_grid("rho1"), mic.download_grid("wtnodes")), want, "context entry point")
    mic.close()


def test_noalloc_edges_outside_markers_clusters_and_empty_nodes(eb, oracle):
    eb.build()
    model = edge_case_model(eb)
    rng = np.random.default_rng(3)
    avg0 = np.asfortranarray(3000.0 + 100.0 * rng.random(model.grids["rho1"].shape))
    model.grids["rho1"] = avg0
    got = noalloc_average(eb, model, avg0)
    want = oracle_average(oracle, model)
    assert_matches(got, want, "edge cases")
    empty = want[1] == 0
    assert empty.sum() >= 100
    assert np.array_equal(got[0][empty], avg0[empty])  # empty nodes keep the caller's value


def test_noalloc_no_markers_then_a_smaller_call_after_a_larger_one(eb, oracle):
    eb.build()
    big = eb.synthetic.config("sinking_block")
    assert_matches(noalloc_average(eb, big), oracle_average(oracle, big), "large call")
    avg, wsum = noalloc_average(eb, big, marknum=0)
    assert np.all(wsum == 0) and np.array_equal(avg, big.grids["rho1"])
    small = eb.synthetic.sinking_block(xnum=41, ynum=31, mpc=3, seed=9)
    assert_matches(noalloc_average(eb, small), oracle_average(oracle, small), "smaller call")
    assert_matches(noalloc_average(eb, big), oracle_average(oracle, big), "large call again")


def test_noalloc_rejects_sizes_beyond_its_limit(eb):
    eb.build()
    fn = _entry(eb)
    err = C.create_string_buffer(256)
    rc = fn(None, None, None, 1 << 20, None, 3, None, 3, None, None, None, err, len(err))
    assert rc == 3 and b"524288" in err.value
    rc = fn(None, None, None, 0, None, 1001, None, 1001, None, None, None, err, len(err))
    assert rc == 3 and b"131072" in err.value
