"""The allocation-free entry point, called through the C-ABI, against the context entry point.

eb_marker_to_basic_grid_average_noalloc is for callers that cannot call
cudaMalloc (their device memory comes from someone else's allocator, or
allocating is not allowed where they run).  It takes device pointers for all
inputs and outputs and works in a fixed 16 MiB static device array.  This test
hands it device buffers, runs it twice in a row (the second call must not see
the first call's partial sums) and compares each result with the density
average of eb_interpolate_marker_stokes_parameters_to_grid, within the parity
tolerance (1e-6 relative).  It lives in a file of its own that pytest
collects last.
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


def test_noalloc_average_matches_context_entry_point(eb):
    import torch
    eb.build()
    fn = _entry(eb)
    model = eb.synthetic.config("sinking_block")
    # reference result: the context entry point (allocating path)
    mic = eb.MarkerInCell(0)
    mic.load_model(model)
    mic.get_marker_inside_flags()
    mic.initialize_bilinear_interpolation()
    mic.interpolate_marker_stokes_parameters_to_grid()
    want = mic.download_grid("rho1")
    want_w = mic.download_grid("wtnodes")
    mic.close()

    dev = torch.device("cuda:0")
    x = torch.tensor(model.markers["x"], device=dev)
    y = torch.tensor(model.markers["y"], device=dev)
    rho = torch.tensor(model.markers["rho"], device=dev)
    gx = torch.tensor(model.grid.gridx_b, device=dev)
    gy = torch.tensor(model.grid.gridy_b, device=dev)
    X, Y = model.grid.xnum, model.grid.ynum
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        # the output grid starts from the previous density grid (the backup for empty nodes)
        avg = torch.tensor(np.asfortranarray(model.grids["rho1"]).ravel(order="F"), device=dev)
        wsum = torch.zeros(X * Y, dtype=torch.float64, device=dev)
        rc = fn(x.data_ptr(), y.data_ptr(), rho.data_ptr(), model.marknum, gx.data_ptr(), X, gy.data_ptr(), Y,
                avg.data_ptr(), wsum.data_ptr(), C.c_void_p(stream.cuda_stream), err, len(err))
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got = avg.cpu().numpy().reshape((Y, X), order="F")
        got_w = wsum.cpu().numpy().reshape((Y, X), order="F")
        assert np.all(np.abs(got - want) <= RTOL * np.abs(want)), f"call {call}: density average differs"
        assert np.all(np.abs(got_w - want_w) <= RTOL * np.abs(want_w)), f"call {call}: weight sums differ"


def test_noalloc_rejects_sizes_beyond_its_limit(eb):
    eb.build()
    fn = _entry(eb)
    err = C.create_string_buffer(256)
    rc = fn(None, None, None, 1 << 20, None, 3, None, 3, None, None, None, err, len(err))
    assert rc == 3 and b"524288" in err.value
    rc = fn(None, None, None, 0, None, 1001, None, 1001, None, None, None, err, len(err))
    assert rc == 3 and b"131072" in err.value
