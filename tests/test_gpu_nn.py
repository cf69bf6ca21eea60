"""Tensor-core (tcgen05) BF16 GEMM and implicit convolution of the learned preconditioner,
through the C-ABI, against an FP64 product of the same BF16 operands.  The tensor cores
accumulate in FP32, so the bound is a few FP32 ulps of the summed magnitudes."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(a):
    """FP32 array -> (uint16 bits, the FP64 values they represent)."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16)
    bits = t.view(torch.int16).numpy().view(np.uint16).copy()
    return bits, t.to(torch.float64).numpy()


def ptr(a):
    return C.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("M,N,K,splits", [(128, 16, 64, 1), (256, 64, 192, 1), (300, 96, 72, 1), (128, 256, 512, 1),
                                          (1000, 192, 320, 1), (256, 128, 4096, 4), (128, 384, 128, 1)])
def test_gemm_bf16_matches_fp64(eb, M, N, K, splits):
    from earthbox_gb300 import _abi
    lib = _abi.load()
    rng = np.random.default_rng(M + N + K)
    a_bits, a = bf16(rng.normal(size=(M, K)))
    b_bits, b = bf16(rng.normal(size=(N, K)))
    d = np.zeros((M, N), np.float32)
    assert lib.eb_nn_gemm_bf16(M, N, K, ptr(a_bits), ptr(b_bits), ptr(d), splits) == 0
    want = a @ b.T
    scale = np.abs(a) @ np.abs(b).T
    err = np.abs(d - want) / scale
    assert err.max() < 2e-6, err.max()


def conv_ref(x, w, taps, flip):
    """x [B,H,W,C], w [Cout][taps*C] -> [B,H,W,Cout] in FP64, zero padding."""
    B, H, W, Cc = x.shape
    Cout = w.shape[0]
    wt = w.reshape(Cout, taps, Cc)
    y = np.zeros((B, H, W, Cout))
    ya = np.zeros((B, H, W, Cout))
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    for t in range(taps):
        dy, dx = (t // 3 - 1, t % 3 - 1) if taps == 9 else (0, 0)
        if flip:
            dy, dx = -dy, -dx
        xs = xp[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]
        y += xs @ wt[:, t, :].T
        ya += np.abs(xs) @ np.abs(wt[:, t, :]).T
    return y, ya


@pytest.mark.parametrize("B,H,W,Cc,Cout,taps,flip", [(1, 16, 24, 8, 32, 9, 0), (2, 32, 32, 32, 64, 9, 0),
                                                      (1, 20, 12, 64, 16, 9, 1), (1, 16, 16, 32, 16, 1, 0),
                                                      (1, 8, 40, 96, 192, 9, 0)])
def test_conv2d_bf16_matches_fp64(eb, B, H, W, Cc, Cout, taps, flip):
    from earthbox_gb300 import _abi
    lib = _abi.load()
    rng = np.random.default_rng(H * W + Cc)
    x_bits, x = bf16(rng.normal(size=(B, H, W, Cc)))
    w_bits, w = bf16(rng.normal(size=(Cout, taps * Cc)) / np.sqrt(taps * Cc))
    y = np.zeros((B, H, W, Cout), np.float32)
    assert lib.eb_nn_conv2d_bf16(B, H, W, Cc, Cout, taps, flip, ptr(x_bits), ptr(w_bits), None, 0, ptr(y),
                                 None) == 0
    want, scale = conv_ref(x, w, taps, flip)
    err = np.abs(y - want) / np.maximum(scale, 1e-30)
    assert err.max() < 2e-6, err.max()
    # BF16 output with bias and ReLU
    bias = rng.normal(size=Cout).astype(np.float32)
    y16 = np.zeros((B, H, W, Cout), np.uint16)
    assert lib.eb_nn_conv2d_bf16(B, H, W, Cc, Cout, taps, flip, ptr(x_bits), ptr(w_bits), ptr(bias), 1, None,
                                 ptr(y16)) == 0
    import torch
    got = torch.from_numpy(y16.view(np.int16)).view(torch.bfloat16).to(torch.float64).numpy()
    ref = np.maximum(want + bias, 0.0)
    assert np.all(np.abs(got - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-5 * (scale + np.abs(bias)))
