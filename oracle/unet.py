"""CPU oracle (TEST INFRASTRUCTURE ONLY) of the learned preconditioner's U-Net: forward pass,
MSE loss and the gradient of every parameter, in numpy.

The network is the one the GPU trains (earthbox.jl_gb300/csrc/eb_nn_net.cu): 3x3
convolutions with zero padding, ReLU, 2x2 average pooling, nearest upsampling with channel
concatenation [upsampled | skip], and a 1x1 output convolution to 16 channels of which the
first three enter the loss.  Parameters are one flat FP32 vector, per layer the weights
[cout][taps][cin] then the biases [cout].

With bf16=True the oracle rounds to BF16 where the GPU stores BF16 (the input, the weights of
every product, each convolution's output after bias and ReLU, the pooled tensors, and the
output gradient of each layer before its two products) and keeps everything else in FP32;
the products themselves are summed in FP64 here and in FP32 on the tensor cores.  With
bf16=False everything is FP64, which the finite-difference test uses to pin the backward
formulas.  Only tests/ use this module.
"""
from __future__ import annotations

import numpy as np

# name, cin, cout, taps, relu, level
LAYERS = [("e0a", 8, 32, 9, True, 0), ("e0b", 32, 32, 9, True, 0), ("e1a", 32, 64, 9, True, 1),
          ("e1b", 64, 64, 9, True, 1), ("e2a", 64, 128, 9, True, 2), ("e2b", 128, 128, 9, True, 2),
          ("e3a", 128, 128, 9, True, 3), ("e3b", 128, 128, 9, True, 3), ("d2a", 256, 128, 9, True, 2),
          ("d2b", 128, 128, 9, True, 2), ("d1a", 192, 64, 9, True, 1), ("d1b", 64, 64, 9, True, 1),
          ("d0a", 96, 32, 9, True, 0), ("d0b", 32, 32, 9, True, 0), ("out", 32, 16, 1, False, 0)]
OUT_USED = 3


def n_params() -> int:
    return sum(co * t * ci + co for _, ci, co, t, _, _ in LAYERS)


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even), returned as FP32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(params):
    out, off = {}, 0
    for name, ci, co, t, _, _ in LAYERS:
        w = params[off:off + co * t * ci].reshape(co, t, ci)
        off += co * t * ci
        b = params[off:off + co]
        off += co
        out[name] = (w, b)
    return out


def _shift(x, dy, dx):
    """s[b, y, x] = x[b, y + dy, x + dx], zero outside."""
    B, H, W, C = x.shape
    s = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    s[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return s


def _taps(t):
    return [(k // 3 - 1, k % 3 - 1) for k in range(9)] if t == 9 else [(0, 0)]


class UNet:
    def __init__(self, params, bf16: bool = True):
        self.bf16 = bf16
        self.dt = np.float32 if bf16 else np.float64
        self.p = unpack(np.asarray(params, dtype=np.float32 if bf16 else np.float64))

    def _r(self, a):  # storage rounding
        return bf16_round(a) if self.bf16 else a

    def _w(self, name):
        w, b = self.p[name]
        return (bf16_round(w).astype(np.float64) if self.bf16 else w), b

    def conv(self, name, x):
        w, b = self._w(name)
        t = w.shape[1]
        acc = np.zeros(x.shape[:3] + (w.shape[0],))
        for k, (dy, dx) in enumerate(_taps(t)):
            acc += _shift(x, dy, dx).astype(np.float64) @ w[:, k, :].T
        return acc.astype(self.dt) + b.astype(self.dt)

    def pool(self, x):
        s = ((x[:, 0::2, 0::2].astype(self.dt) + x[:, 0::2, 1::2]) + x[:, 1::2, 0::2]) + x[:, 1::2, 1::2]
        return self._r(self.dt(0.25) * s)

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    def forward(self, x):
        r, relu = self._r, (lambda a: np.maximum(a, 0))
        A = {"x0": r(np.asarray(x, dtype=self.dt))}
        A["e0a"] = r(relu(self.conv("e0a", A["x0"])))
        A["e0b"] = r(relu(self.conv("e0b", A["e0a"])))
        A["x1"] = self.pool(A["e0b"])
        A["e1a"] = r(relu(self.conv("e1a", A["x1"])))
        A["e1b"] = r(relu(self.conv("e1b", A["e1a"])))
        A["x2"] = self.pool(A["e1b"])
        A["e2a"] = r(relu(self.conv("e2a", A["x2"])))
        A["e2b"] = r(relu(self.conv("e2b", A["e2a"])))
        A["x3"] = self.pool(A["e2b"])
        A["e3a"] = r(relu(self.conv("e3a", A["x3"])))
        A["e3b"] = r(relu(self.conv("e3b", A["e3a"])))
        A["cat2"] = np.concatenate([self.up(A["e3b"]), A["e2b"]], axis=3)
        A["d2a"] = r(relu(self.conv("d2a", A["cat2"])))
        A["d2b"] = r(relu(self.conv("d2b", A["d2a"])))
        A["cat1"] = np.concatenate([self.up(A["d2b"]), A["e1b"]], axis=3)
        A["d1a"] = r(relu(self.conv("d1a", A["cat1"])))
        A["d1b"] = r(relu(self.conv("d1b", A["d1a"])))
        A["cat0"] = np.concatenate([self.up(A["d1b"]), A["e0b"]], axis=3)
        A["d0a"] = r(relu(self.conv("d0a", A["cat0"])))
        A["d0b"] = r(relu(self.conv("d0b", A["d0a"])))
        A["y"] = self.conv("out", A["d0b"])
        self.A = A
        return A["y"]

    def _layer_back(self, name, x_in, out, g, grads, need_in=True):
        """Weight / bias gradient of layer `name` and (need_in) the gradient of its input."""
        w, _ = self._w(name)
        relu = name != "out"
        d = g * (out > 0) if relu else g
        d = self._r(d).astype(np.float64)
        xi = x_in.astype(np.float64)
        t = w.shape[1]
        gw = np.zeros(w.shape)
        gin = np.zeros(x_in.shape[:3] + (w.shape[2],)) if need_in else None
        for k, (dy, dx) in enumerate(_taps(t)):
            xs = _shift(xi, dy, dx)
            gw[:, k, :] = np.einsum("bhwo,bhwi->oi", d, xs)
            if need_in:
                gin += _shift(d, -dy, -dx) @ w[:, k, :]
        grads[name] = (gw, d.sum(axis=(0, 1, 2)))
        return gin.astype(self.dt) if need_in else None

    def loss_grad(self, x, target):
        y = self.forward(x)
        A = self.A
        n = y.shape[0] * y.shape[1] * y.shape[2] * OUT_USED
        diff = y[..., :OUT_USED].astype(np.float64) - target
        loss = float(np.sum(diff * diff) / n)
        gy = np.zeros(y.shape, self.dt)
        gy[..., :OUT_USED] = (2.0 * diff / n).astype(self.dt)
        G = {}
        g = self._layer_back("out", A["d0b"], A["y"], gy, G)
        g = self._layer_back("d0b", A["d0a"], A["d0b"], g, G)
        gcat0 = self._layer_back("d0a", A["cat0"], A["d0a"], g, G)
        g = self._up_back(gcat0[..., :64])
        g = self._layer_back("d1b", A["d1a"], A["d1b"], g, G)
        gcat1 = self._layer_back("d1a", A["cat1"], A["d1a"], g, G)
        g = self._up_back(gcat1[..., :128])
        g = self._layer_back("d2b", A["d2a"], A["d2b"], g, G)
        gcat2 = self._layer_back("d2a", A["cat2"], A["d2a"], g, G)
        g = self._up_back(gcat2[..., :128])
        g = self._layer_back("e3b", A["e3a"], A["e3b"], g, G)
        gx3 = self._layer_back("e3a", A["x3"], A["e3a"], g, G)
        g = gcat2[..., 128:] + self._pool_back(gx3)
        g = self._layer_back("e2b", A["e2a"], A["e2b"], g, G)
        gx2 = self._layer_back("e2a", A["x2"], A["e2a"], g, G)
        g = gcat1[..., 128:] + self._pool_back(gx2)
        g = self._layer_back("e1b", A["e1a"], A["e1b"], g, G)
        gx1 = self._layer_back("e1a", A["x1"], A["e1a"], g, G)
        g = gcat0[..., 64:] + self._pool_back(gx1)
        g = self._layer_back("e0b", A["e0a"], A["e0b"], g, G)
        self._layer_back("e0a", A["x0"], A["e0a"], g, G, need_in=False)
        flat = np.concatenate([np.concatenate([G[name][0].ravel(), G[name][1].ravel()]) for name, *_ in LAYERS])
        return loss, flat

    def _up_back(self, g):
        return ((g[:, 0::2, 0::2] + g[:, 0::2, 1::2]) + (g[:, 1::2, 0::2] + g[:, 1::2, 1::2])).astype(self.dt)

    def _pool_back(self, g):
        return self.dt(0.25) * self.up(g)


def layer_slices():
    """(name, slice of the weights, slice of the biases) in the flat parameter vector."""
    out, off = [], 0
    for name, ci, co, t, _, _ in LAYERS:
        out.append((name, slice(off, off + co * t * ci), slice(off + co * t * ci, off + co * t * ci + co)))
        off += co * t * ci + co
    return out
