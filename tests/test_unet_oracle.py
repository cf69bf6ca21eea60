"""The U-Net oracle's gradient against central finite differences of its own loss (FP64,
no BF16 rounding): pins the backward formulas that the GPU gradients are compared with.
The step is small (1e-9) so that a random direction rarely carries a ReLU input across zero,
where the loss has a kink and the difference quotient stops being a derivative."""
import numpy as np


def test_unet_oracle_gradient_matches_finite_differences():
    from oracle import unet
    rng = np.random.default_rng(3)
    params = np.zeros(unet.n_params())
    for name, ws, bs in unet.layer_slices():
        fan = {n: ci * t for n, ci, co, t, _, _ in unet.LAYERS}[name]
        params[ws] = rng.normal(0.0, np.sqrt(2.0 / fan), ws.stop - ws.start)
        params[bs] = rng.normal(0.0, 0.1, bs.stop - bs.start)
    x = rng.normal(size=(1, 8, 16, 8))
    t = rng.normal(size=(1, 8, 16, 3))
    net = unet.UNet(params, bf16=False)
    loss, g = net.loss_grad(x, t)
    assert g.shape == params.shape and np.isfinite(loss)
    for trial in range(4):
        d = rng.normal(size=params.shape)
        eps = 1e-9
        lp, _ = unet.UNet(params + eps * d, bf16=False).loss_grad(x, t)
        lm, _ = unet.UNet(params - eps * d, bf16=False).loss_grad(x, t)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ d) <= 1e-5 * max(abs(fd), 1e-3), (fd, g @ d)
    # per-layer: the gradient of each layer's weights alone
    for name, ws, bs in unet.layer_slices()[::5]:
        d = np.zeros_like(params)
        d[ws] = rng.normal(size=ws.stop - ws.start)
        lp, _ = unet.UNet(params + 1e-9 * d, bf16=False).loss_grad(x, t)
        lm, _ = unet.UNet(params - 1e-9 * d, bf16=False).loss_grad(x, t)
        fd = (lp - lm) / 2e-9
        assert abs(fd - g @ d) <= 1e-5 * max(abs(fd), 1e-3), (name, fd, g @ d)
