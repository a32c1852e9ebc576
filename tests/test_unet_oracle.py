"""The U-Net CPU oracle checked by finite differences (no BF16 rounding):
its backward pass is the derivative of its forward pass."""
import numpy as np

from unet_ref import RefUNet, r16


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.001953125, -2.5, 3.0e38], dtype=np.float32)
    y = r16(x)
    assert y[0] == 1.0 and y[4] == -2.5
    assert y[1] == 1.0  # 1 + 2^-8 is half way between 1 and 1 + 2^-7: ties to even
    assert y[2] == 1.0078125  # 3/4 of the way: up
    assert y[3] == 1.0  # 1/4 of the way: down
    assert np.all(np.isfinite(y))


def test_oracle_gradients_match_finite_differences():
    from lbm_gb300.warmstart import layer_specs

    specs = layer_specs()
    n = sum(9 * ci * co + co for _, ci, co, _ in specs)
    rng = np.random.default_rng(0)
    p = (rng.normal(size=n) * 0.05).astype(np.float32)
    # He-like scale so the signal survives the 18 layers
    o = 0
    for _, ci, co, _ in specs:
        p[o:o + 9 * ci * co] *= np.float32(np.sqrt(2.0 / (9 * ci)) / 0.05)
        o += 9 * ci * co + co
    B, H, W = 1, 8, 16
    x = rng.normal(size=(B, H, W, 32)).astype(np.float32)
    t = rng.normal(size=(B, H, W, 3)).astype(np.float32)
    fl = rng.random((B, H, W)) > 0.25
    ref = RefUNet(specs, p, bf16=False)
    _, grads = ref.loss_grad(x, t, fl)
    offs = {}
    o = 0
    for name, ci, co, _ in specs:
        offs[name] = (o, o + 9 * ci * co)
        o += 9 * ci * co + co
    checked = 0
    for name in ("out", "d0a", "u1", "b_b", "e2b", "e0a"):
        gw, gb = grads[name]
        w0, b0 = offs[name]
        flat = gw.ravel()
        for j in rng.choice(flat.size, 3, replace=False):
            h = 1e-2 * max(1e-3, abs(float(p[w0 + j])))
            pp, pm = p.copy(), p.copy()
            pp[w0 + j] += h
            pm[w0 + j] -= h
            lp, _ = RefUNet(specs, pp, bf16=False).loss_grad(x, t, fl)
            lm, _ = RefUNet(specs, pm, bf16=False).loss_grad(x, t, fl)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - flat[j]) <= 2e-2 * max(abs(fd), 1e-4), (name, j, fd, flat[j])
            checked += 1
    assert checked == 18
