"""CPU oracle of the warm-start U-Net (test infrastructure only).

A NumPy restatement of the network of lbm_gb300/warmstart.py -- same layer
table, wiring, concatenation order, pooling tie rule and loss -- with the BF16
roundings of the GPU kernels applied at the same places (inputs, weights,
stored activations and activation gradients), so the GPU forward and backward
passes can be checked against it element for element up to FP32 summation
order.  Nothing in the product imports this file.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np


def r16(a: np.ndarray) -> np.ndarray:
    """Round FP32 to the nearest BF16 (ties to even), returned as FP32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return (u.astype(np.uint32)).view(np.float32).reshape(a.shape)


def im2col(x: np.ndarray) -> np.ndarray:
    B, H, W, C = x.shape
    xp = np.zeros((B, H + 2, W + 2, C), dtype=x.dtype)
    xp[:, 1:-1, 1:-1] = x
    cols = np.empty((B, H, W, 9, C), dtype=x.dtype)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        cols[:, :, :, tap] = xp[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
    return cols.reshape(B, H, W, 9 * C)


def col2im(dcols: np.ndarray, C: int) -> np.ndarray:
    B, H, W, _ = dcols.shape
    d = dcols.reshape(B, H, W, 9, C)
    dp = np.zeros((B, H + 2, W + 2, C), dtype=np.float64)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        dp[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W] += d[:, :, :, tap]
    return dp[:, 1:-1, 1:-1]


def pool_fwd(x):
    B, H, W, C = x.shape
    v = x.reshape(B, H // 2, 2, W // 2, 2, C)
    return v.max(axis=(2, 4))


def pool_bwd(x, dy):
    """Gradient to the first maximum of each window (row-major window order)."""
    B, H, W, C = x.shape
    v = x.reshape(B, H // 2, 2, W // 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(B, H // 2, W // 2, 4, C)
    am = np.argmax(v, axis=3)
    dx = np.zeros((B, H // 2, W // 2, 4, C), dtype=dy.dtype)
    np.put_along_axis(dx, am[:, :, :, None, :], dy[:, :, :, None, :], axis=3)
    return dx.reshape(B, H // 2, W // 2, 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(B, H, W, C)


def up_fwd(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def up_bwd(dy):
    B, H, W, C = dy.shape
    return dy.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4), dtype=np.float64)


class RefUNet:
    """bf16=False drops every rounding (plain FP32/FP64 arithmetic), which is
    what the finite-difference check of the oracle itself uses."""

    def __init__(self, specs: List[Tuple[str, int, int, bool]], params: np.ndarray, bf16: bool = True):
        self.dt = np.float32 if bf16 else np.float64
        self.q = r16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
        self.specs = specs
        self.W: Dict[str, np.ndarray] = {}
        self.b: Dict[str, np.ndarray] = {}
        o = 0
        for name, cin, cout, _ in specs:
            self.W[name] = self.q(params[o:o + 9 * cin * cout].reshape(cout, 9 * cin))
            o += 9 * cin * cout
            self.b[name] = params[o:o + cout].astype(self.dt)
            o += cout
        self.relu = {s[0]: s[3] for s in specs}

    def conv(self, name, x, store16=True):
        y = (im2col(x).astype(np.float64) @ self.W[name].T.astype(np.float64)).astype(self.dt) + self.b[name]
        if self.relu[name]:
            y = np.maximum(y, 0.0)
        return self.q(y) if store16 else y

    def forward(self, x):
        a = {"x": self.q(x)}
        a["e0a"] = self.conv("e0a", a["x"])
        a["e0b"] = self.conv("e0b", a["e0a"])
        a["pool0"] = pool_fwd(a["e0b"])
        a["e1a"] = self.conv("e1a", a["pool0"])
        a["e1b"] = self.conv("e1b", a["e1a"])
        a["pool1"] = pool_fwd(a["e1b"])
        a["e2a"] = self.conv("e2a", a["pool1"])
        a["e2b"] = self.conv("e2b", a["e2a"])
        a["pool2"] = pool_fwd(a["e2b"])
        a["b_a"] = self.conv("b_a", a["pool2"])
        a["b_b"] = self.conv("b_b", a["b_a"])
        prev = "b_b"
        for lvl in (2, 1, 0):
            a[f"up{lvl}"] = up_fwd(a[prev])
            a[f"u{lvl}"] = self.conv(f"u{lvl}", a[f"up{lvl}"])
            a[f"cat{lvl}"] = np.concatenate([a[f"u{lvl}"], a[f"e{lvl}b"]], axis=-1)
            a[f"d{lvl}a"] = self.conv(f"d{lvl}a", a[f"cat{lvl}"])
            a[f"d{lvl}b"] = self.conv(f"d{lvl}b", a[f"d{lvl}a"])
            prev = f"d{lvl}b"
        a["out"] = self.conv("out", a["d0b"], store16=False)
        self.a = a
        return a["out"]

    def conv_bwd(self, name, x, y, dy, need_dx=True):
        dpre = self.q(dy * (y > 0)) if self.relu[name] else dy
        cols = im2col(x)
        B, H, W, cout = dpre.shape
        d2 = dpre.reshape(-1, cout).astype(np.float64)
        gW = (d2.T @ cols.reshape(-1, cols.shape[-1]).astype(np.float64)).astype(self.dt)
        gb = d2.sum(axis=0).astype(self.dt)
        dx = None
        if need_dx:
            dcols = (d2 @ self.W[name].astype(np.float64)).astype(self.dt).reshape(B, H, W, -1)
            dx = self.q(col2im(dcols, x.shape[-1]))
        return gW, gb, dx

    def loss_grad(self, x, target, fluid, nout=3):
        """Masked MSE over fluid pixels and the first nout outputs; returns the
        loss and the per-layer (dW, db)."""
        out = self.forward(x)
        a = self.a
        m = fluid.astype(bool)
        count = max(1, int(m.sum())) * nout
        d = (out[..., :nout] - target) * m[..., None]
        loss = float((d.astype(np.float64) ** 2).sum() / count)
        dout = np.zeros_like(out)
        dout[..., :nout] = self.q(2.0 * d / count)
        grads = {}
        gW, gb, dd = self.conv_bwd("out", a["d0b"], a["out"], dout)
        grads["out"] = (gW, gb)
        skip = {}
        for lvl in (0, 1, 2):
            gW, gb, dd = self.conv_bwd(f"d{lvl}b", a[f"d{lvl}a"], a[f"d{lvl}b"], dd)
            grads[f"d{lvl}b"] = (gW, gb)
            gW, gb, dcat = self.conv_bwd(f"d{lvl}a", a[f"cat{lvl}"], a[f"d{lvl}a"], dd)
            grads[f"d{lvl}a"] = (gW, gb)
            c = a[f"u{lvl}"].shape[-1]
            skip[lvl] = dcat[..., c:]
            gW, gb, dup = self.conv_bwd(f"u{lvl}", a[f"up{lvl}"], a[f"u{lvl}"], dcat[..., :c])
            grads[f"u{lvl}"] = (gW, gb)
            dd = self.q(up_bwd(dup))
        gW, gb, dd = self.conv_bwd("b_b", a["b_a"], a["b_b"], dd)
        grads["b_b"] = (gW, gb)
        gW, gb, dpool = self.conv_bwd("b_a", a["pool2"], a["b_a"], dd)
        grads["b_a"] = (gW, gb)
        for lvl in (2, 1, 0):
            de = self.q(skip[lvl] + pool_bwd(a[f"e{lvl}b"], dpool))
            gW, gb, dd = self.conv_bwd(f"e{lvl}b", a[f"e{lvl}a"], a[f"e{lvl}b"], de)
            grads[f"e{lvl}b"] = (gW, gb)
            below = {0: "x", 1: "pool0", 2: "pool1"}[lvl]
            gW, gb, dpool = self.conv_bwd(f"e{lvl}a", a[below], a[f"e{lvl}a"], dd, need_dx=lvl > 0)
            grads[f"e{lvl}a"] = (gW, gb)
        return loss, grads
