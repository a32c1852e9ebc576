"""Learned warm start for the D2Q9 channel: a convolutional U-Net predicts the
steady (rho, u) from the geometry and Reynolds number, and the prediction
initialises the populations of the plain LBM, which then iterates to the same
residual as from rest.

* Network: 4 levels of width 32, 64, 128, 256 (two 3x3 convolutions with
  ReLU per level, 2x2 max pooling down, nearest 2x upsampling followed by a
  3x3 convolution up, skip connections by concatenation), a final 3x3
  convolution to (rho - 1, u_x, u_y) in normalised units.  Input channels:
  fluid mask, Re / 200, x / nx, y / ny (zero-padded to 32).
* Kernels: every convolution, its data and weight gradients, pooling,
  upsampling, the loss and Adam run in the project's own CUDA kernels
  (csrc/unet.cu: BF16 tensor-core mma, FP32 accumulation) through the C ABI
  of include/lbm_unet.h.  PyTorch only allocates device memory.
* Training data: steady fields of the FP64 LBM (dense-box engine) on seeded
  channels; several channels with one Reynolds number run together as the
  z-slices of one D2Q9 box.
* Warm start: f = f_eq(rho, u) + f_neq, f_neq from the Chapman-Enskog
  estimate -3 tau w_i rho Q_i:grad(u) of the predicted velocity gradient,
  then two period-2 filters (at the first step and after 2,000 steps) that
  remove the undamped staggered mode a non-rest initial state excites.  The
  timing of the warm start includes the prediction, the population build and
  the filters.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import cases
from ._lib import load

W_D2Q9 = np.array([1 / 9] * 4 + [1 / 36] * 4 + [4 / 9])
C_D2Q9 = np.array([[-1, 0], [1, 0], [0, -1], [0, 1], [1, 1], [1, -1], [-1, -1], [-1, 1], [0, 0]])

_NN = {
    "lbm_nn_conv3x3_fwd": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                           C.c_int, C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_conv3x3_wgrad": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_int, C.c_int,
                             C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_bias_grad": [C.c_void_p, C.c_int, C.c_int64, C.c_int, C.c_void_p, C.c_void_p],
    "lbm_nn_flip_weights": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_relu_bwd": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int64, C.c_int, C.c_void_p],
    "lbm_nn_pool_fwd": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_pool_bwd": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                        C.c_void_p],
    "lbm_nn_up_fwd": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_up_bwd": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "lbm_nn_mse": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_void_p],
    "lbm_nn_adam": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float,
                    C.c_int, C.c_void_p],
    "lbm_nn_to_bf16": [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p],
    "lbm_nn_set_conv_path": [C.c_int],
    "lbm_nn_conv_uses_tc": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                            C.c_int],
    "lbm_nn_conv_status": [C.c_void_p],
    "lbm_nn_conv_test_wait": [C.c_int64, C.c_int32],
}


def nn_lib():
    lib = load()
    for name, args in _NN.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    return lib


def _ck(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc})")


# layer table: name, cin, cout, relu
def layer_specs(width: int = 32) -> List[Tuple[str, int, int, bool]]:
    c = [width << l for l in range(4)]
    return [
        ("e0a", 32, c[0], True), ("e0b", c[0], c[0], True),
        ("e1a", c[0], c[1], True), ("e1b", c[1], c[1], True),
        ("e2a", c[1], c[2], True), ("e2b", c[2], c[2], True),
        ("b_a", c[2], c[3], True), ("b_b", c[3], c[3], True),
        ("u2", c[3], c[2], True), ("d2a", 2 * c[2], c[2], True), ("d2b", c[2], c[2], True),
        ("u1", c[2], c[1], True), ("d1a", 2 * c[1], c[1], True), ("d1b", c[1], c[1], True),
        ("u0", c[1], c[0], True), ("d0a", 2 * c[0], c[0], True), ("d0b", c[0], c[0], True),
        ("out", c[0], 32, False),
    ]


class UNet:
    """Parameters, activations and the forward / backward passes for a batch
    of B fields of H x W (H, W divisible by 8)."""

    NOUT = 3

    def __init__(self, B: int, H: int, W: int, width: int = 32, seed: int = 0, device: int = 0):
        import torch

        self.torch = torch
        self.lib = nn_lib()
        self.dev = torch.device("cuda", device)
        self.B, self.H, self.W = B, H, W
        self.specs = layer_specs(width)
        self.c = [width << l for l in range(4)]
        rng = np.random.default_rng(seed)
        # flat parameter vector: per layer weights [cout][9 cin] then bias [cout]
        self.off: Dict[str, Tuple[int, int, int]] = {}
        n = 0
        for name, cin, cout, _ in self.specs:
            self.off[name] = (n, n + 9 * cin * cout, cout)
            n += 9 * cin * cout + cout
        self.nparam = n
        w = np.zeros(n, dtype=np.float32)
        for name, cin, cout, relu in self.specs:
            o, ob, _ = self.off[name]
            std = math.sqrt(2.0 / (9 * cin)) if relu else math.sqrt(1.0 / (9 * cin))
            w[o:ob] = rng.normal(0.0, std, 9 * cin * cout).astype(np.float32)
        f32, b16 = torch.float32, torch.bfloat16
        self.w32 = torch.from_numpy(w).to(self.dev)
        self.w16 = torch.zeros(n, dtype=b16, device=self.dev)
        self.g32 = torch.zeros(n, dtype=f32, device=self.dev)
        self.m = torch.zeros(n, dtype=f32, device=self.dev)
        self.v = torch.zeros(n, dtype=f32, device=self.dev)
        self.step_count = 0
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream
        _ck(self.lib.lbm_nn_to_bf16(self.w32.data_ptr(), self.w16.data_ptr(), n, self.stream), "to_bf16")
        self.zero_bias = torch.zeros(512, dtype=f32, device=self.dev)
        maxw = max(9 * cin * cout for _, cin, cout, _ in self.specs)
        self.wflip = torch.zeros(maxw, dtype=b16, device=self.dev)
        self.partial = torch.zeros(8 * 1024 * 1024, dtype=f32, device=self.dev)
        self._alloc()

    # ---- buffers -----------------------------------------------------------
    def _alloc(self):
        t, B, H, W, c = self.torch, self.B, self.H, self.W, self.c
        b16 = t.bfloat16

        def z(h, w, ch, dt=b16):
            return t.zeros((B, h, w, ch), dtype=dt, device=self.dev)

        hw = [(H >> l, W >> l) for l in range(4)]
        self.a: Dict[str, object] = {"x": z(H, W, 32)}
        self.a["e0a"] = z(*hw[0], c[0])
        self.a["cat0"] = z(*hw[0], 2 * c[0])
        self.a["pool0"] = z(*hw[1], c[0])
        self.a["e1a"] = z(*hw[1], c[1])
        self.a["cat1"] = z(*hw[1], 2 * c[1])
        self.a["pool1"] = z(*hw[2], c[1])
        self.a["e2a"] = z(*hw[2], c[2])
        self.a["cat2"] = z(*hw[2], 2 * c[2])
        self.a["pool2"] = z(*hw[3], c[2])
        self.a["b_a"] = z(*hw[3], c[3])
        self.a["b_b"] = z(*hw[3], c[3])
        self.a["up2"] = z(*hw[2], c[3])
        self.a["d2a"] = z(*hw[2], c[2])
        self.a["d2b"] = z(*hw[2], c[2])
        self.a["up1"] = z(*hw[1], c[2])
        self.a["d1a"] = z(*hw[1], c[1])
        self.a["d1b"] = z(*hw[1], c[1])
        self.a["up0"] = z(*hw[0], c[1])
        self.a["d0a"] = z(*hw[0], c[0])
        self.a["d0b"] = z(*hw[0], c[0])
        self.a["out"] = z(*hw[0], 32, t.float32)
        # gradients of the activations (same shapes), plus dense scratch
        self.g = {k: t.zeros_like(v, dtype=b16) for k, v in self.a.items() if k != "x"}
        self.scratch = z(H, W, 2 * c[0]).reshape(-1)
        self.scratch2 = z(H, W, 2 * c[0]).reshape(-1)
        self.fluid = t.zeros(B * H * W, dtype=t.uint8, device=self.dev)
        self.target = t.zeros((B * H * W, self.NOUT), dtype=t.float32, device=self.dev)
        self.loss_part = t.zeros(1024, dtype=t.float32, device=self.dev)
        # conv layer wiring: input (tensor, ld), output (tensor, ld, off), level
        self.wiring = {
            "e0a": ("x", 32, "e0a", c[0], 0, 0), "e0b": ("e0a", c[0], "cat0", 2 * c[0], c[0], 0),
            "e1a": ("pool0", c[0], "e1a", c[1], 0, 1), "e1b": ("e1a", c[1], "cat1", 2 * c[1], c[1], 1),
            "e2a": ("pool1", c[1], "e2a", c[2], 0, 2), "e2b": ("e2a", c[2], "cat2", 2 * c[2], c[2], 2),
            "b_a": ("pool2", c[2], "b_a", c[3], 0, 3), "b_b": ("b_a", c[3], "b_b", c[3], 0, 3),
            "u2": ("up2", c[3], "cat2", 2 * c[2], 0, 2), "d2a": ("cat2", 2 * c[2], "d2a", c[2], 0, 2),
            "d2b": ("d2a", c[2], "d2b", c[2], 0, 2),
            "u1": ("up1", c[2], "cat1", 2 * c[1], 0, 1), "d1a": ("cat1", 2 * c[1], "d1a", c[1], 0, 1),
            "d1b": ("d1a", c[1], "d1b", c[1], 0, 1),
            "u0": ("up0", c[1], "cat0", 2 * c[0], 0, 0), "d0a": ("cat0", 2 * c[0], "d0a", c[0], 0, 0),
            "d0b": ("d0a", c[0], "d0b", c[0], 0, 0),
            "out": ("d0b", c[0], "out", 32, 0, 0),
        }

    def _p(self, name: str):
        o, ob, cout = self.off[name]
        el16 = self.w16.element_size()
        return (self.w16.data_ptr() + o * el16, self.w32.data_ptr() + ob * 4, self.g32.data_ptr() + o * 4, self.g32.data_ptr() + ob * 4)

    def _dims(self, level: int):
        return self.B, self.H >> level, self.W >> level

    # ---- forward -----------------------------------------------------------
    def _conv(self, name: str):
        _, cin, cout, relu = next(s for s in self.specs if s[0] == name)
        src, ldx, dst, ldy, offy, lvl = self.wiring[name]
        w16, bias, _, _ = self._p(name)
        B, h, w = self._dims(lvl)
        out_f32 = 1 if name == "out" else 0
        _ck(self.lib.lbm_nn_conv3x3_fwd(self.a[src].data_ptr(), ldx, w16, bias, self.a[dst].data_ptr(), ldy, offy, B, h, w, cin, cout,
                                        1 if relu else 0, out_f32, self.stream), f"conv {name}")

    def forward(self, x_host: Optional[np.ndarray] = None):
        """x_host: (B, H, W, 32) float array of the input channels, or None to
        keep the input already on the device."""
        t, L, a, c = self.torch, self.lib, self.a, self.c
        if x_host is not None:
            a["x"].copy_(t.from_numpy(np.ascontiguousarray(x_host, dtype=np.float32)).to(self.dev).to(t.bfloat16))
        s = self.stream
        self._conv("e0a")
        self._conv("e0b")
        for lvl, (cat, pool) in enumerate((("cat0", "pool0"), ("cat1", "pool1"), ("cat2", "pool2"))):
            B, h, w = self._dims(lvl)
            _ck(L.lbm_nn_pool_fwd(a[cat].data_ptr(), 2 * c[lvl], c[lvl], a[pool].data_ptr(), B, h, w, c[lvl], s), "pool")
            if lvl == 0:
                self._conv("e1a"), self._conv("e1b")
            elif lvl == 1:
                self._conv("e2a"), self._conv("e2b")
            else:
                self._conv("b_a"), self._conv("b_b")
        for lvl, (src, up, cs) in ((2, ("b_b", "up2", c[3])), (1, ("d2b", "up1", c[2])), (0, ("d1b", "up0", c[1]))):
            B, h, w = self._dims(lvl + 1)
            _ck(L.lbm_nn_up_fwd(a[src].data_ptr(), a[up].data_ptr(), cs, B, h, w, cs, s), "up")
            self._conv(f"u{lvl}")
            self._conv(f"d{lvl}a")
            self._conv(f"d{lvl}b")
        self._conv("out")
        return a["out"]

    # ---- backward ----------------------------------------------------------
    def _conv_bwd(self, name: str, dy, lddy: int, offdy: int, dx=None):
        """Gradients of one convolution given the gradient of its output (dy
        at stride lddy / offset offdy); writes its weight and bias gradients
        and, if dx is given, the gradient of its input (dense, cin channels)."""
        L, s = self.lib, self.stream
        _, cin, cout, relu = next(sp for sp in self.specs if sp[0] == name)
        src, ldx, dst, ldy, offy, lvl = self.wiring[name]
        B, h, w = self._dims(lvl)
        npix = B * h * w
        w16, _, gw, gb = self._p(name)
        if relu:
            dpre = self.scratch
            _ck(L.lbm_nn_relu_bwd(dy.data_ptr(), lddy, offdy, self.a[dst].data_ptr(), ldy, offy, dpre.data_ptr(), cout, npix, cout, s), "relu")
            dp, ldp = dpre, cout
        else:
            dp, ldp = dy, lddy
        _ck(L.lbm_nn_conv3x3_wgrad(self.a[src].data_ptr(), ldx, dp.data_ptr(), ldp, self.partial.data_ptr(), self.partial.numel(), gw,
                                   B, h, w, cin, cout, s), f"wgrad {name}")
        _ck(L.lbm_nn_bias_grad(dp.data_ptr(), ldp, npix, cout, gb, s), "bias grad")
        if dx is not None:
            _ck(L.lbm_nn_flip_weights(w16, self.wflip.data_ptr(), cin, cout, s), "flip")
            _ck(L.lbm_nn_conv3x3_fwd(dp.data_ptr(), ldp, self.wflip.data_ptr(), self.zero_bias.data_ptr(), dx.data_ptr(), cin, 0, B, h, w,
                                     cout, cin, 0, 0, s), f"dgrad {name}")

    def backward(self):
        """Gradient of the loss (whose output gradient k_mse left in g['out'])
        with respect to every parameter, into g32."""
        L, s, a, g, c = self.lib, self.stream, self.a, self.g, self.c
        self._conv_bwd("out", g["out"], 32, 0, g["d0b"])
        # decoder, from the finest level down
        for lvl in (0, 1, 2):
            cat = f"cat{lvl}"
            self._conv_bwd(f"d{lvl}b", g[f"d{lvl}b"], c[lvl], 0, g[f"d{lvl}a"])
            self._conv_bwd(f"d{lvl}a", g[f"d{lvl}a"], c[lvl], 0, g[cat])  # dense 2 c[lvl] channels
            self._conv_bwd(f"u{lvl}", g[cat], 2 * c[lvl], 0, g[f"up{lvl}"])
            B, h, w = self._dims(lvl + 1)
            src = {0: "d1b", 1: "d2b", 2: "b_b"}[lvl]
            cs = c[lvl + 1]
            _ck(L.lbm_nn_up_bwd(g[f"up{lvl}"].data_ptr(), cs, g[src].data_ptr(), B, h, w, cs, s), "up bwd")
        # bottleneck, then the encoder from the bottom
        self._conv_bwd("b_b", g["b_b"], c[3], 0, g["b_a"])
        self._conv_bwd("b_a", g["b_a"], c[3], 0, g["pool2"])
        for lvl in (2, 1, 0):
            B, h, w = self._dims(lvl)
            cat = f"cat{lvl}"
            # pooling gradient added to the skip half of the concatenation gradient
            _ck(L.lbm_nn_pool_bwd(a[cat].data_ptr(), 2 * c[lvl], c[lvl], g[f"pool{lvl}"].data_ptr(), g[cat].data_ptr(), 2 * c[lvl], c[lvl],
                                  B, h, w, c[lvl], s), "pool bwd")
            self._conv_bwd(f"e{lvl}b", g[cat], 2 * c[lvl], c[lvl], g[f"e{lvl}a"])
            below = {0: None, 1: "pool0", 2: "pool1"}[lvl]
            self._conv_bwd(f"e{lvl}a", g[f"e{lvl}a"], c[lvl], 0, g[below] if below else None)

    # ---- loss, update ------------------------------------------------------
    def set_batch(self, x: np.ndarray, target: np.ndarray, fluid: np.ndarray):
        t = self.torch
        self.a["x"].copy_(t.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(self.dev).to(t.bfloat16))
        self.target.copy_(t.from_numpy(np.ascontiguousarray(target, dtype=np.float32).reshape(-1, self.NOUT)).to(self.dev))
        self.fluid.copy_(t.from_numpy(np.ascontiguousarray(fluid, dtype=np.uint8).reshape(-1)).to(self.dev))

    def loss_and_grad(self) -> float:
        """Forward, masked MSE (mean over fluid cells and outputs), backward."""
        self.forward()
        npix = self.B * self.H * self.W
        count = max(1, int(self.fluid.sum().item())) * self.NOUT
        nb = 512
        _ck(self.lib.lbm_nn_mse(self.a["out"].data_ptr(), 32, self.target.data_ptr(), self.fluid.data_ptr(), npix, self.NOUT, 1.0 / count,
                                self.g["out"].data_ptr(), self.loss_part.data_ptr(), nb, self.stream), "mse")
        self.backward()
        loss = float(self.loss_part[:nb].double().sum().item()) / count
        _ck(self.lib.lbm_nn_conv_status(self.stream), "tensor-core convolution (a pipeline wait ran out)")
        return loss

    def adam(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        _ck(self.lib.lbm_nn_adam(self.w32.data_ptr(), self.w16.data_ptr(), self.g32.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                 self.nparam, lr, b1, b2, eps, self.step_count, self.stream), "adam")

    def predict(self, x: np.ndarray) -> np.ndarray:
        """(B, H, W, 3) FP32 prediction for input channels x."""
        out = self.forward(x)
        pred = out[..., : self.NOUT].float().cpu().numpy()
        _ck(self.lib.lbm_nn_conv_status(self.stream), "tensor-core convolution (a pipeline wait ran out)")
        return pred

    def get_params(self) -> np.ndarray:
        return self.w32.cpu().numpy()

    def set_params(self, w: np.ndarray):
        t = self.torch
        self.w32.copy_(t.from_numpy(np.ascontiguousarray(w, dtype=np.float32)).to(self.dev))
        _ck(self.lib.lbm_nn_to_bf16(self.w32.data_ptr(), self.w16.data_ptr(), self.nparam, self.stream), "to_bf16")


# ---- inputs, targets, warm start ------------------------------------------------

def net_width(nx: int) -> int:
    """Network width for an nx-wide periodic channel: nx rounded up to a
    multiple of 8 (the extra columns wrap around periodically)."""
    return (nx + 7) // 8 * 8


def wrap_columns(a: np.ndarray, W: int) -> np.ndarray:
    """Extend the x axis (axis 1) of a periodic field to W columns."""
    nx = a.shape[1]
    return a[:, np.arange(W) % nx] if W != nx else a


def input_channels(flags2d: np.ndarray, re: float) -> np.ndarray:
    """(H, W, 32) network input of one channel geometry (flags (ny, nx)),
    W = net_width(nx): fluid mask, Re / 200, x / nx, y / ny, zeros."""
    H, nx = flags2d.shape
    W = net_width(nx)
    x = np.zeros((H, W, 32), dtype=np.float32)
    x[..., 0] = wrap_columns((flags2d != cases.SOLID).astype(np.float32), W)
    x[..., 1] = re / 200.0
    x[..., 2] = ((np.arange(W) % nx)[None, :] + 0.5) / nx
    x[..., 3] = (np.arange(H)[:, None] + 0.5) / H
    return x


class Scales:
    """Normalisation of the outputs: (rho - 1) / s_rho, u / u_ref."""

    def __init__(self, s_rho: float, u_ref: float):
        self.s_rho, self.u_ref = float(s_rho), float(u_ref)

    def to_net(self, rho, ux, uy):
        return np.stack([(rho - 1.0) / self.s_rho, ux / self.u_ref, uy / self.u_ref], axis=-1).astype(np.float32)

    def from_net(self, y):
        return 1.0 + y[..., 0] * self.s_rho, y[..., 1] * self.u_ref, y[..., 2] * self.u_ref


def populations_from_fields(rho: np.ndarray, ux: np.ndarray, uy: np.ndarray, solid: np.ndarray, tau: float) -> np.ndarray:
    """FP64 populations (9, ny*nx) of a predicted field: equilibrium plus the
    first-order non-equilibrium part -3 tau w_i rho Q_i:grad u (Q_i = c_i c_i -
    I/3), central differences inside, one-sided at the edges.  The density is
    rescaled so the fluid mass is that of the rest state (a closed periodic
    channel conserves it); solids get the rest state."""
    fluid = ~solid
    rho = np.where(solid, 1.0, rho)
    rho = rho * (fluid.sum() / rho[fluid].sum()) if fluid.any() else rho
    ux = np.where(solid, 0.0, ux)
    uy = np.where(solid, 0.0, uy)
    dux_dy, dux_dx = np.gradient(ux)
    duy_dy, duy_dx = np.gradient(uy)
    usq = ux * ux + uy * uy
    f = np.empty((9,) + rho.shape)
    for i in range(9):
        cx, cy = C_D2Q9[i]
        cu = cx * ux + cy * uy
        feq = W_D2Q9[i] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
        qxx, qyy, qxy = cx * cx - 1.0 / 3, cy * cy - 1.0 / 3, cx * cy
        qs = qxx * dux_dx + qyy * duy_dy + qxy * (dux_dy + duy_dx)
        f[i] = feq - 3.0 * tau * W_D2Q9[i] * rho * qs
    f[:, solid] = W_D2Q9[:, None]
    return f.reshape(9, -1)


def period2_filter(g) -> None:
    """Replace the state s(t) by (s(t) + s(t+1)) / 2 (one step taken).

    A warm-start state, unlike the state at rest, has a component along the
    undamped period-2 (staggered) mode of BGK + bounce-back: left alone it
    keeps the one-step residual near 1e-4 for ever.  Averaging two consecutive
    states removes the eigenvalue -1 component exactly (to first order) and
    halves every other mode's amplitude by (1 + lambda) / 2."""
    s0 = g.populations()
    g.step(1)
    s1 = g.populations()
    g.set_populations(0.5 * (s0 + s1))


def channel_momentum(g, n: int) -> np.ndarray:
    """Total x momentum of each of the n stacked channels."""
    rho, u = g.moments()
    return (rho * u[0]).reshape(n, -1).sum(axis=1)


def aitken_scales(pa: np.ndarray, pb: np.ndarray, pc: np.ndarray) -> np.ndarray:
    """Per channel, P_inf / P(c) for momenta sampled at equally spaced steps
    a < b < c of an exponential relaxation P(t) = P_inf + A exp(-t / T):
    with r = (P(c) - P(b)) / (P(b) - P(a)) = exp(-(c - b) / T), Aitken's
    extrapolation P_inf = P(c) + (P(c) - P(b)) r / (1 - r).  1 where the samples
    do not contract (0 < r < 0.95), clipped to [0.2, 5]."""
    pa, pb, pc = (np.asarray(v, dtype=np.float64) for v in (pa, pb, pc))
    d1, d2 = pb - pa, pc - pb
    r = np.divide(d2, d1, out=np.zeros_like(d2), where=np.abs(d1) > 0)
    ok = (r > 0.0) & (r < 0.95) & (np.abs(pc) > 0)
    p_inf = pc + d2 * r / np.where(ok, 1.0 - r, 1.0)
    return np.where(ok, np.clip(p_inf / np.where(ok, pc, 1.0), 0.2, 5.0), 1.0)


def rescale_flow(g, chans: List[Dict], scale: np.ndarray) -> None:
    """Scale the flow of each stacked channel k by scale[k], as a Stokes flow
    scales with its forcing: f -> f_eq(1 + s (rho - 1), s u) + s (f - f_eq(rho, u))
    in every fluid cell (u the Guo velocity (j + F / 2) / rho)."""
    f = g.populations()
    n = len(chans)
    ny_nx = f.shape[1] // n
    rho = f.sum(axis=0)
    jx = (C_D2Q9[:, 0, None] * f).sum(axis=0)
    jy = (C_D2Q9[:, 1, None] * f).sum(axis=0)
    fluid = np.concatenate([(c["flags"] != cases.SOLID).reshape(-1) for c in chans])
    gx = np.concatenate([np.full(ny_nx, c["g"]) for c in chans])
    sc = np.repeat(np.asarray(scale, dtype=np.float64), ny_nx)
    rho = np.where(fluid, rho, 1.0)  # solids keep their populations below; no division by their (zero) density
    ux = np.where(fluid, (jx + 0.5 * gx) / rho, 0.0)
    uy = np.where(fluid, jy / rho, 0.0)

    def feq(r, vx, vy):
        usq = vx * vx + vy * vy
        out = np.empty((9,) + r.shape)
        for i in range(9):
            cu = C_D2Q9[i, 0] * vx + C_D2Q9[i, 1] * vy
            out[i] = W_D2Q9[i] * r * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
        return out

    new = feq(1.0 + sc * (rho - 1.0), sc * ux, sc * uy) + sc * (f - feq(rho, ux, uy))
    g.set_populations(np.where(fluid[None, :], new, f))


def run_stack(chans: List[Dict], storage: str, max_steps: int, tol: Optional[float] = None, check: int = 2000,
              init: Optional[np.ndarray] = None, filters=(0, 2000), project: Optional[Tuple[int, int, int]] = None) -> Dict:
    """Forced channels sharing one Re as the z-slices of one D2Q9 box, from
    rest (or from populations `init`, (9, ncells)), for max_steps or until the
    residual summed over the slices, divided by their number, is below tol
    (checked every `check` steps: the reference's convergence test with
    conv_interval = check).  A warm start applies period2_filter at the steps
    in `filters` (a start from rest too, when `init` holds the rest state).

    project = (a, b, c): the flow-rate projection.  The slowest mode of a
    forced channel is its flow rate, which relaxes exponentially towards the
    balance of drag and body force on the time P / F (thousands of steps for
    the 128-high channels).  The total x momentum of each channel is sampled
    at steps a < b < c (b - a = c - b); Aitken's extrapolation of the three
    gives the momentum P_inf the channel relaxes to, and at step c the flow
    is scaled by P_inf / P(c) (rescale_flow), which removes that mode.  A
    channel whose samples are not a contracting monotone sequence is left as
    it is; the period-2 filter follows the rescaling (the rescaled state has a
    component along that undamped mode again).  Returns fields, steps, wall
    time, residual and the scales."""
    from .solver import BoxSolver

    st = cases.stacked_forced(chans)
    g = BoxSolver(st["lattice"], st["shape"], st["omega"], storage, **cases.box_kwargs(st))
    g.initial_condition()
    g.synchronize()
    t0 = time.perf_counter()
    pending = sorted(filters) if init is not None else []
    samples = list(project) if project else []
    moms: List[np.ndarray] = []
    scales = None
    if init is not None:
        g.set_populations(init)
    n = len(chans)
    done, res = 0, np.full(3, np.inf)
    while done < max_steps:
        if pending and pending[0] <= done:
            pending.pop(0)
            period2_filter(g)
            done += 1
            continue
        if samples and samples[0] <= done:
            samples.pop(0)
            moms.append(channel_momentum(g, n))
            if len(moms) == 3:
                scales = aitken_scales(*moms)
                rescale_flow(g, chans, scales)
                # the rescaled state has a component along the undamped
                # period-2 mode again: filter it out
                period2_filter(g)
                done += 1
            continue
        k = min(check, max_steps - done)
        if pending:
            k = min(k, max(2, pending[0] - done))
        if samples:
            k = min(k, samples[0] - done)
        g.step(k)
        done += k
        if tol is not None and k >= 2:
            res = g.residual() / n
            if float(np.max(res)) < tol:
                break
    g.synchronize()
    wall = time.perf_counter() - t0
    if tol is None or not np.all(np.isfinite(res)):
        res = g.residual() / n
    rho, u = g.moments()
    nx, ny = chans[0]["shape"]
    g.close()
    return dict(rho=rho.reshape(n, ny, nx), ux=u[0].reshape(n, ny, nx), uy=u[1].reshape(n, ny, nx), steps=done, wall=wall,
                residual=float(np.max(res)), flow_scales=None if scales is None else [float(x) for x in scales])


def make_dataset(seeds: List[int], per_batch: int, steps: int, storage: str = "f32", nx: int = 512, ny: int = 128,
                 rng_seed: int = 0, re_range=(20.0, 200.0), log=None) -> Dict:
    """Near-steady fields for the training channels: the seeds are grouped
    `per_batch` at a time, each group shares a Reynolds number drawn
    uniformly from [20, 200], and runs `steps` steps as one stacked box."""
    rng = np.random.default_rng(rng_seed)
    xs, ys, masks, res, flux = [], [], [], [], []
    for k in range(0, len(seeds), per_batch):
        re = float(rng.uniform(*re_range))
        chans = [cases.forced_channel(s, nx, ny, re=re) for s in seeds[k:k + per_batch]]
        out = run_stack(chans, storage, steps)
        W = net_width(nx)
        for j, c in enumerate(chans):
            xs.append(input_channels(c["flags"], re))
            ys.append(wrap_columns(np.stack([out["rho"][j], out["ux"][j], out["uy"][j]], axis=-1), W))
            masks.append(wrap_columns(c["flags"] != cases.SOLID, W))
            flux.append(float(out["ux"][j][c["flags"] != cases.SOLID].mean()))
        res.append(out["residual"])
        if log:
            log(f"dataset batch {k // per_batch}: Re {re:.1f}, {len(chans)} channels, {steps} steps, residual/slice {out['residual']:.2e}, "
                f"{out['wall']:.1f} s")
    return dict(x=np.stack(xs), fields=np.stack(ys), fluid=np.stack(masks), residuals=res, flux=np.asarray(flux))


def normalize_by_flux(data: Dict) -> Dict:
    """The dataset with every field divided by its channel's flow rate (mean
    u_x over the fluid): (rho - 1) / q, u / q.  In Stokes flow both scale with
    the flow rate, which is a channel-wide quantity (set by every obstacle
    along the channel) that flux_balance supplies at inference; the network
    learns the flow pattern only."""
    q = np.asarray(data["flux"])[:, None, None]
    f = data["fields"].copy()
    f[..., 0] = 1.0 + (f[..., 0] - 1.0) / q
    f[..., 1] /= q
    f[..., 2] /= q
    return dict(data, fields=f)


def train(net: "UNet", data: Dict, scales: Scales, epochs: int, lr: float = 1e-3, seed: int = 0, log=None) -> List[float]:
    rng = np.random.default_rng(seed)
    n = data["x"].shape[0]
    target = scales.to_net(data["fields"][..., 0], data["fields"][..., 1], data["fields"][..., 2])
    losses = []
    steps_per_epoch = max(1, n // net.B)
    total = epochs * steps_per_epoch
    it = 0
    for ep in range(epochs):
        order = rng.permutation(n)
        acc = 0.0
        for b in range(steps_per_epoch):
            idx = order[b * net.B:(b + 1) * net.B]
            net.set_batch(data["x"][idx], target[idx], data["fluid"][idx])
            acc += net.loss_and_grad()
            it += 1
            # cosine decay of the learning rate
            net.adam(lr=lr * 0.5 * (1.0 + math.cos(math.pi * it / total)))
        losses.append(acc / steps_per_epoch)
        if log:
            log(f"epoch {ep}: loss {losses[-1]:.4e}")
    return losses


def predict_fields(net: "UNet", chans: List[Dict], scales: Scales,
                   flux: Optional[float] = None) -> List[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """(rho, u_x, u_y) per channel; a network trained on flux-normalised
    fields (normalize_by_flux) gets the flow rate `flux` to scale by."""
    out = []
    for k in range(0, len(chans), net.B):
        group = chans[k:k + net.B]
        x = np.zeros((net.B, net.H, net.W, 32), dtype=np.float32)
        for j, c in enumerate(group):
            x[j] = input_channels(c["flags"], c["re"])
        y = net.predict(x)
        for j, c in enumerate(group):
            nx = c["flags"].shape[1]
            r, ux, uy = scales.from_net(y[j][:, :nx])
            out.append((r, ux, uy) if flux is None else (1.0 + flux * (r - 1.0), flux * ux, flux * uy))
    return out


def flux_balance(chans: List[Dict], fields, iters: int = 3, settle: int = 0, window: int = 2):
    """Rescale each predicted field so that the drag of the walls and
    cylinders balances the body force, as it does in the steady state.

    The network predicts the flow pattern per unit flow rate
    (normalize_by_flux); the flow rate of a channel is set by every obstacle
    along it.  For each channel the predicted state steps in FP64, and the
    change of its total x momentum per step over `window` steps (after
    `settle`) is the body force minus the drag, D = F N - dP/dt.  Velocity and
    density deviation are scaled by F N / D, as a Stokes flow scales with its
    forcing; `iters` fixed-point passes take up the inertial part.  The
    estimate is taken over the first steps: the flow rate relaxes towards the
    balance on the time P / F (a few hundred steps), so a longer window
    measures a drag already partly relaxed.  Returns the corrected fields and
    each channel's total scale."""
    from .solver import BoxSolver

    st = cases.stacked_forced(chans)
    n = len(chans)
    fluid = np.stack([c["flags"] != cases.SOLID for c in chans]).reshape(n, -1)
    force = np.array([c["g"] for c in chans]) * fluid.sum(axis=1)
    fields = [(r.copy(), ux.copy(), uy.copy()) for r, ux, uy in fields]
    total = np.ones(n)
    g = BoxSolver(st["lattice"], st["shape"], st["omega"], "f64", **cases.box_kwargs(st))
    try:
        for _ in range(iters):
            g.set_populations(warm_start_populations(chans, fields))
            if settle:
                g.step(settle)
            r0, u0 = g.moments()
            g.step(window)
            r1, u1 = g.moments()
            p0 = (r0 * u0[0]).reshape(n, -1).sum(axis=1)
            p1 = (r1 * u1[0]).reshape(n, -1).sum(axis=1)
            drag = force - (p1 - p0) / window
            ok = drag > 0.05 * force
            alpha = np.where(ok, np.clip(force / np.where(ok, drag, 1.0), 0.2, 5.0), 1.0)
            fields = [(1.0 + a * (r - 1.0), a * ux, a * uy) for (r, ux, uy), a in zip(fields, alpha)]
            total *= alpha
    finally:
        g.close()
    return fields, total


def warm_start_populations(chans: List[Dict], fields) -> np.ndarray:
    fs = [populations_from_fields(r, ux, uy, c["flags"] == cases.SOLID, c["tau"]) for c, (r, ux, uy) in zip(chans, fields)]
    return np.concatenate(fs, axis=1)


def experiment(n_train: int = 1024, per_batch: int = 64, train_steps: int = 300000, epochs: int = 20, n_eval: int = 16,
               per_eval: int = 8, tol: float = 1e-8, max_steps: int = 1500000, nx: int = 511, ny: int = 128, batch: int = 8,
               re_range=(20.0, 200.0), lr: float = 1e-3, filtered_rest: bool = True, normalize_flux: bool = True,
               project: Optional[Tuple[int, int, int]] = (2500, 4500, 6500), log=print) -> Dict:
    """The whole warm-start study: FP32 training fields, training with the
    project's kernels, then for held-out channels the plain FP64 LBM from rest
    and from the network's prediction to the same residual.

    The periodic length is odd (511 by default): with an even one, some
    geometries keep an undamped period-2 (staggered) mode of the BGK +
    bounce-back scheme, seen identically in the CPU oracle, and the
    reference's one-step residual then never falls below ~1e-4."""
    import torch

    t0 = time.perf_counter()
    data = make_dataset(list(range(n_train)), per_batch, train_steps, "f32", nx, ny, re_range=re_range, log=log)
    t_data = time.perf_counter() - t0
    flux_guess = None
    if normalize_flux:
        # the network learns the flow pattern per unit flow rate; a held-out
        # channel starts from the training set's median flow rate, which
        # flux_balance then corrects
        train_data = normalize_by_flux(data)
        flux_guess = float(np.median(data["flux"]))
        scales = Scales(float(np.std(train_data["fields"][..., 0][data["fluid"]])) or 1e-3, 1.0)
    else:
        train_data = data
        scales = Scales(float(np.std(data["fields"][..., 0][data["fluid"]])) or 1e-3, 0.08)
    net = UNet(batch, ny, net_width(nx), seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = train(net, train_data, scales, epochs, lr=lr, log=log)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    flops = 3 * net_flops(net) * epochs * (n_train // batch) * batch
    rng = np.random.default_rng(12345)
    rows = []
    for k in range(0, n_eval, per_eval):
        re = float(rng.uniform(*re_range))
        chans = [cases.forced_channel(100000 + k + j, nx, ny, re=re) for j in range(per_eval)]
        cold = run_stack(chans, "f64", max_steps, tol)
        # the same filters applied from rest, to separate their share of the gain from the network's
        rest = rest_p = None
        rest_init = warm_start_populations(chans, [(np.ones((ny, nx)), np.zeros((ny, nx)), np.zeros((ny, nx))) for _ in chans])
        if filtered_rest:
            rest = run_stack(chans, "f64", max_steps, tol, init=rest_init)
            # and with the flow-rate projection, which is physics, not learned
            rest_p = run_stack(chans, "f64", max_steps, tol, init=rest_init, project=project)
        fluid = np.stack([c["flags"] != cases.SOLID for c in chans])

        def err_of(fl):
            u_pred = np.stack([f[1] for f in fl])
            return float(np.linalg.norm((u_pred - cold["ux"])[fluid]) / np.linalg.norm(cold["ux"][fluid]))

        # the network's prediction alone, then with the flow rate balanced
        tp = time.perf_counter()
        fields = predict_fields(net, chans, scales, flux_guess)
        init = warm_start_populations(chans, fields)
        t_pred = time.perf_counter() - tp
        warm_net = run_stack(chans, "f64", max_steps, tol, init=init)
        tp = time.perf_counter()
        fields = predict_fields(net, chans, scales, flux_guess)
        fields_b, alpha = flux_balance(chans, fields)
        init = warm_start_populations(chans, fields_b)
        t_pred_b = time.perf_counter() - tp
        warm = run_stack(chans, "f64", max_steps, tol, init=init, project=project)
        rows.append(dict(re=re, cold_steps=cold["steps"], cold_wall=cold["wall"], cold_res=cold["residual"],
                         rest_filtered_steps=rest["steps"] if rest else None, rest_filtered_wall=rest["wall"] if rest else None,
                         rest_projected_steps=rest_p["steps"] if rest_p else None,
                         rest_projected_wall=rest_p["wall"] if rest_p else None,
                         rest_projected_scales=rest_p["flow_scales"] if rest_p else None, warm_projected_scales=warm["flow_scales"],
                         net_steps=warm_net["steps"], net_wall=warm_net["wall"] + t_pred, ux_rel_l2_net=err_of(fields),
                         warm_steps=warm["steps"], warm_wall=warm["wall"] + t_pred_b, warm_res=warm["residual"], predict_s=t_pred_b,
                         ux_rel_l2_pred=err_of(fields_b), flux_scale=[float(a) for a in alpha]))
        if log:
            log(f"held-out Re {re:.1f}: cold {cold['steps']} steps {cold['wall']:.1f} s; rest+filters "
                f"{rest['steps'] if rest else '-'}; rest+filters+projection {rest_p['steps'] if rest_p else '-'}; "
                f"net {warm_net['steps']} steps (u_x error {err_of(fields):.3e}); "
                f"warm {warm['steps']} steps {warm['wall'] + t_pred_b:.1f} s (u_x error {err_of(fields_b):.3e})")
    cs = sum(r["cold_steps"] for r in rows)
    ws = sum(r["warm_steps"] for r in rows)
    cw = sum(r["cold_wall"] for r in rows)
    ww = sum(r["warm_wall"] for r in rows)
    nw = sum(r["net_wall"] for r in rows)
    rr = [r for r in rows if r["rest_filtered_wall"] is not None]
    rcw = sum(r["cold_wall"] for r in rr)
    return dict(n_train=n_train, train_steps=train_steps, epochs=epochs, dataset_s=t_data, train_s=t_train, final_loss=losses[-1],
                train_tflops=flops / t_train / 1e12, eval=rows, steps_ratio=ws / cs, wall_ratio=ww / cw, net_only_wall_ratio=nw / cw,
                rest_filtered_wall_ratio=(sum(r["rest_filtered_wall"] for r in rr) / rcw) if rr else None,
                rest_projected_wall_ratio=(sum(r["rest_projected_wall"] for r in rr) / rcw) if rr else None,
                project=list(project) if project else None, tol=tol, max_steps=max_steps)


def net_flops(net: "UNet") -> float:
    """Forward multiply-add FLOPs of one sample: 2 cin cout 9 H W per convolution."""
    lvl = {name: w[5] for name, w in net.wiring.items()}
    return float(sum(2 * 9 * cin * cout * (net.H >> lvl[name]) * (net.W >> lvl[name]) for name, cin, cout, _ in net.specs))
