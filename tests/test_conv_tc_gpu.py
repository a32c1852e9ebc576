"""The warm-start network's 3x3 convolution on the tcgen05 tensor-core kernel
(lbm_gb300/csrc/conv_tc.cu) against an FP64 convolution of the same
BF16-rounded activations and weights, and against the mma.sync kernel.

Every shape class the U-Net uses: image rows of 128 pixels or more (one row
segment per 128-pixel tile) and narrower images (128 / W whole rows per tile,
W = 64, 32, 16); input channels 32-256 read from a wider buffer (a
concatenation view, ldx > cin); 32-256 output channels written into a
channel offset of a wider buffer; ReLU or not; BF16 or FP32 output.  FP32
output agrees to FP32 accumulation error (relative 1e-5 of the output scale);
BF16 output to one BF16 rounding (2^-8 relative) plus that.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# B, H, W, cin, ldx, cout, ldy, offy, relu, out_f32
SHAPES = [
    (2, 4, 256, 32, 32, 32, 32, 0, True, False),
    (1, 6, 128, 64, 64, 64, 128, 64, True, False),
    (2, 16, 64, 32, 64, 128, 128, 0, False, False),
    (1, 16, 32, 128, 256, 256, 256, 0, True, False),
    (2, 8, 16, 256, 256, 64, 64, 0, True, False),
    (1, 8, 512, 64, 64, 32, 32, 0, False, True),
    (2, 32, 64, 32, 32, 32, 32, 0, False, True),
]


def _lib():
    from lbm_gb300.warmstart import nn_lib

    return nn_lib()


def _bf16(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16)


def _reference(x, w, bias, relu):
    """FP64 3x3 convolution, zero padding 1: x (B,H,W,cin), w (cout, 3, 3, cin)."""
    B, H, W, cin = x.shape
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((B, H, W, w.shape[0]))
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W], w[:, ky, kx, :])
    y += bias
    return np.maximum(y, 0.0) if relu else y


def _run(lib, shape, path, seed=0):
    import torch

    B, H, W, cin, ldx, cout, ldy, offy, relu, out_f32 = shape
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda", 0)
    xbuf = _bf16(rng.normal(size=(B, H, W, ldx))).to(dev)
    w16 = _bf16(rng.normal(size=(cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin))).to(dev)
    bias = torch.from_numpy(rng.normal(size=cout).astype(np.float32) * 0.1).to(dev)
    ydt = torch.float32 if out_f32 else torch.bfloat16
    y = torch.full((B, H, W, ldy), 7.0, dtype=ydt, device=dev)  # untouched channels must keep this
    assert lib.lbm_nn_set_conv_path(path) == 0
    stream = torch.cuda.current_stream(dev).cuda_stream
    uses = lib.lbm_nn_conv_uses_tc(xbuf.data_ptr(), ldx, w16.data_ptr(), y.data_ptr(), ldy, offy, B, H, W, cin, cout, int(out_f32))
    rc = lib.lbm_nn_conv3x3_fwd(xbuf.data_ptr(), ldx, w16.data_ptr(), bias.data_ptr(), y.data_ptr(), ldy, offy, B, H, W, cin, cout,
                                int(relu), int(out_f32), C.c_void_p(stream))
    assert rc == 0
    assert lib.lbm_nn_conv_status(C.c_void_p(stream)) == 0
    lib.lbm_nn_set_conv_path(0)
    x = xbuf.float().cpu().numpy()[..., :cin].astype(np.float64)
    wt = w16.float().cpu().numpy().astype(np.float64).reshape(cout, 3, 3, cin)
    ref = _reference(x, wt, bias.cpu().numpy().astype(np.float64), relu)
    return uses, y.float().cpu().numpy(), ref


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "B{}H{}W{}_cin{}of{}_cout{}of{}at{}_{}_{}".format(
    s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], "relu" if s[8] else "lin", "f32" if s[9] else "bf16"))
def test_tensor_core_convolution_matches_fp64(shape):
    lib = _lib()
    uses, y, ref = _run(lib, shape, 0)
    assert uses == 1, "this shape qualifies for the tensor-core kernel"
    _, _, _, _, _, cout, ldy, offy, _, out_f32 = shape
    got = y[..., offy:offy + cout]
    scale = float(np.abs(ref).max())
    err = np.abs(got - ref)
    bound = 1e-5 * scale + (0.0 if out_f32 else 2.0 ** -8 * np.abs(ref))
    assert np.all(err <= bound), (float(err.max()), scale)
    # the channels outside [offy, offy + cout) are untouched
    rest = np.concatenate([y[..., :offy], y[..., offy + cout:]], axis=-1)
    assert np.all(rest == 7.0)


@pytest.mark.parametrize("shape", SHAPES[:4])
def test_tensor_core_and_mma_sync_kernels_agree(shape):
    lib = _lib()
    _, y_tc, ref = _run(lib, shape, 0, seed=4)
    uses, y_mma, _ = _run(lib, shape, 1, seed=4)
    assert uses == 0
    _, _, _, _, _, cout, _, offy, _, out_f32 = shape
    a, b = y_tc[..., offy:offy + cout], y_mma[..., offy:offy + cout]
    scale = float(np.abs(ref).max())
    tol = 2e-5 * scale + (0.0 if out_f32 else 2.0 ** -7 * np.abs(ref))
    assert np.all(np.abs(a - b) <= tol)


def test_shapes_outside_the_tensor_core_kernel_fall_back():
    """cout above 256, or an image narrower than 128 whose height is not a
    multiple of 128 / W, runs on the mma.sync kernel (and stays correct)."""
    import torch

    lib = _lib()
    dev = torch.device("cuda", 0)
    x = torch.zeros((1, 4, 8, 32), dtype=torch.bfloat16, device=dev)
    w = torch.zeros((320, 9 * 32), dtype=torch.bfloat16, device=dev)
    y = torch.zeros((1, 4, 8, 320), dtype=torch.bfloat16, device=dev)
    assert lib.lbm_nn_conv_uses_tc(x.data_ptr(), 32, w.data_ptr(), y.data_ptr(), 320, 0, 1, 4, 8, 32, 320, 0) == 0  # cout 320
    assert lib.lbm_nn_conv_uses_tc(x.data_ptr(), 32, w.data_ptr(), y.data_ptr(), 32, 0, 1, 4, 8, 32, 32, 0) == 0  # 4 rows of 8 < 16
    assert lib.lbm_nn_conv_uses_tc(x.data_ptr(), 32, w.data_ptr(), y.data_ptr(), 32, 0, 1, 16, 8, 32, 32, 0) == 1
    uses, y, ref = _run(lib, (1, 4, 8, 32, 32, 64, 64, 0, True, False), 0)
    assert uses == 0
    assert np.all(np.abs(y - ref) <= 1e-5 * float(np.abs(ref).max()) + 2.0 ** -8 * np.abs(ref))


def test_pipeline_wait_that_runs_out_reports_status_without_a_fault():
    """With a 1 ms limit and every CTA's first K chunk left unloaded, the
    tensor-core convolution's bounded waits run out: lbm_nn_conv_status
    reports -6, and with the defaults restored the same call is correct
    again (the context stayed usable)."""
    import torch

    lib = _lib()
    dev = torch.device("cuda", 0)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    shape = SHAPES[2]
    B, H, W, cin, ldx, cout, ldy, offy, relu, out_f32 = shape
    x = torch.zeros((B, H, W, ldx), dtype=torch.bfloat16, device=dev)
    w = torch.zeros((cout, 9 * cin), dtype=torch.bfloat16, device=dev)
    b = torch.zeros(cout, dtype=torch.float32, device=dev)
    y = torch.zeros((B, H, W, ldy), dtype=torch.bfloat16, device=dev)
    assert lib.lbm_nn_conv_uses_tc(x.data_ptr(), ldx, w.data_ptr(), y.data_ptr(), ldy, offy, B, H, W, cin, cout, 0) == 1
    assert lib.lbm_nn_conv_test_wait(1_000_000, 1) == 0
    try:
        assert lib.lbm_nn_conv3x3_fwd(x.data_ptr(), ldx, w.data_ptr(), b.data_ptr(), y.data_ptr(), ldy, offy, B, H, W, cin, cout,
                                      int(relu), 0, stream) == 0
        assert lib.lbm_nn_conv_status(stream) == -6
    finally:
        assert lib.lbm_nn_conv_test_wait(200_000_000, 0) == 0
    assert lib.lbm_nn_conv_test_wait(0, 0) == -1 and lib.lbm_nn_conv_test_wait(1000, 2) == -1
    uses, out, ref = _run(lib, shape, 0)
    assert uses == 1
    got = out[..., offy:offy + cout]
    assert np.all(np.abs(got - ref) <= 1e-5 * float(np.abs(ref).max()) + 2.0 ** -8 * np.abs(ref))
