"""The 16-bit storage LBM_STORE_E3M12_DEV (1 sign, 3 exponent, 12 mantissa
bits of s / 1024; lbm_gb300/csrc/step_common.cuh, e3m12_encode /
e3m12_decode) against the rounding the storage study emulates
(oracle/storage_floor.c, store 7: round to 13 significant bits, exponent
floor 2^-6, saturating at 2 - 2^-12).

The device functions are integer operations on FP32 bit patterns, one
FP32-to-integer conversion with round-to-nearest-even and products by
powers of two, all exact; the NumPy lines below perform the same operations
on the same bit patterns, so they give the device's codes.  Every FP32 value
of the ranges that matter, and ties, must round as the study rounds.
"""
import numpy as np


def encode(s):
    s = np.ascontiguousarray(s, dtype=np.float32)
    u = s.view(np.uint32)
    a = u & np.uint32(0x7FFFFFFF)
    r = a + np.uint32(0x3FF) + ((a >> np.uint32(11)) & np.uint32(1))
    with np.errstate(over="ignore", invalid="ignore"):  # each branch is only used where it applies
        normal = np.minimum((r >> np.uint32(11)) - np.uint32(130 << 12), np.uint32(0x7FFF))
        small = np.rint(np.minimum(a.view(np.float32), np.float32(16.0)) * np.float32(256.0)).astype(np.uint32)
    code = np.where(a >= np.uint32(0x41800000), normal, small) | ((u >> np.uint32(16)) & np.uint32(0x8000))
    return code.astype(np.uint16)


def decode(c):
    c = np.asarray(c, dtype=np.uint32)
    bits = ((c & np.uint32(0x7FFF)) << np.uint32(11)) | ((c & np.uint32(0x8000)) << np.uint32(16))
    return bits.astype(np.uint32).view(np.float32) * np.float32(2.0 ** 127) * np.float32(8.0)


def study_rounding(s):
    """storage_floor.c store 7, in FP64: round_fp(s / 4096 * 4, 13, -6, 2 - 2^-12) / 4 * 4096."""
    t = np.asarray(s, dtype=np.float64) / 1024.0
    a = np.abs(t)
    maxv = 2.0 - 2.0 ** -12
    _, e = np.frexp(a)
    lead = np.maximum(e - 1, -6)
    q = np.ldexp(1.0, lead - 12)
    r = np.rint(a / q) * q
    r = np.where(a >= maxv, maxv, r)
    r = np.where(a == 0, 0.0, r)
    return np.copysign(r, t) * 1024.0


def test_random_values_round_as_the_study():
    rng = np.random.default_rng(7)
    mag = np.exp(rng.uniform(np.log(1e-6), np.log(1e4), 4_000_000)).astype(np.float32)
    s = np.where(rng.random(mag.size) < 0.5, -mag, mag).astype(np.float32)
    got = decode(encode(s)).astype(np.float64)
    want = study_rounding(s)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, (s[bad[:5]], got[bad[:5]], want[bad[:5]])


def test_ties_boundaries_and_saturation():
    # every representable code and the midpoints between neighbours
    codes = np.arange(0, 0x8000, dtype=np.uint32)
    vals = decode(codes).astype(np.float64)
    assert np.all(np.diff(vals) > 0)                       # monotonic, no gaps or overlaps
    assert vals[0x1000] == 16.0 and vals[0x7FFF] == (2.0 - 2.0 ** -12) * 1024
    assert np.array_equal(encode(vals.astype(np.float32)), codes.astype(np.uint16))  # exact round trip
    mids = ((vals[1:] + vals[:-1]) / 2).astype(np.float32)  # exact in FP32: 14 significant bits at most
    assert np.array_equal(mids.astype(np.float64), (vals[1:] + vals[:-1]) / 2)
    got = decode(encode(mids)).astype(np.float64)
    assert np.array_equal(got, study_rounding(mids))        # ties to even, as the study
    big = np.array([2047.9, 2048.0, 3000.0, 1e30, np.inf], dtype=np.float32)
    assert np.all(decode(encode(big)) == np.float32((2.0 - 2.0 ** -12) * 1024))
    assert np.all(decode(encode(-big)) == -np.float32((2.0 - 2.0 ** -12) * 1024))
    z = decode(encode(np.array([0.0, -0.0], dtype=np.float32)))
    assert z[0] == 0 and z[1] == 0


def test_precision_over_the_shifted_state_range():
    """13 significant bits from |s| = 16 up to the saturation at 2048 - 1/2
    (FP16: 11), and an absolute spacing of 2^-8 below 16."""
    s = np.float32(16.0) * np.float32(1.0 + 2.0 ** -13)
    assert abs(float(decode(encode([s]))[0]) - float(s)) <= 16.0 * 2.0 ** -13
    x = np.linspace(0.001, 15.99, 100_001).astype(np.float32)
    assert np.max(np.abs(decode(encode(x)).astype(np.float64) - x)) <= 2.0 ** -9
