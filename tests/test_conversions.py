"""The integer-pipe FP64 <-> FP32 conversions of the mixed path
(gf_d2f / gf_f2d in geoflac_gb300/csrc/gf_kernels.cuh), restated here step
for step with numpy integer operations and checked against IEEE conversion
(numpy's float32 cast rounds to nearest even): equal bits for every normal
result, ties included; signed zero below the float range; infinity above."""
import numpy as np


def d2f(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sign = hi & np.uint32(0x80000000)
    e = ((hi >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 1023 + 127
    m = ((hi & np.uint32(0xFFFFF)) << np.uint32(3)) | (lo >> np.uint32(29))
    rem = lo & np.uint32(0x1FFFFFFF)
    half = np.uint32(0x10000000)
    up = (rem > half) | ((rem == half) & ((m & np.uint32(1)) == 1))
    m = m + up.astype(np.uint32)
    bits = sign + (np.clip(e, 0, 255).astype(np.uint32) << np.uint32(23)) + m
    bits = np.where(e <= 0, sign, bits)
    bits = np.where(e >= 255, sign | np.uint32(0x7F800000), bits)
    return bits.astype(np.uint32).view(np.float32)


def f2d(f):
    u = np.asarray(f, dtype=np.float32).view(np.uint32)
    sign = u & np.uint32(0x80000000)
    e = (u >> np.uint32(23)) & np.uint32(0xFF)
    m = u & np.uint32(0x7FFFFF)
    ed = np.where(e == 255, np.uint32(0x7FF), e.astype(np.int64) - 127 + 1023).astype(np.uint32)
    hi = sign | (ed << np.uint32(20)) | (m >> np.uint32(3))
    bits = (hi.astype(np.uint64) << np.uint64(32)) | ((m & np.uint32(7)).astype(np.uint64) << np.uint64(29))
    bits = np.where(e == 0, sign.astype(np.uint64) << np.uint64(32), bits)
    return bits.view(np.float64)


def test_d2f_rounds_like_ieee_for_normal_results():
    rng = np.random.default_rng(3)
    x = rng.standard_normal(200000) * 10.0 ** rng.uniform(-30, 30, 200000)
    # exact ties between two floats, and values one double ulp either side
    f = rng.standard_normal(20000).astype(np.float32)
    nxt = np.nextafter(f, np.float32(np.inf))
    tie = (f.astype(np.float64) + nxt.astype(np.float64)) / 2
    x = np.concatenate([x, tie, np.nextafter(tie, -np.inf), np.nextafter(tie, np.inf), [0.0, -0.0, 1.0, -2.5]])
    ref = x.astype(np.float32)
    normal = np.abs(ref) >= np.finfo(np.float32).tiny
    assert np.array_equal(d2f(x)[normal].view(np.uint32), ref[normal].view(np.uint32))
    # rounding up across a power of two
    assert d2f(np.array([np.nextafter(2.0, 0.0)]))[0] == np.float32(2.0)


def test_d2f_range_ends():
    tiny = np.array([1e-40, -1e-45, 1e-300])
    out = d2f(tiny)
    assert (out == 0).all() and np.signbit(out[1]) and not np.signbit(out[0])
    big = d2f(np.array([1e39, -1e300]))
    assert np.isinf(big).all() and big[1] < 0


def test_f2d_is_exact_and_splits_recombine():
    rng = np.random.default_rng(4)
    f = (rng.standard_normal(200000) * 10.0 ** rng.uniform(-30, 30, 200000)).astype(np.float32)
    f = f[np.abs(f) >= np.finfo(np.float32).tiny]
    assert np.array_equal(f2d(f), f.astype(np.float64))
    # x = hi + lo with hi = float(x), lo = float(x - hi): as the device splits
    x = rng.uniform(-3e5, 3e5, 100000)
    h = d2f(x)
    lo = d2f(x - f2d(h))
    assert np.array_equal(h, x.astype(np.float32))
    assert np.abs(f2d(h) + f2d(lo) - x).max() <= np.abs(x).max() * 2.0 ** -47
