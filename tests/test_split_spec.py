"""The bit algorithm of split_tf32_fast (apyib_gb300/csrc/fsplit.cuh), restated on the two
32-bit words of each FP64 value with NumPy integer operations, step for step: x = hi + lo
with both parts TF32 (low 13 FP32 mantissa bits zero) and |x - hi - lo| <= 2^-23 |x| for
|x| in the FP32 normal range, over 60 decades, signs, rounding carries into the exponent
and negative remainders.  The device code is exercised by the 3xTF32 GEMM accuracy tests;
this pins the algorithm those tests rely on."""
import numpy as np


def split_tf32_fast(x):
    u = np.asarray(x, dtype=np.float64).view(np.uint64)
    hw = (u >> np.uint64(32)).astype(np.uint32)
    lw = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sign = hw & np.uint32(0x80000000)
    e = ((hw >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64)
    hr = (hw + np.uint32(0x200)) & np.uint32(0xFFFFFC00)
    eh = ((hr >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64)
    hi = sign | (((eh - 896).clip(0, 255)).astype(np.uint32) << np.uint32(23)) | \
        ((hr & np.uint32(0x000FFC00)) << np.uint32(3))
    hi = np.where(e > 896, hi, sign)
    q = (((hw & np.uint32(0x3FF)) << np.uint32(22)) | (lw >> np.uint32(10))).view(np.int32)
    qf = q.astype(np.float32).view(np.uint32).astype(np.int64)
    sh = e - 1023 - 42
    ne = ((qf >> 23) & 0xFF) + sh
    lo = np.where((q != 0) & (ne > 0) & (e > 896), (qf + (sh << 23)) & 0xFFFFFFFF, 0).astype(np.uint32)
    lo = (lo + np.uint32(0x1000)) & np.uint32(0xFFFFE000)
    lo = lo ^ sign
    return hi.view(np.float32), lo.view(np.float32)


def test_split_tf32_fast_spec():
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.standard_normal(200000) * 10.0 ** rng.integers(-30, 30, 200000),
        np.array([0.0, -0.0, 1.0, -1.0, 1.0 - 2 ** -53, 2.0 - 2 ** -40, 1.0 + 2 ** -11, 1.0 + 2 ** -11 + 2 ** -40,
                  -(1.0 + 2 ** -11), 65000.0, 1.5, 2.0 ** -126, 3.0e38, -2.0 ** 100 * (1 - 2 ** -30)])])
    hi, lo = split_tf32_fast(x)
    assert np.all((hi.view(np.uint32) & 0x1FFF) == 0)
    assert np.all((lo.view(np.uint32) & 0x1FFF) == 0)
    err = np.abs(x - (hi.astype(np.float64) + lo.astype(np.float64)))
    normal = (np.abs(x) >= 2.0 ** -100) & (np.abs(x) < 3.3e38)
    assert np.all(err[normal] <= 2.0 ** -23 * np.abs(x[normal]))
    assert np.all(hi[np.abs(x) < 2.0 ** -126] == 0) and np.all(lo[np.abs(x) < 2.0 ** -126] == 0)
    # hi is x rounded to 11 significant bits (half away from zero)
    big = normal & (np.abs(x) > 0)
    assert np.all(np.abs(hi[big].astype(np.float64) - x[big]) <= 2.0 ** -11 * np.abs(x[big]))
