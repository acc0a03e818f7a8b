"""The division sweeps' float -> double widening (widen_scaled in
cuda-pro-cell_gb300/csrc/pc_sweeps.cuh), restated on the bits with numpy: shifting the
float's bits arithmetically by 3, masking with 0x8FFFFFFF and appending the low 3 mantissa
bits gives exactly z x 2^-896 for every finite float, zero and subnormals included. The sweeps
pair it with sd stored as sd x 2^896 (an exact scaling), so the fused product, and the timer
fma(sd, z, mean), are those of the unscaled values bit for bit."""
from fractions import Fraction

import numpy as np

SHIFT = 896


def widen_scaled(z):
    f = np.asarray(z, dtype=np.float32).view(np.uint32)
    hi = ((f.view(np.int32) >> 3).view(np.uint32) & np.uint32(0x8FFFFFFF)).astype(np.uint64)
    lo = (f << np.uint32(29)).astype(np.uint64)
    return ((hi << np.uint64(32)) | lo).view(np.float64)


def test_widen_is_an_exact_power_of_two_scaling():
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2 ** 32, size=2_000_000, dtype=np.uint64).astype(np.uint32)
    z = bits.view(np.float32)
    z = z[np.isfinite(z)]
    special = np.array([0.0, -0.0, 1.0, -1.0, 1e-10, -1e-10, 3.4028235e38, -3.4028235e38,
                        1.17549435e-38, 1.4e-45, -1.4e-45, 5.877472e-39], dtype=np.float32)
    z = np.concatenate([z, special])
    got = widen_scaled(z)
    want = np.ldexp(z.astype(np.float64), -SHIFT)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_scaled_product_is_the_product():
    rng = np.random.default_rng(2)
    for sd, z in zip(rng.uniform(-50.0, 50.0, 200), rng.standard_normal(200).astype(np.float32)):
        s = np.ldexp(float(sd), SHIFT)
        w = float(widen_scaled(np.float32(z)))
        assert Fraction(s) * Fraction(w) == Fraction(float(sd)) * Fraction(float(z))
