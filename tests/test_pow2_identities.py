"""The exponent identities the block-step arithmetic uses in place of
divisions (csrc/p3t_phys.cuh: rem_pow2, recip_pow2_or_div): for d = 2^k, a
normal double below 2^1023, the double whose biased exponent is 2046 minus
d's is exactly 1/d, and t * (1/d) is the same double as t / d -- so the
remainder t - floor(t/d) d and the corrector's 1/dt are unchanged bit for
bit.  Checked here on the host's IEEE doubles, the device's being the same
format."""
import numpy as np


def recip_pow2(d):
    b = np.array([d], np.float64).view(np.uint64)[0]
    return np.array([np.uint64(0x7FE0000000000000) - b], np.uint64).view(np.float64)[0]


def test_reciprocal_of_powers_of_two_is_exact():
    for k in range(-1021, 1023):
        d = np.ldexp(1.0, k)
        assert recip_pow2(d) == 1.0 / d, k


def test_product_equals_quotient():
    rng = np.random.default_rng(5)
    t = rng.random(20000) * 10.0 ** rng.integers(-6, 4, 20000)
    for k in range(-60, 8):
        d = np.ldexp(1.0, k)
        np.testing.assert_array_equal(t * recip_pow2(d), t / d)
        np.testing.assert_array_equal(t - np.floor(t * recip_pow2(d)) * d, t - np.floor(t / d) * d)
