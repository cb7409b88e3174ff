"""The FP64 pass compares projections as unsigned integer keys
(ordered_key in k_prec_fp64): -0 is made +0, then a negative double's bits
are inverted and a non-negative one's sign bit is set. For finite doubles
the key order must be the double order, with -0 == +0, so that the pass's
min / max / strict comparisons give the FP64 formula's answer."""
import numpy as np


def ordered_key(d):
    b = np.asarray(d, dtype=np.float64).view(np.uint64).copy()
    sign = np.uint64(1 << 63)
    b[b == sign] = 0
    neg = (b & sign) != 0
    return np.where(neg, ~b, b | sign)


def test_key_order_is_double_order():
    rng = np.random.default_rng(7)
    x = np.concatenate([
        rng.standard_normal(20000) * 10.0 ** rng.uniform(-300, 300, 20000),
        np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, -2.2250738585072014e-308,
                  1.7976931348623157e308, -1.7976931348623157e308, 1.0, -1.0]),
        rng.standard_normal(2000) * 1e-310,  # subnormals
    ])
    i = rng.integers(0, len(x), 200000)
    j = rng.integers(0, len(x), 200000)
    a, b = x[i], x[j]
    ka, kb = ordered_key(a), ordered_key(b)
    assert np.array_equal(ka < kb, a < b)
    assert np.array_equal(ka == kb, a == b)  # -0 == +0 included
    assert np.array_equal(ka > kb, a > b)
