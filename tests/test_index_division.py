"""The variable-order kernels decode item and face indices with an FP32-reciprocal quotient
(dg_var.cuh: quot): q = trunc((n + 1/2) * rn(1/d)). This checks, with IEEE single-precision
arithmetic on the host (numpy float32: correctly rounded reciprocal, product and sum), that it equals
the integer quotient for every n < 2^15 and divisor d <= 1024. The kernels decode item nodes
(n < 1024, d = the element's node count <= 512 or a line length <= 8 or a plane <= 64), trace tasks
of an item (n <= 3 x 1024, d = an element's 6 P^2 face points <= 384) and face points (n < 64,
d <= 8)."""
import numpy as np


def test_fp32_reciprocal_quotient_is_exact():
    n = np.arange(1 << 15, dtype=np.int64)
    nf = n.astype(np.float32) + np.float32(0.5)
    for d in range(1, 1025):
        r = np.float32(1.0) / np.float32(d)
        q = np.trunc(nf * r).astype(np.int64)
        assert np.array_equal(q, n // d), d
