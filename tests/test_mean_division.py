"""The mean kernels divide an exact integer sum S by the window size N with
a 32-bit multiply-high by m = ceil(2^32 / N).  For |S| < 2^24 and
2 <= N < 256 this equals trunc(S / N), which also equals trunc(fl(S / N))
of the reference's float division (mean_separable_3d_x.cl:24-28 followed by
the truncating convert).  Checked here for every N at the worst case of
every quotient (remainder N - 1) and at exact multiples."""
import numpy as np


def recip32(n):
    return ((1 << 32) + n - 1) // n


def test_multiply_high_equals_integer_division():
    for n in range(2, 256):
        k = np.arange(0, (1 << 24) // n + 1, dtype=np.uint64)
        for s in (k * n, k * n + (n - 1)):
            s = s[s < (1 << 24)]
            q = (s * np.uint64(recip32(n))) >> np.uint64(32)
            assert np.array_equal(q, s // np.uint64(n)), n


def test_integer_division_equals_float_division():
    for n in (2, 3, 5, 7, 11, 13, 31, 61, 127, 255):
        s = np.arange(0, 1 << 24, dtype=np.int64)
        f = np.trunc(s.astype(np.float32) / np.float32(n)).astype(np.int64)
        assert np.array_equal(f, s // n), n
