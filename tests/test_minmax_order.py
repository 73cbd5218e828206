"""The float minimum / maximum of the fused separables and the line passes
evaluate the reference's loop (res = centre, then res = min(res, x) over the
taps with OpenCL's min: x < res ? x : res; max alike) as the van Herk /
Gil-Werman split with the operator "the earlier operand unless the later one
is strictly more extreme or the earlier one is NaN", taking the centre first
unless it is NaN.  This restates that evaluation order in numpy and checks
it bit for bit against the reference loop on windows full of NaNs, signed
zeros and infinities (no GPU)."""
import numpy as np
import pytest


def ref_loop(w, R, is_max):
    res = w[R]
    for x in w:
        if (res < x) if is_max else (x < res):
            res = x
    return res


def first(a, b, is_max):
    take = ((a < b) if is_max else (b < a)) or (a != a)
    return b if take else a


def van_herk(w, M, R, is_max):
    """Outputs j = 0..M-1 over w[j .. j+2R] (len(w) = M + 2R), 2R >= M."""
    suf = [None] * M
    suf[M - 1] = w[M - 1]
    for j in range(M - 2, -1, -1):
        suf[j] = first(w[j], suf[j + 1], is_max)
    pre = w[M]
    for k in range(M + 1, 2 * R + 1):
        pre = first(pre, w[k], is_max)
    out = [first(suf[0], pre, is_max)]
    for j in range(1, M):
        pre = first(pre, w[j + 2 * R], is_max)
        out.append(first(suf[j], pre, is_max))
    res = []
    for j in range(M):
        c = w[j + R]
        res.append(c if c != c else first(c, out[j], is_max))
    return res


@pytest.mark.parametrize("is_max", [False, True])
@pytest.mark.parametrize("M,R", [(8, 4), (8, 5), (8, 8), (4, 2), (4, 3), (8, 15), (8, 30)])
def test_van_herk_with_leftmost_rule_equals_reference_loop(is_max, M, R):
    rng = np.random.default_rng(100 * M + R + (7 if is_max else 0))
    pool = np.array([np.nan, 0.0, -0.0, np.inf, -np.inf, 1.0, -1.0, 2.5, -2.5], dtype=np.float32)
    for _ in range(400):
        n = M + 2 * R
        w = rng.choice(pool, size=n).astype(np.float32)
        if rng.random() < 0.5:  # some windows with ordinary values between the special ones
            k = rng.random(n) < 0.5
            w[k] = (rng.standard_normal(int(k.sum())) * 3).astype(np.float32)
        got = van_herk(list(w), M, R, is_max)
        for j in range(M):
            want = ref_loop(list(w[j:j + 2 * R + 1]), R, is_max)
            assert np.float32(got[j]).tobytes() == np.float32(want).tobytes(), (w, j)
