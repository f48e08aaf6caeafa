"""The ray kernel walks RayIterator in closed form: after k steps axis b has
moved n_b(k) = floor((2 k d_b + max) / (2 max)) cells. This checks that form
(and its incremental stride-W update) against the iterative Bresenham of
probabilistic_map.hpp:162-203 for every delta in [-12, 12]^3."""
import itertools

import numpy as np
import pytest


def iterative(d):
    m = max(abs(v) for v in d)
    if m == 0:
        return []
    s = [(-1 if v < 0 else 1) for v in d]
    a = [abs(v) for v in d]
    err = [0, 0, 0]
    c = [0, 0, 0]
    out = [tuple(c)]
    for _ in range(m - 1):
        for k in range(3):
            err[k] += a[k]
        for k in range(3):
            if (err[k] << 1) >= m:
                c[k] += s[k]
                err[k] -= m
        out.append(tuple(c))
    return out


def closed(d):
    m = max(abs(v) for v in d)
    if m == 0:
        return []
    return [tuple((-1 if v < 0 else 1) * ((2 * k * abs(v) + m) // (2 * m)) for v in d)
            for k in range(m)]


def strided(d, W):
    """The kernel's per-lane (n, r) state advanced by the quotient/remainder of
    2*W*d by 2*max."""
    m = max(abs(v) for v in d)
    if m == 0:
        return []
    cells = [None] * m
    for lane in range(W):
        st = []
        for v in d:
            a = abs(v)
            n, r = divmod(2 * lane * a + m, 2 * m)
            Q, R = divmod(2 * W * a, 2 * m)
            st.append([n, r, Q, R, -1 if v < 0 else 1])
        k = lane
        while k < m:
            cells[k] = tuple(s[4] * s[0] for s in st)
            for s in st:
                s[0] += s[2]
                s[1] += s[3]
                if s[1] >= 2 * m:
                    s[0] += 1
                    s[1] -= 2 * m
            k += W
    return cells


def test_closed_form_exhaustive():
    r = range(-12, 13)
    for d in itertools.product(r, r, r):
        assert closed(d) == iterative(d), d


@pytest.mark.parametrize("W", [1, 8, 16, 32])
def test_strided_matches(W):
    r = range(-9, 10, 2)
    for d in itertools.product(r, r, r):
        assert strided(d, W) == iterative(d), (d, W)
    rng = np.random.default_rng(W)
    for d in rng.integers(-400, 401, (200, 3)):
        d = tuple(int(x) for x in d)
        assert strided(d, W) == closed(d)


def test_float_divmod_estimate_exact():
    """divmod_small's float estimate + one correction equals exact divmod for
    the ranges the kernel uses (quotient < 2^20)."""
    rng = np.random.default_rng(0)
    for _ in range(20000):
        den = int(rng.integers(2, 2 ** 27))
        q_true = int(rng.integers(0, 64))
        num = min(q_true * den + int(rng.integers(0, den)), 2 ** 32 - 1)
        rden = np.float32(1.0) / np.float32(den)
        qe = int(np.float32(num) * rden)  # truncation like __fmul_rz + cvt
        rr = num - qe * den
        while rr < 0:
            qe -= 1
            rr += den
        while rr >= den:
            qe += 1
            rr -= den
        assert (qe, rr) == divmod(num, den)
