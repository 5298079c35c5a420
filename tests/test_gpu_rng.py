"""The device's Box-Muller normals against the host build of the same
header (include/dml_rng.h), bit for bit.

Both the plain and the chosen form draw their Ermak, Brownian and Maxwell
noise through dml_normal_pair32f.  On the device its integer-to-float steps
(RN32(a + 1), the angle fraction, the exponent of the log) are integer
operations, because GB300 issues conversion instructions on its narrow FP64
pipe; they must give the conversions' own results.  Checked over random
words and the edges: a = 0 and a = 2^32 - 1 (u1 = 1), words whose a + 1 is
a rounding tie (round to even, with and without a carry into the next
binade), every quadrant boundary of the angle and the words next to them.
"""
import numpy as np
import pytest

from tests import oracle_lib
import dml

pytestmark = pytest.mark.gpu


def host_normals(words):
    w = np.ascontiguousarray(words, np.uint32)
    out = np.zeros(w.shape, np.float32)
    oracle_lib.load().orc_rng_normal_pairs(w.ctypes.data, w.size // 2, out.ctypes.data)
    return out


def test_device_normals_equal_host_normals():
    dml.build()
    rng = np.random.default_rng(11)
    a = list(rng.integers(0, 2 ** 32, 300000, dtype=np.uint64))
    b = list(rng.integers(0, 2 ** 32, 300000, dtype=np.uint64))
    edges_a = [0, 1, 2, 0xFFFFFFFF, 0xFFFFFFFE, 0xFFFFFF7F, 0xFFFFFF80, 0xFFFFFF81,
               0x00FFFFFF, 0x00FFFFFE, 0x01000000, 0x01000001, 0x01000002, 0x7FFFFF3F,
               0x7FFFFF40, 0x7FFFFFBF, 0x7FFFFFC0, 0x80000000, 0x8000007F, 0x80000080]
    edges_b = []
    for q in range(4):
        x = q << 22
        for dx in (-1, 0, 1, 0x200000 - 1, 0x200000, 0x200001):
            edges_b.append((((x + dx) & 0xFFFFFF) << 8) | 0xAB)
    for ea in edges_a:
        for eb in edges_b[:8]:
            a.append(ea)
            b.append(eb)
    for eb in edges_b:
        a.append(12345)
        b.append(eb)
    w = np.empty(2 * len(a), np.uint32)
    w[0::2] = np.array(a, np.uint64).astype(np.uint32)
    w[1::2] = np.array(b, np.uint64).astype(np.uint32)
    got = dml.check_normals(w, dml.PRECISION_FP64)
    want = host_normals(w)
    bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    assert len(bad) == 0, (len(bad), w[2 * (bad[0] // 2)], w[2 * (bad[0] // 2) + 1])
    assert np.isfinite(got).all()
    assert abs(float(got.mean())) < 0.01 and abs(float(got.var()) - 1.0) < 0.01


def test_chosen_form_normals_close_to_exact_ones():
    """The chosen form's integrators take the same words through the
    hardware's approximate log2, sin and cos.  The log2 error is absolute
    (about 2^-22), so the radius r = sqrt(-2 ln u1) is within 2e-6 (1 + r)
    of the exact one where r > 0.05, and within 1e-3 where r is smaller
    (u1 within 1e-3 of 1); standard moments, tails to 6.6 sigma."""
    rng = np.random.default_rng(12)
    n = 400000
    w = rng.integers(0, 2 ** 32, 2 * n, dtype=np.uint64).astype(np.uint32)
    w[0], w[2], w[4] = 0xFFFFFFFF, 0, 1  # u1 = 1 and the two smallest u1
    fast = dml.check_normals(w, dml.PRECISION_MIXED)
    exact = host_normals(w)
    assert np.isfinite(fast).all()
    r = np.hypot(exact[0::2].astype(np.float64), exact[1::2]).repeat(2)
    diff = np.abs(fast.astype(np.float64) - exact)
    big = r > 0.05
    assert (diff[big] / (1.0 + r[big])).max() < 2e-6
    assert diff.max() < 1e-3
    assert fast[0] == 0.0 and fast[1] == 0.0
    assert np.abs(fast[2:6]).max() > 6.0
    v = fast[6:].astype(np.float64)
    assert abs(v.mean()) < 0.005 and abs(v.var() - 1.0) < 0.005
    assert abs((v ** 4).mean() - 3.0) < 0.05

