"""The shared random-stream header (include/dml_rng.h), host build.

Checks the Philox4x32-10 core against the known-answer vectors published with
the Random123 library (Salmon et al., SC'11), and the project-written log and
sin/cos against libm within the stated error bounds.
"""
import ctypes
import math

import numpy as np

from tests import oracle_lib


def philox_ref(c0, c1, c2, c3, k0, k1):
    """Pure-Python Philox4x32-10 (independent restatement for the test)."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    m32 = 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & m32, p1 & m32, ((p0 >> 32) ^ c3 ^ k1) & m32, p0 & m32
        k0 = (k0 + W0) & m32
        k1 = (k1 + W1) & m32
    return [c0, c1, c2, c3]


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10.
    assert philox_ref(0, 0, 0, 0, 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox_ref(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF) == \
        [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox_ref(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_draw_matches_python_philox():
    lib = oracle_lib.load()
    out = np.zeros(4, np.uint32)
    for seed, step, aid, stream, sub in [(0, 0, 0, 0, 0), (12345, 7, 99, 1, 2),
                                         (2**63 + 5, 2**40 + 3, 2**33 + 17, 4, 9)]:
        lib.orc_rng_draw(seed, step, aid, stream, sub, out.ctypes.data)
        st = step & (2**64 - 1)
        c = [aid & 0xFFFFFFFF, ((stream << 24) | (sub & 0xFFFFFF)) & 0xFFFFFFFF, st & 0xFFFFFFFF,
             ((st >> 32) ^ (aid >> 32)) & 0xFFFFFFFF]
        assert list(out) == philox_ref(*c, seed & 0xFFFFFFFF, seed >> 32)


def test_log_accuracy():
    lib = oracle_lib.load()
    rng = np.random.default_rng(1)
    xs = np.concatenate([(rng.integers(0, 2**32, 20000) + 1.0) * 2.0**-32,
                         [2.0**-32, 0.5, 1.0, 0.70710678, 0.75]]).astype(np.float32)
    worst = 0.0
    for x in xs:
        got = lib.orc_rng_logf(float(x))
        ref = math.log(float(x))
        if ref != 0.0:
            worst = max(worst, abs(got - ref) / abs(ref))
        else:
            assert got == 0.0
    assert worst < 2e-7


def test_sincos_accuracy():
    lib = oracle_lib.load()
    s, c = ctypes.c_float(), ctypes.c_float()
    rng = np.random.default_rng(2)
    us = np.floor(rng.random(20000) * 2.0**24) / 2.0**24
    us = np.concatenate([us, [0.0, 0.125, 0.25, 0.375, 0.5, 0.75, 1 - 2.0**-24]])
    worst = 0.0
    for u in us:
        lib.orc_rng_sincosf_2pi(float(u), ctypes.byref(s), ctypes.byref(c))
        a = 2.0 * math.pi * float(u)
        worst = max(worst, abs(s.value - math.sin(a)), abs(c.value - math.cos(a)))
    assert worst < 2e-7


def test_normals_moments():
    lib = oracle_lib.load()
    w = np.zeros(4, np.uint32)
    n = np.zeros(4)
    vals = []
    for i in range(10000):
        lib.orc_rng_draw(7, i, 3, 1, 0, w.ctypes.data)
        lib.orc_rng_normal_quad(w.ctypes.data, n.ctypes.data)
        vals += list(n)
    v = np.array(vals)
    assert abs(v.mean()) < 0.02
    assert abs(v.var() - 1.0) < 0.03
    assert abs((v**4).mean() - 3.0) < 0.15
    # independence of the two pairs of one draw
    a = v.reshape(-1, 4)
    assert abs(np.corrcoef(a[:, 0], a[:, 2])[0, 1]) < 0.03
