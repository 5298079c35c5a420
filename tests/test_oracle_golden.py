"""The oracle is pinned against the reference's own known-answer tests.

tests/{ermak,brown,gcmc}/ref.xyz of the reference hold the last frame of
three full runs (Ermak + piston, Brownian + chunks, Brownian + GCMC).  The
oracle in NR random-number mode must reproduce every coordinate bit for bit.
"""
import os

import numpy as np
import pytest

from tests import oracle_lib

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference")


@pytest.mark.parametrize("case", ["ermak", "brown", "gcmc"])
def test_reference_golden_bit_exact(case):
    d = os.path.join(GOLD, case)
    ref_pos, ref_z, ref_zmax = oracle_lib.read_xyz_frame(os.path.join(d, "ref.xyz"))
    pos, z, zmax, _ = oracle_lib.run_reference_case(d)
    assert pos.shape == ref_pos.shape
    assert np.array_equal(z, ref_z)
    # bit-exact: compare the raw 64-bit patterns
    assert np.array_equal(pos.view(np.uint64), ref_pos.view(np.uint64))
    assert zmax == ref_zmax
