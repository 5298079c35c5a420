"""The device's random sequential addition (dml_gen_ions_batch) against the
oracle's serial generator (oracle/oracle_gen.cpp), bit for bit.

pos_inic (src/dana.F90:330-396) places one ion after another; the device
places a window of ions per round and must reach the same configuration:
the same try accepted for every ion, the same coordinates to the last bit,
and the same failure when some ion cannot be placed.  Cases: axes of one,
two and many cells (every cell once below three), the config-1, config-5
and config-2 ion counts, a batch of config-4 replicas of uneven size up to
the tallest 1 M box, empty systems, and a failing system inside a batch.
"""
import numpy as np
import pytest

from tests import oracle_lib, systems  # noqa: F401  (systems sets sys.path)
import dml

pytestmark = pytest.mark.gpu


def _same(spec):
    want, st = oracle_lib.gen_ions(*spec)
    got, gst, rc = dml.random_ions_batch([spec])
    assert gst[0] == st and rc == st, (spec, gst, st)
    if st == 0:
        assert np.array_equal(got[0].view(np.uint64), want.view(np.uint64)), spec
    return want


@pytest.mark.parametrize("spec", [
    (7, 200, 35.1, 35.1, 10.0, 60.0, 2.5),     # config 1 (14 x 14 x 20 cells)
    (3, 12, 6.0, 6.0, 0.0, 30.0, 2.5),         # two cells along x and y
    (5, 6, 4.0, 4.0, 0.0, 40.0, 3.2),          # one cell along x and y
    (9, 602, 100.0, 100.0, 0.0, 100.0, 3.2),   # the reference's tests/gcmc count (1 M)
    (11, 300, 20.0, 20.0, 0.0, 20.0, 0.0),     # no separation
])
def test_small_systems_match_the_serial_rule(spec):
    _same(spec)


def test_config5_replica_and_config2_system():
    a = _same((11 * 7919, 20000, 140.4, 140.4, 15.0, 300.0, 3.2))
    assert len(a) == 20000
    b = _same((7, 200000, 351.0, 351.0, 15.0, 300.0, 2.5))
    d = np.diff(np.sort(b[:, 2]))
    assert d.max() < 1.0  # spread over the whole height


def test_uneven_batch_with_tall_replicas_empty_and_failing_systems():
    """64 config-4-like replicas (L in 5..40 cells, 50..20 000 ions, 1 M
    height) plus the tallest (20 000 ions over 5 x 5 cells: about 1.3e5 Å),
    an empty system and one that cannot be filled, in one launch."""
    rng = np.random.default_rng(21)
    a = 3.51
    specs = []
    for r in range(64):
        cells = int(rng.integers(5, 41))
        n = int(round(float(np.exp(rng.uniform(np.log(50.0), np.log(20000.0))))))
        L = cells * a
        lz = 10.0 + max(20.0, n / (6.022e-4 * L * L))
        specs.append((1300 + r, n, L, L, 10.0, lz, 3.2))
    L = 5 * a
    specs.append((77, 20000, L, L, 10.0, 10.0 + 20000 / (6.022e-4 * L * L), 3.2))
    specs.append((78, 0, 20.0, 20.0, 0.0, 20.0, 3.2))
    specs.append((79, 1000, 10.0, 10.0, 0.0, 10.0, 5.0))  # cannot be filled
    got, st, rc = dml.random_ions_batch(specs)
    assert rc == dml.E_RSA and st[-1] == dml.E_RSA
    for spec, g, s in zip(specs[:-1], got[:-1], st[:-1]):
        want, ost = oracle_lib.gen_ions(*spec)
        assert ost == 0 and s == 0
        assert np.array_equal(g.view(np.uint64), want.view(np.uint64)), spec
    assert got[-2].shape == (0, 3)
