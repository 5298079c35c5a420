"""Chosen (mixed-precision) force form: error statistics against the FP64 path.

At identical positions the mixed form (FP32 pair math on FP64 differences,
int64 fixed-point sums) must give forces within 1e-6 relative of the
bit-exact FP64 path.  The error metric has a floor: |dF| / max(|F|, F_rms),
because near the cut-off the WCA force goes to zero.  Sums are order
independent, so repeated runs give identical bits.
"""
import numpy as np
import pytest

from tests import systems
import dml

pytestmark = pytest.mark.gpu

TOL_FORCE = 1e-6   # max relative force error (with the F_rms floor)
TOL_ENERGY = 1e-6  # relative error of the total potential energy


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def force_error(atoms, params):
    pp = systems.c1_params() if params is None else params
    pm = systems.c1_params() if params is None else params
    pp.precision = dml.PRECISION_FP64
    g64 = dml.Simulation(pp)
    g64.set_atoms(atoms)
    g64.setup()
    import copy

    pm = copy.copy(pp)
    pm.precision = dml.PRECISION_MIXED
    g32 = dml.Simulation(pm)
    g32.set_atoms(atoms)
    g32.setup()
    a, b = g64.get_atoms(), g32.get_atoms()
    f64, f32 = a["force"], b["force"]
    mag = np.linalg.norm(f64, axis=1)
    rms = np.sqrt((mag ** 2).mean())
    err = np.linalg.norm(f32 - f64, axis=1) / np.maximum(mag, rms)
    e64, e32 = a["epot"].sum(), b["epot"].sum()
    return err.max(), np.sqrt((err ** 2).mean()), abs(e32 - e64) / max(abs(e64), 1e-30), rms


def test_force_error_config1():
    mx, rms_err, e_err, frms = force_error(systems.c1_atoms(), None)
    assert frms > 0
    assert mx <= TOL_FORCE, (mx, rms_err)
    assert e_err <= TOL_ENERGY, e_err


def test_force_error_dense_overlaps():
    # 2.2 Å minimum separation: many pairs deep inside the repulsive core
    mx, rms_err, e_err, frms = force_error(systems.c1_atoms(dmin=2.2, n_ion=300), None)
    assert mx <= TOL_FORCE, (mx, rms_err)
    assert e_err <= TOL_ENERGY, e_err


def test_mixed_is_deterministic():
    p = systems.c1_params()
    p.precision = dml.PRECISION_MIXED
    out = []
    for _ in range(2):
        g = dml.Simulation(p)
        g.set_atoms(systems.c1_atoms())
        g.setup()
        g.step(100)
        out.append(g.get_atoms())
        g.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
