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


def test_device_conversions_match_ieee():
    """The device conversions behind the FP32 position copies and the
    integrators' FP32 increments equal IEEE 754 round-to-nearest-even (numpy)
    over random bit patterns, positions in the box range, halfway cases,
    mantissa carries and the subnormal, overflow, zero, inf and NaN edges."""
    rng = np.random.default_rng(3)
    bits = rng.integers(0, 2 ** 64, 200000, dtype=np.uint64)
    anyd = bits.view(np.float64)
    box = rng.uniform(-50.0, 400.0, 200000)
    f = rng.uniform(-300.0, 300.0, 50000).astype(np.float32).astype(np.float64)
    ulp = np.spacing(f.astype(np.float32)).astype(np.float64)
    ties = np.concatenate([f + ulp / 2, f - ulp / 2, f + ulp / 2 * (1 + 2 ** -40)])
    carry = np.array([1.0 - 2 ** -25, 2.0 - 2 ** -24, 255.99999999, -(2.0 - 2 ** -25)])
    fmax = float(np.finfo(np.float32).max)
    tiny = float(np.finfo(np.float32).tiny)
    edges = np.array([0.0, -0.0, 5e-324, -5e-324, tiny, -tiny, tiny * (1 - 2 ** -30),
                      tiny * 2 ** -10, fmax, -fmax, fmax * (1 + 2 ** -25), fmax * 2,
                      np.inf, -np.inf, np.nan, 1e-45, 1.4e-45, 3e-39, 1e300, -1e-300])
    x = np.concatenate([anyd, box, ties, carry, edges])
    f32, back = dml.check_conversions(x)
    with np.errstate(over="ignore", invalid="ignore"):
        want = x.astype(np.float32)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(f32), nan)
    assert np.array_equal(f32[~nan].view(np.uint32), want[~nan].view(np.uint32))
    wb = f32.astype(np.float64)
    assert np.array_equal(np.isnan(back), nan)
    assert np.array_equal(back[~nan].view(np.uint64), wb[~nan].view(np.uint64))


def _sorted_rows(nn, lst):
    return [np.sort(lst[k, : nn[k]]) for k in range(len(nn))]


@pytest.mark.parametrize("factor", [1.2, 1.5])
def test_cell_factor_keeps_list_sets_and_forces(factor):
    """The chosen form's larger cells: after the rebuild each row holds the
    same atoms as with the reference grid (in another order), and the
    fixed-point forces at those positions are the same bits."""
    import copy

    p = systems.c5_small_params(nadj=32)
    p.precision = dml.PRECISION_MIXED
    p.skin = 2.0
    atoms = systems.c1_atoms(seed=21, dmin=2.2, n_ion=300)
    sims = []
    for f in (1.0, factor):
        g = dml.Simulation(copy.copy(p))
        g.set_atoms(atoms)
        g.setup()
        if f != 1.0:
            g.set_cell_factor(f)
        assert g.test_update() == (1 if f != 1.0 else 0)
        g.fuerza()
        sims.append(g)
    (n1, l1), (n2, l2) = [g.get_neighbors(p.mnb) for g in sims]
    assert np.array_equal(n1, n2)
    for a, b in zip(_sorted_rows(n1, l1), _sorted_rows(n2, l2)):
        assert np.array_equal(a, b)
    a, b = sims[0].get_atoms(), sims[1].get_atoms()
    assert np.array_equal(a["force"].view(np.uint64), b["force"].view(np.uint64))
    assert np.abs(a["force"]).max() > 0
    for g in sims:
        g.close()
    # GCMC steps and rebuilds on the coarser grid (ions start rc apart: closer
    # ones would be moved back forever without a piston, as in the reference)
    g = dml.Simulation(copy.copy(p))
    g.set_atoms(systems.c1_atoms(seed=22, dmin=3.2))
    g.setup()
    g.set_cell_factor(factor)
    g.step(60)
    c = g.counters()
    assert c["nupd"] >= 2 and c["gcmc_ins"] > 0
    g.close()


def test_cell_tuning_picks_a_factor():
    p, reps, atoms = systems.c4_batch(n_rep=24, seed=5)
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    g.setup()
    best = g.tune_cells(steps=3)
    t = g.cell_tuning()
    assert 1.0 <= best <= 1.5 and t["factor"] == best
    assert all(v > 0 for v in t["us_per_step"].values())
    g.step(10)
    g.close()


def test_cell_factor_refused_for_the_plain_form():
    p = systems.c1_params()
    g = dml.Simulation(p)
    g.set_atoms(systems.c1_atoms())
    with pytest.raises(dml.DmlError) as e:
        g.set_cell_factor(1.3)
    assert e.value.code == dml.E_UNSUPPORTED
    g.close()
