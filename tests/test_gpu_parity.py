"""Plain FP64 CUDA path vs the oracle: bit-exact, routine by routine.

Both sides start from the same seeded system and draw from the same keyed
Philox stream.  Every state array (positions, velocities, accelerations,
forces, energies, elements, skip flags, old positions), the neighbour lists
and the counters must agree bit for bit (integer and index work exactly;
floating point to the last bit, tolerance 0).
"""
import numpy as np
import pytest

from tests import oracle_lib, systems
import dml

pytestmark = pytest.mark.gpu

FIELDS = ["pos", "vel", "acel", "force", "epot", "z", "skip", "old_cg", "pos_old", "in_ref", "id"]
COUNTERS = ["try_", "depo", "choques", "choques3", "nupd", "n_ref", "n_atoms", "zmax", "rho"]


def assert_same_state(g, o, where, fields=FIELDS):
    a, b = g.get_atoms(), o.get_atoms()
    for k in fields:
        x, y = a[k], b[k]
        if x.dtype.kind == "f":
            same = np.array_equal(x.view(np.uint64), y.view(np.uint64))
        else:
            same = np.array_equal(x, y)
        if not same:
            bad = np.argwhere(x != y)
            i = bad[0][0] if len(bad) else -1
            raise AssertionError("%s: field %s differs at atom %d: gpu %r oracle %r (%d entries)"
                                 % (where, k, i, x[i], y[i], len(bad)))


def assert_same_counters(g, o, where, keys=COUNTERS):
    a, b = g.counters(), o.counters()
    for k in keys:
        assert a[k] == b[k], "%s: counter %s gpu %r oracle %r" % (where, k, a[k], b[k])


def assert_same_lists(g, o, where, ld=2048):
    n1, l1 = g.get_neighbors(ld)
    n2, l2 = o.get_neighbors(ld)
    assert np.array_equal(n1, n2), where + ": neighbour counts differ"
    for k in range(len(n1)):
        assert np.array_equal(l1[k, : n1[k]], l2[k, : n2[k]]), "%s: list row %d differs" % (where, k)


def make_pair(params, atoms):
    g = dml.Simulation(params)
    o = oracle_lib.Oracle(params)
    g.set_atoms(atoms)
    o.set_atoms(atoms)
    return g, o


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def test_setup_lists_forces_rho0():
    g, o = make_pair(systems.c1_params(), systems.c1_atoms())
    g.setup()
    o.setup()
    assert_same_lists(g, o, "setup")
    assert_same_state(g, o, "setup")
    assert_same_counters(g, o, "setup")
    assert g.counters()["rho0"] == o.counters()["rho0"]


@pytest.mark.parametrize("integrator", [dml.INTEGRATOR_ERMAK, dml.INTEGRATOR_BROWNIAN])
def test_routine_by_routine(integrator):
    """Each reference routine called separately, compared after every call."""
    p = systems.c1_params(integrator=integrator)
    g, o = make_pair(p, systems.c1_atoms())
    g.setup()
    o.setup()
    for step in range(1, 31):
        if integrator == dml.INTEGRATOR_ERMAK:
            g.ermak_a(step)
            o.ermak_a(step)
            assert_same_state(g, o, "ermak_a %d" % step)
            g.fuerza()
            o.fuerza()
            assert_same_state(g, o, "fuerza %d" % step)
            g.ermak_b()
            o.ermak_b()
            assert_same_state(g, o, "ermak_b %d" % step)
        else:
            g.cbrownian_hs(step)
            o.cbrownian_hs(step)
            assert_same_state(g, o, "brownian %d" % step)
        assert g.test_update() == o.test_update()
        assert_same_lists(g, o, "test_update %d" % step)
        g.overlap_moveback(step)
        o.overlap_moveback(step)
        assert_same_state(g, o, "overlap %d" % step)
        assert_same_counters(g, o, "overlap %d" % step)
        assert g.test_update() == o.test_update()
        assert g.capture_commit() == o.capture_commit()
        assert g.calc_rho() == o.calc_rho()
        g.maxz()
        o.maxz()
        assert_same_state(g, o, "maxz %d" % step)
        assert_same_counters(g, o, "step %d" % step)


@pytest.mark.parametrize("integrator,reservoir,nsteps", [
    (dml.INTEGRATOR_ERMAK, dml.RESERVOIR_PISTON, 300),
    (dml.INTEGRATOR_BROWNIAN, dml.RESERVOIR_PISTON, 200),
    (dml.INTEGRATOR_BROWNIAN, dml.RESERVOIR_NONE, 200),
])
def test_fused_steps(integrator, reservoir, nsteps):
    """dml_step (CUDA graph of the whole loop body) vs the oracle loop."""
    p = systems.c1_params(integrator=integrator, reservoir=reservoir)
    if integrator == dml.INTEGRATOR_BROWNIAN:
        p.h = 1e-3
    atoms = systems.c1_atoms(dmin=3.2 if reservoir != dml.RESERVOIR_PISTON else 2.5)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    done = 0
    for chunk in [1, 9, 40, nsteps - 50]:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_state(g, o, "after %d steps" % done)
        assert_same_counters(g, o, "after %d steps" % done)
    assert_same_lists(g, o, "end")
    c = g.counters()
    assert c["nupd"] >= 1


def test_verlet_path_small_box():
    """All cell counts below 4: the all-pairs list builder (ngroup_verlet)."""
    p = systems.c1_params()
    p.box[2] = 40.0
    p.zmax = 40.0
    p.z0 = 20.0
    atoms = systems.slab_system(10, 10, 2, 40.0, 120, 10.0, 40.0, 11)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    assert_same_lists(g, o, "verlet setup")
    g.step(100)
    o.step(100)
    assert_same_state(g, o, "verlet 100 steps")
    assert_same_counters(g, o, "verlet 100 steps")


def test_capture_events_happen_and_match():
    """Ions started next to the electrode are captured; counts match exactly."""
    p = systems.c1_params(integrator=dml.INTEGRATOR_BROWNIAN, reservoir=dml.RESERVOIR_NONE)
    p.h = 1e-2  # sqrt(2*250*0.01) = 2.2 Å per step: reaches the slab quickly
    atoms = systems.slab_system(10, 10, 2, 60.0, 150, 5.0, 20.0, 3, dmin=3.2)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    g.step(100)
    o.step(100)
    assert_same_state(g, o, "capture run")
    assert_same_counters(g, o, "capture run")
    assert g.counters()["depo"] > 0


def test_error_parity_empty_reservoir_piston():
    """No ion above z0 at start: rho0 = 0, the piston factor is 0/0 and the
    positions become NaN; both sides stop with 'Particle out of tessellation'
    at the same step (the reference would stop in cgroup_sort, Cells.F90:293)."""
    p = systems.c1_params(integrator=dml.INTEGRATOR_BROWNIAN)
    p.h = 1e-2
    atoms = systems.slab_system(10, 10, 2, 60.0, 150, 5.0, 20.0, 3, dmin=3.2)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    fail_g = fail_o = None
    for step in range(1, 30):
        if fail_g is None:
            try:
                g.step(1)
            except dml.DmlError as e:
                fail_g = (step, e.code)
        if fail_o is None:
            try:
                o.step(1)
            except RuntimeError as e:
                fail_o = (step, "OUT_OF_TESSELLATION" in str(e))
        if fail_g and fail_o:
            break
    assert fail_g == (fail_o[0], 4) and fail_o[1]
