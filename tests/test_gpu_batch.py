"""Replica batches (dml_create_batch) vs one oracle run per replica.

Every kernel of a batch context covers all replicas in one launch; each
replica must still give, bit for bit, what the oracle gives for that replica
alone (plain FP64), and what a one-replica context gives (mixed form).
"""
import ctypes

import numpy as np
import pytest

from tests import oracle_lib, systems
from tests.test_gpu_parity import COUNTERS, FIELDS
import dml

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def replica_params(p, rep):
    """A copy of p carrying one replica's box, planes and seed."""
    q = dml.Params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(p))
    q.box[:] = list(rep.box)
    q.z0, q.zmax, q.z1, q.seed = rep.z0, rep.zmax, rep.z1, rep.seed
    return q


def same_bits(x, y):
    if x.dtype.kind == "f":
        return np.array_equal(x.view(np.uint64), y.view(np.uint64))
    return np.array_equal(x, y)


def check_replica(g, r, o, where, lists=True, ld=2048):
    a, b = g.get_atoms(replica=r), o.get_atoms()
    for k in FIELDS:
        if not same_bits(a[k], b[k]):
            bad = np.argwhere(a[k] != b[k])
            i = bad[0][0] if len(bad) else -1
            raise AssertionError("%s replica %d: %s differs at atom %d (%d entries)"
                                 % (where, r, k, i, len(bad)))
    cg, co = g.counters(replica=r), o.counters()
    for k in COUNTERS:
        assert cg[k] == co[k], "%s replica %d: counter %s gpu %r oracle %r" % (
            where, r, k, cg[k], co[k])
    if lists:
        n1, l1 = g.get_neighbors(ld, replica=r)
        n2, l2 = o.get_neighbors(ld)
        assert np.array_equal(n1, n2), "%s replica %d: neighbour counts differ" % (where, r)
        for k in range(len(n1)):
            assert np.array_equal(l1[k, : n1[k]], l2[k, : n2[k]]), (
                "%s replica %d: list row %d differs" % (where, r, k))


def run_batch_vs_oracles(p, reps, atoms, steps):
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    orcs = []
    for rep, at in zip(reps, atoms):
        o = oracle_lib.Oracle(replica_params(p, rep))
        o.set_atoms(at)
        o.setup()
        orcs.append(o)
    g.setup()
    for r, o in enumerate(orcs):
        check_replica(g, r, o, "setup")
    done = 0
    for chunk in steps:
        g.step(chunk)
        for o in orcs:
            o.step(chunk)
        done += chunk
        for r, o in enumerate(orcs):
            check_replica(g, r, o, "after %d steps" % done, lists=(chunk == steps[-1]))
    return g, orcs


def uneven_replicas(p):
    """Four replicas of uneven size: two electrode boxes that use cells, a
    wider one, and a short box whose lists come from the all-pairs builder."""
    reps = [
        dml.replica_of(p, seed=1234),
        dml.replica_of(p, seed=99),
        dml.replica_of(p, box=[42.12, 42.12, 60.0], seed=5),
        dml.replica_of(p, box=[35.1, 35.1, 40.0], z0=20.0, zmax=40.0, seed=17),
    ]
    atoms = [
        systems.slab_system(10, 10, 2, 60.0, 200, 10.0, 60.0, 7),
        systems.slab_system(10, 10, 2, 60.0, 90, 10.0, 60.0, 8),
        systems.slab_system(12, 12, 2, 60.0, 320, 10.0, 60.0, 9),
        systems.slab_system(10, 10, 2, 40.0, 120, 10.0, 40.0, 11),
    ]
    return reps, atoms


@pytest.mark.parametrize("integrator", [dml.INTEGRATOR_ERMAK, dml.INTEGRATOR_BROWNIAN])
def test_uneven_batch_matches_oracle_per_replica(integrator):
    p = systems.c1_params(integrator=integrator)
    reps, atoms = uneven_replicas(p)
    g, orcs = run_batch_vs_oracles(p, reps, atoms, [1, 9, 40, 100])
    assert g.counters()["nupd"] >= 4  # every replica built its list


def test_many_replicas_exact_displacement_pass():
    """160 replicas: the displacement test's exact FP64 pass runs one block
    per replica (more than 152 replicas), and every replica whose FP32 top-2
    lands within the margin of the skin must decide as the oracle does.
    Skin 1 A, so lists are rebuilt several times in 150 steps."""
    p = systems.c1_params(reservoir=dml.RESERVOIR_NONE)
    p.skin = 1.0
    reps = [dml.replica_of(p, box=[21.06, 21.06, 60.0], seed=500 + r) for r in range(160)]
    atoms = [systems.slab_system(6, 6, 2, 60.0, 60, 10.0, 60.0, 300 + r, dmin=3.2)
             for r in range(160)]
    g, orcs = run_batch_vs_oracles(p, reps, atoms, [1, 49, 100])
    tests = exact = 0
    for r in range(160):
        t, e = g.test_counts(replica=r)
        tests += t
        exact += e
        assert g.counters(replica=r)["nupd"] == orcs[r].counters()["nupd"]
    assert tests >= 160 * 300 and exact > 0, (tests, exact)


def test_batch_capture_events():
    """Ions next to the electrode, Brownian, no reservoir: captures happen in
    every replica and match the oracle per replica."""
    p = systems.c1_params(integrator=dml.INTEGRATOR_BROWNIAN, reservoir=dml.RESERVOIR_NONE)
    p.h = 1e-2
    reps = [dml.replica_of(p, seed=s) for s in (3, 4, 5)]
    atoms = [systems.slab_system(10, 10, 2, 60.0, n, 5.0, 20.0, s, dmin=3.2)
             for n, s in ((150, 3), (100, 4), (60, 5))]
    g, orcs = run_batch_vs_oracles(p, reps, atoms, [50, 50])
    for r in range(3):
        assert g.counters(replica=r)["depo"] > 0


def test_batch_gcmc_matches_oracle_per_replica():
    """GCMC reservoir: one block per replica runs its sequential trials.

    Ions start at least rc apart: without the piston, two ions left within
    rc of each other at their step-start positions are moved back forever
    (overlap_moveback recurses without end, dana.F90:916-940), which both
    sides report as DML_E_OVERLAP_PASSES."""
    p = systems.c5_small_params(nadj=32)
    reps = [dml.replica_of(p, seed=s) for s in (7, 8, 9)]
    atoms = [systems.c1_atoms(seed=s, n_ion=n, dmin=3.2)
             for s, n in ((7, 200), (8, 150), (9, 260))]
    g, orcs = run_batch_vs_oracles(p, reps, atoms, [1, 9, 20])
    c = g.counters()
    assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0


def test_mixed_batch_equals_single_contexts():
    """Mixed form: int64 fixed-point sums do not depend on the order of the
    atomics, so a replica in a batch equals the same system run alone."""
    p = systems.c1_params()
    p.precision = dml.PRECISION_MIXED
    reps, atoms = uneven_replicas(p)
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    g.setup()
    g.step(60)
    for r, (rep, at) in enumerate(zip(reps, atoms)):
        s = dml.Simulation(replica_params(p, rep))
        s.set_atoms(at)
        s.setup()
        s.step(60)
        a, b = g.get_atoms(replica=r), s.get_atoms()
        for k in FIELDS:
            assert same_bits(a[k], b[k]), "replica %d: %s differs from the lone run" % (r, k)
        s.close()


def test_batch_api_errors():
    p = systems.c1_params()
    reps, atoms = uneven_replicas(p)
    g = dml.Simulation(p, replicas=reps[:2])
    with pytest.raises(ValueError):
        g.set_atoms(atoms[:1])
    g.set_atoms(atoms[:2])
    with pytest.raises(dml.DmlError):
        g.counters(replica=2)
    # the one-replica entry points refuse a context of several
    lib = dml.lib()
    a = dml.atoms_struct(dict(atoms[0]), len(atoms[0]["z"]))
    assert lib.dml_get_atoms(g.h, ctypes.byref(a)) == 1
    assert lib.dml_num_replicas(g.h) == 2


@pytest.mark.parametrize("precision", [dml.PRECISION_FP64, dml.PRECISION_MIXED])
def test_batch_download_equals_per_replica(precision):
    """dml_get_atoms_batch packs every replica on the device: each replica's
    arrays equal dml_get_atoms_replica's, for every member and for a subset,
    after GCMC has left holes in sys%alist."""
    p = systems.c5_small_params(nadj=32)
    p.precision = precision
    reps = [dml.replica_of(p, seed=s) for s in (7, 8, 9)]
    atoms = [systems.c1_atoms(seed=s, n_ion=n, dmin=3.2)
             for s, n in ((7, 200), (8, 150), (9, 260))]
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    g.setup()
    g.step(15)
    full = g.get_atoms_batch()
    sub = g.get_atoms_batch(fields=("pos", "z"))
    assert len(full) == len(sub) == 3
    for r in range(3):
        one = g.get_atoms(replica=r)
        assert set(full[r]) == set(one)
        for k in one:
            assert same_bits(full[r][k], one[k]), "replica %d member %s" % (r, k)
        assert set(sub[r]) == {"pos", "z"}
        assert same_bits(sub[r]["pos"], one["pos"]) and np.array_equal(sub[r]["z"], one["z"])


@pytest.mark.parametrize("precision", [dml.PRECISION_FP64, dml.PRECISION_MIXED])
def test_steps_per_graph_do_not_change_results(precision):
    """dml_step queues runs of graph_steps steps as one CUDA graph (each step
    with its own conditional rebuild nodes): 1, 7 and 100 steps per graph
    give the same state, bit for bit, after 150 GCMC + Ermak steps."""
    p = systems.c5_small_params(nadj=64)
    p.precision = precision
    p.skin = 1.0  # list rebuilds inside the run
    reps = [dml.replica_of(p, seed=3), dml.replica_of(p, seed=4)]
    atoms = [systems.c1_atoms(seed=s, dmin=3.2) for s in (5, 6)]
    out = []
    for k in (1, 7, 100):
        g = dml.Simulation(p, replicas=reps)
        g.set_atoms(atoms)
        g.setup()
        g.set_graph_steps(k)
        g.step(150)
        out.append([g.get_atoms(replica=r) for r in range(2)] + [g.counters()])
        g.close()
    assert out[0][2]["nupd"] >= 4 and out[0][2]["gcmc_ins"] > 0
    for other in out[1:]:
        for r in range(2):
            for key in FIELDS:
                assert same_bits(out[0][r][key], other[r][key]), (r, key)
        assert out[0][2] == other[2]
