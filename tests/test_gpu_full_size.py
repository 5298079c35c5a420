"""Plain FP64 CUDA path vs the oracle at the benchmark configurations' own sizes.

The other parity tests run systems of a few hundred atoms; these run the
systems the benchmarks time, where list capacities, the per-replica FP32
pre-filter margins, the cell grids and the GCMC paths meet their largest
cases.  Each compares bit for bit (tolerance 0) every state array, the
neighbour lists and the counters (captures and capture attempts, overlap
move-backs, list rebuilds, GCMC insertions and deletions) with the oracle
run of the same replica, fed the same keyed Philox streams:

  config 5  two full replicas of the GCMC batch (40 x 40 x 2-cell electrode,
            20 000 Li+, 128 trials per step, Ermak, skin 2 Å), 100 steps with
            list rebuilds, both replicas on the parallel GCMC path and the
            force scan walking flagged rows between full scans;
  config 2  the 280 000-atom system: the set-up list build and 20 steps,
            forces also checked within 1e-12 relative (src/dana.F90:173-265);
  config 1  the full 10 000-step run, captures compared every 1000 steps;
  config 4  the tallest replica the 1 M rule allows for the batch's smallest
            electrode (5 x 5 cells, 20 000 ions, about 108 000 Å high),
            batched with a short replica, Brownian with the piston.
"""
import numpy as np
import pytest

from tests import oracle_lib, systems
from tests.test_gpu_batch import replica_params, same_bits
from tests.test_gpu_parity import COUNTERS, FIELDS
import dml

pytestmark = pytest.mark.gpu

GCMC_COUNTERS = COUNTERS + ["gcmc_ins", "gcmc_del"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def check_state(g, o, where, replica=None, counters=COUNTERS):
    a = g.get_atoms(replica=replica) if replica is not None else g.get_atoms()
    b = o.get_atoms()
    for k in FIELDS:
        if not same_bits(a[k], b[k]):
            bad = np.argwhere(a[k] != b[k])
            i = bad[0][0] if len(bad) else -1
            raise AssertionError("%s: %s differs at atom %d (%d entries)" % (where, k, i, len(bad)))
    cg = g.counters(replica=replica) if replica is not None else g.counters()
    co = o.counters()
    for k in counters:
        assert cg[k] == co[k], "%s: counter %s gpu %r oracle %r" % (where, k, cg[k], co[k])
    return a, cg


def check_lists(g, o, where, ld, replica=None):
    n1, l1 = g.get_neighbors(ld, replica=replica) if replica is not None else g.get_neighbors(ld)
    n2, l2 = o.get_neighbors(ld)
    assert np.array_equal(n1, n2), where + ": neighbour counts differ"
    used = np.arange(ld)[None, :] < n1[:, None]
    bad = np.argwhere(used & (l1 != l2))
    assert len(bad) == 0, "%s: list row %d entry %d differs (%d entries)" % (
        where, bad[0][0], bad[0][1], len(bad))
    return int(n1.sum())


def test_config5_replicas_full_size():
    p, reps, atoms = systems.c5_batch(2, precision=dml.PRECISION_FP64)
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    g.set_scan_lanes(1)  # the benchmark's mapping: flagged-row scans between full ones
    orcs = []
    for rep, at in zip(reps, atoms):
        o = oracle_lib.Oracle(replica_params(p, rep))
        o.set_atoms(at)
        o.setup()
        orcs.append(o)
    g.setup()
    nupd0 = [o.counters()["nupd"] for o in orcs]
    for r, o in enumerate(orcs):
        check_state(g, o, "c5 setup r%d" % r, replica=r, counters=GCMC_COUNTERS)
        check_lists(g, o, "c5 setup r%d" % r, p.mnb, replica=r)
    done = 0
    for chunk in (1, 9, 40, 50):
        g.step(chunk)
        for o in orcs:
            o.step(chunk)
        done += chunk
        for r, o in enumerate(orcs):
            check_state(g, o, "c5 after %d steps r%d" % (done, r), replica=r,
                        counters=GCMC_COUNTERS)
    for r, o in enumerate(orcs):
        check_lists(g, o, "c5 end r%d" % r, p.mnb, replica=r)
        c = o.counters()
        assert c["nupd"] > nupd0[r], "no list rebuild in %d steps" % done
        assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0 and c["choques"] > 0
        par, seq = g.gcmc_paths(replica=r)
        assert par == done and seq == 0, (r, par, seq)
        full, partial = g.scan_counts(replica=r)
        assert full + partial == done and partial > 0, (r, full, partial)
    # the exact displacement pass, several blocks per replica (two replicas)
    assert sum(g.test_counts(replica=r)[1] for r in range(2)) > 0
    g.close()


def test_config2_full_system():
    p = systems.c2_params()
    atoms = systems.c2_atoms()
    g = dml.Simulation(p)
    g.set_atoms(atoms)
    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    g.setup()
    o.setup()
    check_state(g, o, "c2 setup")
    # no reservoir appends: the longest row is the build's
    ld = max(1, int(o.counters()["max_nn"]))
    entries = check_lists(g, o, "c2 setup", ld)
    assert entries > 200000 * 40  # about 55 list entries per ion at 13.2 Å
    done = 0
    for chunk in (1, 4, 15):
        g.step(chunk)
        o.step(chunk)
        done += chunk
        a, c = check_state(g, o, "c2 after %d steps" % done)
    check_lists(g, o, "c2 end", max(1, int(o.counters()["max_nn"])))
    b = o.get_atoms()
    f, fo = a["force"], b["force"]
    scale = np.maximum(np.abs(fo).max(axis=1, keepdims=True), 1e-300)
    assert float((np.abs(f - fo) / scale).max()) <= 1e-12
    assert c["depo"] > 0 and c["try_"] >= c["depo"]
    g.close()


def test_config1_full_run():
    p = systems.c1_params()
    atoms = systems.c1_atoms()
    g = dml.Simulation(p)
    g.set_atoms(atoms)
    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    g.setup()
    o.setup()
    for k in range(10):
        g.step(1000)
        o.step(1000)
        _, c = check_state(g, o, "c1 after %d steps" % (1000 * (k + 1)))
    check_lists(g, o, "c1 end", p.mnb)
    assert c["step"] == 10000 and c["depo"] > 0 and c["nupd"] > 1
    # the exact displacement pass, one replica spread over many blocks
    tests, exact = g.test_counts()
    assert tests >= 20000 and exact > 0, (tests, exact)
    g.close()


def test_config4_tallest_replica():
    a = 3.51
    p = systems.default_params()
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.reservoir = dml.RESERVOIR_PISTON
    p.h, p.skin, p.mnb, p.seed = 5e-5, 2.0, 128, 13
    specs = [(5, 20000, 13 * 100003 + 1), (12, 300, 13 * 100003 + 2)]
    reps, atoms = [], []
    for cells, n_ion, seed in specs:
        L = cells * a
        lz = 10.0 + max(20.0, n_ion / (6.022e-4 * L * L))
        reps.append(dml.replica_of(p, box=[L, L, lz], z0=0.5 * lz, zmax=lz, seed=seed))
        atoms.append(systems.slab_system(cells, cells, 2, lz, n_ion, 10.0, lz, seed, dmin=3.2))
    assert reps[0].box[2] > 1.0e5
    p.box[:] = list(reps[0].box)
    p.z0, p.zmax = reps[0].z0, reps[0].zmax
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    orcs = []
    for rep, at in zip(reps, atoms):
        o = oracle_lib.Oracle(replica_params(p, rep))
        o.set_atoms(at)
        o.setup()
        orcs.append(o)
    g.setup()
    done = 0
    for chunk in (1, 4, 15):
        g.step(chunk)
        for o in orcs:
            o.step(chunk)
        done += chunk
        for r, o in enumerate(orcs):
            check_state(g, o, "c4 after %d steps r%d" % (done, r), replica=r)
    for r, o in enumerate(orcs):
        check_lists(g, o, "c4 end r%d" % r, p.mnb, replica=r)
    g.close()
