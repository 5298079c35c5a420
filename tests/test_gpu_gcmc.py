"""Device gcmc_run vs the oracle, bit-exact (structure, slots, lists).

Insertions reuse the first free slot, go to the head of their cell chain and
are appended to the other atoms' lists; deletions leave limbo slots; captured
atoms leave the gcmc group.  The device must reproduce all of it: every state
array in sys%alist order, the gcmc membership, the neighbour lists (with
limbo entries) and the insertion/deletion counters.
"""
import numpy as np
import pytest

from tests import oracle_lib, systems
from tests.test_gpu_parity import (assert_same_counters, assert_same_lists, assert_same_state,
                                   make_pair)
import dml

pytestmark = pytest.mark.gpu

FIELDS = ["pos", "vel", "acel", "force", "epot", "z", "skip", "old_cg", "pos_old", "in_ref",
          "in_gcmc", "id"]
COUNTERS = ["try_", "depo", "choques", "choques3", "nupd", "n_ref", "n_atoms", "zmax", "rho",
            "gcmc_ins", "gcmc_del"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def test_gcmc_routine_after_setup():
    p = systems.gcmc_params()
    g, o = make_pair(p, systems.gcmc_atoms())
    g.setup()
    o.setup()
    for step in range(1, 6):
        g.gcmc_run(step)
        o.gcmc_run(step)
        assert_same_state(g, o, "gcmc_run %d" % step, FIELDS)
        assert_same_counters(g, o, "gcmc_run %d" % step, COUNTERS)
        assert_same_lists(g, o, "gcmc_run %d" % step, ld=1024)
    c = g.counters()
    assert c["gcmc_ins"] + c["gcmc_del"] > 0


def test_reference_gcmc_case_fused_steps():
    """tests/gcmc configuration (Brownian + GCMC), Philox streams, 400 steps."""
    p = systems.gcmc_params()
    g, o = make_pair(p, systems.gcmc_atoms())
    g.setup()
    o.setup()
    done = 0
    for chunk in [1, 19, 80, 300]:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_state(g, o, "gcmc after %d" % done, FIELDS)
        assert_same_counters(g, o, "gcmc after %d" % done, COUNTERS)
    assert_same_lists(g, o, "gcmc end", ld=1024)
    c = g.counters()
    assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0


@pytest.mark.parametrize("lanes", [0, 1])
def test_ermak_gcmc_with_electrode(lanes):
    """Electrode + Ermak forces + GCMC reservoir (config 5 at test size).
    With one lane per list row the force scan walks only the rows flagged at
    its last full scan (or written by GCMC since) until the atoms have moved
    by the flag margin: the run must still equal the oracle bit for bit, and
    most scans must have been of that kind."""
    p = systems.c5_small_params()
    g, o = make_pair(p, systems.c1_atoms(dmin=3.2))
    g.set_scan_lanes(lanes)
    g.setup()
    o.setup()
    done = 0
    for chunk in [1, 29, 170]:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_state(g, o, "ermak+gcmc after %d" % done, FIELDS)
        assert_same_counters(g, o, "ermak+gcmc after %d" % done, COUNTERS)
    assert_same_lists(g, o, "ermak+gcmc end")
    c = g.counters()
    assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0
    if lanes == 1:
        full, partial = g.scan_counts()
        assert full + partial == done and partial > full, (full, partial)


def test_config5_shape_gcmc_matches_oracle():
    """Config-5 geometry at test size: 15 x 15 x 2-cell electrode (52.65 Å),
    1500 ions, GCMC slab z in [60, 100] with 64 trials per step and the
    activity that balances the slab count.  Three or more cells along every
    axis, so each trial searches its 27 stencil cells; the list rebuilds free
    limbo slots that later insertions take (Brownian moves, small skin)."""
    p = systems.c5_params(seed=3, precision=dml.PRECISION_FP64, nadj=64, cells=15, n_ion=1500)
    p.box[2] = 100.0
    p.z0, p.zmax = 60.0, 100.0
    p.skin = 2.0  # Brownian moves of ~0.4 Å: a rebuild every few steps
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.h = 1e-4
    p.mnb = 512
    atoms = systems.slab_system(15, 15, 2, 100.0, 1500, 15.0, 100.0, 21, dmin=3.2)
    p.act = systems.slab_activity(p, atoms, 3)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    done = 0
    for chunk in [1, 9, 40]:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_state(g, o, "config-5 shape after %d" % done, FIELDS)
        assert_same_counters(g, o, "config-5 shape after %d" % done, COUNTERS)
    assert_same_lists(g, o, "config-5 shape end", ld=512)
    c = g.counters()
    assert c["gcmc_ins"] > 50 and c["gcmc_del"] > 50 and c["nupd"] > 1


@pytest.mark.parametrize("capacity", [0, 600000])
def test_dense_gcmc_many_trials_matches_oracle(capacity):
    """256 trials per step (the most one call decides on the parallel path)
    at a high activity: insertions blocked by earlier insertions of the same
    call, deletions of atoms inserted in the same call, hs%b slots freed and
    taken again within one call, limbo slots freed by rebuilds.  The larger
    capacity keeps the membership bits in global memory instead of shared
    memory."""
    p = systems.c5_params(seed=5, precision=dml.PRECISION_FP64, nadj=256, cells=12, n_ion=900)
    p.box[2] = 80.0
    p.z0, p.zmax = 50.0, 80.0
    p.skin = 2.0
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.h = 1e-4
    p.mnb = 256
    if capacity:
        p.capacity = capacity
    atoms = systems.slab_system(12, 12, 2, 80.0, 900, 15.0, 80.0, 31, dmin=3.2)
    p.act = 3.0 * systems.slab_activity(p, atoms, 5)
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    done = 0
    for chunk in [1, 4, 15]:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_state(g, o, "dense gcmc after %d" % done, FIELDS)
        assert_same_counters(g, o, "dense gcmc after %d" % done, COUNTERS)
        assert_same_lists(g, o, "dense gcmc after %d" % done, ld=256)
    c = g.counters()
    assert c["gcmc_ins"] > 200 and c["gcmc_del"] > 200


def test_deletion_pick_matches_binary64():
    """The integer form of the deletion pick equals int(upick * n) + 1 (capped
    at n) evaluated in binary64, for random draws and counts and for products
    that sit on or next to a rounding boundary."""
    import numpy as np

    rng = np.random.default_rng(11)
    k = rng.integers(0, 2 ** 53, 300000, dtype=np.uint64)
    n = rng.integers(0, 2 ** 31 - 1, 300000).astype(np.int32)
    n[:100000] = rng.integers(0, 40000, 100000)
    # products just below an integer: upick close to j / n
    nn = rng.integers(1, 40000, 50000)
    j = (rng.random(50000) * nn).astype(np.int64)
    base = (j.astype(np.float64) / nn * 2.0 ** 53).astype(np.uint64)
    edge_k = np.concatenate([base - 2, base - 1, base, base + 1, base + 2]).clip(0, 2 ** 53 - 1)
    edge_n = np.tile(nn, 5).astype(np.int32)
    k = np.concatenate([k, edge_k.astype(np.uint64), np.array([0, 2 ** 53 - 1, 2 ** 53 - 1, 1], np.uint64)])
    n = np.concatenate([n, edge_n, np.array([0, 0, 2 ** 31 - 1, 1], np.int32)])
    m = dml.check_pick(k, n)
    upick = k.astype(np.float64) * 2.0 ** -53  # exact: k < 2^53
    want = np.floor(upick * n.astype(np.float64)).astype(np.int64) + 1
    want = np.minimum(want, n.astype(np.int64))
    assert np.array_equal(m.astype(np.int64), want)


def config5_shape(n_fill=1500):
    """The config-5 geometry of test_config5_shape_gcmc_matches_oracle, with
    the activity that balances a slab of n_fill ions."""
    p = systems.c5_params(seed=3, precision=dml.PRECISION_FP64, nadj=64, cells=15, n_ion=n_fill)
    p.box[2] = 100.0
    p.z0, p.zmax = 60.0, 100.0
    p.skin = 2.0
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.h = 1e-4
    p.mnb = 512
    full = systems.slab_system(15, 15, 2, 100.0, n_fill, 15.0, 100.0, 21, dmin=3.2)
    p.act = systems.slab_activity(p, full, 3)
    return p


def test_reservoir_filling_from_few_ions_batch():
    """Replicas that start with 1, 4 and 30 ions under the activity of a
    1500-ion slab: nearly every creation is accepted, so the group grows
    from a single member to hundreds within the run (insertions into
    near-empty cells, first and last members changing, many rebuilds).
    Each replica stays bit-exact to its own oracle run."""
    from tests.test_gpu_batch import run_batch_vs_oracles

    p = config5_shape()
    reps = [dml.replica_of(p, seed=s) for s in (41, 42, 43)]
    atoms = [systems.slab_system(15, 15, 2, 100.0, n, 15.0, 100.0, s, dmin=3.2)
             for n, s in ((1, 41), (4, 42), (30, 43))]
    g, orcs = run_batch_vs_oracles(p, reps, atoms, [1, 9, 30])
    for r, o in enumerate(orcs):
        cg, co = g.counters(replica=r), o.counters()
        for k in ("gcmc_ins", "gcmc_del", "n_ref", "nupd"):
            assert cg[k] == co[k], "replica %d: %s gpu %r oracle %r" % (r, k, cg[k], co[k])
        assert same_membership(g.get_atoms(replica=r), o.get_atoms()), "replica %d" % r
        assert cg["n_ref"] > 300


def same_membership(a, b):
    return np.array_equal(a["in_gcmc"], b["in_gcmc"]) and np.array_equal(a["id"], b["id"])


@pytest.mark.parametrize("geometry", ["cells", "all_pairs"])
def test_error_parity_empty_gcmc_group(geometry):
    """An electrode without ions: the first trial finds no template atom in
    the gcmc group and both sides stop with 'No more particles' at step 1
    (werr, dana.F90:624), on the parallel path (cells) and in gcmc_kernel
    (all-pairs lists)."""
    if geometry == "cells":
        p = config5_shape()
        full = systems.slab_system(15, 15, 2, 100.0, 1, 15.0, 100.0, 5, dmin=3.2)
    else:
        p = systems.c5_small_params(nadj=32)
        p.box[2] = 40.0
        p.z0, p.zmax = 20.0, 40.0
        full = systems.slab_system(10, 10, 2, 40.0, 1, 10.0, 40.0, 5, dmin=3.2)
    keep = full["z"] == dml.Z_CG
    atoms = {k: v[keep] for k, v in full.items()}
    g, o = make_pair(p, atoms)
    g.setup()
    o.setup()
    with pytest.raises(RuntimeError, match="NO_PARTICLES"):
        o.step(1)
    with pytest.raises(dml.DmlError) as e:
        g.step(1)
    assert e.value.code == dml.E_NO_PARTICLES
