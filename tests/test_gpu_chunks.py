"""The chunk reservoir (bloques, src/dana.F90:716-773) on the device against the
oracle, bit for bit.

The reference's tests/brown run keeps the bulk density with chunks: when the
density of the sensor slab [z0, z1] strays from rhomedia by 18.6 % or more,
the planes and the box top rise by the chunk height and a copy of the
301-atom template (tests/golden/reference/brown/chunk.xyz) joins the system;
the list is then rebuilt with the taller box's cells.  Here the same geometry
runs in the keyed Philox streams on both sides (602 Li+ placed by random
sequential addition, Brownian, dt = 0.01 ps, skin 10 Å, box 100 x 100,
z0 = 100, chunk height 50 + rc, z1 = z0 + height, zmax = z1 + height, box
height 100 as pos_inic leaves it), routine by routine and through the fused
step, on one replica and on a batch of two.
"""
import ctypes
import os

import numpy as np
import pytest

from tests import oracle_lib, systems
from tests.test_gpu_batch import replica_params, same_bits
from tests.test_gpu_parity import COUNTERS, FIELDS
import dml

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CHUNK_XYZ = os.path.join(HERE, "golden", "reference", "brown", "chunk.xyz")
ELEMENTS = {"Li": dml.Z_LI, "CG": dml.Z_CG, "cg": dml.Z_CG, "F": dml.Z_F}


def read_chunk():
    lines = open(CHUNK_XYZ).read().splitlines()
    n = int(lines[0].split()[0])
    pos = np.zeros((n, 3))
    z = np.zeros(n, np.int32)
    for j in range(n):
        t = lines[2 + j].split()
        z[j] = ELEMENTS[t[0]]
        pos[j] = [float(t[1]), float(t[2]), float(t[3])]
    return pos, z


def brown_params(seed=77):
    """entrada.ini of tests/brown with config_inic's chunk geometry."""
    p = systems.default_params()
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.reservoir = dml.RESERVOIR_CHUNKS
    p.h = 1e-2
    p.skin = 10.0
    p.prob = 1.0
    p.dif_sc = p.dif_sei = 250.0
    dist = 50.0 + p.rc
    p.box[:] = [100.0, 100.0, 100.0]
    p.z0 = 100.0
    p.z1 = p.z0 + dist
    p.zmax = p.z1 + dist
    p.seed = seed
    p.mnb = 2048
    return p, dist


def brown_atoms(seed=5):
    ions = systems.random_ions(seed, 602, 100.0, 100.0, 0.0, 100.0, 3.2)
    return {"pos": ions, "z": np.full(len(ions), dml.Z_LI, np.int32)}


def check(g, o, where, replica=None, lists=False, ld=2048):
    a = g.get_atoms(replica=replica) if replica is not None else g.get_atoms()
    b = o.get_atoms()
    for k in FIELDS:
        assert len(a[k]) == len(b[k]), "%s: %d atoms on the device, %d in the oracle" % (
            where, len(a[k]), len(b[k]))
        if not same_bits(a[k], b[k]):
            bad = np.argwhere(a[k] != b[k])
            raise AssertionError("%s: %s differs at atom %d (%d entries)"
                                 % (where, k, bad[0][0] if len(bad) else -1, len(bad)))
    cg = g.counters(replica=replica) if replica is not None else g.counters()
    co = o.counters()
    for k in COUNTERS + ["z0"]:
        assert cg[k] == co[k], "%s: counter %s gpu %r oracle %r" % (where, k, cg[k], co[k])
    if lists:
        n1, l1 = g.get_neighbors(ld, replica=replica) if replica is not None else \
            g.get_neighbors(ld)
        n2, l2 = o.get_neighbors(ld)
        assert np.array_equal(n1, n2), where + ": neighbour counts differ"
        used = np.arange(ld)[None, :] < n1[:, None]
        assert not np.any(used & (l1 != l2)), where + ": lists differ"
    return cg


def pair(p, dist, atoms, chunk):
    g = dml.Simulation(p)
    g.set_chunk(chunk[0], chunk[1], dist)
    g.set_atoms(atoms)
    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    o.set_chunk(chunk[0], chunk[1], dist)
    return g, o


def test_bloques_routine_by_routine():
    p, dist = brown_params()
    chunk = read_chunk()
    g, o = pair(p, dist, brown_atoms(), chunk)
    g.setup()
    o.setup()
    check(g, o, "setup", lists=True)
    zmax0 = o.counters()["zmax"]
    for step in range(1, 9):
        g.cbrownian_hs(step)
        o.cbrownian_hs(step)
        assert g.test_update() == o.test_update()
        g.overlap_moveback(step)
        o.overlap_moveback(step)
        assert g.test_update() == o.test_update()
        assert g.capture_commit() == o.capture_commit()
        assert g.calc_rho() == o.calc_rho()
        g.bloques()
        o.bloques()
        check(g, o, "bloques %d" % step, lists=True)
    c = o.counters()
    assert c["zmax"] >= zmax0 + 2 * dist - 1e-9  # at least two chunks arrived
    assert c["n_atoms"] >= 602 + 2 * 301
    g.close()


def test_fused_steps_with_chunks():
    p, dist = brown_params(seed=91)
    chunk = read_chunk()
    g, o = pair(p, dist, brown_atoms(seed=8), chunk)
    g.setup()
    o.setup()
    zmax0 = o.counters()["zmax"]
    done = 0
    for n in (1, 9, 40, 150):
        g.step(n)
        o.step(n)
        done += n
        check(g, o, "after %d steps" % done, lists=(n == 150))
    c = o.counters()
    assert c["zmax"] >= zmax0 + 2 * dist - 1e-9 and c["nupd"] > 5
    g.close()


def test_chunk_batch_matches_oracle_per_replica():
    """Two replicas with their own seeds in one context, each equal to its
    oracle run; one of them starts from a lower box so that its chunks come
    at other steps."""
    p, dist = brown_params(seed=3)
    chunk = read_chunk()
    reps = [dml.replica_of(p, seed=31), dml.replica_of(p, seed=32, z0=90.0, z1=90.0 + dist,
                                                        zmax=90.0 + 2 * dist)]
    atoms = [brown_atoms(seed=40), brown_atoms(seed=41)]
    g = dml.Simulation(p, replicas=reps)
    g.set_chunk(chunk[0], chunk[1], dist)
    g.set_atoms(atoms)
    orcs = []
    for rep, at in zip(reps, atoms):
        o = oracle_lib.Oracle(replica_params(p, rep))
        o.set_atoms(at)
        o.set_chunk(chunk[0], chunk[1], dist)
        o.setup()
        orcs.append(o)
    g.setup()
    done = 0
    for n in (1, 24, 75):
        g.step(n)
        for o in orcs:
            o.step(n)
        done += n
        for r, o in enumerate(orcs):
            check(g, o, "after %d steps r%d" % (done, r), replica=r, lists=(n == 75))
    g.close()


def test_chunk_api_order_and_capacity():
    p, dist = brown_params()
    chunk = read_chunk()
    g = dml.Simulation(p)
    with pytest.raises(dml.DmlError) as e:  # the template must come first
        g.set_atoms(brown_atoms())
    assert e.value.code == dml.E_STATE
    g.close()
    # capacity for one chunk only: the second one stops with DML_E_CAPACITY
    q = dml.Params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(q))
    q.capacity = 602 + 301
    g = dml.Simulation(q)
    g.set_chunk(chunk[0], chunk[1], dist)
    g.set_atoms(brown_atoms())
    g.setup()
    with pytest.raises(dml.DmlError) as e:
        g.step(20)
    assert e.value.code == dml.E_CAPACITY
    g.close()
