"""dml_salida on the device: salida's observables (src/dana.F90:1143-1183).

Plain FP64 form: every record equals the oracle's salida bit for bit, in
the piston, capture and GCMC systems.  Chosen form, batched: every
replica's record equals the reference's loops run on the arrays that
replica's download returns (sequential sums in sys%alist order).  In both,
try and depo are zero afterwards and zmax is the info line's: the value
before the last step's maxz.
"""
import numpy as np
import pytest

from tests import oracle_lib, systems
from tests.test_gpu_batch import uneven_replicas
from tests.test_salida_cpu import capture_params, same_float, salida_sums
import dml

pytestmark = pytest.mark.gpu

KEYS = ["step", "energia", "temp", "rho", "zmax", "try_", "depo", "n_atoms", "n_mobile"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    dml.build()


def case_system(case):
    if case == "ermak_piston":
        return systems.c1_params(), systems.c1_atoms()
    if case == "brownian_captures":
        return capture_params()
    p = systems.c5_small_params(nadj=32)
    return p, systems.c1_atoms(seed=8, n_ion=150, dmin=3.2)


def assert_same_record(a, b, where):
    for k in KEYS:
        same = same_float(a[k], b[k]) if isinstance(a[k], float) else a[k] == b[k]
        assert same, "%s: %s gpu %r oracle %r" % (where, k, a[k], b[k])


@pytest.mark.parametrize("case", ["ermak_piston", "brownian_captures", "gcmc"])
def test_salida_matches_oracle(case):
    p, atoms = case_system(case)
    g = dml.Simulation(p)
    o = oracle_lib.Oracle(p)
    g.set_atoms(atoms)
    o.set_atoms(atoms)
    g.setup()
    o.setup()
    assert_same_record(g.salida()[0], o.salida(), "setup")
    done = 0
    for chunk in (1, 19, 40):
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_record(g.salida()[0], o.salida(), "after %d steps" % done)
        c = g.counters()
        assert c["try_"] == 0 and c["depo"] == 0


def test_salida_batch_mixed_is_the_reference_loops():
    p = systems.c1_params()
    p.precision = dml.PRECISION_MIXED
    reps, atoms = uneven_replicas(p)
    g = dml.Simulation(p, replicas=reps)
    g.set_atoms(atoms)
    g.setup()
    g.step(59)
    zmax_before = [g.counters(replica=r)["zmax"] for r in range(len(reps))]
    g.step(1)
    cnt = [g.counters(replica=r) for r in range(len(reps))]
    arrays = g.get_atoms_batch(fields=("epot", "vel", "z"))
    obs = g.salida()
    assert len(obs) == len(reps)
    for r, (s, c, a) in enumerate(zip(obs, cnt, arrays)):
        e, t, j = salida_sums(a, p)
        where = "replica %d" % r
        assert same_float(s["energia"], e), where
        assert same_float(s["temp"], t), where
        assert s["n_mobile"] == j and s["n_atoms"] == c["n_atoms"] == len(a["z"]), where
        assert s["step"] == 60 and same_float(s["rho"], c["rho"]), where
        assert (s["try_"], s["depo"]) == (c["try_"], c["depo"]), where
        assert s["zmax"] == zmax_before[r], where
        after = g.counters(replica=r)
        assert after["try_"] == 0 and after["depo"] == 0, where
    assert any(c["zmax"] != z for c, z in zip(cnt, zmax_before))
    again = g.salida()
    assert all(s["try_"] == 0 and s["depo"] == 0 for s in again)
