"""The oracle in Philox mode runs the benchmark configurations on the CPU."""
import numpy as np

from tests import oracle_lib, systems


def _c1():
    p = systems.c1_params()
    o = oracle_lib.Oracle(p)
    o.set_atoms(systems.c1_atoms())
    o.setup()
    return o


def test_c1_setup_and_steps():
    o = _c1()
    c0 = o.counters()
    assert c0["nupd"] == 1 and c0["n_ref"] == 200 and c0["n_atoms"] == 600
    nn, lst = o.get_neighbors(2048)
    assert nn.max() > 0
    o.step(50)
    c = o.counters()
    assert c["step"] == 50
    a = o.get_atoms()
    assert np.isfinite(a["pos"]).all()
    assert (a["z"] >= 1).all() and (a["z"] <= 3).all()


def test_c1_is_deterministic():
    a = _c1()
    b = _c1()
    a.step(30)
    b.step(30)
    x, y = a.get_atoms(), b.get_atoms()
    for k in x:
        assert np.array_equal(x[k], y[k]), k


def test_duplicate_stencil_cells_in_c1():
    # 35.1 Å box with a 13.2 Å list radius gives 2 cells in x and y: the
    # stencil visits the other cell twice, so lists hold duplicate entries
    # (src/Cells.F90:378-404).
    o = _c1()
    nn, lst = o.get_neighbors(2048)
    dup = 0
    for k in range(len(nn)):
        row = lst[k, : nn[k]]
        dup += len(row) - len(np.unique(row))
    assert dup > 0


def test_gcmc_reference_case_runs():
    p = systems.gcmc_params()
    o = oracle_lib.Oracle(p)
    o.set_atoms(systems.gcmc_atoms())
    o.setup()
    o.step(200)
    c = o.counters()
    assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0
    a = o.get_atoms()
    assert len(a["z"]) == c["n_atoms"]


def test_c5_small_runs():
    p = systems.c5_small_params()
    o = oracle_lib.Oracle(p)
    o.set_atoms(systems.c1_atoms(dmin=3.2))
    o.setup()
    o.step(200)
    c = o.counters()
    assert c["gcmc_ins"] > 0 and c["gcmc_del"] > 0


def test_list_overflow_stops_at_setup():
    """More list entries than mnb: the reference writes past list(n, mnb)
    unchecked (src/Neighbor.F90:44,149); here the build stops with
    DML_E_NEIGH_OVERFLOW instead."""
    import pytest

    p = systems.c1_params()
    p.mnb = 8
    o = oracle_lib.Oracle(p)
    o.set_atoms(systems.c1_atoms())
    with pytest.raises(RuntimeError, match="NEIGH_OVERFLOW"):
        o.setup()


def test_deposit_above_z0_stops_the_run():
    """A contact capture of an ion above z0 ends the run ('supero z0',
    src/dana.F90:905-908) after try, depo and the element have changed."""
    import pytest

    from tests.test_salida_cpu import capture_params

    p, atoms = capture_params()
    p.z0 = 6.0  # just above the electrode's top layer
    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    o.setup()
    with pytest.raises(RuntimeError, match="DENDRITE"):
        o.step(50)
    c = o.counters()
    assert c["depo"] >= 1 and c["try_"] >= c["depo"]


def test_chunk_reservoir_adds_chunks():
    """The oracle's bloques in the keyed-stream mode: the tests/brown geometry
    takes chunks as the sensor empties (the chunk parity tests on the GPU
    compare the device with this)."""
    from tests.test_gpu_chunks import brown_atoms, brown_params, read_chunk

    p, dist = brown_params()
    pos, z = read_chunk()
    o = oracle_lib.Oracle(p)
    o.set_atoms(brown_atoms())
    o.set_chunk(pos, z, dist)
    o.setup()
    z0 = o.counters()["zmax"]
    o.step(5)
    c = o.counters()
    assert c["zmax"] >= z0 + 2 * dist - 1e-9
    assert c["n_atoms"] == 602 + 301 * round((c["zmax"] - z0) / dist)
