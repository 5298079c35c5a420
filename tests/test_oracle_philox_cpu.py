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
