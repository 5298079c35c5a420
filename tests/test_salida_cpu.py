"""salida's observables in the oracle (src/dana.F90:1143-1183, kion :1342-1376).

energia and kion's temperature are sums in sys%alist order, one term at a
time; the restatement here adds the oracle's own arrays with np.cumsum
(sequential, unlike Python's sum(), which compensates) and must match bit for
bit.  rho, try and depo are the counters, try and depo are zero after the
call, and zmax is the info line's: the value before the step's maxz.
"""
import numpy as np
import pytest

from tests import oracle_lib, systems
import dml


def salida_sums(atoms, p):
    """(energia, temp, j) of salida and kion over one system's arrays."""
    energia = float(np.cumsum(np.concatenate([[0.0], atoms["epot"]]))[-1])
    mob = atoms["z"] != dml.Z_CG
    v = atoms["vel"][mob]
    vd = v[:, 0] * v[:, 0]
    vd = vd + v[:, 1] * v[:, 1]
    vd = vd + v[:, 2] * v[:, 2]
    vd = vd * np.array(list(p.mass))[atoms["z"][mob] - 1]
    vdac = float(np.cumsum(np.concatenate([[0.0], vd]))[-1])
    j = int(mob.sum())
    return energia, vdac / (float(j) * 3.0 * p.kb_driver), j


def same_float(x, y):
    return np.float64(x).view(np.uint64) == np.float64(y).view(np.uint64)


def capture_params():
    """Brownian, no reservoir, ions next to the electrode: captures every
    few steps, so try and depo are non-zero."""
    p = systems.c1_params(integrator=dml.INTEGRATOR_BROWNIAN, reservoir=dml.RESERVOIR_NONE)
    p.h = 1e-2
    return p, systems.slab_system(10, 10, 2, 60.0, 150, 5.0, 20.0, 3, dmin=3.2)


@pytest.mark.parametrize("case", ["ermak_piston", "brownian_captures"])
def test_oracle_salida_is_the_reference_loops(case):
    if case == "ermak_piston":
        p, atoms = systems.c1_params(), systems.c1_atoms()
    else:
        p, atoms = capture_params()
    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    o.setup()
    o.step(59)  # an ion crosses z0 by then, so the piston moves zmax
    zmax_before = o.counters()["zmax"]
    o.step(1)
    c, a = o.counters(), o.get_atoms()
    s = o.salida()
    e, t, j = salida_sums(a, p)
    assert same_float(s["energia"], e) and same_float(s["temp"], t)
    assert s["n_mobile"] == j and s["n_atoms"] == c["n_atoms"] == len(a["z"])
    assert s["step"] == 60 and same_float(s["rho"], c["rho"])
    assert (s["try_"], s["depo"]) == (c["try_"], c["depo"])
    assert s["zmax"] == zmax_before
    if case == "ermak_piston":
        assert c["zmax"] != zmax_before  # the piston moved zmax after the output
        assert t > 0.0 and e > 0.0
    else:
        assert s["try_"] > 0 and s["depo"] > 0
    after = o.counters()
    assert after["try_"] == 0 and after["depo"] == 0
    again = o.salida()
    assert again["try_"] == 0 and again["depo"] == 0
    assert same_float(again["energia"], e)
