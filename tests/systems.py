"""Seeded synthetic systems shared by the tests, the smoke check and bench.py.

The reference measures no public dataset; its configurations are generated.
These follow the benchmark configurations: a frozen bcc Li slab (a = 3.51 Å)
under ions placed by random sequential addition.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "din-mol-li_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

import dml  # noqa: E402


def c1_params(integrator=dml.INTEGRATOR_ERMAK, reservoir=dml.RESERVOIR_PISTON, seed=1234,
              h=1e-3, mnb=1024):
    """Config 1: 35.1 x 35.1 x 60 Å box, piston z0 = 30 Å, skin 10 Å, dt = 1 fs."""
    p = dml.default_params()
    p.box[:] = [35.1, 35.1, 60.0]
    p.z0, p.zmax = 30.0, 60.0
    p.h = h
    p.skin = 10.0
    p.integrator = integrator
    p.reservoir = reservoir
    p.seed = seed
    p.mnb = mnb
    return p


def c1_atoms(seed=7, n_ion=200, dmin=2.5, nz_slab=2):
    """400 frozen electrode atoms (10x10x2 bcc cells) + n_ion Li+ in z in [10, 60)."""
    return dml.slab_system(10, 10, nz_slab, 60.0, n_ion, 10.0, 60.0, seed, dmin=dmin)


def c2_params(seed=1234, mnb=1024):
    """Config 2: 351 x 351 x 320 Å, piston z0 = 160 Å, 1 fs, Ermak."""
    p = dml.default_params()
    p.box[:] = [351.0, 351.0, 320.0]
    p.z0, p.zmax = 160.0, 320.0
    p.h = 1e-3
    p.skin = 10.0
    p.seed = seed
    p.mnb = mnb
    return p


def c2_atoms(seed=7, n_ion=200000, dmin=2.5):
    """80 000 electrode atoms (100x100x4 bcc cells) + 200 000 Li+ in z in [15, 300)."""
    return dml.slab_system(100, 100, 4, 320.0, n_ion, 15.0, 300.0, seed, dmin=dmin)


def scaled_params(nx, box_z, z0, seed=1234):
    a = 3.51
    p = dml.default_params()
    p.box[:] = [nx * a, nx * a, box_z]
    p.z0, p.zmax = z0, box_z
    p.h = 1e-3
    p.skin = 10.0
    p.seed = seed
    return p


def gcmc_params(seed=99, integrator=dml.INTEGRATOR_BROWNIAN):
    """The reference's tests/gcmc run: 100^3 Å box, reservoir z in [80, 100],
    act 0.000627, 10 trials per step, dt = 5e-5 ps, skin 2 Å (Brownian)."""
    p = dml.default_params()
    p.box[:] = [100.0, 100.0, 100.0]
    p.z0, p.zmax = 80.0, 100.0
    p.h = 5e-5
    p.skin = 2.0
    p.integrator = integrator
    p.reservoir = dml.RESERVOIR_GCMC
    p.act = 0.000627
    p.nadj = 10
    p.seed = seed
    p.mnb = 512
    return p


def gcmc_atoms(seed=5):
    """602 Li+ (1 M in the 100^3 Å box, dana.F90:349-353) at >= 3.2 Å separation."""
    import numpy as np

    ions = dml.random_ions(seed, 602, 100.0, 100.0, 0.0, 100.0, 3.2)
    return {"pos": ions, "z": np.full(len(ions), dml.Z_LI, np.int32)}


def c5_small_params(seed=7, nadj=32):
    """Config-5-like electrode system at test size: 35.1 x 35.1 x 60 Å, Ermak,
    GCMC reservoir slab z in [40, 60]."""
    p = c1_params(seed=seed)
    p.reservoir = dml.RESERVOIR_GCMC
    p.z0, p.zmax = 40.0, 60.0
    p.act = 0.0045
    p.nadj = nadj
    # deleted atoms hold limbo slots until the next list rebuild
    p.capacity = 16384
    return p
