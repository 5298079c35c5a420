"""Seeded synthetic systems shared by the tests, the smoke check and bench.py.

The reference measures no public dataset; its configurations are generated.
These follow the benchmark configurations: a frozen bcc Li slab (a = 3.51 Å)
under ions placed by random sequential addition.

Built without the CUDA library: parameters are ctypes structures filled
here, and atoms come from the oracle's serial generators
(oracle/oracle_gen.cpp), which the device generator equals bit for bit
(tests/test_gpu_rsa.py).  So the CPU arms of bench.py and the CPU tests load
nothing of the product.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "din-mol-li_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from dml import _abi as dml  # noqa: E402  (structures and constants only)
from tests import oracle_lib  # noqa: E402

# dml_params_default's list capacity (the reference's mnb = 10000 is sized
# for its host memory; tests/test_abi_cpu.py checks the two defaults agree)
DEFAULT_MNB = 1024


def default_params():
    """dml_params_default: the reference's constants, as the oracle states
    them, with the device's default list capacity."""
    p = oracle_lib.default_params()
    p.mnb = DEFAULT_MNB
    return p


def slab_system(*args, **kw):
    return oracle_lib.slab_system(*args, **kw)


def random_ions(*args):
    return oracle_lib.random_ions(*args)


def c1_params(integrator=dml.INTEGRATOR_ERMAK, reservoir=dml.RESERVOIR_PISTON, seed=1234,
              h=1e-3, mnb=1024):
    """Config 1: 35.1 x 35.1 x 60 Å box, piston z0 = 30 Å, skin 10 Å, dt = 1 fs."""
    p = default_params()
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
    return slab_system(10, 10, nz_slab, 60.0, n_ion, 10.0, 60.0, seed, dmin=dmin)


def c2_params(seed=1234, mnb=1024):
    """Config 2: 351 x 351 x 320 Å, piston z0 = 160 Å, 1 fs, Ermak."""
    p = default_params()
    p.box[:] = [351.0, 351.0, 320.0]
    p.z0, p.zmax = 160.0, 320.0
    p.h = 1e-3
    p.skin = 10.0
    p.seed = seed
    p.mnb = mnb
    return p


def c2_atoms(seed=7, n_ion=200000, dmin=2.5):
    """80 000 electrode atoms (100x100x4 bcc cells) + 200 000 Li+ in z in [15, 300)."""
    return slab_system(100, 100, 4, 320.0, n_ion, 15.0, 300.0, seed, dmin=dmin)


def scaled_params(nx, box_z, z0, seed=1234):
    a = 3.51
    p = default_params()
    p.box[:] = [nx * a, nx * a, box_z]
    p.z0, p.zmax = z0, box_z
    p.h = 1e-3
    p.skin = 10.0
    p.seed = seed
    return p


def gcmc_params(seed=99, integrator=dml.INTEGRATOR_BROWNIAN):
    """The reference's tests/gcmc run: 100^3 Å box, reservoir z in [80, 100],
    act 0.000627, 10 trials per step, dt = 5e-5 ps, skin 2 Å (Brownian)."""
    p = default_params()
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

    ions = random_ions(seed, 602, 100.0, 100.0, 0.0, 100.0, 3.2)
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


C5_CELLS, C5_IONS = 40, 20000


def c5_params(seed=11, precision=dml.PRECISION_MIXED, nadj=128, cells=C5_CELLS, n_ion=C5_IONS):
    """Config 5 replica: 40 x 40 x 2-cell electrode (140.4 Å square), 300 Å
    high, GCMC reservoir slab z in [200, 300] with `nadj` trials per step
    (half creations, half destructions on average), Ermak, dt = 1 fs,
    neighbour skin 2 Å (nb_dcut of the reference's GCMC run, tests/gcmc).
    slab_activity sets the activity that keeps the mean ion count fixed."""
    a = 3.51
    L = cells * a
    p = default_params()
    p.box[:] = [L, L, 300.0]
    p.z0, p.zmax = 200.0, 300.0
    p.h = 1e-3
    p.skin = 2.0
    p.reservoir = dml.RESERVOIR_GCMC
    p.nadj = nadj
    p.act = n_ion / (L * L * (300.0 - 15.0))
    p.precision = precision
    p.seed = seed
    p.mnb = 128
    # room for insertions while deleted atoms wait in limbo for a rebuild
    p.capacity = 2 * cells * cells * 2 + n_ion + 16384
    return p


def c5_batch(n_rep, seed=11, precision=dml.PRECISION_MIXED, nadj=128, cells=C5_CELLS,
             n_ion=C5_IONS):
    """n_rep config-5 replicas, each with its own Philox seed and ion
    placement.  Ions start at least rc = 3.2 Å apart: without a piston,
    ions left within rc of each other at their step-start positions would
    be moved back forever by overlap_moveback."""
    p = c5_params(seed, precision, nadj, cells, n_ion)
    reps = [dml.replica_of(p, seed=seed * 100003 + r) for r in range(n_rep)]
    atoms = [slab_system(cells, cells, 2, 300.0, n_ion, 15.0, 300.0, seed * 7919 + r, dmin=3.2)
             for r in range(n_rep)]
    p.act = slab_activity(p, atoms[0], seed)
    return p, reps, atoms


def slab_activity(p, atoms, seed, samples=20000):
    """Activity that keeps the slab count of `atoms` fixed on average:
    creation and destruction balance when act * V * P_ins = N_slab, with
    P_ins the chance that a uniform point of the slab lies at least rc from
    every ion (the hard-core test), estimated here by sampling."""
    import numpy as np
    from scipy.spatial import cKDTree

    L = p.box[0]
    ions = atoms["pos"][atoms["z"] != dml.Z_CG]
    n_slab = int(((ions[:, 2] >= p.z0) & (ions[:, 2] <= p.zmax)).sum())
    rng = np.random.default_rng(seed)
    pts = np.column_stack([rng.random(samples) * L, rng.random(samples) * L,
                           p.z0 + rng.random(samples) * (p.zmax - p.z0)])
    big = 4.0 * p.box[2] + 100.0  # no wrap along z
    tree = cKDTree(np.mod(ions, [L, L, big]), boxsize=[L, L, big])
    d, _ = tree.query(pts, k=1)
    p_ins = max(float((d >= p.rc).mean()), 1e-3)
    return n_slab / (L * L * (p.zmax - p.z0) * p_ins)


C4_REPLICAS = 1024


def c4_batch(n_rep=C4_REPLICAS, seed=13, precision=dml.PRECISION_MIXED):
    """Config 4: n_rep independent replicas of uneven size.  Replica r: a
    2-cell-thick bcc electrode of L x L cells, L uniform in 5..40; N ions,
    log-uniform in 50..20 000; the height set by the reference's 1 M rule
    (dana.F90:349-353: N = 6.022e-4 Lx Ly h, h above z = 10 Å, at least
    20 Å); its own Philox seed.  Brownian integrator with the reference's
    Brownian GCMC run time step and shell (tests/gcmc: 5e-5 ps, nb_dcut
    2 Å), piston reservoir at half height (the ratio of tests/ermak), ions
    at least rc = 3.2 Å apart."""
    import numpy as np

    rng = np.random.default_rng(seed)
    p = default_params()
    p.integrator = dml.INTEGRATOR_BROWNIAN
    p.reservoir = dml.RESERVOIR_PISTON
    p.h = 5e-5
    p.skin = 2.0
    p.precision = precision
    p.seed = seed
    p.mnb = 128
    a = 3.51
    reps, atoms = [], []
    for r in range(n_rep):
        cells = int(rng.integers(5, 41))
        n_ion = int(round(float(np.exp(rng.uniform(np.log(50.0), np.log(20000.0))))))
        L = cells * a
        height = max(20.0, n_ion / (6.022e-4 * L * L))
        lz = 10.0 + height
        rseed = seed * 100003 + r
        reps.append(dml.replica_of(p, box=[L, L, lz], z0=0.5 * lz, zmax=lz, seed=rseed))
        atoms.append(slab_system(cells, cells, 2, lz, n_ion, 10.0, lz, rseed, dmin=3.2))
    p.box[:] = list(reps[0].box)
    p.z0, p.zmax = reps[0].z0, reps[0].zmax
    return p, reps, atoms
