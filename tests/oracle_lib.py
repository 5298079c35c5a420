"""TEST INFRASTRUCTURE: ctypes loader for the oracle (oracle/dana_oracle.cpp).

The oracle is a serial CPU restatement of the reference's hot path.  It is
the checker for the CUDA path and is never imported by the product.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "din-mol-li_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from dml import _abi  # noqa: E402

RNG_NR = 0
RNG_PHILOX = 1

_lib = None


def oracle_build():
    """oracle/build.py as a module of its own name (not a bare "build",
    which an installed package of that name could shadow)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("_dml_oracle_build",
                                                  os.path.join(ROOT, "oracle", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = oracle_build().build()
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [ctypes.POINTER(_abi.Params), i32, i32]
    lib.orc_destroy.argtypes = [vp]
    for name in ["orc_setup", "orc_force", "orc_ermak_b", "orc_piston", "orc_reset_counters"]:
        getattr(lib, name).argtypes = [vp]
    for name in ["orc_step", "orc_ermak_a", "orc_brownian", "orc_overlap_moveback", "orc_gcmc"]:
        getattr(lib, name).argtypes = [vp, i64]
    lib.orc_set_atoms.argtypes = [vp, ctypes.POINTER(_abi.Atoms)]
    lib.orc_get_atoms.argtypes = [vp, ctypes.POINTER(_abi.Atoms)]
    lib.orc_test_update.argtypes = [vp, ctypes.POINTER(i32)]
    lib.orc_capture_commit.argtypes = [vp, ctypes.POINTER(i32)]
    lib.orc_calc_rho.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    lib.orc_get_neighbors.argtypes = [vp, ctypes.POINTER(i32), vp, vp, i32]
    lib.orc_get_counters.argtypes = [vp, ctypes.POINTER(_abi.Counters)]
    lib.orc_salida.argtypes = [vp, ctypes.POINTER(_abi.Observables)]
    lib.orc_errmsg.restype = ctypes.c_char_p
    lib.orc_errmsg.argtypes = [vp]
    lib.orc_set_step.argtypes = [vp, i64]
    lib.orc_run_reference_case.argtypes = [ctypes.c_char_p, i32, ctypes.POINTER(i32), vp, vp,
                                           ctypes.POINTER(ctypes.c_double), vp]
    lib.orc_rng_draw.argtypes = [ctypes.c_uint64, i64, ctypes.c_uint64, ctypes.c_uint32,
                                 ctypes.c_uint32, vp]
    lib.orc_rng_logf.restype = ctypes.c_float
    lib.orc_rng_logf.argtypes = [ctypes.c_float]
    lib.orc_rng_sincosf_2pi.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_float)]
    lib.orc_rng_normal_quad.argtypes = [vp, vp]
    lib.orc_rng_normal_pairs.argtypes = [vp, i64, vp]
    lib.orc_set_chunk.argtypes = [vp, i32, vp, vp, ctypes.c_double]
    lib.orc_bloques.argtypes = [vp]
    lib.orc_gen_bcc_slab.argtypes = [i32, i32, i32, ctypes.c_double, vp, i32]
    lib.orc_gen_ions.argtypes = [ctypes.c_uint64, i32, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
    _lib = lib
    return lib


def bcc_slab(nx, ny, nz, a=3.51):
    """Frozen bcc Li electrode: 2*nx*ny*nz positions (oracle/oracle_gen.cpp)."""
    n = 2 * nx * ny * nz
    out = np.zeros((n, 3))
    rc = load().orc_gen_bcc_slab(nx, ny, nz, a, out.ctypes.data, n)
    if rc < 0:
        raise RuntimeError("orc_gen_bcc_slab: %s" % _abi.STATUS.get(-rc, rc))
    return out


def gen_ions(seed, n, box_x, box_y, zlo, zhi, dmin):
    """Serial random sequential addition (oracle/oracle_gen.cpp): the checker
    of the device generator.  Returns (positions, status)."""
    out = np.zeros((n, 3))
    rc = load().orc_gen_ions(seed, n, box_x, box_y, zlo, zhi, dmin, out.ctypes.data)
    return out, -rc if rc < 0 else 0


def random_ions(seed, n, box_x, box_y, zlo, zhi, dmin):
    out, st = gen_ions(seed, n, box_x, box_y, zlo, zhi, dmin)
    if st:
        raise RuntimeError("orc_gen_ions: %s" % _abi.STATUS.get(st, st))
    return out


def slab_system(nx, ny, nz_slab, box_z, n_ion, zlo, zhi, seed, a=3.51, dmin=2.5):
    """Electrode slab followed by ions, as sys%alist-ordered arrays."""
    slab = bcc_slab(nx, ny, nz_slab, a)
    ions = random_ions(seed, n_ion, nx * a, ny * a, zlo, zhi, dmin)
    pos = np.concatenate([slab, ions])
    z = np.concatenate([np.full(len(slab), _abi.Z_CG, np.int32),
                        np.full(n_ion, _abi.Z_LI, np.int32)])
    return {"pos": pos, "z": z}


def default_params():
    """The reference constants as the oracle states them (oracle/oracle.h)."""
    p = _abi.Params()
    ctypes.memset(ctypes.byref(p), 0, ctypes.sizeof(p))
    eV_ui = 96.485 * 100.0
    joule_ev = 1.0 / 1.60219e-19
    ui_ev = 1.0e2 * 1.0e2 * 1.6605402e-27 * joule_ev
    ev_ui = 1.0 / ui_ev
    p.box[:] = [100.0, 100.0, 200.0]
    p.z0, p.zmax, p.z1 = 100.0, 200.0, 0.0
    p.h, p.gamma, p.temp = 1.e-2, 1.0, 300.0
    p.kb_driver = 8.617330350e-5 * eV_ui
    p.kb_module = 8.617385e-05 * ev_ui
    r0 = [[3.2, 3.5, 1.564], [3.5, 0.0, 0.0], [1.564, 0.0, 3.61]]
    eps = [[2313.6, 0.0, 529.1], [0.0, 0.0, 0.0], [529.1, 0.0, 121.0]]
    for i in range(3):
        for j in range(3):
            p.r0[i][j] = r0[i][j]
            p.eps[i][j] = eps[i][j]
    p.mass[:] = [6.94, 6.94, 6.94]
    p.rc, p.skin, p.prob = 3.2, 10.0, 1.0
    p.dif_sc, p.dif_sei, p.dif_switch_z, p.tau = 250.0, 250.0, 80.0, 0.1
    p.integrator, p.reservoir = _abi.INTEGRATOR_ERMAK, _abi.RESERVOIR_PISTON
    p.mnb, p.max_passes, p.event_cap = 10000, 64, 64
    return p


class Oracle:
    """One oracle simulation; method names follow the reference routines."""

    def __init__(self, params, rng_mode=RNG_PHILOX, idum=0):
        self.lib = load()
        self.p = params
        self.h = self.lib.orc_create(ctypes.byref(params), rng_mode, idum)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: %s (%s)" % (_abi.STATUS.get(rc, rc),
                                                    self.lib.orc_errmsg(self.h).decode()))
        return rc

    def set_atoms(self, arrays):
        n = len(arrays["z"])
        a = _abi.atoms_struct(dict(arrays), n)
        self._check(self.lib.orc_set_atoms(self.h, ctypes.byref(a)))

    def setup(self):
        self._check(self.lib.orc_setup(self.h))

    def step(self, n=1):
        self._check(self.lib.orc_step(self.h, n))

    def test_update(self):
        r = ctypes.c_int32()
        self._check(self.lib.orc_test_update(self.h, ctypes.byref(r)))
        return r.value

    def fuerza(self):
        self._check(self.lib.orc_force(self.h))

    def ermak_a(self, step):
        self._check(self.lib.orc_ermak_a(self.h, step))

    def ermak_b(self):
        self._check(self.lib.orc_ermak_b(self.h))

    def cbrownian_hs(self, step):
        self._check(self.lib.orc_brownian(self.h, step))

    def overlap_moveback(self, step):
        self._check(self.lib.orc_overlap_moveback(self.h, step))

    def capture_commit(self):
        r = ctypes.c_int32()
        self._check(self.lib.orc_capture_commit(self.h, ctypes.byref(r)))
        return r.value

    def gcmc_run(self, step):
        self._check(self.lib.orc_gcmc(self.h, step))

    def calc_rho(self):
        r = ctypes.c_double()
        self._check(self.lib.orc_calc_rho(self.h, ctypes.byref(r)))
        return r.value

    def maxz(self):
        self._check(self.lib.orc_piston(self.h))

    def set_chunk(self, pos, z, dist):
        """config_chunk: the chunk template (positions as chunk.xyz gives them)."""
        pos = np.ascontiguousarray(pos, np.float64)
        z = np.ascontiguousarray(z, np.int32)
        self._check(self.lib.orc_set_chunk(self.h, len(z), pos.ctypes.data, z.ctypes.data, dist))

    def bloques(self):
        self._check(self.lib.orc_bloques(self.h))

    def set_step(self, step):
        self.lib.orc_set_step(self.h, step)

    def counters(self):
        c = _abi.Counters()
        self._check(self.lib.orc_get_counters(self.h, ctypes.byref(c)))
        return c.as_dict()

    def salida(self):
        r = _abi.Observables()
        self._check(self.lib.orc_salida(self.h, ctypes.byref(r)))
        return r.as_dict()

    def get_atoms(self):
        n = self.counters()["n_atoms"]
        out = _abi.empty_atoms(n)
        a = _abi.atoms_struct(out, n)
        self._check(self.lib.orc_get_atoms(self.h, ctypes.byref(a)))
        return out

    def get_neighbors(self, ld):
        n_ref = self.counters()["n_ref"]
        nn = np.zeros(n_ref, np.int32)
        lst = np.zeros((n_ref, ld), np.int32)
        nr = ctypes.c_int32()
        self._check(self.lib.orc_get_neighbors(self.h, ctypes.byref(nr), nn.ctypes.data,
                                               lst.ctypes.data, ld))
        return nn, lst


def run_reference_case(case_dir, cap=10000):
    lib = load()
    pos = np.zeros((cap, 3))
    z = np.zeros(cap, np.int32)
    n = ctypes.c_int32()
    zmax = ctypes.c_double()
    cnt = np.zeros(4, np.int64)
    rc = lib.orc_run_reference_case(case_dir.encode(), cap, ctypes.byref(n), pos.ctypes.data,
                                    z.ctypes.data, ctypes.byref(zmax), cnt.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle reference case failed: %s" % _abi.STATUS.get(rc, rc))
    return pos[: n.value].copy(), z[: n.value].copy(), zmax.value, cnt


def read_xyz_frame(path):
    """Parses a reference Li.xyz frame (list-directed, 17 significant digits)."""
    lines = open(path).read().splitlines()
    n = int(lines[0].split()[0])
    zmax = float(lines[1].split()[1])
    pos = np.zeros((n, 3))
    z = np.zeros(n, np.int32)
    for i in range(n):
        t = lines[2 + i].split()
        pos[i] = [float(t[1]), float(t[2]), float(t[3])]
        z[i] = int(t[4])
    return pos, z, zmax
