"""Host-side mirror of din-mol-Li's hot-path routines over the GB300 C ABI.

`Simulation` wraps one `dml_ctx` of libdml.so (include/dml.h).  Its methods
carry the names of the reference procedures they replace (src/dana.F90,
src/Neighbor.F90): `test_update`, `fuerza`, `ermak_a`, `ermak_b`,
`cbrownian_hs`, `overlap_moveback`, `capture_commit`, `calc_rho`, `maxz`,
plus `step(n)`, the fused loop body of dana.F90:173-265.

The CUDA library is the only implementation: if libdml.so is missing or
cannot reach a GPU, every call raises.  There is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from ._abi import *  # noqa: F401,F403
from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_DIR, "_build", "libdml.so")

_lib = None


class DmlError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_abi.STATUS.get(code, "?"), code, msg))
        self.code = code


def build(force=False, verbose=False):
    """Compiles libdml.so for sm_103a (din-mol-li_gb300/build.py)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("_dml_build", os.path.join(PKG_DIR, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force, verbose=verbose)


def lib():
    """Loads libdml.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libdml.so not built: run din-mol-li_gb300/build.py (no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    P = ctypes.POINTER
    L.dml_params_default.argtypes = [P(_abi.Params)]
    L.dml_params_default.restype = None
    L.dml_create.argtypes = [P(_abi.Params), P(vp)]
    L.dml_create_batch.argtypes = [P(_abi.Params), i32, P(_abi.Replica), P(vp)]
    L.dml_set_atoms_batch.argtypes = [vp, P(_abi.Atoms)]
    L.dml_num_replicas.argtypes = [vp]
    L.dml_get_atoms_replica.argtypes = [vp, i32, P(_abi.Atoms)]
    L.dml_get_atoms_batch.argtypes = [vp, vp]
    L.dml_get_atom_counts.argtypes = [vp, vp]
    L.dml_get_counters_replica.argtypes = [vp, i32, P(_abi.Counters)]
    L.dml_get_neighbors_replica.argtypes = [vp, i32, P(i32), vp, vp, i32]
    L.dml_destroy.argtypes = [vp]
    L.dml_destroy.restype = None
    L.dml_set_atoms.argtypes = [vp, P(_abi.Atoms)]
    L.dml_get_atoms.argtypes = [vp, P(_abi.Atoms)]
    for name in ["dml_setup", "dml_force", "dml_ermak_b", "dml_piston", "dml_sync",
                 "dml_reset_counters"]:
        getattr(L, name).argtypes = [vp]
    for name in ["dml_ermak_a", "dml_brownian", "dml_overlap_moveback", "dml_gcmc", "dml_step",
                 "dml_step_async"]:
        getattr(L, name).argtypes = [vp, i64]
    L.dml_test_update.argtypes = [vp, P(i32)]
    L.dml_capture_commit.argtypes = [vp, P(i32)]
    L.dml_calc_rho.argtypes = [vp, P(ctypes.c_double)]
    L.dml_get_neighbors.argtypes = [vp, P(i32), vp, vp, i32]
    L.dml_get_counters.argtypes = [vp, P(_abi.Counters)]
    L.dml_salida.argtypes = [vp, vp]
    L.dml_strerror.restype = ctypes.c_char_p
    L.dml_strerror.argtypes = [ctypes.c_int]
    L.dml_last_error.restype = ctypes.c_char_p
    L.dml_last_error.argtypes = [vp]
    L.dml_time_steps.argtypes = [vp, i64, i32, P(ctypes.c_double)]
    L.dml_time_run.argtypes = [vp, i64, P(ctypes.c_double)]
    L.dml_set_graph_steps.argtypes = [vp, i32]
    L.dml_set_chunk.argtypes = [vp, i32, vp, vp, ctypes.c_double]
    L.dml_set_cell_factor.argtypes = [vp, ctypes.c_double]
    L.dml_tune_cells.argtypes = [vp, i32, P(ctypes.c_double)]
    L.dml_get_cell_tuning.argtypes = [vp, P(ctypes.c_double), vp]
    L.dml_bloques.argtypes = [vp]
    L.dml_profile_steps.argtypes = [vp, i64, i32, vp, i32]
    L.dml_launches_per_step.argtypes = [vp, P(i32)]
    L.dml_get_tuning.argtypes = [vp, P(i32), vp]
    L.dml_check_conversions.argtypes = [vp, i64, vp, vp]
    L.dml_check_pick.argtypes = [vp, vp, i64, vp]
    L.dml_check_normals.argtypes = [vp, i64, i32, vp]
    L.dml_gen_bcc_slab.argtypes = [i32, i32, i32, ctypes.c_double, vp, i32]
    L.dml_gen_ions.argtypes = [ctypes.c_uint64, i32, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
    L.dml_gen_ions_batch.argtypes = [i32, P(_abi.IonSpec), vp, vp]
    L.dml_get_gcmc_paths.argtypes = [vp, i32, P(i64), P(i64)]
    L.dml_get_scan_counts.argtypes = [vp, i32, P(i64), P(i64)]
    L.dml_set_scan_lanes.argtypes = [vp, i32]
    L.dml_get_test_counts.argtypes = [vp, i32, P(i64), P(i64)]
    _lib = L
    return L


def default_params():
    p = _abi.Params()
    lib().dml_params_default(ctypes.byref(p))
    return p


def check_conversions(x):
    """The device's float64 -> float32 (round to nearest even) and exact
    float32 -> float64 conversions applied to x: (f32, back)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    f32 = np.zeros(x.shape, np.float32)
    back = np.zeros(x.shape, np.float64)
    rc = lib().dml_check_conversions(x.ctypes.data, x.size, f32.ctypes.data, back.ctypes.data)
    if rc:
        raise DmlError(rc, "dml_check_conversions")
    return f32, back


def check_normals(words, precision=PRECISION_FP64):
    """The device's Box-Muller normals of 32-bit word pairs (uint32 array of
    even length): float32 array of the same length.  PRECISION_FP64: the
    plain form's pair; PRECISION_MIXED: the chosen form's integrators' pair."""
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.zeros(w.shape, np.float32)
    rc = lib().dml_check_normals(w.ctypes.data, w.size // 2, precision, out.ctypes.data)
    if rc:
        raise DmlError(rc, "dml_check_normals")
    return out


def check_pick(k, n):
    """The device's deletion pick int(k * 2^-53 * n) + 1 (capped at n)."""
    k = np.ascontiguousarray(k, dtype=np.uint64)
    n = np.ascontiguousarray(n, dtype=np.int32)
    m = np.zeros(k.shape, np.int32)
    rc = lib().dml_check_pick(k.ctypes.data, n.ctypes.data, k.size, m.ctypes.data)
    if rc:
        raise DmlError(rc, "dml_check_pick")
    return m


def bcc_slab(nx, ny, nz, a=3.51):
    """Frozen bcc Li electrode: 2*nx*ny*nz positions."""
    n = 2 * nx * ny * nz
    out = np.zeros((n, 3))
    rc = lib().dml_gen_bcc_slab(nx, ny, nz, a, out.ctypes.data, n)
    if rc < 0:
        raise DmlError(-rc, "dml_gen_bcc_slab")
    return out


def random_ions(seed, n, box_x, box_y, zlo, zhi, dmin):
    """RSA ions with minimum separation dmin (x,y periodic), placed on the GPU."""
    out = np.zeros((n, 3))
    rc = lib().dml_gen_ions(seed, n, box_x, box_y, zlo, zhi, dmin, out.ctypes.data)
    if rc < 0:
        raise DmlError(-rc, "dml_gen_ions")
    return out


def random_ions_batch(specs):
    """RSA ions of several systems in one GPU launch (dml_gen_ions_batch).
    specs: sequence of (seed, n, box_x, box_y, zlo, zhi, dmin).  Returns
    (list of [n][3] arrays, per-system status array, call status)."""
    arr = (_abi.IonSpec * len(specs))(*[_abi.ion_spec(*s) for s in specs])
    total = sum(int(s[1]) for s in specs)
    out = np.zeros((total, 3))
    st = np.zeros(len(specs), np.int32)
    rc = lib().dml_gen_ions_batch(len(specs), arr, out.ctypes.data, st.ctypes.data)
    parts, off = [], 0
    for s in specs:
        parts.append(out[off:off + int(s[1])].copy())
        off += int(s[1])
    return parts, st, rc


def slab_system(nx, ny, nz_slab, box_z, n_ion, zlo, zhi, seed, a=3.51, dmin=2.5):
    """Electrode slab followed by ions, as sys%alist-ordered arrays."""
    slab = bcc_slab(nx, ny, nz_slab, a)
    ions = random_ions(seed, n_ion, nx * a, ny * a, zlo, zhi, dmin)
    pos = np.concatenate([slab, ions])
    z = np.concatenate([np.full(len(slab), Z_CG, np.int32), np.full(n_ion, Z_LI, np.int32)])
    return {"pos": pos, "z": z}


class Simulation:
    """One device context (dml_ctx); methods mirror the reference routines.

    With `replicas` (a list of `Replica`, see `replica_of`) the context runs
    that many independent systems in every launch (dml_create_batch);
    `set_atoms` then takes one array dict per replica and the per-replica
    getters take `replica=`.
    """

    def __init__(self, params, replicas=None):
        self.lib = lib()
        self.params = params
        h = ctypes.c_void_p()
        if replicas is None:
            self.n_rep = 1
            rc = self.lib.dml_create(ctypes.byref(params), ctypes.byref(h))
        else:
            self.n_rep = len(replicas)
            arr = (_abi.Replica * self.n_rep)(*replicas)
            rc = self.lib.dml_create_batch(ctypes.byref(params), self.n_rep, arr,
                                           ctypes.byref(h))
        if rc != 0:
            raise DmlError(rc, "dml_create")
        self.h = h
        self.batched = replicas is not None

    def close(self):
        if getattr(self, "h", None):
            self.lib.dml_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what=""):
        if rc != 0:
            raise DmlError(rc, "%s: %s" % (what, self.lib.dml_last_error(self.h).decode()))

    def set_atoms(self, arrays):
        if not self.batched:
            n = len(arrays["z"])
            a = _abi.atoms_struct(dict(arrays), n)
            self._check(self.lib.dml_set_atoms(self.h, ctypes.byref(a)), "dml_set_atoms")
            return
        if len(arrays) != self.n_rep:
            raise ValueError("set_atoms: one array dict per replica")
        keep = [dict(x) for x in arrays]
        structs = (_abi.Atoms * self.n_rep)(*[_abi.atoms_struct(x, len(x["z"])) for x in keep])
        self._check(self.lib.dml_set_atoms_batch(self.h, structs), "dml_set_atoms_batch")

    def setup(self):
        self._check(self.lib.dml_setup(self.h), "dml_setup")

    def step(self, n=1):
        self._check(self.lib.dml_step(self.h, n), "dml_step")

    def step_async(self, n=1):
        self._check(self.lib.dml_step_async(self.h, n), "dml_step_async")

    def sync(self):
        self._check(self.lib.dml_sync(self.h), "dml_sync")

    def test_update(self):
        r = ctypes.c_int32()
        self._check(self.lib.dml_test_update(self.h, ctypes.byref(r)), "dml_test_update")
        return r.value

    def fuerza(self):
        self._check(self.lib.dml_force(self.h), "dml_force")

    def ermak_a(self, step):
        self._check(self.lib.dml_ermak_a(self.h, step), "dml_ermak_a")

    def ermak_b(self):
        self._check(self.lib.dml_ermak_b(self.h), "dml_ermak_b")

    def cbrownian_hs(self, step):
        self._check(self.lib.dml_brownian(self.h, step), "dml_brownian")

    def overlap_moveback(self, step):
        self._check(self.lib.dml_overlap_moveback(self.h, step), "dml_overlap_moveback")

    def capture_commit(self):
        r = ctypes.c_int32()
        self._check(self.lib.dml_capture_commit(self.h, ctypes.byref(r)), "dml_capture_commit")
        return r.value

    def gcmc_run(self, step):
        self._check(self.lib.dml_gcmc(self.h, step), "dml_gcmc")

    def calc_rho(self):
        r = ctypes.c_double()
        self._check(self.lib.dml_calc_rho(self.h, ctypes.byref(r)), "dml_calc_rho")
        return r.value

    def maxz(self):
        self._check(self.lib.dml_piston(self.h), "dml_piston")

    def reset_counters(self):
        self._check(self.lib.dml_reset_counters(self.h), "dml_reset_counters")

    def salida(self):
        """salida's observables (dml_salida): one dict per replica with
        energia, temp, rho, zmax (the info line's), try_ and depo; try and
        depo are zero afterwards, as salida leaves them."""
        out = (_abi.Observables * self.n_rep)()
        self._check(self.lib.dml_salida(self.h, out), "dml_salida")
        return [o.as_dict() for o in out]

    def counters(self, replica=None):
        """Counters of one replica, or (replica=None) summed over replicas."""
        c = _abi.Counters()
        if replica is None:
            self._check(self.lib.dml_get_counters(self.h, ctypes.byref(c)), "dml_get_counters")
        else:
            self._check(self.lib.dml_get_counters_replica(self.h, replica, ctypes.byref(c)),
                        "dml_get_counters_replica")
        return c.as_dict()

    def get_atoms(self, n=None, replica=None, fields=None):
        """Atom state in sys%alist order; `fields` (names of dml_atoms
        members) limits what is copied back."""
        if replica is None and self.batched:
            replica = 0 if self.n_rep == 1 else None
            if replica is None:
                raise ValueError("get_atoms: pass replica= on a batch context")
        if n is None:
            n = self.counters(replica)["n_atoms"]
        out = _abi.empty_atoms(n, fields)
        a = _abi.atoms_struct(out, n)
        if replica is None:
            self._check(self.lib.dml_get_atoms(self.h, ctypes.byref(a)), "dml_get_atoms")
        else:
            self._check(self.lib.dml_get_atoms_replica(self.h, replica, ctypes.byref(a)),
                        "dml_get_atoms_replica")
        n = a.n
        return {k: v[:n] for k, v in out.items()}

    def get_atoms_batch(self, fields=None):
        """Every replica's atom state (dml_get_atoms_batch): a list of dicts
        as get_atoms(replica=r) returns, one device pass and one copy per
        replica and field."""
        cnt = np.zeros(self.n_rep, np.int32)
        self._check(self.lib.dml_get_atom_counts(self.h, cnt.ctypes.data), "dml_get_atom_counts")
        counts = [int(n) for n in cnt]
        outs = [_abi.empty_atoms(n, fields) for n in counts]
        arr = (_abi.Atoms * len(outs))()
        for r, (o, n) in enumerate(zip(outs, counts)):
            a = _abi.atoms_struct(o, n)
            arr[r] = a
        self._check(self.lib.dml_get_atoms_batch(self.h, arr), "dml_get_atoms_batch")
        return [{k: v[:arr[r].n] for k, v in o.items()} for r, o in enumerate(outs)]

    def time_steps(self, n, flush_l2=True):
        """Device time [ms] of n steps, each bracketed by CUDA events."""
        ms = ctypes.c_double()
        self._check(self.lib.dml_time_steps(self.h, n, 1 if flush_l2 else 0, ctypes.byref(ms)),
                    "dml_time_steps")
        return ms.value

    PHASES = ["integrate", "force_pairs", "force_sum", "test_update1", "overlap",
              "test_update2", "commit", "gcmc_cells", "gcmc", "rho_piston"]

    def set_chunk(self, pos, z, dist):
        """config_chunk: the chunk reservoir's template (positions as
        chunk.xyz gives them, elements) and chunk height; before set_atoms."""
        pos = np.ascontiguousarray(pos, np.float64)
        z = np.ascontiguousarray(z, np.int32)
        self._check(self.lib.dml_set_chunk(self.h, len(z), pos.ctypes.data, z.ctypes.data,
                                           float(dist)), "dml_set_chunk")

    def set_cell_factor(self, f):
        """Chosen form: cells of edge bound f * (rc + skin) (lists rebuilt)."""
        self._check(self.lib.dml_set_cell_factor(self.h, float(f)), "dml_set_cell_factor")

    def tune_cells(self, steps=10):
        """Chosen form: time the cell factors 1.0 .. 1.5 and keep the fastest."""
        b = ctypes.c_double()
        self._check(self.lib.dml_tune_cells(self.h, steps, ctypes.byref(b)), "dml_tune_cells")
        return b.value

    def cell_tuning(self):
        f = ctypes.c_double()
        us = np.zeros(6, np.float32)
        self._check(self.lib.dml_get_cell_tuning(self.h, ctypes.byref(f), us.ctypes.data),
                    "dml_get_cell_tuning")
        return {"factor": f.value,
                "us_per_step": {"%.1f" % (1.0 + 0.1 * v): float(us[v]) for v in range(6)}}

    def bloques(self):
        self._check(self.lib.dml_bloques(self.h), "dml_bloques")

    def time_run(self, n):
        """Device milliseconds of n steps queued as step(n) queues them."""
        ms = ctypes.c_double()
        self._check(self.lib.dml_time_run(self.h, n, ctypes.byref(ms)), "dml_time_run")
        return ms.value

    def set_graph_steps(self, k):
        self._check(self.lib.dml_set_graph_steps(self.h, k), "dml_set_graph_steps")

    def profile_steps(self, n, flush_l2=True):
        """Per-phase device time [ms] summed over n un-graphed steps."""
        out = np.zeros(len(self.PHASES))
        self._check(self.lib.dml_profile_steps(self.h, n, 1 if flush_l2 else 0, out.ctypes.data,
                                               len(out)), "dml_profile_steps")
        return dict(zip(self.PHASES, out.tolist()))

    def tuning(self):
        """Autotuner choice: {"scan_lanes": L, "scan_us": {1: t, 2: t, ..., 32: t}}."""
        lanes = ctypes.c_int32()
        us = np.zeros(6, np.float32)
        self._check(self.lib.dml_get_tuning(self.h, ctypes.byref(lanes), us.ctypes.data),
                    "dml_get_tuning")
        return {"scan_lanes": lanes.value,
                "scan_us": {l: float(t) for l, t in zip((1, 2, 4, 8, 16, 32), us)}}

    def launches_per_step(self):
        """(kernels per step without a rebuild, extra kernels per rebuild)."""
        r = ctypes.c_int32()
        n = self.lib.dml_launches_per_step(self.h, ctypes.byref(r))
        if n < 0:
            raise DmlError(-n, "dml_launches_per_step")
        return n, r.value

    def gcmc_paths(self, replica=0):
        """(parallel, sequential) gcmc_run calls of a replica so far."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.dml_get_gcmc_paths(self.h, replica, ctypes.byref(a),
                                                 ctypes.byref(b)), "dml_get_gcmc_paths")
        return a.value, b.value

    def scan_counts(self, replica=0):
        """(full, flagged-rows-only) force scans of a replica so far."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.dml_get_scan_counts(self.h, replica, ctypes.byref(a),
                                                  ctypes.byref(b)), "dml_get_scan_counts")
        return a.value, b.value

    def test_counts(self, replica=0):
        """(displacement tests, those decided by the exact FP64 pass) of a replica."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.dml_get_test_counts(self.h, replica, ctypes.byref(a),
                                                  ctypes.byref(b)), "dml_get_test_counts")
        return a.value, b.value

    def set_scan_lanes(self, lanes):
        """Pin the force scan's lanes per row (0: autotuned)."""
        self._check(self.lib.dml_set_scan_lanes(self.h, int(lanes)), "dml_set_scan_lanes")

    def get_neighbors(self, ld, replica=None):
        n_ref = self.counters(replica)["n_ref"]
        nn = np.zeros(max(n_ref, 1), np.int32)
        lst = np.zeros((max(n_ref, 1), ld), np.int32)
        nr = ctypes.c_int32()
        if replica is None:
            rc = self.lib.dml_get_neighbors(self.h, ctypes.byref(nr), nn.ctypes.data,
                                            lst.ctypes.data, ld)
        else:
            rc = self.lib.dml_get_neighbors_replica(self.h, replica, ctypes.byref(nr),
                                                    nn.ctypes.data, lst.ctypes.data, ld)
        self._check(rc, "dml_get_neighbors")
        return nn[: nr.value], lst[: nr.value]
