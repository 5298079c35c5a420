"""ctypes mirror of include/dml.h (structures and constants)."""
import ctypes

DML_OK = 0

STATUS = {
    0: "DML_OK",
    1: "DML_E_ARG",
    2: "DML_E_CUDA",
    3: "DML_E_NOMEM",
    4: "DML_E_OUT_OF_TESSELLATION",
    5: "DML_E_UNSORT",
    6: "DML_E_INDEX",
    7: "DML_E_NO_PARTICLES",
    8: "DML_E_CHOSEN_MISSING",
    9: "DML_E_RESERVOIR",
    10: "DML_E_DENDRITE",
    11: "DML_E_RSA",
    12: "DML_E_OVERLAP_PASSES",
    13: "DML_E_NEIGH_OVERFLOW",
    14: "DML_E_EVENT_OVERFLOW",
    15: "DML_E_FIXEDPOINT_OVERFLOW",
    16: "DML_E_CAPACITY",
    17: "DML_E_UNSUPPORTED",
    18: "DML_E_NEAR_OVERFLOW",
    19: "DML_E_STATE",
}
# E_ARG, E_CUDA, ...: the status codes by name
for _code, _name in STATUS.items():
    globals()[_name[len("DML_"):]] = _code

INTEGRATOR_BROWNIAN, INTEGRATOR_ERMAK = 0, 1
RESERVOIR_NONE, RESERVOIR_PISTON, RESERVOIR_CHUNKS, RESERVOIR_GCMC = 0, 1, 2, 3
PRECISION_FP64, PRECISION_MIXED = 0, 1
Z_LI, Z_CG, Z_F = 1, 2, 3

_d33 = (ctypes.c_double * 3) * 3


class Replica(ctypes.Structure):
    """struct dml_replica: the per-replica values of a batch context."""
    _fields_ = [
        ("box", ctypes.c_double * 3),
        ("z0", ctypes.c_double),
        ("zmax", ctypes.c_double),
        ("z1", ctypes.c_double),
        ("seed", ctypes.c_uint64),
    ]


class IonSpec(ctypes.Structure):
    """struct dml_ion_spec: one system of dml_gen_ions_batch."""
    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("n", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("box_x", ctypes.c_double),
        ("box_y", ctypes.c_double),
        ("zlo", ctypes.c_double),
        ("zhi", ctypes.c_double),
        ("dmin", ctypes.c_double),
    ]


def ion_spec(seed, n, box_x, box_y, zlo, zhi, dmin):
    return IonSpec(seed, n, 0, box_x, box_y, zlo, zhi, dmin)


def replica_of(params, **kw):
    """A Replica with params' box, z0, zmax, z1, seed, overridden by kw."""
    r = Replica()
    r.box[:] = list(kw.get("box", params.box))
    r.z0 = kw.get("z0", params.z0)
    r.zmax = kw.get("zmax", params.zmax)
    r.z1 = kw.get("z1", params.z1)
    r.seed = kw.get("seed", params.seed)
    return r


class Params(ctypes.Structure):
    _fields_ = [
        ("box", ctypes.c_double * 3),
        ("z0", ctypes.c_double),
        ("zmax", ctypes.c_double),
        ("z1", ctypes.c_double),
        ("h", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("temp", ctypes.c_double),
        ("kb_driver", ctypes.c_double),
        ("kb_module", ctypes.c_double),
        ("eps", _d33),
        ("r0", _d33),
        ("mass", ctypes.c_double * 3),
        ("rc", ctypes.c_double),
        ("skin", ctypes.c_double),
        ("prob", ctypes.c_double),
        ("dif_sc", ctypes.c_double),
        ("dif_sei", ctypes.c_double),
        ("dif_switch_z", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("act", ctypes.c_double),
        ("nadj", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("reservoir", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("mnb", ctypes.c_int32),
        ("capacity", ctypes.c_int32),
        ("max_passes", ctypes.c_int32),
        ("event_cap", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


class Atoms(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int32),
        ("pos", ctypes.c_void_p),
        ("vel", ctypes.c_void_p),
        ("acel", ctypes.c_void_p),
        ("force", ctypes.c_void_p),
        ("pos_old", ctypes.c_void_p),
        ("old_cg", ctypes.c_void_p),
        ("epot", ctypes.c_void_p),
        ("z", ctypes.c_void_p),
        ("skip", ctypes.c_void_p),
        ("in_ref", ctypes.c_void_p),
        ("in_gcmc", ctypes.c_void_p),
        ("id", ctypes.c_void_p),
    ]


class Counters(ctypes.Structure):
    _fields_ = [
        ("try_", ctypes.c_int64),
        ("depo", ctypes.c_int64),
        ("choques", ctypes.c_int64),
        ("choques3", ctypes.c_int64),
        ("nupd", ctypes.c_int64),
        ("step", ctypes.c_int64),
        ("gcmc_ins", ctypes.c_int64),
        ("gcmc_del", ctypes.c_int64),
        ("n_atoms", ctypes.c_int32),
        ("n_ref", ctypes.c_int32),
        ("max_nn", ctypes.c_int32),
        ("passes", ctypes.c_int32),
        ("zmax", ctypes.c_double),
        ("z0", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("rho0", ctypes.c_double),
        ("list_builds", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Observables(ctypes.Structure):
    """dml_observables: what salida writes for one replica."""
    _fields_ = [
        ("step", ctypes.c_int64),
        ("energia", ctypes.c_double),
        ("temp", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("zmax", ctypes.c_double),
        ("try_", ctypes.c_int64),
        ("depo", ctypes.c_int64),
        ("n_atoms", ctypes.c_int32),
        ("n_mobile", ctypes.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# Per-atom arrays of dml_atoms: name -> (numpy dtype, components)
ATOM_FIELDS = {
    "pos": ("f8", 3),
    "vel": ("f8", 3),
    "acel": ("f8", 3),
    "force": ("f8", 3),
    "pos_old": ("f8", 3),
    "old_cg": ("f8", 3),
    "epot": ("f8", 1),
    "z": ("i4", 1),
    "skip": ("i1", 1),
    "in_ref": ("i1", 1),
    "in_gcmc": ("i1", 1),
    "id": ("i8", 1),
}


def atoms_struct(arrays, n):
    """Builds a dml_atoms pointing at numpy arrays (absent keys -> NULL)."""
    import numpy as np

    a = Atoms()
    a.n = n
    keep = []
    for name, (dt, comp) in ATOM_FIELDS.items():
        arr = arrays.get(name)
        if arr is None:
            setattr(a, name, None)
            continue
        arr = np.ascontiguousarray(arr, dtype=dt)
        keep.append(arr)
        arrays[name] = arr
        setattr(a, name, arr.ctypes.data)
    a._keep = keep
    return a


def empty_atoms(n, fields=None):
    """Output arrays for n atoms: every field, or only those named in fields."""
    import numpy as np

    out = {}
    for name, (dt, comp) in ATOM_FIELDS.items():
        if fields is not None and name not in fields:
            continue
        shape = (n, comp) if comp > 1 else (n,)
        out[name] = np.empty(shape, dtype=dt)  # every element below the count is written
    return out
