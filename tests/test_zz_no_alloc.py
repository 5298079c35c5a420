"""dml_force_noalloc: the pair force without any device allocation.

Some callers cannot allocate device memory: a host whose device memory
belongs to another allocator or runtime (a Fortran driver whose arrays a
CUDA Fortran or OpenACC runtime owns, a framework whose caching allocator has
reserved the free memory), or a time-stepping loop that must not call
cudaMalloc or cudaFree, which stall the host.  For them dml_force_noalloc
takes device arrays the caller already owns and keeps its scratch in a
fixed-size static device array.  These tests hand it the positions and lists
of a system and check, on two calls in a row, that its forces and energies
equal those of the context entry point dml_force and of the oracle's fuerza
bit for bit (the tolerance of the other force parity tests: zero), and that
its error returns leave the caller's outputs as they were.  Torch makes the
device buffers here, standing in for the caller's.
"""
import ctypes

import numpy as np
import pytest

from tests import oracle_lib, systems
import dml

pytestmark = pytest.mark.gpu

MAX_ATOMS = 16384
EV_CAP = 32


def _lib():
    dml.build()
    L = dml.lib()
    L.dml_force_noalloc.argtypes = [ctypes.POINTER(dml.Params), ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return L


def _call(L, torch, p, pos, z, ref_idx, nn, lst, force, epot, stream=None):
    """One dml_force_noalloc call on torch-owned device copies; returns
    (status, force, epot) as host arrays."""
    dev = torch.device("cuda")
    ld = int(max(1, lst.shape[1]))
    t_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).to(dev)
    t_z = torch.from_numpy(np.ascontiguousarray(z, np.int32)).to(dev)
    t_ref = torch.from_numpy(np.ascontiguousarray(ref_idx, np.int32)).to(dev)
    t_nn = torch.from_numpy(np.ascontiguousarray(nn, np.int32)).to(dev)
    t_list = torch.from_numpy(np.ascontiguousarray(lst, np.int32)).to(dev)
    t_f = torch.from_numpy(np.ascontiguousarray(force, np.float64)).to(dev)
    t_e = torch.from_numpy(np.ascontiguousarray(epot, np.float64)).to(dev)
    torch.cuda.synchronize()
    rc = L.dml_force_noalloc(ctypes.byref(p), len(z), t_pos.data_ptr(), t_z.data_ptr(),
                             len(ref_idx), t_ref.data_ptr(), t_nn.data_ptr(), t_list.data_ptr(),
                             ld, t_f.data_ptr(), t_e.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, t_f.cpu().numpy(), t_e.cpu().numpy()


def _bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def test_noalloc_force_matches_context_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = _lib()
    p = systems.c1_params()
    sim = dml.Simulation(p)
    sim.set_atoms(systems.c1_atoms(dmin=2.2, n_ion=300))  # many interacting pairs
    sim.setup()
    sim.step(5)
    before = sim.get_atoms()
    nn, lst = sim.get_neighbors(2048)
    sim.fuerza()  # existing entry point
    ref_out = sim.get_atoms()
    ref_idx = np.nonzero(before["in_ref"])[0].astype(np.int32)
    assert len(ref_idx) == len(nn)
    ld = int(max(1, nn.max()))
    for call in range(2):
        rc, f, e = _call(L, torch, p, before["pos"], before["z"], ref_idx, nn, lst[:, :ld],
                         before["force"], before["epot"])
        assert rc == 0, dml._abi.STATUS.get(rc, rc)
        assert _bits_equal(f, ref_out["force"]), call
        assert _bits_equal(e, ref_out["epot"]), call
    assert np.abs(ref_out["force"]).max() > 0
    sim.close()


def test_noalloc_force_matches_oracle_on_a_stream():
    """Positions and lists from the oracle after a few steps; the oracle's
    fuerza at that state is the answer.  The call goes on a stream of its
    own, twice."""
    torch = pytest.importorskip("torch")
    L = _lib()
    p = systems.c1_params(seed=4321)
    orc = oracle_lib.Oracle(p)
    orc.set_atoms(systems.c1_atoms(seed=9, dmin=2.2, n_ion=300))
    orc.setup()
    orc.step(4)
    before = orc.get_atoms()
    nn, lst = orc.get_neighbors(2048)
    orc.fuerza()
    want = orc.get_atoms()
    ref_idx = np.nonzero(before["in_ref"])[0].astype(np.int32)
    ld = int(max(1, nn.max()))
    st = torch.cuda.Stream()
    for call in range(2):
        rc, f, e = _call(L, torch, p, before["pos"], before["z"], ref_idx, nn, lst[:, :ld],
                         before["force"], before["epot"], stream=st.cuda_stream)
        assert rc == 0, dml._abi.STATUS.get(rc, rc)
        assert _bits_equal(f, want["force"]), call
        assert _bits_equal(e, want["epot"]), call
    assert np.abs(want["force"]).max() > 0


def _crowded(n_near):
    """Atom 0 at the centre of a 100 Å box with n_near Li+ around it, all
    within r0 = 3.2 Å of it: one hand-made list row of n_near interacting
    entries."""
    rng = np.random.default_rng(5)
    d = rng.normal(size=(n_near, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = 1.5 + 1.5 * rng.random(n_near)
    pos = np.vstack([[50.0, 50.0, 50.0], 50.0 + d * r[:, None]])
    z = np.full(n_near + 1, dml.Z_LI, np.int32)
    lst = np.arange(1, n_near + 1, dtype=np.int32)[None, :]
    return pos, z, np.zeros(1, np.int32), np.array([n_near], np.int32), lst


def test_noalloc_errors_leave_outputs_untouched():
    """More interacting entries for one atom than the scratch holds gives
    DML_E_EVENT_OVERFLOW, a list entry past the atom count DML_E_ARG; both
    are found on the device, and force and epot keep the caller's values."""
    torch = pytest.importorskip("torch")
    L = _lib()
    p = systems.c1_params()
    p.box[:] = [100.0, 100.0, 100.0]
    pos, z, ref_idx, nn, lst = _crowded(EV_CAP + 1)
    f0 = np.full((len(z), 3), 7.25)
    e0 = np.full(len(z), -3.5)
    rc, f, e = _call(L, torch, p, pos, z, ref_idx, nn, lst, f0, e0)
    assert rc == 14  # DML_E_EVENT_OVERFLOW
    assert _bits_equal(f, f0) and _bits_equal(e, e0)
    # the same system at the limit is fine
    pos, z, ref_idx, nn, lst = _crowded(EV_CAP)
    rc, f, e = _call(L, torch, p, pos, z, ref_idx, nn, lst, f0, e0)
    assert rc == 0
    assert np.abs(f[0]).max() > 0
    # an entry that names no atom
    bad = lst.copy()
    bad[0, 3] = len(z) + 5
    rc, f, e = _call(L, torch, p, pos, z, ref_idx, nn, bad, f0, e0)
    assert rc == 1  # DML_E_ARG
    assert _bits_equal(f, f0) and _bits_equal(e, e0)
    # and the next good call works again on the shared scratch
    rc, f, e = _call(L, torch, p, pos, z, ref_idx, nn, lst, f0, e0)
    assert rc == 0


def test_noalloc_rejects_sizes_beyond_its_maximum():
    L = _lib()
    p = systems.c1_params()
    dummy = ctypes.c_double()
    rc = L.dml_force_noalloc(ctypes.byref(p), MAX_ATOMS + 1, ctypes.addressof(dummy),
                             ctypes.addressof(dummy), 0, None, None, None, 0,
                             ctypes.addressof(dummy), ctypes.addressof(dummy), None)
    assert rc == 16  # DML_E_CAPACITY, before anything is launched
