"""dml_force_noalloc: the pair force without any device allocation.

Some callers cannot allocate device memory: code that runs while a stream is
captured into a CUDA graph (cudaMalloc is not allowed there), drivers whose
device buffers belong to another runtime, loops that must not allocate.  For
them dml_force_noalloc takes caller-provided device arrays and keeps its
scratch in a fixed-size static device array.  This test hands it the
positions and lists of a system and checks, on two calls in a row, that its
forces and energies equal those of the context entry point dml_force bit for
bit (the tolerance of the other force parity tests: zero).  Its own device
buffers are made by torch here, standing in for the caller's.
"""
import ctypes

import numpy as np
import pytest

from tests import systems
import dml

pytestmark = pytest.mark.gpu

MAX_ATOMS = 16384


def _lib():
    dml.build()
    L = dml.lib()
    L.dml_force_noalloc.argtypes = [ctypes.POINTER(dml.Params), ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return L


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
    n = len(before["z"])
    ref_idx = np.nonzero(before["in_ref"])[0].astype(np.int32)
    assert len(ref_idx) == len(nn)
    ld = int(max(1, nn.max()))
    dev = torch.device("cuda")
    t_pos = torch.from_numpy(np.ascontiguousarray(before["pos"])).to(dev)
    t_z = torch.from_numpy(before["z"].astype(np.int32)).to(dev)
    t_ref = torch.from_numpy(ref_idx).to(dev)
    t_nn = torch.from_numpy(nn.astype(np.int32)).to(dev)
    t_list = torch.from_numpy(np.ascontiguousarray(lst[:, :ld]).astype(np.int32)).to(dev)
    for call in range(2):
        t_f = torch.from_numpy(np.ascontiguousarray(before["force"])).to(dev)
        t_e = torch.from_numpy(np.ascontiguousarray(before["epot"])).to(dev)
        torch.cuda.synchronize()
        rc = L.dml_force_noalloc(ctypes.byref(p), n, t_pos.data_ptr(), t_z.data_ptr(),
                                 len(ref_idx), t_ref.data_ptr(), t_nn.data_ptr(),
                                 t_list.data_ptr(), ld, t_f.data_ptr(), t_e.data_ptr(), None)
        assert rc == 0, dml._abi.STATUS.get(rc, rc)
        f = t_f.cpu().numpy()
        e = t_e.cpu().numpy()
        assert np.array_equal(f.view(np.uint64), ref_out["force"].view(np.uint64)), call
        assert np.array_equal(e.view(np.uint64), ref_out["epot"].view(np.uint64)), call
    assert np.abs(ref_out["force"]).max() > 0
    sim.close()


def test_noalloc_rejects_sizes_beyond_its_maximum():
    L = _lib()
    p = systems.c1_params()
    dummy = ctypes.c_double()
    rc = L.dml_force_noalloc(ctypes.byref(p), MAX_ATOMS + 1, ctypes.addressof(dummy),
                             ctypes.addressof(dummy), 0, None, None, None, 0,
                             ctypes.addressof(dummy), ctypes.addressof(dummy), None)
    assert rc == 16  # DML_E_CAPACITY, before anything is launched
