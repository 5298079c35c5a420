"""CPU checks of the product library: it builds, loads without a GPU and
exports every entry point include/dml.h declares; host-side generators."""
import ctypes
import os
import re

import numpy as np

from tests import systems  # noqa: F401  (sets sys.path)
import dml

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for hdr in ["dml.h"]:
        text = open(os.path.join(ROOT, "include", hdr)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(dml_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_all_symbols():
    path = dml.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert "dml_create" in names and "dml_step" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_default_params_match_reference_constants():
    p = dml.default_params()
    assert p.eps[0][0] == 2313.6 and p.r0[0][0] == 3.2
    assert p.r0[0][1] == 3.5 and p.eps[0][1] == 0.0
    assert p.eps[0][2] == 529.1 and p.r0[0][2] == 1.564
    assert p.eps[2][2] == 121.0 and p.r0[2][2] == 3.61
    assert p.kb_driver == 8.617330350e-5 * (96.485 * 100.0)
    assert abs(p.kb_module / p.kb_driver - 1) < 1e-4
    assert p.rc == 3.2 and p.tau == 0.1 and p.gamma == 1.0 and p.temp == 300.0


def test_strerror_names_reference_messages():
    lib = dml.lib()
    assert lib.dml_strerror(4) == b"Particle out of tessellation"
    assert lib.dml_strerror(7) == b"No more particles"


def test_bcc_slab_and_ions():
    """The product's electrode lattice (host code) equals the oracle's; the
    oracle's serial ion placement (the checker of the device generator and
    the source of every test system) keeps the separation."""
    from tests import oracle_lib

    slab = dml.bcc_slab(10, 10, 2)
    assert slab.shape == (400, 3)
    assert slab[:, 2].max() == 1.5 * 3.51
    assert np.array_equal(slab.view(np.uint64), oracle_lib.bcc_slab(10, 10, 2).view(np.uint64))
    ions = oracle_lib.random_ions(7, 200, 35.1, 35.1, 10.0, 60.0, 2.5)
    d = ions[:, None, :] - ions[None, :, :]
    d[..., :2] -= 35.1 * np.round(d[..., :2] / 35.1)
    r2 = (d ** 2).sum(-1) + np.eye(len(ions)) * 1e9
    assert r2.min() >= 2.5 ** 2
    # too many ions for the volume: every try of some ion is rejected
    _, st = oracle_lib.gen_ions(3, 400, 10.0, 10.0, 0.0, 10.0, 3.2)
    assert st == dml.E_RSA


def test_test_systems_use_the_library_defaults():
    """tests/systems.py fills parameters without the library; they equal
    dml_params_default byte for byte."""
    a = dml.default_params()
    b = systems.default_params()
    assert bytes(a) == bytes(b)


def test_create_rejects_unsupported_options_without_gpu():
    p = systems.c1_params()
    p.box[0] = 10.0  # minimum image ambiguous at the list radius
    h = ctypes.c_void_p()
    assert dml.lib().dml_create(ctypes.byref(p), ctypes.byref(h)) == 1


def test_ctypes_mirrors_match_header_layout(tmp_path):
    """Every ctypes mirror of a dml.h struct has the header's size and field
    offsets, as gcc lays the header out on this host."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest

        pytest.skip("no C compiler")
    mirrors = {"dml_params": dml.Params, "dml_replica": dml.Replica, "dml_atoms": dml.Atoms,
               "dml_counters": dml.Counters, "dml_observables": dml.Observables,
               "dml_ion_spec": dml.IonSpec}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "dml.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                           str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in mirrors.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[cname + "." + f]) == getattr(py, f).offset, cname + "." + f


def test_ion_placement_errors():
    """Random sequential addition that cannot place every ion stops with
    DML_E_RSA (the reference's own stop, src/dana.F90:386-389), in the
    oracle's serial generator here and in the device generator on the GPU
    (tests/test_gpu_rsa.py); malformed boxes are DML_E_ARG before the
    device is touched."""
    import pytest

    from tests import oracle_lib

    _, st = oracle_lib.gen_ions(1, 1000, 10.0, 10.0, 0.0, 10.0, 5.0)  # 1000 ions 5 Å apart
    assert st == dml.E_RSA
    _, st = oracle_lib.gen_ions(1, 10, -1.0, 10.0, 0.0, 10.0, 1.0)
    assert st == dml.E_ARG
    with pytest.raises(dml.DmlError) as e:
        dml.random_ions(1, 10, -1.0, 10.0, 0.0, 10.0, 1.0)
    assert e.value.code == dml.E_ARG
    assert dml.random_ions(1, 0, 10.0, 10.0, 0.0, 10.0, 1.0).shape == (0, 3)


def kernel_bodies(src):
    """(name, first statement) of every __global__ definition in a source."""
    out = []
    for m in re.finditer(r"__global__", src):
        k, depth, seen = m.end(), 0, False
        while True:
            c = src[k]
            if c == "(":
                depth, seen = depth + 1, True
            elif c == ")":
                depth -= 1
            elif depth == 0 and seen and c in ";{":
                break
            k += 1
        if src[k] == ";":
            continue  # a declaration
        head = src[m.end():k]
        name = re.findall(r"(\w+)\s*\(", re.sub(r"__launch_bounds__\s*\([^)]*\)", "", head))[0]
        out.append((name, src[k + 1:].lstrip().split(";", 1)[0]))
    return out


def test_every_graph_kernel_waits_for_its_predecessor():
    """The step graphs' kernel-to-kernel edges are programmatic, so a kernel
    may be launched before the one it follows has completed; each kernel
    must begin with the grid-dependency wait before it touches memory."""
    csrc = os.path.join(ROOT, "din-mol-li_gb300", "csrc")
    seen = 0
    for f in ("dml_kernels.cu", "dml_noalloc.cu"):
        for name, first in kernel_bodies(open(os.path.join(csrc, f)).read()):
            seen += 1
            assert first == "DML_GRID_WAIT()", (f, name, first)
    assert seen >= 60
