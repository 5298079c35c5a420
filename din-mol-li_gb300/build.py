"""Builds libdml.so, the GB300 (sm_103a) implementation behind include/dml.h.

Four translation units compiled in parallel and linked into one shared
library in din-mol-li_gb300/_build/:
  csrc/dml_kernels.cu  device kernels, --fmad=false (no contraction: the
                       plain form is bit-exact to the reference order)
  csrc/dml_api.cu      C ABI and host orchestration (-ffp-contract=off)
  csrc/dml_gen.cu      initial configurations: bcc electrode (host), random
                       sequential addition of ions (device), --fmad=false
  csrc/dml_noalloc.cu  dml_force_noalloc, scratch in a static device array
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdml.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not os.path.exists(NVCC):
    NVCC = "nvcc"

HEADERS = [os.path.join(ROOT, "include", "dml.h"), os.path.join(ROOT, "include", "dml_rng.h"),
           os.path.join(CSRC, "dml_internal.h")]

UNITS = [
    ("dml_kernels.cu", [NVCC, "-std=c++17", "-O3", "-lineinfo", "--fmad=false"] + ARCH +
     ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v"]),
    ("dml_noalloc.cu", [NVCC, "-std=c++17", "-O3", "-lineinfo", "--fmad=false"] + ARCH +
     ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]),
    ("dml_api.cu", [NVCC, "-std=c++17", "-O2"] + ARCH +
     ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]),
    ("dml_gen.cu", [NVCC, "-std=c++17", "-O3", "-lineinfo", "--fmad=false"] + ARCH +
     ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]),
]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compiles and links libdml.so when a source is newer than the library."""
    os.makedirs(OUT, exist_ok=True)
    objs, procs = [], []
    for src, cmd in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + HEADERS):
            full = cmd + ["-I", os.path.join(ROOT, "include"), "-c", s, "-o", o]
            if verbose:
                print(" ".join(full))
            log = open(o + ".log", "w")
            procs.append((src, subprocess.Popen(full, stdout=log, stderr=subprocess.STDOUT), o))
    failed = []
    for src, p, o in procs:
        if p.wait() != 0:
            failed.append(src)
    if failed:
        for src in failed:
            sys.stderr.write(open(os.path.join(OUT, src + ".o.log")).read())
        raise RuntimeError("libdml build failed: %s" % ", ".join(failed))
    if force or procs or _stale(LIB, objs):
        link = [NVCC, "-shared"] + ARCH + objs + ["-o", LIB + ".tmp", "-lcudart"]
        if verbose:
            print(" ".join(link))
        subprocess.check_call(link)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
