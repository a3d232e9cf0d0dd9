"""Builds libgdtk_chem.so (in this directory) from csrc/ with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared library.  The
chemistry kernels are compiled with --fmad=false: the reference's x86-64 build evaluates
a*b+c with two roundings, and the kernels restate its arithmetic in the same order.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgdtk_chem.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")

SOURCES = [
    ("chem_kernels.cu", ["--fmad=false"]),
    ("fp64_probe.cu", []),
    ("chem_api.cpp", []),
    ("mechanism.cpp", []),
    ("lua_table.cpp", []),
]
HEADERS = ["chem_types.h", "chem_launch.h", "cea_thermo.h", "lua_table.h", "mechanism.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, src + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
           [os.path.join(HERE, "..", "include", "gdtk_chem.h"), __file__]
    if not _newer(obj, deps):
        return obj
    cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                           "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(*s), SOURCES))
    if _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
