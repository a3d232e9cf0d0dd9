"""Builds libgdtk_chem.so (in this directory) from csrc/ with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared library.  The
reference-order chemistry kernels (chem_kernels.cu) are compiled with --fmad=false: the reference's
x86-64 build evaluates a*b+c with two roundings, and those kernels restate its arithmetic in the same
order.
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
    ("chem_warp.cu", []),
    ("twotemp_kernels.cu", []),
    ("twotemp.cpp", []),
    ("codegen.cpp", []),
    ("fp64_probe.cu", []),
    ("noalloc.cu", []),
    ("mlp_kernels.cu", []),
    ("mlp_tcgen05.cu", []),
    ("surrogate_kernels.cu", []),
    ("surrogate.cpp", []),
    ("chem_api.cpp", []),
    ("mechanism.cpp", []),
    ("lua_table.cpp", []),
]
HEADERS = ["chem_kernels.cu", "chem_types.h", "chem_launch.h", "cea_thermo.h", "lua_table.h", "mechanism.h", "codegen.h", "fast_exp.h",
           "chem_fast.cuh", "mix_thermo.cuh", "api_internal.h", "mlp_launch.h", "surrogate_launch.h", "twotemp.h"]
# sources compiled at run time by NVRTC, embedded in the library as string literals
EMBEDDED = [("kFastCuhSource", "chem_fast.cuh"), ("kFastExpSource", "fast_exp.h")]


def _write_embedded():
    path = os.path.join(OUT_DIR, "embedded_sources.cpp")
    parts = ["// generated by buildlib.py from csrc/: sources compiled at run time by NVRTC",
             "namespace gdtk {"]
    for name, fn in EMBEDDED:
        with open(os.path.join(CSRC, fn)) as f:
            text = f.read()
        if ")GDTKSRC\"" in text:
            raise RuntimeError("embedded source contains the raw-string delimiter")
        parts.append('extern const char* const %s = R"GDTKSRC(%s)GDTKSRC";' % (name, text))
    parts.append("}")
    new = "\n".join(parts) + "\n"
    old = open(path).read() if os.path.exists(path) else None
    if old != new:
        with open(path, "w") as f:
            f.write(new)
    return path


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    srcpath = src if os.path.isabs(src) else os.path.join(CSRC, src)
    deps = [srcpath] + [os.path.join(CSRC, h) for h in HEADERS] + \
           [os.path.join(HERE, "..", "include", h) for h in ("gdtk_chem.h", "gdtk_surrogate.h")] + [__file__]
    if not _newer(obj, deps):
        return obj
    cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                           "-I", CSRC, "-c", srcpath, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def _which(prog):
    for d in os.environ.get("PATH", "").split(os.pathsep):
        c = os.path.join(d, prog)
        if os.path.isfile(c) and os.access(c, os.X_OK):
            return os.path.realpath(c)
    return "/usr/local/cuda/bin/nvcc"


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    sources = SOURCES + [(_write_embedded(), [])]
    with ThreadPoolExecutor(max_workers=len(sources)) as ex:
        objs = list(ex.map(lambda s: _compile(*s), sources))
    if _newer(LIB, objs):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(_which(NVCC))), "lib64")
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lnvrtc",
                                                             "-Xlinker", "-rpath," + cuda_lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
