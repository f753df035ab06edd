"""Build libmacgpu.so (the C-ABI force path) for sm_103a with nvcc.

Each translation unit is compiled in parallel into macsimus_gb300/_build/,
then linked into one shared library.  No torch, no cmake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmacgpu.so")
SOURCES = ["mg_tables.cpp", "mg_kernels.cu", "mg_kspace.cu", "mg_api.cu", "mg_noalloc.cu", "mg_drude.cu", "mg_nlist.cu", "mg_widom.cu", "mg_adjoint.cu", "mg_thermo.cu", "mg_sites.cu", "mg_tc.cu", "mg_kspace_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _flags():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                   "-I" + os.path.join(HERE, "..", "include"), "-I" + CSRC]


def _compile(src, verbose):
    s = os.path.join(CSRC, src)
    o = os.path.join(BUILD, src + ".o")
    deps = [s] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    deps.append(os.path.join(HERE, "..", "include", "macgpu.h"))
    if os.path.exists(o) and all(os.path.getmtime(o) >= os.path.getmtime(d) for d in deps):
        return o
    cmd = [nvcc()] + _flags() + (["-Xptxas", "-v"] if verbose else []) + ["-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return o


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
