"""Build the GB300 rasteriser library (libubs_gb300.so) from csrc/ with nvcc.

Translation units are compiled in parallel for sm_103a only and linked into
one shared library inside the package tree (_build/), which is what the
ctypes loader in ubs._lib opens.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB_NAME = "libubs_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-diag-suppress", "128"]
# Every translation unit is built with fast math, as the reference's own CUDA
# operators are (submodules/setup.py), except those that must round like
# PyTorch's IEEE elementwise kernels (the parameter activations of the fused
# render: scene_act.cu).
FAST_MATH = ["--use_fast_math"]
IEEE_SOURCES = ("scene_act.cu",)


def _flags(src):
    return NVCC_FLAGS + ([] if os.path.basename(src) in IEEE_SOURCES else FAST_MATH)


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 rasteriser needs the CUDA toolkit to build")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _fingerprint():
    h = hashlib.sha256()
    files = _sources() + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                if f.endswith((".cuh", ".h")))
    files.append(os.path.join(INCLUDE, "ubs.h"))
    for f in files:
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + FAST_MATH + list(IEEE_SOURCES)).encode())
    return h.hexdigest()


def build(force=False, verbose=False, jobs=None):
    """Compile (if sources changed) and return the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp.txt")
    fp = _fingerprint()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB_PATH
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmds.append([nvcc] + ARCH + _flags(src) + ["-I", INCLUDE, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        return r

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs)
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
