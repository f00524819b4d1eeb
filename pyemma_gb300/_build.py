"""Builds libkmgpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit under ``pyemma_gb300/csrc`` is compiled in parallel
into ``pyemma_gb300/_build/`` and linked into
``pyemma_gb300/_lib/libkmgpu.so``.  An object is rebuilt only when its source
or a header is newer.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libkmgpu.so")
INCLUDE_DIR = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["capi.cu", "assign_fp32.cu", "assign_tc.cu", "update.cu", "kmpp.cu", "serve.cu", "regspace.cu", "counts.cu", "featurize.cu", "minrmsd.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr",
              "-I" + INCLUDE_DIR]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _headers():
    out = [os.path.join(INCLUDE_DIR, "kmgpu.h")]
    for f in os.listdir(SRC_DIR):
        if f.endswith((".h", ".cuh")):
            out.append(os.path.join(SRC_DIR, f))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, extra_flags=None):
    """Compile and link; returns the path of libkmgpu.so."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    flags = NVCC_FLAGS + list(extra_flags or [])

    def compile_one(src):
        path = os.path.join(SRC_DIR, src)
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        if not _stale(obj, [path] + headers):
            return obj
        cmd = [nvcc] + ARCH + flags + ["-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if _stale(LIB_PATH, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
