"""nvcc build recipe of libspringsteel_gpu.so (sm_103a only).

Each translation unit is compiled in parallel, then linked into
``springsteel.jl_gb300/lib/libspringsteel_gpu.so`` in-tree.  The library has a
plain C ABI (``include/springsteel_gpu.h``); nothing here depends on torch.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
OUT_DIR = os.path.join(PKG_DIR, "lib")
OBJ_DIR = os.path.join(PKG_DIR, "_build")
LIB = os.path.join(OUT_DIR, "libspringsteel_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["ss_setup.cpp", "ss_kernels.cu", "ss_sa_f32.cu", "ss_api.cu", "ss_batch.cu", "ss_solver.cu", "ss_mlp.cu",
           "ss_regular.cu", "ss_io.cpp"]


def _nvcc():
    n = shutil.which("nvcc")
    if n:
        return n
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _deps():
    out = [os.path.join(ROOT, "include", "springsteel_gpu.h"), __file__]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force=False, verbose=False, extra_flags=()):
    """Compile every CUDA/C++ source of the library for sm_103a and link it."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    flags = _flags() + list(extra_flags)

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
