"""Build recipe of the FP64 CPU oracle (test infrastructure only).

Compiles ``oracle/ss_oracle.c`` into ``oracle/_build/libss_oracle.so`` with
gcc.  ``-ffp-contract=off`` keeps multiply-adds unfused so x86_64 and aarch64
hosts produce identical oracle results; no ``-march`` flag is used.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libss_oracle.so")
SOURCES = [os.path.join(HERE, "ss_oracle.c")]
HEADERS = [os.path.join(HERE, "ss_oracle.h"), os.path.join(ROOT, "include", "springsteel_gpu.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or out of date."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
           "-I", os.path.join(ROOT, "include"), *SOURCES, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
