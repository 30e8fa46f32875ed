"""Build recipe for oracle/_ref (TEST INFRASTRUCTURE ONLY).

Compiles oracle/nsvg_ref.c against vkvg's vendored nanoSVG, read in place
from the reference tree (src/nsvg/nanosvg.h), into oracle/_ref/libnsvg_ref.so.
Nothing of the reference is copied; the library exists only where the
reference tree does (build() calls this when it is present), and only the
CPU tests and the fixture script load it.

    python oracle/build_ref.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: VKVG_REFERENCE, else where this build keeps it
REFERENCE = os.environ.get("VKVG_REFERENCE", "/root/reference")
NSVG_DIR = os.path.join(REFERENCE, "src", "nsvg")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libnsvg_ref.so")


def available():
    return os.path.isfile(os.path.join(NSVG_DIR, "nanosvg.h"))


def build(verbose=False):
    """path of the built library, or None when the reference tree is absent"""
    if not available():
        return None
    src = os.path.join(HERE, "nsvg_ref.c")
    if os.path.isfile(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fvisibility=hidden", "-w",
           "-I", NSVG_DIR, src, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(verbose=True)
    print(p if p else "reference tree absent: nothing built")
    sys.exit(0)
