"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/*.c into oracle/_build/libvko.so with IEEE single-precision
semantics (-ffp-contract=off, no fast-math) so that the same sources give the
same bits on x86-64 and aarch64 hosts.  Used by tests/, by
__graft_entry__.build() and by bench.py's CPU-baseline leg only.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvko.so")
SOURCES = ["vko_geom.c", "vko_raster.c", "vko_api.c", "vko_png.c", "vko_analytic.c"]
HEADERS = ["vko.h", "vko_internal.h", "vko_pmath.h"]
CFLAGS = ["-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
          "-fvisibility=hidden", "-Wall", "-Wno-unused-function", "-pthread"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in SOURCES + HEADERS + ["build.py"]:
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


def build(force=False, verbose=False):
    """Compile the oracle library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc"] + CFLAGS + [os.path.join(HERE, s) for s in SOURCES] + ["-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
