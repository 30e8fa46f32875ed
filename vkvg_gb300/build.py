"""Build recipe for libvkvg_gb300.so (sm_103a).

Geometry units (flatten, stroke, setup) are compiled with -fmad=false and
IEEE division / square root so that their float steps match the CPU
restatement bit for bit; the raster and scan units keep FMA contraction.  Host
C++ is compiled with -ffp-contract=off for the same reason.  Units compile in
parallel; the result is linked with the static CUDA runtime.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvkvg_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_GEOM = ["flatten.cu", "stroke.cu", "setup.cu", "analytic_flat.cu"]
CU_FAST = ["raster.cu", "raster_rows.cu", "scan.cu", "analytic.cu"]
CPP = ["api.cpp", "pipeline.cpp", "extras.cpp", "png.cpp", "svg.cpp", "batch.cpp", "analytic.cpp"]
HEADERS = ["gb_types.h", "pmath.h", "launch.h", "host.h", "xdiv.cuh", "bezier.cuh", "analytic.h", "raster_common.cuh"]

NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                      "-I" + CSRC, "-I" + INC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-fno-fast-math",
             "-Wall", "-Wno-unused-function", "-I" + CSRC, "-I" + INC, "-I" + os.path.join(CUDA_HOME, "include")]


def _cmds():
    cmds = []
    for f in CU_GEOM:
        cmds.append((f, [NVCC] + NVCC_COMMON + ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                                                "-c", os.path.join(CSRC, f), "-o", os.path.join(OUT, f + ".o")]))
    for f in CU_FAST:
        cmds.append((f, [NVCC] + NVCC_COMMON + ["-c", os.path.join(CSRC, f), "-o", os.path.join(OUT, f + ".o")]))
    for f in CPP:
        cmds.append((f, ["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, f), "-o", os.path.join(OUT, f + ".o")]))
    return cmds


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in CU_GEOM + CU_FAST + CPP + HEADERS]
    deps += [os.path.join(INC, f) for f in ("vkvg.h", "vkvg_gb300.h", "vkvg-svg.h")] + [os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile the CUDA library if missing or older than its sources; returns its path."""
    if not force and not _stale():
        return LIB
    if shutil.which(NVCC) is None and not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s: cannot build libvkvg_gb300.so" % NVCC)
    os.makedirs(OUT, exist_ok=True)
    cmds = _cmds()

    def run(item):
        name, cmd = item
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiling %s failed:\n%s%s" % (name, r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        for msg in ex.map(run, cmds):
            if verbose and msg.strip():
                print(msg)
    objs = [os.path.join(OUT, f + ".o") for f, _ in [(c[0], None) for c in cmds]]
    tmp = LIB + ".tmp%d" % os.getpid()
    link = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-ldl", "-lrt"]
    if verbose:
        print(" ".join(link), flush=True)
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking libvkvg_gb300.so failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
