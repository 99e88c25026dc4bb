"""Build recipe for the sm_103a backend library (libsimradar_gb300.so).

The library is built in-tree (simradar_gb300/lib/) with nvcc directly: one
translation unit, one -gencode, -fmad=false so that every a*b+c in the
kernels is the same two rounded operations as in the reference arithmetic
(the elementary functions use explicit fmaf; see csrc/rsmath.h).
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libsimradar_gb300.so")
SOURCES = ["rsc.cu", "rsc_iq.cpp", "rsc_populate.cpp", "rsc_les.cpp"]
DEPS = ["rsc.cu", "rsc_iq.cpp", "rsc_populate.cpp", "rsc_populate.h", "rsc_les.cpp", "rsc_les.h", "rsc_batch.cuh", "rsc_sort.cuh", "rsc_step.cuh", "rsc_pulse.cuh", "rsc_kernels.cuh", "rsc_physics.cuh", "rsmath.h"]
GENCODE = "arch=compute_103a,code=sm_103a"


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build simradar_gb300")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(HERE, "..", "include", "rsc.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile the backend if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), "-std=c++17", "-O3", "-lineinfo", "-gencode", GENCODE, "-fmad=false",
           "-Xcompiler", "-fPIC", "-shared", "-o", tmp] + [os.path.join(CSRC, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True, cwd=CSRC)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
