"""In-tree build of the CUDA library for GB300 (sm_103a)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libtnsp_gb300.so")
SOURCES = [os.path.join(CSRC, f)
           for f in ("sampler_f64.cu", "sampler_dd.cu", "sampler_f32.cu", "sampler_mixed.cu", "tnsp_capi.cu", "noalloc.cu",
                     "made.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("sampler_kernels.cuh", "cta_linalg.cuh", "ddfloat.cuh", "launch.h",
                                                  "capi_internal.h")] + [
    os.path.join(os.path.dirname(HERE), "include", "tnsp_gb300.h")
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def up_to_date():
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(p) <= t for p in DEPS if os.path.exists(p))


def build(force=False, verbose=False):
    """Compiles libtnsp_gb300.so next to this file unless it is newer than its sources.  The seven
    translation units compile in parallel, then link into one shared library."""
    if not force and up_to_date():
        return OUT
    objdir = os.path.join(os.path.dirname(HERE), "_build")
    os.makedirs(objdir, exist_ok=True)
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append(subprocess.Popen(cmd))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("nvcc failed")
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", OUT + ".tmp"] + objs
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(OUT)
