"""In-tree build of the GPU library (libvbm3d_gb300.so) with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into
vbm3d_gb300/_build/libvbm3d_gb300.so.  Flags: --fmad=false keeps every
multiply and add separately rounded, as the reference's C++ computes them
(the kernels write FMAs explicitly where wanted); -prec-div / -prec-sqrt
stay IEEE (no fast-math).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvbm3d_gb300.so")
SOURCES = ["api.cu", "batch.cu", "batch_step1.cu", "batch_step2.cu", "bm.cu", "bm2.cu", "det_agg.cu", "filter.cu",
           "linear.cu", "misc.cu", "multiscaler.cu", "noalloc.cu", "tvl1.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "vbm3d_gb300.h"),
                                                                 os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, res.stdout, res.stderr))
        return obj, res.stderr

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-cudart", "static", "-o", tmp] + [o for o, _ in results]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
