"""Build the RBRP CUDA library in-tree: ``librbrp_gb300.so`` next to this file.

Each translation unit under ``csrc/`` is compiled for sm_103a only, in
parallel, then linked into one shared library that exports the C ABI of
``include/rbrp_gb300.h``.  Run ``python -m robust_blockwise_random_pivoting_gb300.build``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librbrp_gb300.so")
SOURCES = ["rbrp_capi.cu", "rbrp_f64.cu", "rbrp_f32.cu", "rbrp_noalloc.cu", "rbrp_batched.cu",
           "rbrp_adjoint.cu", "rbrp_sketch.cu", "rbrp_lupp.cu", "rbrp_compare.cu", "rbrp_matdivide.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
           "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the RBRP library")
    return exe


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cudalib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-Xlinker", f"-rpath,{cudalib}", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
