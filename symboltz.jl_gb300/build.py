"""Builds libsymboltz_gb300.so (sm_103a) in-tree: symboltz.jl_gb300/lib/libsymboltz_gb300.so.

Translation units compile in parallel with one -gencode (sm_103a); host C++ uses portable flags
only (the same recipe runs on x86_64 and aarch64).  The CUDA runtime is linked statically.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libsymboltz_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SRCS = ["sbz_pt.cu", "sbz_pt_f32_w1.cu", "sbz_pt_f32_w24.cu", "sbz_pt_f64_w1.cu", "sbz_pt_f64_w24.cu", "sbz_los.cu", "sbz_capi.cu", "sbz_noalloc.cu", "sbz_mlp.cu", "sbz_surrogate.cu", "sbz_table.cu"]
CXX_SRCS = ["sbz_background.cpp", "sbz_setup.cpp", "sbz_trainset.cpp"]


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "symboltz_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "-Xptxas", "-v", "-c", path, "-o", obj]
    else:
        cmd = [NVCC, "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = CUDA_SRCS + CXX_SRCS
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log:
                print(o, "\n", log)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
