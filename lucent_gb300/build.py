"""Builds liblucent_gpu.so in-tree (lucent_gb300/_build/) with nvcc for sm_103a.

Each .cu file compiles to an object in parallel; the objects link into one
shared library exporting the C ABI declared in include/lucent.h. The CUDA
runtime is linked statically so the library has no dependency on where a
given host keeps libcudart.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblucent_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code restates reference arithmetic too (the environment sampler's
# binary64 weights and alias table): no contraction into FMA on the host
# side either, whatever the host compiler's default on the machine.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
# Per-file extra flags. The BVH builder's binary64 arithmetic must match
# JavaScript operation by operation, so no contraction into FMA there; the
# denoiser and display pass keep the shaders' separate multiply and add so
# that variance differences (second moment minus squared mean) round the
# same way as the unfused restatement they are tested against.
EXTRA = {"bvh_build.cu": ["-fmad=false"], "denoise.cu": ["-fmad=false"], "texture.cu": ["-fmad=false"]}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def _compile(src, verbose):
    obj = os.path.join(BUILD, src[:-3] + ".o")
    path = os.path.join(CSRC, src)
    newest = max([os.path.getmtime(path), os.path.getmtime(__file__)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + EXTRA.get(src, []) + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    return obj


def build(verbose=False, jobs=None):
    """Compile every CUDA source for sm_103a and link liblucent_gpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
