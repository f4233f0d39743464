"""Builds the oracle (test infrastructure only) into oracle/_build/.

The oracle is the CPU checker for the CUDA product: a C++ restatement of the
reference's TypeScript/GLSL arithmetic. Flags keep binary64/binary32 results
identical to JavaScript's: no FMA contraction, no fast-math. The same recipe
runs on x86_64 and on aarch64 (no -march flags).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SOURCES = ["lucent_oracle.cpp", "oracle_render.cpp"]
LIB = os.path.join(BUILD, "liblucent_oracle.so")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + ["lucent_oracle.h", "oracle_render.h", "build_oracle.py"]
    return any(os.path.getmtime(os.path.join(HERE, s)) > t for s in deps if os.path.exists(os.path.join(HERE, s)))


def build(force=False, verbose=False):
    """Compile liblucent_oracle.so if any source is newer than it."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++"] + FLAGS + srcs + ["-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
