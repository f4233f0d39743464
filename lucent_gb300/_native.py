"""ctypes binding of liblucent_gpu.so (the C ABI in include/lucent.h).

The library is built in-tree by lucent_gb300/build.py. There is no fallback:
if the library is missing or fails to load, every entry point raises.
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblucent_gpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "lucent.h")

LUCENT_OK = 0
STATUS_NAMES = {1: "INVALID", 2: "CUDA", 3: "OOM", 4: "DEVICE", 5: "UNSUPPORTED"}


class LucentError(RuntimeError):
    """A C-ABI call returned a non-zero lucent_status."""

    def __init__(self, status, message):
        super().__init__("%s (%s)" % (message, STATUS_NAMES.get(status, status)))
        self.status = status


class NativeMissing(ImportError):
    pass


_lib = None
P = C.POINTER


class BvhOpts(C.Structure):
    """lucent_bvh_opts (include/lucent.h)."""
    _fields_ = [("max_leaf_size", C.c_uint32), ("bins", C.c_uint32)]

F32P, F64P, I32P, U32P, U8P = P(C.c_float), P(C.c_double), P(C.c_int32), P(C.c_uint32), P(C.c_uint8)
VP = C.c_void_p


def _sig(L, name, args, res=C.c_int32):
    fn = getattr(L, name)
    fn.argtypes = args
    fn.restype = res


def _declare(L):
    _sig(L, "lucent_last_error", [], C.c_char_p)
    _sig(L, "lucent_version", [])
    _sig(L, "lucent_bvh_build", [F32P, C.c_uint64, VP, F32P, U32P, U32P, F64P, P(VP), VP])
    _sig(L, "lucent_bvh_build_device", [VP, C.c_uint32, VP, P(VP), VP])
    _sig(L, "lucent_bvh_download", [VP, F32P, U32P])
    _sig(L, "lucent_bvh_create", [F32P, C.c_uint32, U32P, C.c_uint32, F32P, P(VP)])
    _sig(L, "lucent_bvh_destroy", [VP], None)
    _sig(L, "lucent_bvh_info", [VP, U32P, U32P])
    _sig(L, "lucent_bvh_set_mode", [VP, C.c_int32])
    _sig(L, "lucent_bvh_intersect", [VP, F32P, C.c_uint32, C.c_double, C.c_double, I32P, F32P, F32P, F32P, VP])
    _sig(L, "lucent_bvh_intersect_device", [VP, VP, C.c_uint32, C.c_double, C.c_double, VP, VP, VP, VP, VP])
    _sig(L, "lucent_bvh_check", [VP, VP])
    _sig(L, "lucent_bvh_intersect_f64", [VP, F64P, C.c_uint32, C.c_double, C.c_double, I32P, F64P, F64P, F64P, VP])
    try:
        from . import _native_render
        _native_render.declare(L, _sig)
        _native_render.declare_batch(L, _sig)
    except ImportError:
        pass


def lib():
    """Loads liblucent_gpu.so (raises NativeMissing if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeMissing("liblucent_gpu.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(status):
    if status != LUCENT_OK:
        msg = lib().lucent_last_error().decode("utf-8", "replace")
        raise LucentError(status, msg or "lucent call failed")


def declared_symbols():
    """Function names declared in include/lucent.h (and its siblings)."""
    names = set()
    inc = os.path.dirname(HEADER)
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(lucent_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def ptr(a, ct):
    """ctypes pointer to a numpy array's data."""
    return a.ctypes.data_as(P(ct))
