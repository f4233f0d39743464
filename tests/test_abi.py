"""CPU-only checks of the C ABI library: it loads without a GPU and exports
every function include/*.h declares."""
import ctypes

import pytest

from lucent_gb300 import _native as N


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = N.declared_symbols()
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_error_text_without_gpu():
    L = N.lib()
    assert L.lucent_version() >= 100
    assert L.lucent_last_error() == b""


def test_null_arguments_rejected_before_any_device_work():
    L = N.lib()
    h = ctypes.c_void_p()
    st = L.lucent_bvh_create(None, 0, None, 0, None, ctypes.byref(h))
    assert st == 1 and b"null" in L.lucent_last_error()
    with pytest.raises(N.LucentError):
        N.check(st)


def test_renderer_calls_reject_null_handles_without_device_work():
    # Argument checks run before any CUDA call, so they hold without a GPU;
    # the pipelining switch and the asynchronous read-back included.
    from lucent_gb300 import _native_render  # noqa: F401  (declares the renderer signatures)
    L = N.lib()
    buf = (ctypes.c_float * 4)()
    for st in (L.lucent_renderer_set_pipelining(None, 1),
               L.lucent_renderer_read_color_async(None, buf, None),
               L.lucent_renderer_set_wide_bvh(None, 1),
               L.lucent_renderer_set_ray_sort(None, 1),
               L.lucent_renderer_trace(None, 1, None)):
        assert st == 1 and b"null" in L.lucent_last_error()
