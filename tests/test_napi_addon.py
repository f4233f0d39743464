"""The Node-API addon source (addon/lucent_napi.c) compiles against the C ABI
header and the Node-API signatures, and calls only entry points the built
library exports. Node's own headers and runtime are absent from this image,
so the addon is compiled (not linked or run) against a declarations-only
stand-in of node_api.h (tests/napi/node_api.h)."""
import os
import re
import shutil
import subprocess

import pytest

from lucent_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(ROOT, "addon", "lucent_napi.c")


def test_addon_compiles_against_the_abi():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    out = subprocess.run([cc, "-std=c11", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
                          "-I" + os.path.join(HERE, "napi"), "-I" + os.path.join(ROOT, "include"), SRC],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def test_addon_calls_only_exported_entry_points():
    used = set(re.findall(r"\b(lucent_[a-z0-9_]+)\s*\(", open(SRC).read()))
    declared = set(N.declared_symbols())
    assert used and used <= declared, used - declared
    L = N.lib()
    for name in used:
        getattr(L, name)  # raises AttributeError if the library does not export it
