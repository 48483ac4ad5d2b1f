"""The C ABI library (no GPU): it loads, and exports every function include/gpc.h declares.

The declarations are read from the header itself, so a function added to the
header but not to the library (or misspelled) fails here.  Nothing is called
that needs a GPU.
"""

from __future__ import annotations

import ctypes
import re

from conftest import ROOT
from greenpeas_gb300 import _native


def _declared() -> set:
    text = (ROOT / "include" / "gpc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(gpc_[a-z0-9_]+)\s*\(", text))


def test_header_declares_the_binding_list():
    assert _declared() == set(_native.EXPORTS)


def test_library_exports_every_declared_function():
    lib = ctypes.CDLL(str(_native.LIB_PATH))
    missing = [f for f in sorted(_declared()) if not hasattr(lib, f)]
    assert not missing, missing


def test_error_reporting_without_a_gpu():
    L = _native.lib()
    h = ctypes.c_void_p()
    # a null text is rejected before any CUDA call
    assert L.gpc_get_driver(None, 0, 2, None, ctypes.byref(h)) == -1
    assert b"null" in L.gpc_last_error()
    assert L.gpc_get_driver(b"H 0\n", 4, 7, None, ctypes.byref(h)) == -1  # bad correlation level
    # tape lowering is host-only
    t = ctypes.c_void_p()
    assert L.gpc_tape_lower(b"FOO 0\n", 6, 2, ctypes.byref(t)) == -3


def test_static_merge_rejects_a_stride_too_large_for_32_bit_counts():
    import pytest

    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("argument checks only: stand-in addresses must never reach a device")
    L = _native.lib()
    fake = ctypes.c_void_p(0x1000)  # non-null, 16-byte aligned, never dereferenced
    # 8,192 mechanisms x stride 2^20 = 2^33 targets: more than 32-bit counts hold
    st = L.gpc_merge_mechanisms_static(fake, fake, 1 << 20, fake, 1 << 13, fake, fake, fake, 0, fake, None)
    assert st == -8  # GPC_ERR_CAPACITY, before any CUDA call
