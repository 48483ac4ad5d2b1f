"""ctypes wrapper of the CPU FP64 oracle (oracle/dem_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of bench.py, never by the product package.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
SRC = HERE / "dem_oracle.cpp"


def build(force: bool = False) -> Path:
    """Compiles the oracle with g++ (host code only, no GPU)."""
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < SRC.stat().st_mtime:
        LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
        tmp = LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
        subprocess.run(
            ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-o", str(tmp), str(SRC)],
            check=True,
        )
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.oracle_compile.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_compile.restype = ctypes.c_int
        L.oracle_last_error.restype = ctypes.c_char_p
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.oracle_info.argtypes = [ctypes.c_void_p, u32p, u32p, u32p, u32p,
                                  ctypes.POINTER(ctypes.c_uint64), u32p]
        L.oracle_arrays.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), u32p, u32p]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        for f in ("oracle_split_dep1", "oracle_split_dep2"):
            getattr(L, f).argtypes = [ctypes.c_double]
            getattr(L, f).restype = ctypes.c_double
        L.oracle_xor_merge.argtypes = [ctypes.c_double, ctypes.c_double]
        L.oracle_xor_merge.restype = ctypes.c_double
        _lib = L
    return _lib


@dataclass
class OracleDem:
    """Merged mechanisms in the oracle's order plus circuit counts."""

    probs: list
    offsets: list
    targets: list
    num_detectors: int
    num_observables: int
    num_raw: int
    num_qubits: int

    def errors(self):
        """Yields (targets tuple, p) per merged mechanism; target >= num_detectors is an observable."""
        for i, p in enumerate(self.probs):
            yield tuple(self.targets[self.offsets[i]:self.offsets[i + 1]]), p

    def canonical(self):
        """Sorted list of (targets tuple, p): the order-free form used for comparisons."""
        return sorted(self.errors())


class OracleError(RuntimeError):
    pass


def compile_text(text: str, level: int = 2, threads: int = 1) -> OracleDem:
    L = lib()
    raw = text.encode()
    h = ctypes.c_void_p()
    if L.oracle_compile(raw, len(raw), level, threads, ctypes.byref(h)) != 0:
        raise OracleError(L.oracle_last_error().decode())
    try:
        ne, nt, nd, no, nq = (ctypes.c_uint32() for _ in range(5))
        nr = ctypes.c_uint64()
        L.oracle_info(h, ctypes.byref(ne), ctypes.byref(nt), ctypes.byref(nd), ctypes.byref(no),
                      ctypes.byref(nr), ctypes.byref(nq))
        probs = (ctypes.c_double * ne.value)()
        offs = (ctypes.c_uint32 * (ne.value + 1))()
        tg = (ctypes.c_uint32 * max(1, nt.value))()
        L.oracle_arrays(h, probs, offs, tg)
        return OracleDem(list(probs), list(offs), list(tg[:nt.value]), nd.value, no.value, nr.value, nq.value)
    finally:
        L.oracle_free(h)


def time_compile(text: str, level: int = 2, threads: int = 1) -> None:
    """Compiles and discards the result (used for CPU-baseline timing)."""
    L = lib()
    raw = text.encode()
    h = ctypes.c_void_p()
    if L.oracle_compile(raw, len(raw), level, threads, ctypes.byref(h)) != 0:
        raise OracleError(L.oracle_last_error().decode())
    L.oracle_free(h)
