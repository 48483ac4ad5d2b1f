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
        L.oracle_num_ticks.argtypes = [ctypes.c_void_p]
        L.oracle_num_ticks.restype = ctypes.c_uint32
        L.oracle_raw.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 5
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
    num_ticks: int = 1
    raw: dict = None  # provenance arrays of the raw components (compile_text(..., provenance=True))

    def errors(self):
        """Yields (targets tuple, p) per merged mechanism; target >= num_detectors is an observable."""
        for i, p in enumerate(self.probs):
            yield tuple(self.targets[self.offsets[i]:self.offsets[i + 1]]), p

    def canonical(self):
        """Sorted list of (targets tuple, p): the order-free form used for comparisons."""
        return sorted(self.errors())


class OracleError(RuntimeError):
    pass


def compile_text(text: str, level: int = 2, threads: int = 1, provenance: bool = False) -> OracleDem:
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
        raw_info = None
        if provenance:
            import numpy as np
            n = nr.value
            raw_info = {"group": np.zeros(n, np.int32), "q": np.zeros(n), "src": np.zeros(n, np.uint32),
                        "chan": np.zeros(n, np.uint8), "arg": np.zeros(n)}
            L.oracle_raw(h, *(raw_info[k].ctypes.data for k in ("group", "q", "src", "chan", "arg")))
        return OracleDem(list(probs), list(offs), list(tg[:nt.value]), nd.value, no.value, nr.value, nq.value,
                         int(L.oracle_num_ticks(h)), raw_info)
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


def noise_gradient(dem: OracleDem, dl_dp) -> "np.ndarray":
    """CPU FP64 reference gradient dL/dnoise[tick, class] from dL/dp of each merged mechanism.

    ``dem`` comes from ``compile_text(..., provenance=True)``.  Each merged
    probability is the XOR-fold p = (1 - prod_j (1 - 2 q_j)) / 2 of its
    components, so dp/dq_m = prod_{j != m} (1 - 2 q_j) (prefix and suffix
    products, no division); dq/dp of the channel is 1 for X/Y/Z_ERROR and
    measurement flips, 1 / (3 sqrt(1 - 4p/3)) for DEPOLARIZE1 and
    (1 - 16p/15)^(1/8) / (15 (1 - 16p/15)) for DEPOLARIZE2."""
    import numpy as np
    r = dem.raw
    grad = np.zeros(dem.num_ticks * 4)
    dl = np.asarray(dl_dp, dtype=np.float64)
    group, q = r["group"], r["q"]
    keep = np.nonzero(group >= 0)[0]
    order = keep[np.argsort(group[keep], kind="stable")]
    g_sorted = group[order]
    bounds = np.flatnonzero(np.diff(g_sorted)) + 1
    dq = np.zeros(group.size)
    for seg in np.split(np.arange(order.size), bounds):
        if seg.size == 0:
            continue
        ms = order[seg]
        u = 1.0 - 2.0 * q[ms]
        pre = np.concatenate(([1.0], np.cumprod(u[:-1])))
        suf = np.concatenate((np.cumprod(u[::-1][:-1])[::-1], [1.0]))
        dq[ms] = dl[group[ms[0]]] * pre * suf
    p, chan, src = r["arg"], r["chan"], r["src"]
    slope = np.ones_like(p)
    d1 = chan == 1
    slope[d1] = 1.0 / (3.0 * np.sqrt(1.0 - 4.0 * p[d1] / 3.0))
    d2 = chan == 2
    x = 1.0 - 16.0 * p[d2] / 15.0
    slope[d2] = x ** 0.125 / (15.0 * x)
    ok = (src != 0xFFFFFFFF) & (group >= 0)
    np.add.at(grad, src[ok].astype(np.int64), dq[ok] * slope[ok])
    return grad.reshape(dem.num_ticks, 4)
