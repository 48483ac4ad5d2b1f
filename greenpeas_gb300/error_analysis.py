"""``get_driver(circuit).compile_detector_error_model(circuit)`` on the GB300 path.

Python surface of GreenPeas' error-analysis bindings
(source/QEC/ErrorAnalysis/ErrorAnalysis.pybind.cu:47-79): ``CorrelationLevel``,
``Driver`` with the one- and zero-argument ``compile_detector_error_model``
overloads, and ``get_driver(circuit, correlation_level=CorrelationLevel.L2)``.
Circuits cross the boundary as stim text (a ``stim.Circuit`` is converted with
``str()``), the compile runs in libgpc.so through the C ABI, and the result is
a ``stim.DetectorErrorModel`` when stim is importable, else this package's
``DetectorErrorModel`` with the same text form.
"""

from __future__ import annotations

import ctypes
import enum

import numpy as np

from . import _native
from .dem import DetectorErrorModel


FALLBACK_NAMES = ("batch_per_circuit", "global_sort", "wider_lists", "full_key_resort", "target_regrowth")


class CorrelationLevel(enum.IntEnum):
    """Pauli components kept per depolarizing channel (Mixer.hpp:13-20)."""

    L0 = 0  # X, Z, IX, IZ, XI, XX, ZI, ZZ
    L1 = 1  # + Y, IY, XZ, YI, ZX
    L2 = 2  # all 3 / 15 components


def _text(circuit) -> bytes:
    if circuit is None:
        return None
    if isinstance(circuit, bytes):
        return circuit
    return str(circuit).encode()


_as_utf8 = None


def _text_ref(circuit):
    """(address, length, keep-alive) of the circuit text's UTF-8 bytes, without a copy: bytes as
    they are, a str through the UTF-8 buffer CPython keeps for it (for ASCII text, the str's own
    storage).  The address is valid while the keep-alive object lives; the library only reads it.
    None gives (None, 0, None)."""
    global _as_utf8
    if circuit is None:
        return None, 0, None
    if isinstance(circuit, bytes):
        return ctypes.cast(ctypes.c_char_p(circuit), ctypes.c_void_p).value, len(circuit), circuit
    text = circuit if isinstance(circuit, str) else str(circuit)
    if _as_utf8 is None:
        f = ctypes.pythonapi.PyUnicode_AsUTF8AndSize
        f.restype = ctypes.c_void_p
        f.argtypes = [ctypes.py_object, ctypes.POINTER(ctypes.c_ssize_t)]
        _as_utf8 = f
    n = ctypes.c_ssize_t()
    addr = _as_utf8(text, ctypes.byref(n))
    return addr, n.value, text


def _stim_available() -> bool:
    try:
        import stim  # noqa: F401
        return True
    except ImportError:
        return False


class _DemHandle:
    """Owns a gpc_dem; frees it when the last array viewing it is collected."""

    def __init__(self, h: ctypes.c_void_p):
        self.h = h

    def __del__(self):
        try:
            _native.lib().gpc_dem_free(self.h)
        except Exception:
            pass


def dem_from_handle(h: ctypes.c_void_p) -> DetectorErrorModel:
    """Wraps a gpc_dem in a DetectorErrorModel without copying its arrays (numpy views over the
    library's host arrays, made on first use); the handle is freed once the DEM and every array
    taken from it are gone."""
    L = _native.lib()
    try:
        nd, no = ctypes.c_uint32(), ctypes.c_uint32()
        raw = ctypes.c_uint64()
        _native.check(L.gpc_dem_info(h, ctypes.byref(nd), ctypes.byref(no), ctypes.byref(raw)))
    except Exception:
        L.gpc_dem_free(h)
        raise
    owner = _DemHandle(h)

    def views():
        offs = ctypes.POINTER(ctypes.c_uint32)()
        tg = ctypes.POINTER(ctypes.c_uint32)()
        pr = ctypes.POINTER(ctypes.c_double)()
        n = ctypes.c_uint32()
        _native.check(L.gpc_dem_arrays(owner.h, ctypes.byref(offs), ctypes.byref(tg), ctypes.byref(pr),
                                       ctypes.byref(n)))
        ne = n.value
        offsets = _owned(offs, ne + 1, np.uint32, owner)
        targets = _owned(tg, int(offsets[-1]), np.uint32, owner)
        probs = _owned(pr, ne, np.float64, owner)
        return probs, offsets, targets

    return DetectorErrorModel._deferred(views, nd.value, no.value, raw.value)


class _View:
    """Array-interface exporter of n elements at an address; it holds the gpc_dem's owner, so
    the numpy array made from it (whose base it becomes) keeps the handle alive.  Cheaper than
    a ctypes array type per array (a new type for every size)."""

    __slots__ = ("__array_interface__", "owner")

    def __init__(self, addr: int, n: int, typestr: str, owner):
        self.__array_interface__ = {"data": (addr, True), "shape": (n,), "typestr": typestr, "version": 3}
        self.owner = owner


def _owned(ptr, n: int, dtype, owner) -> np.ndarray:
    """Read-only numpy view of n elements at ptr whose base keeps ``owner`` (the gpc_dem) alive."""
    if n == 0:
        return np.zeros(0, dtype=dtype)
    addr = ctypes.cast(ptr, ctypes.c_void_p).value
    return np.asarray(_View(addr, n, np.dtype(dtype).str, owner))


class Driver:
    """Owns a libgpc driver: device buffers, a CUDA stream, the parsed circuit."""

    def __init__(self, circuit, correlation_level: CorrelationLevel = CorrelationLevel.L2, *,
                 device: int = 0, sort_bits: int = 0, global_sort: bool = False, walk_qpt: int = 0,
                 bucket_mean: int = 0, walk_words: int = 0, key_split: int = 0, walk_queue: int = 0,
                 walk_segment: int = 0, wait_limit_us: int = 0, test_hold_tile: int = 0,
                 test_fail_alloc: int = 0, heap_results: bool = False, incremental: bool = False):
        """``incremental``: in batches, lower each circuit against the previous one of its lowering
        thread (branches of one circuit re-parse only the statements that differ and reschedule only
        the time segments those change; see ``Lowerer``).  The DEMs are the same.  A single circuit
        is lowered whole on all host threads."""
        L = _native.lib()
        self._h = ctypes.c_void_p()
        self.correlation_level = CorrelationLevel(correlation_level)
        self.device = device
        opts = _native.Options()
        opts.device = device
        opts.sort_bits = sort_bits
        opts.global_sort = 1 if global_sort else 0
        opts.walk_qpt = walk_qpt
        opts.bucket_mean = bucket_mean
        opts.walk_words = walk_words
        opts.key_split = key_split
        opts.walk_queue = walk_queue
        opts.walk_segment = walk_segment
        opts.wait_limit_us = wait_limit_us
        opts.test_hold_tile = test_hold_tile
        opts.test_fail_alloc = test_fail_alloc
        opts.heap_results = 1 if heap_results else 0
        opts.incremental = 1 if incremental else 0
        text = _text(circuit)
        _native.check(L.gpc_get_driver(text, len(text), int(self.correlation_level), ctypes.byref(opts),
                                       ctypes.byref(self._h)))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _native.lib().gpc_driver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def alloc_counts(self) -> dict:
        """Device allocations and frees of this driver's buffers since its creation."""
        a, f = ctypes.c_uint64(), ctypes.c_uint64()
        _native.check(_native.lib().gpc_alloc_counts(self._h, ctypes.byref(a), ctypes.byref(f)))
        return {"allocs": a.value, "frees": f.value}

    def fallback_counts(self) -> dict:
        """How often this driver left the fast path (gpc_fallback_counts)."""
        c = (ctypes.c_uint64 * 5)()
        _native.check(_native.lib().gpc_fallback_counts(self._h, c))
        return dict(zip(FALLBACK_NAMES, (int(x) for x in c)))

    def walk_segments(self) -> dict:
        """The segmented walk of the prepared single circuit: segments (0: not segmented) and the
        CTAs of its two launches."""
        L = _native.lib()
        a, b, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _native.check(L.gpc_walk_segments(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"segments": a.value, "items_first": b.value, "items_rest": c.value}

    def compile(self, circuit=None) -> DetectorErrorModel:
        """Compiles ``circuit`` (or the driver's current circuit) to this package's DEM type."""
        L = _native.lib()
        out = ctypes.c_void_p()
        addr, n, keep = _text_ref(circuit)
        _native.check(L.gpc_compile(self._h, addr, n, ctypes.byref(out)))
        del keep
        return dem_from_handle(out)

    def compile_detector_error_model(self, circuit=None):
        """Reference-compatible entry point: a stim.DetectorErrorModel when stim is importable."""
        dem = self.compile(circuit)
        return dem.to_stim() if _stim_available() else dem

    @staticmethod
    def _batch_args(circuits):
        refs = [_text_ref(c) for c in circuits]
        n = len(refs)
        arr = (ctypes.c_void_p * n)(*[r[0] for r in refs])
        lens = (ctypes.c_size_t * n)(*[r[1] for r in refs])
        arr._keep = refs  # the texts outlive the call that reads them
        return n, arr, lens

    def compile_batch(self, circuits) -> list:
        """Compiles many circuits in one batched pipeline; one DEM per circuit, in order."""
        L = _native.lib()
        n, arr, lens = self._batch_args(circuits)
        outs = (ctypes.c_void_p * n)()
        _native.check(L.gpc_compile_batch(self._h, arr, lens, n, outs))
        return [dem_from_handle(ctypes.c_void_p(outs[i])) for i in range(n)]

    def autotune(self, circuits, reps: int = 3) -> dict:
        """Times the batched pipeline of ``circuits`` in each walk configuration (detector words per
        walk CTA x qubits per walk thread x per-class launches or one persistent launch) and keeps the
        fastest for this driver's batches; the DEMs do not depend on it.  Returns the choice and every
        configuration's time (ms, best of reps)."""
        n, arr, lens = self._batch_args(circuits)
        t = _native.Tuning()
        _native.check(_native.lib().gpc_autotune(self._h, arr, lens, n, int(reps), ctypes.byref(t)))
        self._batch_n = n
        tried = [{"walk_words": e.walk_words, "walk_qpt": e.walk_qpt, "walk_queue": e.walk_queue,
                  "ms": float(e.ms)} for e in t.tried[:t.num_tried]]
        return {"walk_words": t.walk_words, "walk_qpt": t.walk_qpt, "walk_queue": t.walk_queue,
                "ms": float(t.ms), "tried": tried}

    def prepare_batch(self, circuits) -> None:
        n, arr, lens = self._batch_args(circuits)
        self._batch_n = n
        _native.check(_native.lib().gpc_prepare_batch(self._h, arr, lens, n))

    def fetch_batch(self) -> list:
        n = self._batch_n
        outs = (ctypes.c_void_p * n)()
        _native.check(_native.lib().gpc_fetch_batch(self._h, outs, n))
        return [dem_from_handle(ctypes.c_void_p(outs[i])) for i in range(n)]

    def device_dem(self, circuit: int = 0):
        """Circuit ``circuit``'s merged mechanisms of the last run as device arrays, without a copy.

        Returns (probs, offsets, targets) as torch CUDA tensors viewing the
        driver's buffers (valid until its next prepare/run/compile; do not
        write them): probs[E] float64, offsets[E + 1] int32 positions in
        targets (the run's whole target array, so offsets need not start at
        0)."""
        import torch
        L = _native.lib()
        pp, po, pt = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        n, end = ctypes.c_uint32(), ctypes.c_uint32()
        _native.check(L.gpc_device_dem(self._h, int(circuit), ctypes.byref(pp), ctypes.byref(po), ctypes.byref(pt),
                                       ctypes.byref(n), ctypes.byref(end)))

        class _View:
            def __init__(self, ptr, count, typestr):
                self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr,
                                                 "data": (ptr or 0, False), "version": 3, "strides": None}

        dev = torch.device("cuda", self.device)
        probs = torch.as_tensor(_View(pp.value, n.value, "<f8"), device=dev)
        offsets = torch.as_tensor(_View(po.value, n.value + 1, "<i4"), device=dev)
        targets = torch.as_tensor(_View(pt.value, end.value, "<i4"), device=dev)
        return probs, offsets, targets

    # device-resident stages
    def prepare(self, circuit=None) -> None:
        addr, n, keep = _text_ref(circuit)
        _native.check(_native.lib().gpc_prepare(self._h, addr, n))
        del keep

    def run_device(self) -> None:
        _native.check(_native.lib().gpc_run_device(self._h))

    def fetch(self) -> DetectorErrorModel:
        out = ctypes.c_void_p()
        _native.check(_native.lib().gpc_fetch(self._h, ctypes.byref(out)))
        return dem_from_handle(out)

    def set_stage_timing(self, on: bool = True) -> None:
        """Records CUDA events between the pipeline's stages from the next run on (off by default:
        the event nodes of a captured graph cost a few microseconds each)."""
        _native.check(_native.lib().gpc_set_stage_timing(self._h, 1 if on else 0))

    def last_timings(self) -> dict:
        """Stage times (ms) of the last run; stage timing must have been on for it."""
        ms = (ctypes.c_float * 5)()
        _native.check(_native.lib().gpc_last_timings(self._h, ms))
        return dict(zip(("walk", "key", "sort", "merge", "total"), [float(x) for x in ms]))

    def walk_config(self) -> dict:
        """Walk configuration of this driver's batches: detector words per walk CTA, qubits per
        walk thread, persistent launch (0: defaults); set by autotune, or taken from the
        configurations autotune kept for batches of the same bitset widths."""
        w, q, z = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _native.check(_native.lib().gpc_walk_config(self._h, ctypes.byref(w), ctypes.byref(q), ctypes.byref(z)))
        return {"walk_words": w.value, "walk_qpt": q.value, "walk_queue": z.value}

    def walk_form(self) -> dict:
        """Walk launches per run of the prepared circuits and whether they form one persistent launch."""
        n, q = ctypes.c_int32(), ctypes.c_int32()
        _native.check(_native.lib().gpc_walk_form(self._h, ctypes.byref(n), ctypes.byref(q)))
        return {"launches": n.value, "persistent": bool(q.value)}

    def last_host_timings(self) -> dict:
        """Host wall-clock phases (ms) of the last prepare and fetch."""
        ms = (ctypes.c_double * 6)()
        _native.check(_native.lib().gpc_last_host_timings(self._h, ms))
        return dict(zip(("lower", "layout", "stage", "wait", "d2h", "split"), [float(x) for x in ms]))

    def last_sizes(self) -> dict:
        raw, pts = ctypes.c_uint64(), ctypes.c_uint64()
        ep, w, nq = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _native.check(_native.lib().gpc_last_sizes(self._h, ctypes.byref(raw), ctypes.byref(pts), ctypes.byref(ep),
                                                   ctypes.byref(w), ctypes.byref(nq)))
        return {"raw": raw.value, "points": pts.value, "epochs": ep.value, "words": w.value, "qubits": nq.value}

    def last_traffic(self) -> dict:
        """Algorithmic bytes per kernel of the last run (see gpc_last_traffic)."""
        b = (ctypes.c_double * 4)()
        _native.check(_native.lib().gpc_last_traffic(self._h, b))
        return dict(zip(("walk", "key", "bucket", "merge"), [float(x) for x in b]))

    def last_io_bytes(self) -> tuple:
        h2d, d2h = ctypes.c_uint64(), ctypes.c_uint64()
        _native.check(_native.lib().gpc_last_io_bytes(self._h, ctypes.byref(h2d), ctypes.byref(d2h)))
        return h2d.value, d2h.value

    @property
    def stream(self) -> int:
        return _native.lib().gpc_driver_stream(self._h) or 0


def tune_cache_clear() -> None:
    """Forgets the walk configurations autotune kept for the process (gpc_tune_cache_clear)."""
    _native.lib().gpc_tune_cache_clear()


def get_driver(circuit, correlation_level: CorrelationLevel = CorrelationLevel.L2, **kw) -> Driver:
    """greenpeas.get_driver: a driver sized for ``circuit`` (stim.Circuit or stim text)."""
    return Driver(circuit, correlation_level, **kw)


class Tape:
    """The lowered device tape of a circuit, as numpy arrays (host only, no GPU)."""

    def __init__(self, circuit, correlation_level: int = 2, segment_target: int | None = None, cuts=None):
        """``segment_target``: also set ``walk_bounds``, the epoch boundaries a single-circuit
        compile cuts the walk at for that segment cost (slots + 2 per epoch).  ``cuts``: cut the
        backward pass at these instruction indices (descending, from the instruction count to 0)."""
        L = _native.lib()
        h = ctypes.c_void_p()
        text = _text(circuit)
        if cuts is None:
            _native.check(L.gpc_tape_lower(text, len(text), int(correlation_level), ctypes.byref(h)), tape=True)
        else:
            c = (ctypes.c_uint64 * len(cuts))(*[int(x) for x in cuts])
            _native.check(L.gpc_tape_lower_cuts(text, len(text), int(correlation_level), c, len(cuts),
                                                ctypes.byref(h)), tape=True)
        self._load(h, segment_target)

    @classmethod
    def _from_handle(cls, h, segment_target=None) -> "Tape":
        t = cls.__new__(cls)
        t._load(h, segment_target)
        return t

    def _load(self, h, segment_target) -> None:
        """Copies the tape's arrays out of the gpc_tape `h` and frees it."""
        L = _native.lib()
        try:
            v = _native.TapeView()
            _native.check(L.gpc_tape_get_view(h, ctypes.byref(v)), tape=True)

            def arr(ptr, n):
                return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, dtype=ptr._type_)

            for f in ("num_qubits", "qpad", "num_measurements", "num_detectors", "num_observables", "words",
                      "num_epochs", "kmax", "num_points", "num_mechanisms", "num_records"):
                setattr(self, f, int(getattr(v, f)))
            self.ops = arr(v.ops, int(v.num_ops))
            self.ep_opoff = arr(v.ep_opoff, v.num_epochs)
            self.ep_k = arr(v.ep_k, v.num_epochs)
            self.ep_ptoff = arr(v.ep_ptoff, v.num_epochs + 1)
            self.inj_lo = arr(v.inj_lo, v.words)
            self.inj_hi = arr(v.inj_hi, v.words)
            self.rec = arr(v.rec, v.num_records)
            self.rec_p = arr(v.rec_p, v.num_records)
            self.rec_moff = arr(v.rec_moff, v.num_records + 1)
            self.rec_src = arr(v.rec_src, v.num_records)
            self.num_ticks = int(v.num_ticks)
            if segment_target is not None:
                n = ctypes.c_uint32()
                cap = int(v.num_epochs) + 2
                buf = (ctypes.c_uint32 * cap)()
                _native.check(L.gpc_tape_walk_segments(h, int(segment_target), buf, cap, ctypes.byref(n)), tape=True)
                self.walk_bounds = np.array(buf[: n.value], dtype=np.int64)
        finally:
            L.gpc_tape_free(h)


class Lowerer:
    """Lowers circuit after circuit, each against the one before it (host only, no GPU).

    With ``incremental`` the statements between the two texts' common prefix and suffix are
    parsed again, and a time segment of the backward pass over unchanged statements is taken
    over unless its measurements' detector bits or its noise sources changed other than by one
    shift (gpc_lowerer_create).  Every tape equals ``Tape(circuit, cuts=lowerer.cuts)``.
    """

    def __init__(self, correlation_level: int = 2, incremental: bool = True):
        self._h = ctypes.c_void_p()
        _native.check(_native.lib().gpc_lowerer_create(int(correlation_level), 1 if incremental else 0,
                                                       ctypes.byref(self._h)), tape=True)

    def tape(self, circuit, segment_target: int | None = None) -> Tape:
        h = ctypes.c_void_p()
        text = _text(circuit)
        _native.check(_native.lib().gpc_lowerer_lower(self._h, text, len(text), ctypes.byref(h)), tape=True)
        return Tape._from_handle(h, segment_target)

    def lower(self, circuit) -> None:
        """Lowers ``circuit`` (the next circuit is lowered against it) without copying its tape out."""
        h = ctypes.c_void_p()
        text = _text(circuit)
        L = _native.lib()
        _native.check(L.gpc_lowerer_lower(self._h, text, len(text), ctypes.byref(h)), tape=True)
        L.gpc_tape_free(h)

    @property
    def stats(self) -> dict:
        """The last lowering: incremental (lowered against the previous circuit), segments,
        reused (segments taken over), parsed_bytes."""
        st = _native.LowerStats()
        _native.check(_native.lib().gpc_lowerer_stats(self._h, ctypes.byref(st), None, 0, None), tape=True)
        return {"incremental": bool(st.incremental), "segments": int(st.segments), "reused": int(st.reused),
                "parsed_bytes": int(st.parsed_bytes)}

    @property
    def cuts(self) -> np.ndarray:
        """The last lowering's backward-pass cuts (descending instruction indices)."""
        L = _native.lib()
        n = ctypes.c_uint32()
        _native.check(L.gpc_lowerer_stats(self._h, None, None, 0, ctypes.byref(n)), tape=True)
        buf = (ctypes.c_uint64 * n.value)()
        _native.check(L.gpc_lowerer_stats(self._h, None, buf, n.value, ctypes.byref(n)), tape=True)
        return np.array(buf[: n.value], dtype=np.int64)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _native.lib().gpc_lowerer_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
