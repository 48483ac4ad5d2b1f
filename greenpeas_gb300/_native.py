"""ctypes binding of the C ABI in include/gpc.h (libgpc.so, built in tree).

The library is loaded from ``greenpeas_gb300/_lib/libgpc.so``; if it is
missing this module raises instead of falling back to anything else --
run ``python -c "import __graft_entry__ as g; g.build()"`` (or
``python greenpeas_gb300/build.py``) first.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgpc.so"

GPC_OK = 0
STATUS_NAMES = {
    -1: "GPC_ERR_INVALID", -2: "GPC_ERR_PARSE", -3: "GPC_ERR_UNSUPPORTED", -4: "GPC_ERR_CUDA",
    -5: "GPC_ERR_OOM", -6: "GPC_ERR_COLLISION", -7: "GPC_ERR_TIMEOUT", -8: "GPC_ERR_CAPACITY",
}

# every symbol include/gpc.h declares
EXPORTS = [
    "gpc_get_driver", "gpc_compile", "gpc_compile_batch", "gpc_dem_arrays", "gpc_dem_info",
    "gpc_dem_text", "gpc_dem_free", "gpc_driver_destroy", "gpc_last_error", "gpc_prepare",
    "gpc_run_device", "gpc_fetch", "gpc_driver_stream", "gpc_last_timings", "gpc_set_stage_timing", "gpc_last_sizes",
    "gpc_tape_lower", "gpc_tape_get_view", "gpc_tape_free", "gpc_tape_last_error", "gpc_tape_walk_segments",
    "gpc_last_traffic",
    "gpc_last_io_bytes", "gpc_merge_mechanisms_static", "gpc_prepare_batch", "gpc_fetch_batch",
    "gpc_param_prepare", "gpc_param_forward", "gpc_param_probs", "gpc_param_backward",
    "gpc_server_create", "gpc_server_submit", "gpc_server_wait", "gpc_server_stats", "gpc_server_destroy",
    "gpc_device_dem", "gpc_autotune", "gpc_last_host_timings", "gpc_walk_form", "gpc_walk_segments",
    "gpc_walk_config", "gpc_tune_cache_clear",
    "gpc_fallback_counts", "gpc_server_fallback_counts", "gpc_alloc_counts",
    "gpc_tape_lower_cuts", "gpc_lowerer_create", "gpc_lowerer_lower", "gpc_lowerer_stats", "gpc_lowerer_free",
]


class GpcError(RuntimeError):
    """A C-ABI call returned a non-zero gpc_status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class ServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("correlation_level", ctypes.c_int32), ("slots", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("hbm_budget", ctypes.c_uint64), ("lower_threads", ctypes.c_uint32),
                ("incremental", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 2)]


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("sort_bits", ctypes.c_int32), ("global_sort", ctypes.c_int32),
                ("walk_qpt", ctypes.c_int32), ("bucket_mean", ctypes.c_int32), ("walk_words", ctypes.c_int32),
                ("key_split", ctypes.c_int32), ("walk_queue", ctypes.c_int32), ("walk_segment", ctypes.c_int32),
                ("wait_limit_us", ctypes.c_int32), ("test_hold_tile", ctypes.c_int32),
                ("test_fail_alloc", ctypes.c_int32), ("heap_results", ctypes.c_int32), ("incremental", ctypes.c_int32)]


class LowerStats(ctypes.Structure):
    _fields_ = [("incremental", ctypes.c_uint32), ("segments", ctypes.c_uint32), ("reused", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("parsed_bytes", ctypes.c_uint64)]


class TuningEntry(ctypes.Structure):
    _fields_ = [("walk_words", ctypes.c_int32), ("walk_qpt", ctypes.c_int32), ("walk_queue", ctypes.c_int32),
                ("ms", ctypes.c_float)]


class Tuning(ctypes.Structure):
    _fields_ = [("walk_words", ctypes.c_int32), ("walk_qpt", ctypes.c_int32), ("walk_queue", ctypes.c_int32),
                ("ms", ctypes.c_float), ("num_tried", ctypes.c_int32), ("tried", TuningEntry * 12)]


class TapeView(ctypes.Structure):
    _fields_ = [
        ("num_qubits", ctypes.c_uint32), ("qpad", ctypes.c_uint32), ("num_measurements", ctypes.c_uint32),
        ("num_detectors", ctypes.c_uint32), ("num_observables", ctypes.c_uint32), ("words", ctypes.c_uint32),
        ("num_epochs", ctypes.c_uint32), ("kmax", ctypes.c_uint32), ("num_points", ctypes.c_uint32),
        ("num_mechanisms", ctypes.c_uint32), ("num_records", ctypes.c_uint32), ("num_ops", ctypes.c_uint64),
        ("ops", ctypes.POINTER(ctypes.c_uint64)), ("ep_opoff", ctypes.POINTER(ctypes.c_uint32)),
        ("ep_k", ctypes.POINTER(ctypes.c_uint32)), ("ep_ptoff", ctypes.POINTER(ctypes.c_uint32)),
        ("inj_lo", ctypes.POINTER(ctypes.c_uint32)), ("inj_hi", ctypes.POINTER(ctypes.c_uint32)),
        ("rec", ctypes.POINTER(ctypes.c_uint64)), ("rec_p", ctypes.POINTER(ctypes.c_double)),
        ("rec_moff", ctypes.POINTER(ctypes.c_uint32)),
        ("rec_src", ctypes.POINTER(ctypes.c_uint32)),
        ("num_ticks", ctypes.c_uint32),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    """Loads libgpc.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build the native library first "
                          "(python greenpeas_gb300/build.py)")
    L = ctypes.CDLL(str(LIB_PATH))
    vp, sz, i32, u32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_uint32
    u32p, u64p = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64)
    L.gpc_get_driver.argtypes = [ctypes.c_char_p, sz, i32, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.gpc_compile.argtypes = [vp, vp, sz, ctypes.POINTER(vp)]  # text: bytes or an address
    L.gpc_compile_batch.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz), i32, ctypes.POINTER(vp)]
    L.gpc_dem_arrays.argtypes = [vp, ctypes.POINTER(u32p), ctypes.POINTER(u32p),
                                 ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), u32p]
    L.gpc_dem_info.argtypes = [vp, u32p, u32p, u64p]
    L.gpc_dem_text.argtypes = [vp, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(sz)]
    L.gpc_dem_free.argtypes = [vp]
    L.gpc_dem_free.restype = None
    L.gpc_driver_destroy.argtypes = [vp]
    L.gpc_driver_destroy.restype = None
    L.gpc_last_error.restype = ctypes.c_char_p
    L.gpc_prepare.argtypes = [vp, vp, sz]
    L.gpc_run_device.argtypes = [vp]
    L.gpc_fetch.argtypes = [vp, ctypes.POINTER(vp)]
    L.gpc_driver_stream.argtypes = [vp]
    L.gpc_driver_stream.restype = vp
    L.gpc_last_timings.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.gpc_set_stage_timing.argtypes = [vp, i32]
    L.gpc_last_host_timings.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.gpc_walk_form.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.gpc_walk_config.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.gpc_tune_cache_clear.argtypes = []
    L.gpc_tune_cache_clear.restype = None
    L.gpc_last_sizes.argtypes = [vp, u64p, u64p, u32p, u32p, u32p]
    L.gpc_last_traffic.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.gpc_last_io_bytes.argtypes = [vp, u64p, u64p]
    L.gpc_merge_mechanisms_static.argtypes = [vp, vp, u32, vp, u32, vp, vp, vp, u32, vp, vp]
    L.gpc_prepare_batch.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz), i32]
    L.gpc_fetch_batch.argtypes = [vp, ctypes.POINTER(vp), i32]
    L.gpc_autotune.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz), i32, i32, ctypes.POINTER(Tuning)]
    L.gpc_tape_lower.argtypes = [ctypes.c_char_p, sz, i32, ctypes.POINTER(vp)]
    L.gpc_tape_get_view.argtypes = [vp, ctypes.POINTER(TapeView)]
    L.gpc_tape_walk_segments.argtypes = [vp, u32, u32p, u32, u32p]
    L.gpc_walk_segments.argtypes = [vp, u32p, u32p, u32p]
    L.gpc_fallback_counts.argtypes = [vp, u64p]
    L.gpc_alloc_counts.argtypes = [vp, u64p, u64p]
    L.gpc_server_fallback_counts.argtypes = [vp, u64p]
    L.gpc_tape_free.argtypes = [vp]
    L.gpc_tape_free.restype = None
    L.gpc_tape_lower_cuts.argtypes = [ctypes.c_char_p, sz, i32, u64p, u32, ctypes.POINTER(vp)]
    L.gpc_lowerer_create.argtypes = [i32, i32, ctypes.POINTER(vp)]
    L.gpc_lowerer_lower.argtypes = [vp, ctypes.c_char_p, sz, ctypes.POINTER(vp)]
    L.gpc_lowerer_stats.argtypes = [vp, ctypes.POINTER(LowerStats), u64p, u32, u32p]
    L.gpc_lowerer_free.argtypes = [vp]
    L.gpc_lowerer_free.restype = None
    L.gpc_tape_last_error.restype = ctypes.c_char_p
    L.gpc_device_dem.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), u32p, u32p]
    L.gpc_server_create.argtypes = [ctypes.POINTER(ServerOptions), ctypes.POINTER(vp)]
    L.gpc_server_submit.argtypes = [vp, vp, sz, u64p]
    L.gpc_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(vp),
                                  ctypes.POINTER(ctypes.c_double)]
    L.gpc_server_stats.argtypes = [vp, u64p, u64p, u64p, u64p]
    L.gpc_server_destroy.argtypes = [vp]
    L.gpc_server_destroy.restype = None
    L.gpc_param_prepare.argtypes = [vp, ctypes.c_char_p, sz, u32p]
    L.gpc_param_forward.argtypes = [vp, vp, vp, u32p]
    L.gpc_param_probs.argtypes = [vp, vp, vp]
    L.gpc_param_backward.argtypes = [vp, vp, vp, vp]
    for f in ("gpc_param_prepare", "gpc_param_forward", "gpc_param_probs", "gpc_param_backward",
              "gpc_server_create", "gpc_server_submit", "gpc_server_wait", "gpc_server_stats", "gpc_device_dem",
              "gpc_get_driver", "gpc_compile", "gpc_compile_batch", "gpc_dem_arrays", "gpc_dem_info",
              "gpc_dem_text", "gpc_prepare", "gpc_run_device", "gpc_fetch", "gpc_last_timings", "gpc_set_stage_timing",
              "gpc_last_sizes", "gpc_tape_lower", "gpc_tape_get_view", "gpc_last_traffic", "gpc_last_io_bytes",
              "gpc_merge_mechanisms_static", "gpc_prepare_batch", "gpc_fetch_batch", "gpc_last_host_timings", "gpc_walk_form",
              "gpc_tape_walk_segments", "gpc_walk_segments", "gpc_fallback_counts", "gpc_walk_config",
              "gpc_server_fallback_counts", "gpc_alloc_counts", "gpc_tape_lower_cuts", "gpc_lowerer_create",
              "gpc_lowerer_lower", "gpc_lowerer_stats"):
        getattr(L, f).restype = i32
    _lib = L
    return L


def check(status: int, tape: bool = False) -> None:
    if status != GPC_OK:
        L = lib()
        msg = (L.gpc_tape_last_error() if tape else L.gpc_last_error()) or b""
        raise GpcError(status, msg.decode(errors="replace"))
