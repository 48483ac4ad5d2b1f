"""Serving form: a continuous-batching compile server over the C ABI.

    with Server(slots=4, max_batch=16, hbm_budget=120 << 30) as srv:
        t = srv.submit(circuit)           # returns at once
        dem = srv.result(t)               # blocks until compiled

The loop itself is native (``gpc_server_*`` in include/gpc.h): requests are
lowered on host threads as they arrive; GPU workers with resident drivers
form batches from whatever is lowered when they free up, admitted by
device-memory footprint.  ``replay`` drives a server
with timed arrivals and reports throughput and latency percentiles.
"""

from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import _native
from .error_analysis import _text_ref, dem_from_handle

__all__ = ["Server", "replay"]


class Server:
    def __init__(self, slots: int = 4, max_batch: int = 16, hbm_budget: int = 120 << 30, correlation_level: int = 2,
                 device: int = 0, lower_threads: int = 0, incremental: bool = False):
        o = _native.ServerOptions(device=device, correlation_level=int(correlation_level), slots=slots,
                                  max_batch=max_batch, hbm_budget=int(hbm_budget), lower_threads=lower_threads,
                                  incremental=1 if incremental else 0)
        h = ctypes.c_void_p()
        _native.check(_native.lib().gpc_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h is not None and self._h.value:
            _native.lib().gpc_server_destroy(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, circuit) -> int:
        addr, n, keep = _text_ref(circuit)
        t = ctypes.c_uint64()
        _native.check(_native.lib().gpc_server_submit(self._h, addr, n, ctypes.byref(t)))  # copies the text
        del keep
        return int(t.value)

    def result(self, ticket: int, timeout: float = 600.0, with_latency: bool = False):
        """The DEM of ``ticket`` (raises GpcError on failure or timeout); optionally (dem, latency_s)."""
        out = ctypes.c_void_p()
        lat = ctypes.c_double()
        _native.check(_native.lib().gpc_server_wait(self._h, ctypes.c_uint64(ticket), float(timeout),
                                                    ctypes.byref(out), ctypes.byref(lat)))
        dem = dem_from_handle(out)
        return (dem, lat.value) if with_latency else dem

    def stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(4)]
        _native.check(_native.lib().gpc_server_stats(self._h, *(ctypes.byref(x) for x in v)))
        return dict(zip(("completed", "batches", "budget_used", "budget_peak"), (int(x.value) for x in v)))

    def fallback_counts(self) -> dict:
        """Fallbacks taken by the workers' drivers, summed (Driver.fallback_counts)."""
        from .error_analysis import FALLBACK_NAMES
        c = (ctypes.c_uint64 * 5)()
        _native.check(_native.lib().gpc_server_fallback_counts(self._h, c))
        return dict(zip(FALLBACK_NAMES, (int(x) for x in c)))


def replay(server: Server, requests, keep=None) -> dict:
    """Submits ``requests`` -- (arrival time in s, circuit text or a callable returning it) -- at their
    arrival times (relative to the call) and collects every result.

    Returns throughput (DEMs/s over the span from the first arrival to the
    last completion), latency percentiles (submit -> done, measured natively)
    and, for tickets whose index is in ``keep``, the DEMs."""
    n = len(requests)
    tickets = [0] * n
    submitted = threading.Event()
    errors: list = []

    def submitter():
        t0 = time.perf_counter()
        try:
            for i, (at, c) in enumerate(requests):
                text = c() if callable(c) else c
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets[i] = server.submit(text)
                if i == 0:
                    submitted.set()
        except Exception as e:  # pragma: no cover - surfaced below
            errors.append(e)
            submitted.set()

    start = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    lat = np.zeros(n)
    kept = {}
    late = 0.0
    for i in range(n):
        while tickets[i] == 0:
            if errors:
                raise errors[0]
            time.sleep(1e-4)
        dem, lat[i] = server.result(tickets[i], with_latency=True)
        if keep is not None and i in keep:
            kept[i] = dem
        late = time.perf_counter()
    th.join()
    span = late - start
    return {"requests": n, "seconds": span, "dems_per_s": n / span, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "mean_ms": 1e3 * float(lat.mean()),
            "max_ms": 1e3 * float(lat.max()), "dems": kept, "stats": server.stats()}
