"""Serving form: continuous batching through the native server (needs a GPU).

Each DEM a request gets in a mix equals the DEM of the same circuit compiled
alone (bit for bit: symptoms, probabilities, order), and the oracle's.
"""

from __future__ import annotations

import numpy as np
import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from greenpeas_gb300.serving import Server, replay
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mix(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        p = float(10 ** rng.uniform(-4, -2))
        if rng.random() < 0.5:
            d = int(rng.choice([3, 5, 7]))
            out.append(gp.SurfaceCode(d).get_memory(d, p, noise="uniform"))
        else:
            out.append(gp.BBCode(6).get_memory(int(rng.choice([2, 6])), p, noise="uniform"))
    return out


def test_results_are_the_same_alone_and_in_the_mix():
    circs = _mix(48, seed=2)
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(0.002, size=len(circs)))
    with Server(slots=3, max_batch=8) as srv:
        rep = replay(srv, list(zip(arrivals, circs)), keep=set(range(len(circs))))
        st = srv.stats()
    assert rep["requests"] == len(circs) and st["completed"] == len(circs)
    for i, text in enumerate(circs):
        assert rep["dems"][i] == gp.get_driver(text).compile(text)
    for i in (0, 1, 7):
        ref = O.compile_text(circs[i], 2)
        compare_errors(dict(rep["dems"][i].errors()), dict(ref.errors()), rel=1e-12)


def test_a_burst_is_batched():
    """Requests that arrive together while the only worker is busy leave in shared batches."""
    circs = _mix(24, seed=4)
    with Server(slots=1, max_batch=8) as srv:
        rep = replay(srv, [(0.0, c) for c in circs], keep=set(range(len(circs))))
        st = srv.stats()
    assert st["completed"] == len(circs)
    assert st["batches"] < len(circs)
    for i, text in enumerate(circs):
        assert rep["dems"][i] == gp.get_driver(text).compile(text)


def test_admission_by_device_memory():
    """A budget that holds about one request at a time: every request still completes (workers wait
    and give buffers back); a request larger than the whole budget fails alone."""
    small = [gp.SurfaceCode(5).get_memory(5, 1e-3, noise="uniform") for _ in range(6)]
    big = gp.BBCode(12).get_memory(12, 1e-3, noise="uniform")
    with Server(slots=3, max_batch=1, hbm_budget=48 << 20) as srv:
        ts = [srv.submit(c) for c in small]
        tb = srv.submit(big)
        ts += [srv.submit(c) for c in small]
        for t, c in zip(ts, small + small):
            assert srv.result(t) == gp.get_driver(c).compile(c)
        with pytest.raises(gp.GpcError) as e:
            srv.result(tb)
        assert e.value.status == -8  # GPC_ERR_CAPACITY
        st = srv.stats()
        assert st["budget_peak"] <= 48 << 20


def test_a_bad_request_fails_alone():
    good = _mix(6, seed=5)
    with Server(slots=1, max_batch=8) as srv:
        ts = [srv.submit(c) for c in good[:3]]
        tb = srv.submit("H 0\nFOO 1\n")
        ts += [srv.submit(c) for c in good[3:]]
        for t, c in zip(ts, good):
            assert srv.result(t) == gp.get_driver(c).compile(c)
        with pytest.raises(gp.GpcError):
            srv.result(tb)
