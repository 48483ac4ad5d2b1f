"""Failure paths, made to happen without faulting a GPU (needs a GPU).

* A bounded device wait that runs out: a test option keeps the first radix
  tile of the global sort from publishing its counts, so the decoupled
  look-back of the tiles after it waits for a status nothing will write; with
  a 2 ms limit every such wait gives up, the kernel records DEV_ERR_TIMEOUT
  and returns, and the compile fails with GPC_ERR_TIMEOUT.  The driver (same
  stream, same buffers) then compiles correctly.
* A device allocation that fails: the driver's allocation counter (the
  reference's tests count allocations of a host storage policy,
  tests/Helpers/CountingStorage.hpp:9-51) fails the k-th allocation once, as
  an out-of-memory device would; the compile returns GPC_ERR_OOM and the next
  one succeeds.
"""

from __future__ import annotations

import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from greenpeas_gb300._native import GpcError
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GPC_ERR_OOM, GPC_ERR_TIMEOUT = -5, -7


def _check(dem, text):
    compare_errors(dict(dem.errors()), dict(O.compile_text(text, 2).errors()), rel=1e-12)


def test_lookback_wait_runs_out_and_the_driver_recovers():
    text = gp.SurfaceCode(5).get_memory(5, 1e-3, noise="uniform")  # ~10k mechanisms: several sort tiles
    drv = gp.get_driver(text, global_sort=True, wait_limit_us=2000, test_hold_tile=1)
    with pytest.raises(GpcError) as e:
        drv.compile(text)
    assert e.value.status == GPC_ERR_TIMEOUT
    _check(drv.compile(text), text)  # the hold applied to one run only
    _check(drv.compile(text), text)


def test_injected_allocation_failure_leaves_the_driver_usable():
    small = gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    big = gp.SurfaceCode(7).get_memory(7, 1e-3, noise="uniform")
    probe = gp.get_driver(small)
    created = probe.alloc_counts()["allocs"]  # allocations a driver makes when it is created
    assert created >= 1
    probe.compile(small)
    probe.compile(small)
    assert probe.alloc_counts()["allocs"] == created  # a repeated compile allocates nothing
    del probe

    drv = gp.get_driver(small, test_fail_alloc=created + 1)  # the first allocation after creation fails
    _check(drv.compile(small), small)
    with pytest.raises(GpcError) as e:
        drv.compile(big)  # needs a larger arena
    assert e.value.status == GPC_ERR_OOM
    _check(drv.compile(big), big)
    _check(drv.compile(small), small)
    c = drv.alloc_counts()
    assert c["frees"] <= c["allocs"]
