"""Incremental lowering on the compile path (needs a GPU).

A driver or a server created with ``incremental`` has each host thread lower
a circuit against the previous one it lowered.  Its DEMs must equal those of
a driver that lowers every circuit whole: the same symptoms and the same
probabilities, bit for bit.  Each must also equal the oracle's.
"""

from __future__ import annotations

import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from greenpeas_gb300.serving import Server
from greenpeas_gb300.workloads import branches
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _family():
    s = gp.SurfaceCode(7)
    out = [s.get_memory(7, 1e-3, noise="uniform", switch_rounds=sw) for sw in ([], [2], [2, 3], [1, 5], [6], [0, 6])]
    out += [s.get_memory(r, 1e-3, noise="uniform") for r in (8, 6, 7)]
    return out


def test_batches_match_whole_lowering():
    texts = _family() + branches(12, d=6, rounds=6)
    inc = gp.get_driver(texts[0], incremental=True)
    whole = gp.get_driver(texts[0])
    for rep in range(3):  # the later batches are lowered against the earlier ones' circuits
        order = texts[rep:] + texts[:rep]
        a = inc.compile_batch(order)
        b = whole.compile_batch(order)
        for x, y in zip(a, b):
            assert x.canonical() == y.canonical()
    for i in (0, 3, 7):
        compare_errors(dict(a[i].errors()), dict(O.compile_text(order[i], 2).errors()), rel=1e-12)


def test_single_compiles_with_the_option():
    texts = _family()[:4]
    inc = gp.get_driver(texts[0], incremental=True)
    for t in texts:
        assert inc.compile(t).canonical() == gp.get_driver(t).compile(t).canonical()


def test_server_with_incremental_lowering():
    texts = _family() * 2
    with Server(slots=2, max_batch=4, incremental=True) as srv:
        tickets = [srv.submit(t) for t in texts]
        got = [srv.result(t) for t in tickets]
    whole = gp.get_driver(texts[0])
    for t, d in zip(texts, got):
        assert d.canonical() == whole.compile(t).canonical()
