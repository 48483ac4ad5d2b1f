"""The segmented walk against the plain walk and the oracle (needs a GPU).

A single circuit's walk can be cut into time segments walked side by side:
first parts from zero rows, later segments from entry rows composed through
each segment's GF(2) transfer matrix (found by walking unit rows) and its walk
from zero rows.  The DEM must not depend on the cut: symptoms bit-exact and
probabilities equal (the merge sees the same mechanisms in the same order),
and equal to the oracle within 1e-12 relative.
"""

from __future__ import annotations

import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors, repetition_with_repeat
from oracle import oracle as O
from test_lowering import SMALL

pytestmark = pytest.mark.gpu
REL = 1e-12


def _circuits():
    return {
        "surface3": gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"),
        "surface5_ref": gp.SurfaceCode(5).get_memory(5, 1e-3),
        "surface9": gp.SurfaceCode(9).get_memory(9, 1e-3, noise="uniform"),
        "bb6": gp.BBCode(6).get_memory(6, 1e-3, noise="uniform"),
        "bb12": gp.BBCode(12).get_memory(12, 1e-3, noise="uniform"),
        "repetition_repeat": repetition_with_repeat(9),
    }


def _plain(text):
    return gp.get_driver(text, walk_segment=-1).compile(text)


@pytest.mark.parametrize("name", list(_circuits()))
@pytest.mark.parametrize("target", [6, 16, 40])
def test_segmented_walk_equals_the_plain_walk(name, target):
    text = _circuits()[name]
    drv = gp.get_driver(text, walk_segment=target)
    plan = drv.walk_segments()
    dem = drv.compile(text)
    if plan["segments"] == 0:
        pytest.skip("too short to cut at this target")
    ref = _plain(text)
    assert dict(dem.errors()) == dict(ref.errors())  # bit for bit, probabilities included
    if name != "bb12":  # the oracle on bb12 takes a while on the CPU; test_codes covers it
        o = O.compile_text(text, 2)
        compare_errors(dict(dem.errors()), dict(o.errors()), rel=REL)


def test_auto_policy_segments_the_headline_circuit():
    text = _circuits()["bb12"]
    drv = gp.get_driver(text)
    plan = drv.walk_segments()
    assert plan["segments"] >= 3 and plan["items_rest"] > 0
    assert dict(drv.compile(text).errors()) == dict(_plain(text).errors())


@pytest.mark.parametrize("text", SMALL)
def test_small_circuits_with_tiny_segments(text):
    """Every circuit of the gate-set tests, cut as finely as the plan allows."""
    dem = gp.get_driver(text, walk_segment=1).compile(text)
    compare_errors(dict(dem.errors()), dict(O.compile_text(text, 2).errors()), rel=REL)


def test_graph_replays_and_driver_reuse():
    """The same driver alternates between segmented and short circuits; the segmented pipeline
    runs from its CUDA graph after the second identical compile."""
    c = _circuits()
    drv = gp.get_driver(c["bb12"], walk_segment=12)
    want_bb = dict(_plain(c["bb12"]).errors())
    want_s5 = dict(_plain(c["surface5_ref"]).errors())
    for _ in range(3):
        assert dict(drv.compile(c["bb12"]).errors()) == want_bb
    assert dict(drv.compile(c["surface5_ref"]).errors()) == want_s5
    assert dict(drv.compile(c["bb12"]).errors()) == want_bb
    assert dict(drv.compile().errors()) == want_bb  # the no-argument overload


@pytest.mark.parametrize("level", [0, 1])
def test_segmented_walk_at_other_correlation_levels(level):
    text = _circuits()["surface9"]
    dem = gp.get_driver(text, gp.CorrelationLevel(level), walk_segment=8).compile(text)
    compare_errors(dict(dem.errors()), dict(O.compile_text(text, level).errors()), rel=REL)
