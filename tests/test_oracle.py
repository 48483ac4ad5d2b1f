"""The CPU FP64 oracle pinned against the reference's golden DEMs and known-answer tests."""

from __future__ import annotations

import json

import pytest

from conftest import GOLDEN, compare_errors, load_canonical_dem, to_named
from greenpeas_gb300.codes import SurfaceCode
from oracle import oracle as O

KATS = json.loads((GOLDEN / "kats.json").read_text())


def test_kat_dep1_split():
    k = KATS["dep1_split_p1e-3"]
    assert abs(O.lib().oracle_split_dep1(1e-3) - k["value"]) <= k["tol"]


def test_kat_dep2_split():
    k = KATS["dep2_split_p1e-3"]
    assert abs(O.lib().oracle_split_dep2(1e-3) - k["value"]) <= k["tol"]


def test_kat_xor_merge():
    assert O.lib().oracle_xor_merge(0.25, 0.75) == KATS["xor_merge_0.25_0.75"]["value"]


@pytest.mark.parametrize("d", [3, 5])
@pytest.mark.parametrize("level", [0, 1, 2])
def test_oracle_matches_reference_golden(d, level):
    """python/tests/test_error_analysis.py:27-45: surface d, rounds=d, p=1e-3, levels L0-L2."""
    text = SurfaceCode(d).get_memory(d, 1e-3)
    r = O.compile_text(text, level)
    actual = {to_named(t, r.num_detectors): p for t, p in r.errors()}
    expected = load_canonical_dem(GOLDEN / "dems" / f"surface{d}_L{level}.dem")
    compare_errors(actual, expected, rel=1e-12)


def test_oracle_threads_agree():
    text = SurfaceCode(5).get_memory(5, 1e-3)
    a = O.compile_text(text, 2, threads=1).canonical()
    b = O.compile_text(text, 2, threads=4).canonical()
    assert a == b


def test_oracle_small_cases():
    # X error before a measurement flips exactly that detector.
    r = O.compile_text("R 0\nX_ERROR(0.1) 0\nM 0\nDETECTOR rec[-1]\n")
    assert r.canonical() == [((0,), 0.1)]
    # CX propagates an X on the control to the target.
    r = O.compile_text("R 0 1\nX_ERROR(0.2) 0\nCX 0 1\nM 0 1\nDETECTOR rec[-1]\nDETECTOR rec[-2]\n")
    assert r.canonical() == [((0, 1), 0.2)]
    # Z error before a Z measurement is invisible; an empty symptom is dropped.
    r = O.compile_text("R 0\nZ_ERROR(0.3) 0\nM 0\nDETECTOR rec[-1]\n")
    assert r.canonical() == []
    # measurement flip with an observable.
    r = O.compile_text("R 0\nM(0.01) 0\nOBSERVABLE_INCLUDE(2) rec[-1]\n")
    assert r.num_observables == 3 and r.canonical() == [((2,), 0.01)]
    # equal symptoms merge with p1(1-p2)+p2(1-p1)
    r = O.compile_text("R 0\nX_ERROR(0.1) 0\nX_ERROR(0.2) 0\nM 0\nDETECTOR rec[-1]\n")
    (t, p), = r.canonical()
    assert t == (0,) and abs(p - (0.1 * 0.8 + 0.2 * 0.9)) < 1e-15


def test_oracle_rejects_bad_input():
    for bad in ["FOO 0\n", "CX 0\n", "DEPOLARIZE1(0.9) 0\n", "REPEAT 2 {\nH 0\n", "DETECTOR rec[-1]\n"]:
        with pytest.raises(O.OracleError):
            O.compile_text(bad)
