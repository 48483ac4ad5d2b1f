"""Noise-rate templates and the CPU FP64 reference gradient (no GPU).

The device lowering tags each noise record with its (tick, class) source; the
oracle classifies its raw components independently, and
greenpeas_gb300.noise restates the rule on text.  Here the three agree, and
the oracle's analytic gradient matches central differences of the oracle.
"""

from __future__ import annotations

import math
from collections import Counter

import numpy as np
import pytest

from greenpeas_gb300 import error_analysis as ea
from greenpeas_gb300 import noise as N
from greenpeas_gb300.codes import BBCode, SurfaceCode
from conftest import repetition_with_repeat
from oracle import oracle as O


def _tape_sources(text, level=2):
    t = ea.Tape(text, level)
    comps = np.diff(t.rec_moff)
    c = Counter()
    for s, k in zip(t.rec_src, comps):
        if s != 0xFFFFFFFF:
            c[int(s)] += int(k)
    return t, c


@pytest.mark.parametrize("text", [SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"),
                                  SurfaceCode(3).get_memory(2, 1e-3, noise="reference"),
                                  BBCode(6).get_memory(2, 1e-3, noise="uniform"),
                                  repetition_with_repeat(4)])
def test_sources_agree_between_lowering_oracle_and_text(text):
    t, tape = _tape_sources(text)
    assert t.num_ticks == N.num_ticks(text)
    d = O.compile_text(text, 2, provenance=True)
    assert d.num_ticks == t.num_ticks
    assert Counter(int(s) for s in d.raw["src"] if s != 0xFFFFFFFF) == tape
    classes = {s % 4 for s in tape}
    assert {0, 1, 2, 3} >= classes and len(classes) >= 3


def test_reset_and_measurement_flips_are_told_apart():
    text = "R 0 1\nTICK\nX_ERROR(0.01) 0 1\nH 1\nTICK\nX_ERROR(0.02) 0 1\nM(0.03) 0 1\nDETECTOR rec[-1]\nDETECTOR rec[-2]\n"
    _, c = _tape_sources(text)
    # tick 1: both qubits right after their reset; tick 2: qubit 0 still, qubit 1 after H; two M flips
    assert c == Counter({1 * 4 + 3: 2, 2 * 4 + 3: 1, 2 * 4 + 2: 3})
    inst = N.instantiate(text, (np.arange(12, dtype=float).reshape(3, 4) + 1) / 1000)
    assert "X_ERROR(0.008) 0 1\n" in inst and "X_ERROR(0.012) 0\nX_ERROR(0.011) 1\n" in inst
    assert "M(0.011) 0 1\n" in inst


def test_instantiate_with_the_template_rates_gives_the_same_dem():
    text = SurfaceCode(3).get_memory(3, 2e-3, noise="uniform")
    rates = np.full((N.num_ticks(text), 4), 2e-3)
    a = O.compile_text(text, 2).canonical()
    b = O.compile_text(N.instantiate(text, rates), 2).canonical()
    assert [x[0] for x in a] == [x[0] for x in b]
    assert np.allclose([x[1] for x in a], [x[1] for x in b], rtol=1e-15, atol=0)


def test_symptom_weights_are_a_function_of_the_symptom():
    off = [0, 2, 3, 3, 6]
    tg = [4, 9, 4, 1, 2, 3]
    w = N.symptom_weights(off, tg, seed=1)
    assert w.shape == (4,) and np.all(np.isfinite(w))
    assert N.symptom_weights([0, 2], [4, 9], seed=1)[0] == w[0]
    assert N.symptom_weights([0, 2], [4, 9], seed=2)[0] != w[0]
    rng = np.random.default_rng(0)
    many = N.symptom_weights(np.arange(0, 20001, 2), rng.integers(0, 1 << 20, 20000), seed=1)
    assert abs(many.mean()) < 0.05 and abs(many.std() - 1) < 0.05


def _loss(tmpl, rates, w, level):
    p = O.compile_text(N.instantiate(tmpl, rates), level).probs
    return math.fsum(wk * math.log(pk) for wk, pk in zip(w, p))


@pytest.mark.parametrize("level", [0, 1, 2])
def test_reference_gradient_matches_central_differences(level):
    tmpl = SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    rates = N.sample_rates(N.num_ticks(tmpl), 5e-4, 2e-3, seed=1)
    d = O.compile_text(N.instantiate(tmpl, rates), level, provenance=True)
    w = N.symptom_weights(d.offsets, d.targets, seed=1)
    g = O.noise_gradient(d, w / np.array(d.probs))
    live = np.argwhere(g != 0)
    rng = np.random.default_rng(level)
    h = 1e-7
    for i, j in live[rng.choice(len(live), 8, replace=False)]:
        rp, rm = rates.copy(), rates.copy()
        rp[i, j] += h
        rm[i, j] -= h
        fd = (_loss(tmpl, rp, w, level) - _loss(tmpl, rm, w, level)) / (2 * h)
        assert abs(fd - g[i, j]) <= 1e-6 * abs(g[i, j]), (i, j, fd, g[i, j])
