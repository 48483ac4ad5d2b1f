"""CUDA path against the oracle at the benchmark configurations' full sizes (needs a GPU).

The configurations the benchmarks are quoted on, each compiled on the GPU and
by the CPU FP64 oracle: symptoms bit-exact, probabilities within 1e-12
relative, same detector and observable counts.
  * [[288,12,18]] bivariate-bicycle memory, 18 rounds (the serving mix's
    largest BB circuit; 5,196 detector bits);
  * rotated surface-code memory at d = 11, 21 (the batch's largest) and 25
    (the serving mix's largest), rounds = d;
  * a 32-circuit slice of the seed-0 mixed-size batch (time-varying noise,
    basis-switch rounds) compiled as one batch, every circuit checked.
"""

from __future__ import annotations

import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from oracle import oracle as O

pytestmark = pytest.mark.gpu
REL = 1e-12


def _check(dem, text):
    ref = O.compile_text(text, 2)
    assert dem.num_detectors == ref.num_detectors and dem.num_observables == ref.num_observables
    compare_errors(dict(dem.errors()), dict(ref.errors()), rel=REL)


def test_bb18_rounds_18():
    text = gp.BBCode(18).get_memory(18, 1e-3, noise="uniform")
    drv = gp.get_driver(text)
    _check(drv.compile(text), text)


@pytest.mark.parametrize("d", [11, 21, 25])
def test_surface_rounds_d(d):
    text = gp.SurfaceCode(d).get_memory(d, 1e-3, noise="uniform")
    _check(gp.get_driver(text).compile(text), text)


def test_batch_slice_matches_oracle():
    from greenpeas_gb300.workloads import batch_surface

    texts = batch_surface()[:32]
    drv = gp.get_driver(texts[0])
    for text, dem in zip(texts, drv.compile_batch(texts)):
        _check(dem, text)
