"""Differentiation form on the GPU: noise-rate forward, FP64 adjoint, autograd.

Forward: the merged mechanisms for a [num_ticks, 4] rate tensor equal the
oracle's DEM of the instantiated circuit (symptoms exact, p within 1e-12).
Backward: the adjoint equals the CPU FP64 reference gradient (1e-10
relative) and central differences with h = 1e-7 (1e-6 relative; the loss is
summed exactly with math.fsum, so unaffected terms cancel exactly).
"""

from __future__ import annotations

import math

import numpy as np
import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors, repetition_with_repeat
from greenpeas_gb300 import noise as N
from greenpeas_gb300.autograd import NoiseRateDEM
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _setup(tmpl, level, seed=1, lo=5e-4, hi=2e-3):
    model = NoiseRateDEM(tmpl, correlation_level=level)
    rates = N.sample_rates(model.num_ticks, lo, hi, seed)
    noise = torch.tensor(rates, dtype=torch.float64, device="cuda")
    return model, rates, noise


CASES = {
    "surface3-L2": (lambda: gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"), 2),
    "surface3-L0": (lambda: gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"), 0),
    "surface5-reference-L1": (lambda: gp.SurfaceCode(5).get_memory(5, 1e-3, noise="reference"), 1),
    "bb72-L2": (lambda: gp.BBCode(6).get_memory(6, 1e-3, noise="uniform"), 2),
    "repetition-repeat-L2": (lambda: repetition_with_repeat(6), 2),
}


@pytest.mark.parametrize("case", list(CASES))
def test_forward_and_adjoint_match_the_oracle(case):
    make, level = CASES[case]
    tmpl = make()
    model, rates, noise = _setup(tmpl, level)
    noise.requires_grad_(True)
    p = model(noise)
    dem = model.last_dem()
    assert np.array_equal(p.detach().cpu().numpy(), dem.probs)
    inst = N.instantiate(tmpl, rates)
    # the rate tensor and the instantiated text compile to the same DEM, bit for bit
    assert dem == gp.get_driver(inst, correlation_level=level).compile(inst)
    ref = O.compile_text(inst, level, provenance=True)
    compare_errors(dict(dem.errors()), dict(ref.errors()), rel=1e-12)
    w_gpu = N.symptom_weights(dem.offsets, dem.targets, seed=1)
    w = torch.tensor(w_gpu, device="cuda")
    loss = (w * torch.log(p)).sum()
    loss.backward()
    g = noise.grad.cpu().numpy()
    # reference: same loss, the oracle's merged order
    w_ref = N.symptom_weights(ref.offsets, ref.targets, seed=1)
    g_ref = O.noise_gradient(ref, w_ref / np.array(ref.probs))
    scale = np.abs(g_ref).max()
    assert np.all(np.abs(g - g_ref) <= 1e-10 * np.abs(g_ref) + 1e-13 * scale)
    assert np.count_nonzero(g) == np.count_nonzero(g_ref)


def test_central_differences_on_the_bb_144_12_12_memory():
    """The [[144,12,12]] memory, 12 rounds, rates log-uniform in [5e-4, 2e-3] (seed 1):
    64 random entries of the rate tensor against central differences, h = 1e-7."""
    tmpl = gp.BBCode(12).get_memory(12, 1e-3, noise="uniform")
    model, rates, noise = _setup(tmpl, 2)
    noise.requires_grad_(True)
    p = model(noise)
    dem = model.last_dem()
    w_np = N.symptom_weights(dem.offsets, dem.targets, seed=1)
    (torch.tensor(w_np, device="cuda") * torch.log(p)).sum().backward()
    g = noise.grad.cpu().numpy()

    def loss(r):
        with torch.no_grad():
            q = model(torch.tensor(r, dtype=torch.float64, device="cuda")).cpu().numpy()
        return math.fsum(w_np * np.log(q))

    rng = np.random.default_rng(1)
    idx = rng.choice(rates.size, 64, replace=False)
    h = 1e-7
    worst = 0.0
    for k in idx:
        i, j = divmod(int(k), 4)
        rp, rm = rates.copy(), rates.copy()
        rp[i, j] += h
        rm[i, j] -= h
        fd = (loss(rp) - loss(rm)) / (2 * h)
        if g[i, j] == 0:
            assert fd == 0
            continue
        worst = max(worst, abs(fd - g[i, j]) / abs(g[i, j]))
    assert worst <= 1e-6, worst


def test_backward_needs_its_own_forward():
    tmpl = gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    model, rates, noise = _setup(tmpl, 2)
    noise.requires_grad_(True)
    p1 = model(noise)
    model(noise.detach())
    with pytest.raises(RuntimeError):
        p1.sum().backward()


def test_rates_outside_a_channel_are_rejected():
    tmpl = gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    model, rates, noise = _setup(tmpl, 2)
    bad = noise.clone()
    bad[:, 1] = 0.9  # DEPOLARIZE1 above 3/4
    with pytest.raises(gp.GpcError):
        model(bad)
