"""Circuit generators against the reference's fixture circuits (data/circuits/*.stim).

Surface- and BB-code circuits must match byte for byte (the BB codes take the
reference's logical basis, greenpeas_gb300/bb_logicals.py); the [[288,12,18]]
code, which has no fixture circuit, must have the reference's check matrices.
"""

from __future__ import annotations

import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN
from greenpeas_gb300.codes import BBCode, SurfaceCode

CIRC = json.loads((GOLDEN / "circuits.json").read_text())


def _strip_obs(text):
    return "\n".join(l for l in text.splitlines() if not l.startswith("OBSERVABLE_INCLUDE")) + "\n"


@pytest.mark.parametrize("d", [3, 5, 7, 9])
def test_surface_matches_reference(d):
    text = SurfaceCode(d).get_memory(rounds=d, p=0.001)
    assert hashlib.sha256(text.encode()).hexdigest() == CIRC[f"surface{d}"]["sha256"]


@pytest.mark.parametrize("d", [6, 10, 12])
def test_bb_matches_reference(d):
    text = BBCode(d).get_memory(rounds=d, p=0.001)
    assert hashlib.sha256(_strip_obs(text).encode()).hexdigest() == CIRC[f"bb{d}"]["sha256"]
    assert hashlib.sha256(text.encode()).hexdigest() == CIRC[f"bb{d}"]["sha256_full"]


def test_bb18_check_matrices_match_reference():
    """[[288,12,18]] (l = m = 12): the X and Z checks, their data qubits and CNOT layers equal the
    reference's data/codes/bb/d18/H{x,z}.mtx (digests in tests/golden/codes.json)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    triples_digest = mg.triples_digest
    codes = json.loads((GOLDEN / "codes.json").read_text())
    c = BBCode(18)
    for name, sup, lay in (("Hx", c.x_support, c.x_layers), ("Hz", c.z_support, c.z_layers)):
        triples = [(r, q, l) for r, (qs, ls) in enumerate(zip(sup, lay)) for q, l in zip(qs, ls)]
        assert triples_digest(triples) == codes[f"bb18_{name}"], name


@pytest.mark.parametrize("d,k", [(6, 12), (10, 8), (12, 12), (18, 12)])
def test_bb_logicals_valid(d, k):
    c = BBCode(d)
    n = c.num_data
    hx = np.zeros((c.num_x, n), dtype=np.uint8)
    for r, s in enumerate(c.x_support):
        hx[r, s] = 1
    assert len(c.logical_z) == k
    for sup in c.logical_z:
        v = np.zeros(n, dtype=np.uint8)
        v[sup] = 1
        assert not ((hx.astype(int) @ v) % 2).any()


def test_uniform_noise_counts():
    """Uniform noise: raw mechanisms = 15*CX + 3*data*rounds + 2*(resets + measurements)."""
    from oracle import oracle as O
    d, r = 3, 3
    text = SurfaceCode(d).get_memory(rounds=r, p=1e-3, noise="uniform")
    res = O.compile_text(text, 2)
    assert res.num_raw == 15 * 4 * d * (d - 1) * r + 3 * d * d * r + 2 * ((d * d - 1) * r + d * d)
    assert res.num_qubits == 2 * d * d - 1 and res.num_detectors == r * (d * d - 1)


def test_time_varying_noise_and_switch_rounds():
    from greenpeas_gb300.workloads import batch_surface, serving_mix
    code = SurfaceCode(3)
    base = code.get_memory(3, 1e-3, noise="uniform")
    ps = iter([1e-4 * (k + 1) for k in range(1000)])
    tv = code.get_memory(3, 1e-3, noise="uniform", p_sampler=lambda: next(ps))
    assert base.count("\n") == tv.count("\n") and base != tv
    # one draw per noise instruction
    n_noise = sum(1 for ln in base.splitlines() if ln.startswith(("X_ERROR", "DEPOLARIZE")))
    assert next(ps) == pytest.approx(1e-4 * (n_noise + 1))
    sw = code.get_memory(3, 1e-3, noise="uniform", switch_rounds=[1])
    assert sorted(sw.splitlines()) == sorted(base.splitlines()) and sw != base
    with pytest.raises(ValueError):
        code.get_memory(3, 1e-3, p_sampler=lambda: 1e-3)
    a, b = batch_surface(n=4, distances=(3, 5)), batch_surface(n=4, distances=(3, 5))
    assert a == b  # seeded
    mix = serving_mix(6, rate_hz=100.0)
    assert len(mix) == 6 and all(t1 <= t2 for (t1, _), (t2, _) in zip(mix, mix[1:]))
