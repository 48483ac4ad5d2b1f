"""The reference's concatenated (iceberg + surface) fixture circuits (no GPU).

Static and adaptive outer-check schedules, circuit-level and phenomenological
noise (ConcatenatedSurfaceCode.hpp:737-868 made them).  The adaptive fixtures
are noiseless in the reference data; ``noisy`` gives every zero-rate noise
instruction a rate so their schedules produce mechanisms.  The lowering, run
by the CPU tape interpreter, matches the oracle.
"""

from __future__ import annotations

import gzip
import re

import pytest

from conftest import GOLDEN, compare_errors
from greenpeas_gb300 import error_analysis as ea
from oracle import oracle as O
from tape_interp import compile_tape

NAMES = [f"iceberg_surface_{d}_{s}_{n}" for d in (4, 6) for s in ("static", "adaptive") for n in ("circl", "pheno")]


def load(name: str) -> str:
    return gzip.decompress((GOLDEN / "circuits" / f"{name}.stim.gz").read_bytes()).decode()


def noisy(text: str, p: float = 1e-3) -> str:
    return re.sub(r"^(X_ERROR|Z_ERROR|DEPOLARIZE1|DEPOLARIZE2|M)\(0\)", lambda m: f"{m.group(1)}({p})", text,
                  flags=re.M)


@pytest.mark.parametrize("name", [n for n in NAMES if "_4_" in n])
def test_lowering_matches_oracle(name):
    text = noisy(load(name))
    t = ea.Tape(text)
    assert t.num_mechanisms > 0
    got = compile_tape(t)
    ref = dict(O.compile_text(text, 2).errors())
    compare_errors(got, ref, rel=1e-12)


def test_fixtures_lower():
    for name in NAMES:
        t = ea.Tape(noisy(load(name)))
        assert t.num_detectors > 0 and t.num_mechanisms > 0
