"""Shared pytest configuration: the ``gpu`` marker and fixture helpers."""

from __future__ import annotations

import re
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def repetition_with_repeat(rounds: int = 5, p: float = 1e-3) -> str:
    """A distance-3 repetition-code memory whose later rounds sit in a REPEAT block
    (the block's targets are stored once and occur once per repetition)."""
    layer = (f"DEPOLARIZE1({p}) 0 2 4\nCX 0 1 2 3\nDEPOLARIZE2({p}) 0 1 2 3\nTICK\n"
             f"CX 2 1 4 3\nDEPOLARIZE2({p}) 2 1 4 3\nTICK\nX_ERROR({p}) 1 3\nMR 1 3\n")
    return ("R 0 1 2 3 4\nTICK\n" + layer + "DETECTOR rec[-2]\nDETECTOR rec[-1]\n"
            f"REPEAT {rounds} {{\nTICK\n" + layer + "DETECTOR rec[-2] rec[-4]\nDETECTOR rec[-1] rec[-3]\n}\n"
            f"X_ERROR({p}) 0 2 4\nM 0 2 4\nDETECTOR rec[-3] rec[-2] rec[-5]\nDETECTOR rec[-2] rec[-1] rec[-4]\n"
            "OBSERVABLE_INCLUDE(0) rec[-1]\n")


def flatten_repeats(text: str) -> str:
    """The same circuit with its (non-nested) REPEAT blocks written out."""
    out, body, reps = [], None, 0
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("REPEAT"):
            reps, body = int(s.split()[1]), []
        elif s == "}" and body is not None:
            out += body * reps
            body = None
        elif body is not None:
            body.append(line)
        else:
            out.append(line)
    return "\n".join(out) + "\n"


def load_canonical_dem(path: Path):
    """Parses a canonical fixture DEM into {targets tuple: p} (observable k -> 'L', k)."""
    out = {}
    for line in path.read_text().splitlines():
        m = re.fullmatch(r"error\(([^)]*)\)\s*(.*)", line.strip())
        if not m:
            continue
        ts = tuple(m.group(2).split())
        out[ts] = float(m.group(1))
    return out


def to_named(targets, num_detectors):
    """Maps merged-mechanism target indices to DEM names (D<k>, L<k>), detectors first."""
    dets = sorted(t for t in targets if t < num_detectors)
    obs = sorted(t - num_detectors for t in targets if t >= num_detectors)
    return tuple([f"D{d}" for d in dets] + [f"L{o}" for o in obs])


def compare_errors(actual: dict, expected: dict, rel: float = 1e-12):
    """Asserts equal symptom sets and probabilities within ``rel`` relative error."""
    missing = set(expected) - set(actual)
    extra = set(actual) - set(expected)
    assert not missing and not extra, f"{len(missing)} missing, {len(extra)} extra symptoms"
    worst = 0.0
    for k, p in expected.items():
        q = actual[k]
        err = abs(q - p) / max(abs(p), 1e-300)
        worst = max(worst, err)
    assert worst <= rel, f"max relative probability error {worst:.3e} > {rel:.0e}"
    return worst


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libgpc.so and the oracle once per session (no-op when up to date)."""
    import __graft_entry__
    __graft_entry__.build()
    yield
