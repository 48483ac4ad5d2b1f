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
