"""Regenerates the golden fixtures in this directory from the GreenPeas sources.

Run from the repository root with the reference checkout available:

    python tests/golden/make_golden.py --reference /path/to/GreenPeas

It writes:

* ``dems/surface{3,5}_L{0,1,2}.dem`` -- the reference's golden DEMs
  (data/dems/*.dem, pinned by python/tests/test_error_analysis.py:27-45),
  rewritten in canonical form: targets sorted within an error, errors sorted
  by target list, probabilities printed with ``repr`` (exact round trip).
* ``circuits.json`` -- SHA-256 digests of the reference's fixture circuits
  (data/circuits/*.stim), hashed whole (BB-code circuits also without their
  OBSERVABLE_INCLUDE lines, which a generator with another logical basis
  would differ in).
* ``codes.json`` -- SHA-256 digests of the reference's check matrices for
  the BB codes without a fixture circuit (data/codes/bb/d18/H{x,z}.mtx, as
  sorted (row, column, CNOT layer) triples, 0-based), so the generator's
  [[288,12,18]] code is checked against the reference's definition.
* ``kats.json`` -- known-answer values from the reference's unit tests.
* ``circuits/iceberg_*.stim.gz`` -- the reference's concatenated
  (iceberg + surface) fixture circuits, static and adaptive outer-check
  schedules, circuit-level and phenomenological (data/circuits/iceberg_*.stim,
  produced by ConcatenatedSurfaceCode.hpp:737-868), gzip-compressed verbatim.

The tests never read the reference checkout; they read only these files.
"""

from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import re
from pathlib import Path

HERE = Path(__file__).resolve().parent


def canonical_dem(text: str) -> str:
    rows = []
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        m = re.fullmatch(r"error\(([^)]*)\)\s*(.*)", line)
        if not m:
            raise ValueError(f"unexpected DEM line: {line!r}")
        p = float(m.group(1))
        dets, obs = [], []
        for t in m.group(2).split():
            (dets if t[0] == "D" else obs).append(int(t[1:]))
        rows.append((tuple(sorted(dets)), tuple(sorted(obs)), p))
    rows.sort(key=lambda r: (r[0], r[1]))
    out = []
    for dets, obs, p in rows:
        ts = " ".join([f"D{d}" for d in dets] + [f"L{o}" for o in obs])
        out.append(f"error({p!r}) {ts}")
    return "\n".join(out) + "\n"


def triples_digest(triples) -> str:
    """SHA-256 of sorted 0-based (row, column, value) triples, one 'r c v' line each."""
    return hashlib.sha256("".join(f"{r} {c} {v}\n" for r, c, v in sorted(triples)).encode()).hexdigest()


def mtx_digest(path: Path) -> str:
    triples, header = [], False
    for line in path.read_text().splitlines():
        if line.startswith("%") or not line.strip():
            continue
        if not header:
            header = True
            continue
        r, c, v = (int(x) for x in line.split())
        triples.append((r - 1, c - 1, v))
    return triples_digest(triples)


def strip_observables(text: str) -> str:
    return "\n".join(l for l in text.splitlines() if not l.startswith("OBSERVABLE_INCLUDE")) + "\n"


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, type=Path)
    args = ap.parse_args()
    ref = args.reference
    (HERE / "dems").mkdir(exist_ok=True)
    for name in ("surface3", "surface5"):
        for lvl in ("L0", "L1", "L2"):
            src = ref / "data" / "dems" / f"{name}_{lvl}.dem"
            (HERE / "dems" / f"{name}_{lvl}.dem").write_text(canonical_dem(src.read_text()))
    circ = {}
    for path in sorted((ref / "data" / "circuits").glob("*.stim")):
        text = path.read_text()
        if path.stem.startswith("surface"):
            circ[path.stem] = {"sha256": hashlib.sha256(text.encode()).hexdigest(), "observables": True}
        elif path.stem.startswith("bb"):
            circ[path.stem] = {"sha256": hashlib.sha256(strip_observables(text).encode()).hexdigest(),
                               "observables": False,
                               "sha256_full": hashlib.sha256(text.encode()).hexdigest()}
    (HERE / "circuits.json").write_text(json.dumps(circ, indent=1, sort_keys=True) + "\n")
    codes = {}
    for d in (18,):
        for m in ("Hx", "Hz"):
            codes[f"bb{d}_{m}"] = mtx_digest(ref / "data" / "codes" / "bb" / f"d{d}" / f"{m}.mtx")
    (HERE / "codes.json").write_text(json.dumps(codes, indent=1, sort_keys=True) + "\n")
    (HERE / "circuits").mkdir(exist_ok=True)
    for path in sorted((ref / "data" / "circuits").glob("iceberg_*.stim")):
        with open(HERE / "circuits" / (path.name + ".gz"), "wb") as f:
            f.write(gzip.compress(path.read_bytes(), mtime=0))
    kats = {
        "dep1_split_p1e-3": {"value": 0.00033344451858030588, "tol": 1e-15,
                             "source": "tests/QEC/ErrorAnalysis/MixerTest.cpp:112"},
        "dep2_split_p1e-3": {"value": 6.6697798534409714e-05, "tol": 1e-15,
                             "source": "tests/QEC/ErrorAnalysis/MixerTest.cpp:144"},
        "xor_merge_0.25_0.75": {"value": 0.625, "tol": 0.0,
                                "source": "tests/QEC/ErrorAnalysis/STEPGTest.cpp:199-210"},
    }
    (HERE / "kats.json").write_text(json.dumps(kats, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
