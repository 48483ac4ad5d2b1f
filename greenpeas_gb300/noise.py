"""Noise-rate templates: per-(tick, class) rates for a circuit's noise instructions.

A circuit's noise instructions are grouped by source: the tick of an
instruction is the number of TICKs before it (REPEAT blocks unrolled) and its
class is

  0  DEPOLARIZE2
  1  DEPOLARIZE1
  2  measurement flip: X/Y/Z_ERROR on a qubit whose last operation was not a
     reset, or the flip argument of a measurement
  3  reset flip: X/Y/Z_ERROR on a qubit whose last operation was a reset

so a rate tensor of shape [num_ticks, 4] describes time-varying noise.  The
device lowering applies the same rule to each noise record; this module
restates it on stim text, to write a circuit whose text rates are the
tensor's (``instantiate``).  PAULI_CHANNEL_1 and E keep their rates.

``symptom_weights`` gives the N(0, 1) weights keyed by a hash of each
canonical symptom that the calibration loss sum_k w_k log p_k uses.
"""

from __future__ import annotations

import math
import re

import numpy as np

NUM_CLASSES = 4
DEP2, DEP1, MEAS_FLIP, RESET_FLIP = range(NUM_CLASSES)

_RESETS = {"R", "RZ", "RX", "RY"}
_MEAS = {"M", "MZ", "MX", "MY"}
_MEAS_RESET = {"MR", "MRZ", "MRX", "MRY"}
_FLIPS = {"X_ERROR", "Y_ERROR", "Z_ERROR"}
_NOT_GATES = {"TICK", "DETECTOR", "OBSERVABLE_INCLUDE", "QUBIT_COORDS", "SHIFT_COORDS", "MPAD",
              "DEPOLARIZE1", "DEPOLARIZE2", "PAULI_CHANNEL_1", "E", "CORRELATED_ERROR"} | _FLIPS
_LINE = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)(\[[^\]]*\])?(\(([^)]*)\))?\s*(.*?)\s*$")


def _flatten(text: str) -> list:
    """(name, args text or None, target tokens) per instruction, REPEAT blocks unrolled."""
    out: list = []
    stack: list = [(1, out)]
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if line == "}":
            reps, body = stack.pop()
            stack[-1][1].extend(body * reps)
            continue
        if line.upper().startswith("REPEAT"):
            stack.append((int(line.split()[1]), []))
            continue
        m = _LINE.match(line)
        if not m:
            raise ValueError(f"cannot parse line: {raw!r}")
        name = m.group(1).upper()
        stack[-1][1].append((name, m.group(4), m.group(5).split()))
    if len(stack) != 1:
        raise ValueError("unterminated REPEAT block")
    return out


def _sources(ins: list):
    """Per instruction: per-target source (tick * 4 + class) or None; and the tick count."""
    tick = 0
    after_reset: dict = {}
    src = []
    for name, _, tg in ins:
        s = [None] * len(tg)
        if name == "TICK":
            tick += 1
        elif name == "DEPOLARIZE2":
            s = [tick * NUM_CLASSES + DEP2] * len(tg)
        elif name == "DEPOLARIZE1":
            s = [tick * NUM_CLASSES + DEP1] * len(tg)
        elif name in _FLIPS:
            s = [tick * NUM_CLASSES + (RESET_FLIP if after_reset.get(int(t), False) else MEAS_FLIP) for t in tg]
        elif name in _MEAS or name in _MEAS_RESET:
            s = [tick * NUM_CLASSES + MEAS_FLIP] * len(tg)
            for t in tg:
                after_reset[int(t.lstrip("!"))] = name in _MEAS_RESET
        elif name in _RESETS:
            for t in tg:
                after_reset[int(t)] = True
        elif name not in _NOT_GATES:
            for t in tg:
                if t.lstrip("!").isdigit():
                    after_reset[int(t.lstrip("!"))] = False
        src.append(s)
    return src, tick + 1


def num_ticks(text: str) -> int:
    """TICK instructions + 1: the first dimension of the rate tensor."""
    return _sources(_flatten(text))[1]


def _fmt(x: float) -> str:
    r = repr(float(x))
    return r[:-2] if r.endswith(".0") else r


def instantiate(text: str, noise) -> str:
    """The circuit with every sourced noise rate read from noise[tick, class].

    Instructions whose targets have different classes are split into runs of
    equal class (target order kept).  Measurements without a flip argument stay
    noiseless, as in the template."""
    rates = np.asarray(noise, dtype=np.float64).reshape(-1)
    ins = _flatten(text)
    src, nt = _sources(ins)
    if rates.size != nt * NUM_CLASSES:
        raise ValueError(f"noise has {rates.size} entries, the circuit needs {nt} x {NUM_CLASSES}")
    lines = []
    for (name, args, tg), s in zip(ins, src):
        if any(v is not None for v in s) and (args is not None or name not in _MEAS | _MEAS_RESET):
            k = 0
            while k < len(tg):
                j = k
                while j < len(tg) and s[j] == s[k]:
                    j += 1
                lines.append(f"{name}({_fmt(rates[s[k]])}) " + " ".join(tg[k:j]))
                k = j
        else:
            a = f"({args})" if args is not None else ""
            lines.append(f"{name}{a} " + " ".join(tg) if tg else f"{name}{a}")
    return "\n".join(lines) + "\n"


def _splitmix(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return x ^ (x >> np.uint64(31))


def symptom_weights(offsets, targets, seed: int = 1) -> np.ndarray:
    """w_k ~ N(0, 1) per merged mechanism, a function of its canonical (sorted) symptom only.

    The symptom's key is the wrapping sum of splitmix64(target) over its
    targets (independent of order); two further splitmix64 draws of the key
    give a Box-Muller normal."""
    off = np.asarray(offsets, dtype=np.int64)
    tg = np.asarray(targets, dtype=np.uint64)
    n = off.size - 1
    with np.errstate(over="ignore"):
        mixed = _splitmix(tg + np.uint64(seed) * np.uint64(0x632BE59BD9B4E019))
        key = np.zeros(n, dtype=np.uint64)
        lens = np.diff(off)
        nz = lens > 0
        if tg.size:
            sums = np.add.reduceat(mixed, off[:-1][nz])
            key[nz] = sums
        a = _splitmix(key)
        b = _splitmix(key ^ np.uint64(0xD1B54A32D192ED03))
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 0.5) / float(1 << 53)
    u2 = (b >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


def sample_rates(n_ticks: int, lo: float, hi: float, seed: int) -> np.ndarray:
    """[n_ticks, 4] rates drawn log-uniform in [lo, hi] (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    return 10.0 ** rng.uniform(np.log10(lo), np.log10(hi), size=(n_ticks, NUM_CLASSES))
