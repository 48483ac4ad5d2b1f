"""Seeded synthetic workloads: the batch of mixed-size surface codes and the serving mix.

Batch (seed 0, 256 circuits): rotated surface-code memory-Z with d drawn
uniformly from {3, 5, ..., 21} and rounds = d; time-varying uniform noise --
every channel instance (one per tick and gate class, i.e. per noise
instruction) draws its own p log-uniform in [1e-4, 1e-2]; every round takes
the basis-switch branch (its Z-check CNOT layers run before its X-check
layers) independently with probability 0.1.

Branches (seed 5, 256 circuits): bivariate-bicycle [[144,12,12]] memory, 12
rounds, uniform p=1e-3, each circuit a distinct set of basis-switch rounds
(every round switched with probability 0.1, at least one): the branches of
one circuit that the incremental lowering compiles against each other.
Noise variants (seed 6, 256 circuits): the same circuit with uniform p=1e-3
except one noise instruction per variant, drawn at random, at a rate
log-uniform in [1e-4, 1e-2] (a what-if sweep over one channel instance).

Serving (seed 2): 50% surface memory with d uniform in {5, ..., 25}, rounds =
d; 50% bivariate-bicycle memory drawn equally from [[72,12,6]],
[[144,12,12]], [[288,12,18]] with rounds = d; each circuit with one p
log-uniform in [1e-4, 1e-2] (uniform noise); Poisson arrival times at a given
rate.
"""

from __future__ import annotations

import numpy as np

from .codes import BBCode, SurfaceCode

_surface_cache: dict = {}
_bb_cache: dict = {}


def _surface(d):
    if d not in _surface_cache:
        _surface_cache[d] = SurfaceCode(d)
    return _surface_cache[d]


def _bb(d):
    if d not in _bb_cache:
        _bb_cache[d] = BBCode(d)
    return _bb_cache[d]


def batch_surface(n: int = 256, seed: int = 0, switch_prob: float = 0.1, p_lo: float = 1e-4,
                  p_hi: float = 1e-2, distances=tuple(range(3, 23, 2))) -> list[str]:
    """The mixed-size surface-code batch with time-varying noise and basis-switch branches."""
    rng = np.random.default_rng(seed)
    ds = rng.choice(np.array(distances), size=n)
    lo, hi = np.log10(p_lo), np.log10(p_hi)
    out = []
    for d in ds:
        d = int(d)
        switch = [r for r in range(d) if rng.random() < switch_prob]
        out.append(_surface(d).get_memory(d, 1e-3, noise="uniform",
                                          p_sampler=lambda: float(10 ** rng.uniform(lo, hi)),
                                          switch_rounds=switch))
    return out


def branches(n: int = 256, seed: int = 5, d: int = 12, rounds: int = 12, p: float = 1e-3,
             switch_prob: float = 0.1) -> list[str]:
    """Distinct branches of one circuit: bivariate-bicycle memory (d in 6, 10, 12, 18) with uniform
    noise, each branch taking the basis-switch branch in every round independently with probability
    ``switch_prob`` and in at least one round; no two branches alike (seeded)."""
    rng = np.random.default_rng(seed)
    code = _bb(d)
    seen, out = set(), []
    while len(out) < n:
        sw = tuple(r for r in range(rounds) if rng.random() < switch_prob)
        if not sw or sw in seen:
            continue
        seen.add(sw)
        out.append(code.get_memory(rounds, p, noise="uniform", switch_rounds=list(sw)))
    return out


def noise_variants(n: int = 256, seed: int = 6, d: int = 12, rounds: int = 12, p: float = 1e-3,
                   p_lo: float = 1e-4, p_hi: float = 1e-2) -> list[str]:
    """Variants of one circuit for a noise what-if sweep: bivariate-bicycle memory with uniform
    noise ``p``, except that in each variant one noise instruction (one channel instance: a tick
    and gate class), drawn at random, takes a rate log-uniform in [p_lo, p_hi] (seeded)."""
    rng = np.random.default_rng(seed)
    code = _bb(d)
    count = [0]

    def counting():
        count[0] += 1
        return p

    code.get_memory(rounds, p, noise="uniform", p_sampler=counting)
    lo, hi = np.log10(p_lo), np.log10(p_hi)
    out = []
    for _ in range(n):
        k, q = int(rng.integers(count[0])), float(10 ** rng.uniform(lo, hi))
        calls = [0]

        def sample():
            calls[0] += 1
            return q if calls[0] - 1 == k else p

        out.append(code.get_memory(rounds, p, noise="uniform", p_sampler=sample))
    return out


_SENTINEL = 0.000123456789


class ServingMix:
    """The serving mix as per-request closures over cached templates.

    A template per (code, d) is generated once with a sentinel rate; a
    request's text replaces the sentinel with its own rate, so generating
    10,000 requests costs one string substitution each."""

    def __init__(self, seed: int = 2, p_lo: float = 1e-4, p_hi: float = 1e-2):
        self.rng = np.random.default_rng(seed)
        self.lo, self.hi = np.log10(p_lo), np.log10(p_hi)
        self._tmpl: dict = {}

    def _template(self, kind, d):
        key = (kind, d)
        if key not in self._tmpl:
            from .codes import fmt_float
            code = _surface(d) if kind == "surface" else _bb(d)
            text = code.get_memory(d, _SENTINEL, noise="uniform")
            # the template's bytes split at the sentinel rate: a request is one join
            self._tmpl[key] = text.encode().split(f"({fmt_float(_SENTINEL)})".encode())
        return self._tmpl[key]

    def draw(self):
        """(kind, d, p) of the next request."""
        p = float(10 ** self.rng.uniform(self.lo, self.hi))
        if self.rng.random() < 0.5:
            return "surface", int(self.rng.choice(np.arange(5, 26, 2))), p
        return "bb", int(self.rng.choice([6, 12, 18])), p

    def text(self, kind, d, p) -> bytes:
        """The request's stim text (bytes)."""
        from .codes import fmt_float
        return f"({fmt_float(p)})".encode().join(self._template(kind, d))

    def requests(self, n: int, rate_hz: float):
        """n (arrival time, text factory) pairs with Poisson arrivals at rate_hz (rate 0: all at once)."""
        draws = [self.draw() for _ in range(n)]
        t = np.cumsum(self.rng.exponential(1.0 / rate_hz, size=n)) if rate_hz > 0 else np.zeros(n)
        for kind, d, _ in draws:
            self._template(kind, d)
        return [(float(a), (lambda k=k, d=d, p=p: self.text(k, d, p))) for a, (k, d, p) in zip(t, draws)]


def serving_mix(n: int, rate_hz: float, seed: int = 2, p_lo: float = 1e-4, p_hi: float = 1e-2):
    """n requests: (arrival time in s, circuit text) with Poisson arrivals at rate_hz."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log10(p_lo), np.log10(p_hi)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n))
    out = []
    for i in range(n):
        p = float(10 ** rng.uniform(lo, hi))
        if rng.random() < 0.5:
            d = int(rng.choice(np.arange(5, 26, 2)))
            text = _surface(d).get_memory(d, p, noise="uniform")
        else:
            d = int(rng.choice([6, 12, 18]))
            text = _bb(d).get_memory(d, p, noise="uniform")
        out.append((float(t[i]), text))
    return out
