"""Memory-experiment circuit generators (rotated surface code, bivariate-bicycle codes).

Mirrors GreenPeas' ``gp::Code`` generator (QEC/Codes/Code.hpp:286-407) and the
``greenpeas.codes`` Python surface (``SurfaceCode(d).get_memory(rounds, p)``,
``BBCode(d).get_memory(...)``), but builds the parity-check matrices and CNOT
schedules from the code geometry instead of loading ``.mtx`` files:

* rotated surface code: data qubit (r, c) has index r*d + c; a check is the
  plaquette whose top-left corner is (r, c), X-type when r + c is even and
  Z-type otherwise; boundary X checks sit on the left/right edges and boundary
  Z checks on the top/bottom edges.  X checks touch their corners in the order
  BR, TR, BL, TL and Z checks in the order BR, BL, TR, TL (one CNOT layer per
  position).  The Z logical is the main diagonal and the X logical the last row.
* bivariate-bicycle code with ``l, m`` and polynomials ``A = A1 + A2 + A3``,
  ``B = B1 + B2 + B3``: Hx = [A | B], Hz = [B^T | A^T]; X checks are scheduled
  A1, B1, B2, B3, A2, A3 and Z checks A2, A3, B1, B2, B3, A1.  The logical
  operators are a basis computed here by GF(2) elimination.

Two noise models are provided:

* ``noise="reference"`` -- the reference generator's model (Code.hpp:189-203,
  286-326): X_ERROR(p) after resets, DEPOLARIZE1(p/10) on idle qubits every
  tick, DEPOLARIZE2(p) after each CNOT layer and M(p) measurement flips.
* ``noise="uniform"`` -- uniform circuit-level noise: DEPOLARIZE2(p) after each
  CNOT, DEPOLARIZE1(p) on data qubits before each round, X_ERROR(p) after each
  reset and before each measurement, no idle noise.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

__all__ = ["Code", "SurfaceCode", "BBCode", "BB_PARAMS", "fmt_float"]


def fmt_float(x: float) -> str:
    """Shortest round-tripping decimal form of a float, as stim prints arguments."""
    r = repr(float(x))
    if r.endswith(".0"):
        r = r[:-2]
    return r


def _gf2_rank_basis(rows: np.ndarray) -> np.ndarray:
    """Row-reduces ``rows`` over GF(2); returns the independent reduced rows."""
    a = rows.copy() % 2
    r = 0
    ncols = a.shape[1]
    for c in range(ncols):
        piv = None
        for i in range(r, a.shape[0]):
            if a[i, c]:
                piv = i
                break
        if piv is None:
            continue
        a[[r, piv]] = a[[piv, r]]
        for i in range(a.shape[0]):
            if i != r and a[i, c]:
                a[i] ^= a[r]
        r += 1
        if r == a.shape[0]:
            break
    return a[:r]


def _gf2_nullspace(h: np.ndarray) -> np.ndarray:
    """Basis of {v : h v = 0} over GF(2)."""
    a = h.copy() % 2
    m, n = a.shape
    pivots = []
    r = 0
    for c in range(n):
        piv = None
        for i in range(r, m):
            if a[i, c]:
                piv = i
                break
        if piv is None:
            continue
        a[[r, piv]] = a[[piv, r]]
        for i in range(m):
            if i != r and a[i, c]:
                a[i] ^= a[r]
        pivots.append(c)
        r += 1
        if r == m:
            break
    free = [c for c in range(n) if c not in set(pivots)]
    basis = []
    for f in free:
        v = np.zeros(n, dtype=np.uint8)
        v[f] = 1
        for i, pc in enumerate(pivots):
            if a[i, f]:
                v[pc] = 1
        basis.append(v)
    return np.array(basis, dtype=np.uint8).reshape(len(basis), n)


def _logicals(h_commute: np.ndarray, h_stab: np.ndarray) -> list[list[int]]:
    """Logical operators commuting with ``h_commute`` and independent of ``h_stab``'s rows."""
    ker = _gf2_nullspace(h_commute)
    span = _gf2_rank_basis(h_stab)
    rank = span.shape[0]
    out = []
    for v in ker:
        trial = np.vstack([span, v[None, :]])
        red = _gf2_rank_basis(trial)
        if red.shape[0] > rank:
            span, rank = red, red.shape[0]
            out.append([int(i) for i in np.nonzero(v)[0]])
    return out


@dataclass
class Code:
    """A CSS code with CNOT schedules (qubits: data, then X checks, then Z checks)."""

    num_data: int
    x_support: list  # per X check: data qubits in schedule order
    z_support: list
    x_layers: list  # per X check: CNOT layer of each support entry
    z_layers: list
    logical_z: list = field(default_factory=list)  # per logical: data qubits (ascending)

    @property
    def num_x(self) -> int:
        return len(self.x_support)

    @property
    def num_z(self) -> int:
        return len(self.z_support)

    @property
    def num_checks(self) -> int:
        return self.num_x + self.num_z

    @property
    def num_qubits(self) -> int:
        return self.num_data + self.num_checks

    def _schedule(self, support, layers, first_id, x_basis):
        nl = 1 + max((l for ls in layers for l in ls), default=-1)
        sched = [[] for _ in range(nl)]
        for chk, (sup, ls) in enumerate(zip(support, layers)):
            for q, l in zip(sup, ls):
                sched[l].append((chk, q))
        out = []
        for layer in sched:
            pairs = []
            for chk, q in sorted(layer, key=lambda t: t[0]):
                anc = first_id + chk
                pairs += [anc, q] if x_basis else [q, anc]
            out.append(pairs)
        return out

    def get_memory(self, rounds: int, p: float, include_x_detectors: bool = True,
                   noise: str = "reference", p_sampler=None, switch_rounds=()) -> str:
        """Stim text of a memory-Z experiment with ``rounds`` syndrome rounds.

        ``p_sampler`` (uniform noise only): called once per noise instruction --
        one channel instance per tick and gate class -- and returns its
        probability, for time-varying noise.  ``switch_rounds``: rounds (0-based)
        that take the basis-switch branch, running the Z-check CNOT layers
        before the X-check layers.
        """
        if noise not in ("reference", "uniform"):
            raise ValueError("noise must be 'reference' or 'uniform'")
        if p_sampler is not None and noise != "uniform":
            raise ValueError("p_sampler needs noise='uniform'")
        switch = set(switch_rounds)
        if rounds < 1:
            raise ValueError("rounds must be >= 1")
        n, nx, nz, nc = self.num_data, self.num_x, self.num_z, self.num_checks
        data = list(range(n))
        checks = list(range(n, n + nc))
        xchecks = list(range(n, n + nx))
        allq = list(range(n + nc))
        xs = self._schedule(self.x_support, self.x_layers, n, True)
        zs = self._schedule(self.z_support, self.z_layers, n + nx, False)
        ps, pi = fmt_float(p), fmt_float(p / 10)
        ref = noise == "reference"
        L = []

        def ins(name, targets, arg=None):
            a = f"({arg})" if arg is not None else ""
            L.append(f"{name}{a} " + " ".join(map(str, targets)) if targets else f"{name}{a}")

        def pu():  # probability of the next uniform-noise instruction
            return fmt_float(p_sampler()) if p_sampler is not None else ps

        def round_(r):
            ins("R", checks)
            ins("TICK", [])
            ins("X_ERROR", checks, ps if ref else pu())
            ins("DEPOLARIZE1", data, pi if ref else pu())
            if nx:
                ins("H", xchecks)
                ins("TICK", [])
                if ref:
                    ins("DEPOLARIZE1", allq, pi)
            for layer in (zs + xs if r in switch else xs + zs):
                ins("CX", layer)
                ins("TICK", [])
                ins("DEPOLARIZE2", layer, ps if ref else pu())
                if ref:
                    active = set(layer)
                    idle = [q for q in allq if q not in active]
                    if idle:
                        ins("DEPOLARIZE1", idle, pi)
            if nx:
                ins("H", xchecks)
                ins("TICK", [])
                if ref:
                    ins("DEPOLARIZE1", allq, pi)
            if ref:
                ins("M", checks, ps)
            else:
                ins("X_ERROR", checks, pu())
                ins("M", checks)

        # head
        ins("R", data)
        ins("TICK", [])
        ins("X_ERROR", data, ps if ref else pu())
        if ref:
            ins("DEPOLARIZE1", checks, pi)
        # rounds
        round_(0)
        for i in range(nz):
            L.append(f"DETECTOR rec[-{nz - i}]")
        for r in range(1, rounds):
            round_(r)
            lo = 0 if include_x_detectors else nx
            for i in range(lo, nc):
                L.append(f"DETECTOR rec[-{nc - i}] rec[-{2 * nc - i}]")
        # tail
        if ref:
            ins("M", data, ps)
        else:
            ins("X_ERROR", data, pu())
            ins("M", data)
        for chk, sup in enumerate(self.z_support):
            if not sup:
                continue
            recs = [f"rec[-{n - q}]" for q in sup] + [f"rec[-{n + nz - chk}]"]
            L.append("DETECTOR " + " ".join(recs))
        for k, sup in enumerate(self.logical_z):
            L.append(f"OBSERVABLE_INCLUDE({k}) " + " ".join(f"rec[-{n - q}]" for q in sup))
        return "\n".join(L) + "\n"


class SurfaceCode(Code):
    """Rotated planar surface code of distance ``d``."""

    def __init__(self, d: int):
        if d < 2:
            raise ValueError("distance must be >= 2")
        self.d = d

        def inside(r, c):
            return 0 <= r < d and 0 <= c < d

        xs, zs = [], []
        for r in range(-1, d):
            for c in range(-1, d):
                bulk = 0 <= r <= d - 2 and 0 <= c <= d - 2
                is_x = (r + c) % 2 == 0
                if is_x and (bulk or (c in (-1, d - 1) and 0 <= r <= d - 2)):
                    xs.append((r, c))
                elif not is_x and (bulk or (r in (-1, d - 1) and 0 <= c <= d - 2)):
                    zs.append((r, c))

        def sched(corner, order):
            r, c = corner
            pos = {"TL": (r, c), "TR": (r, c + 1), "BL": (r + 1, c), "BR": (r + 1, c + 1)}
            sup, lay = [], []
            for layer, name in enumerate(order):
                rr, cc = pos[name]
                if inside(rr, cc):
                    sup.append(rr * d + cc)
                    lay.append(layer)
            return sup, lay

        xo, zo = ("BR", "TR", "BL", "TL"), ("BR", "BL", "TR", "TL")
        xsl = [sched(k, xo) for k in xs]
        zsl = [sched(k, zo) for k in zs]
        super().__init__(
            num_data=d * d,
            x_support=[s for s, _ in xsl], x_layers=[l for _, l in xsl],
            z_support=[s for s, _ in zsl], z_layers=[l for _, l in zsl],
            logical_z=[[i * (d + 1) for i in range(d)]],
        )


# (l, m, A terms, B terms); a term (a, b) is x^a y^b, listed in schedule order.
BB_PARAMS = {
    6: (6, 6, [(3, 0), (0, 1), (0, 2)], [(1, 0), (2, 0), (0, 3)]),
    10: (15, 3, [(9, 0), (0, 1), (0, 2)], [(0, 0), (2, 0), (7, 0)]),
    12: (12, 6, [(3, 0), (0, 1), (0, 2)], [(1, 0), (2, 0), (0, 3)]),
    18: (12, 12, [(0, 2), (3, 0), (0, 7)], [(1, 0), (2, 0), (0, 3)]),
}


class BBCode(Code):
    """Bivariate-bicycle code [[2lm, k, d]] for d in ``BB_PARAMS`` (6, 10, 12, 18)."""

    def __init__(self, d: int, params=None):
        if params is None:
            if d not in BB_PARAMS:
                raise ValueError(f"no bivariate-bicycle parameters for distance {d}")
            params = BB_PARAMS[d]
        l, m, A, B = params
        self.d, self.l, self.m = d, l, m
        nb = l * m

        def idx(i, j):
            return (i % l) * m + (j % m)

        xsup, xlay, zsup, zlay = [], [], [], []
        x_order = [("A", 0), ("B", 0), ("B", 1), ("B", 2), ("A", 1), ("A", 2)]
        z_order = [("A", 1), ("A", 2), ("B", 0), ("B", 1), ("B", 2), ("A", 0)]
        for i in range(l):
            for j in range(m):
                s, ly = [], []
                for layer, (poly, t) in enumerate(x_order):
                    a, b = (A if poly == "A" else B)[t]
                    base = 0 if poly == "A" else nb
                    s.append(base + idx(i + a, j + b))
                    ly.append(layer)
                xsup.append(s)
                xlay.append(ly)
                s, ly = [], []
                for layer, (poly, t) in enumerate(z_order):
                    a, b = (A if poly == "A" else B)[t]
                    base = nb if poly == "A" else 0  # Hz = [B^T | A^T]
                    s.append(base + idx(i - a, j - b))
                    ly.append(layer)
                zsup.append(s)
                zlay.append(ly)
        n = 2 * nb
        hx = np.zeros((nb, n), dtype=np.uint8)
        hz = np.zeros((nb, n), dtype=np.uint8)
        for r, s in enumerate(xsup):
            hx[r, s] = 1
        for r, s in enumerate(zsup):
            hz[r, s] = 1
        # the reference's logical basis for its own codes (bb_logicals); a basis
        # computed from the check matrices for other parameters
        from .bb_logicals import BB_LOGICAL_Z
        lz = BB_LOGICAL_Z[d] if params == BB_PARAMS.get(d) and d in BB_LOGICAL_Z else _logicals(hx, hz)
        super().__init__(num_data=n, x_support=xsup, x_layers=xlay, z_support=zsup, z_layers=zlay,
                         logical_z=lz)
