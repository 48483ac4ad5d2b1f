"""CPU interpreter of the lowered device tape (test infrastructure).

Executes ``greenpeas_gb300.Tape`` exactly as the walk kernel does -- per
64-bit word, epoch by epoch, two-qubit Cliffords reading the partner rows
published at the epoch barrier, stopping once all rows are zero after the
word's last measurement -- then merges mechanisms the way the merge kernel
does.  It checks the host lowering against the oracle without a GPU.
"""

from __future__ import annotations

import numpy as np

OP_NOP, OP_C1, OP_C2, OP_R, OP_M, OP_INJ, OP_SNAP, OP_SNAPD, OP_XPX, OP_ZPZ, OP_XPZ = range(11)
# components of each record type as (Pauli a, Pauli b); Pauli 1 X, 2 Z, 3 Y
_T2 = [(0, 1), (0, 3), (0, 2), (1, 0), (1, 1), (1, 3), (1, 2), (3, 0), (3, 1), (3, 3), (3, 2), (2, 0), (2, 1), (2, 3), (2, 2)]
REC_COMPS = {
    1: [(1, 0), (2, 0)],
    2: [(1, 0), (3, 0), (2, 0)],
    3: [(0, 1), (0, 2), (1, 0), (1, 1), (2, 0), (2, 2)],
    4: [(0, 1), (0, 3), (0, 2), (1, 0), (1, 1), (1, 2), (3, 0), (2, 0), (2, 1), (2, 2)],
    5: _T2,
}
NONE = 0xFFFFFFFF
U64 = np.uint64


def _sel2(m, x, z):
    m = m.astype(np.uint64)
    return (x & (U64(0) - (m & U64(1)))) ^ (z & (U64(0) - ((m >> U64(1)) & U64(1))))


def _decoded(t):
    if not hasattr(t, "_dec"):
        t._dec = ((t.ops & U64(0xFF)).astype(np.uint32), ((t.ops >> U64(8)) & U64(0xFF)).astype(np.uint32),
                  (t.ops >> U64(32)).astype(np.int64))
    return t._dec


def walk(t):
    """Returns (snap [w, npoints, 2] uint64, band [w, 2])."""
    w, qpad, nE = t.words, t.qpad, t.num_epochs
    snap = np.zeros((w, max(1, t.num_points), 2), dtype=np.uint64)
    band = np.zeros((w, 2), dtype=np.int64)
    for j in range(w):
        e0 = int(t.inj_lo[j])
        if e0 == NONE or e0 >= nE:
            continue
        X = np.zeros(qpad, dtype=np.uint64)
        Z = np.zeros(qpad, dtype=np.uint64)
        e = walk_range(t, j, e0, nE, int(t.inj_hi[j]), X, Z, snap)
        band[j] = (int(t.ep_ptoff[e0]), int(t.ep_ptoff[min(e, nE)]))
    return snap, band


def walk_range(t, j, e_begin, e_end, elast, X, Z, snap=None, inject=True):
    """Walks epochs [e_begin, e_end) of word j from rows X, Z (updated in place), the way the
    walk kernel does; stops early, before an epoch e > elast, once every row is zero.  With
    ``snap`` given, snapshots are stored in it; ``inject=False`` leaves out the measurements'
    bits (the linear part of the walk).  Returns the epoch it stopped before."""
    qpad = t.qpad
    opc_all, sub_all, arg_all = _decoded(t)
    last = np.zeros(qpad, dtype=np.uint64)
    acc = np.zeros(qpad, dtype=np.uint64)
    e = e_begin
    while True:
        pX, pZ = X.copy(), Z.copy()
        anynz = bool(np.any(X | Z))
        if (not anynz and e > elast) or e >= e_end:
            break
        off = int(t.ep_opoff[e])
        for k in range(int(t.ep_k[e])):
            sl = slice(off + k * qpad, off + (k + 1) * qpad)
            opc, sub, arg = opc_all[sl], sub_all[sl], arg_all[sl]
            m = opc == OP_C1
            if m.any():
                x, z = X[m], Z[m]
                X[m] = _sel2(sub[m] & 3, x, z)
                Z[m] = _sel2(sub[m] >> 2, x, z)
            m = opc == OP_C2
            if m.any():
                x, z = X[m], Z[m]
                px, pz = pX[arg[m]], pZ[arg[m]]
                s = sub[m]
                X[m] = _sel2(s & 3, x, z) ^ _sel2((s >> 2) & 3, px, pz)
                Z[m] = _sel2((s >> 4) & 3, x, z) ^ _sel2((s >> 6) & 3, px, pz)
            m = opc == OP_XPX
            X[m] ^= pX[arg[m]]
            m = opc == OP_ZPZ
            Z[m] ^= pZ[arg[m]]
            m = opc == OP_XPZ
            X[m] ^= pZ[arg[m]]
            m = opc == OP_R
            X[m] = 0
            Z[m] = 0
            jlo = 64 * j if inject else -(1 << 40)
            for q in np.nonzero(opc == OP_INJ)[0]:
                b1, b2 = int(arg[q]), (int(t.ops[off + k * qpad + q]) >> 8) & 0xFFFFFF
                for b in (b1, b2):
                    if b != 0xFFFFFF and 0 <= b - jlo < 64:
                        acc[q] |= U64(1 << (b - jlo))
            for q in np.nonzero(opc == OP_M)[0]:
                inj = int(acc[q])
                b1 = int(arg[q])
                if 0 <= b1 - jlo < 64:
                    inj |= 1 << (b1 - jlo)
                acc[q] = 0
                inj = U64(inj)
                if sub[q] & 4:
                    X[q] = 0
                    Z[q] = 0
                if (sub[q] & 3) != 1:
                    X[q] ^= inj
                if (sub[q] & 3) != 0:
                    Z[q] ^= inj
                last[q] = inj
            if snap is None:
                continue
            m = opc == OP_SNAP
            if m.any():
                snap[j, arg[m], 0] = X[m]
                snap[j, arg[m], 1] = Z[m]
            m = opc == OP_SNAPD
            if m.any():
                snap[j, arg[m], 0] = last[m]
                snap[j, arg[m], 1] = 0
        e += 1
    return e


def _unpack(X, Z):
    """Rows (X of slots 0..qpad-1, then Z) as a (2 qpad, 64) 0/1 matrix."""
    v = np.concatenate([X, Z])
    return ((v[:, None] >> np.arange(64, dtype=np.uint64)[None, :]) & U64(1)).astype(np.int64)


def _pack(bits):
    return (bits.astype(np.uint64) << np.arange(64, dtype=np.uint64)[None, :]).sum(axis=1, dtype=np.uint64)


def transfer_matrix(t, a, b):
    """The (2 qpad x 2 qpad) 0/1 matrix A with rows at epoch b = A rows at epoch a over GF(2),
    for the walk of [a, b) without the measurements' bits: column by column, as the transfer
    walk kernel finds it, walking 64 unit rows at a time."""
    n = 2 * t.qpad
    A = np.zeros((n, n), dtype=np.int64)
    for c in range(0, n, 64):
        idx = np.arange(n)
        unit = np.where((idx >= c) & (idx < c + 64), U64(1) << (idx - c).clip(0, 63).astype(np.uint64), U64(0))
        X, Z = unit[: t.qpad].copy(), unit[t.qpad:].copy()
        walk_range(t, 0, a, b, -1, X, Z, inject=False)
        A[:, c: c + 64] = _unpack(X, Z)[:, : min(64, n - c)]
    return A


def walk_segmented(t, bounds):
    """The walk cut into time segments at ``bounds`` (0 = b_0 < ... < b_S = num_epochs), as
    the segmented walk kernels run it: a word whose walk spans segments s0 .. K walks its first
    part [e0, b_{s0+1}) from zero; each later segment s is walked from its entry rows, composed
    from the first part's exit rows through the segments between as rows_{s+1} = A_s rows_s ^
    c_s, where A_s is the segment's transfer matrix and c_s its walk from zero rows.  A word
    holding observables walks to the end; a detector word's last segment is the one holding its
    last measurement, walked on until its rows vanish.  Same (snap, band) contract as walk()."""
    w, qpad, nE = t.words, t.qpad, t.num_epochs
    bounds = [int(b) for b in bounds]
    S = len(bounds) - 1
    seg_of = lambda e: int(np.searchsorted(bounds, e, side="right")) - 1  # noqa: E731
    snap = np.zeros((w, max(1, t.num_points), 2), dtype=np.uint64)
    band = np.zeros((w, 2), dtype=np.int64)
    A = {}
    for j in range(w):
        e0 = int(t.inj_lo[j])
        if e0 == NONE or e0 >= nE:
            continue
        elast = int(t.inj_hi[j])
        s0 = seg_of(e0)
        K = S - 1 if (j + 1) * 64 > t.num_detectors else seg_of(elast)
        X = np.zeros(qpad, dtype=np.uint64)
        Z = np.zeros(qpad, dtype=np.uint64)
        end0 = nE if K == s0 else bounds[s0 + 1]
        e = walk_range(t, j, e0, end0, elast, X, Z, snap)
        band[j] = (int(t.ep_ptoff[e0]), int(t.ep_ptoff[e if e < end0 else nE]))
        rows = _unpack(X, Z)
        for s in range(s0 + 1, K + 1):
            if s > s0 + 1:  # compose through segment s - 1
                p = s - 1
                if p not in A:
                    A[p] = transfer_matrix(t, bounds[p], bounds[p + 1])
                cX = np.zeros(qpad, dtype=np.uint64)
                cZ = np.zeros(qpad, dtype=np.uint64)
                if bounds[p] <= elast:
                    walk_range(t, j, bounds[p], bounds[p + 1], elast, cX, cZ)
                rows = (A[p] @ rows + _unpack(cX, cZ)) & 1
            v = _pack(rows)
            X, Z = v[:qpad].copy(), v[qpad:].copy()
            end = nE if s == K else bounds[s + 1]
            e = walk_range(t, j, bounds[s], end, elast, X, Z, snap)
            if e < end:
                band[j, 1] = min(band[j, 1], int(t.ep_ptoff[e]))
    return snap, band


def expand(t):
    """Per-mechanism (pa, Pa, pb, Pb, p) arrays, expanding records like the key kernel."""
    pa, Pa, pb, Pb, p = [], [], [], [], []
    for r in range(t.num_records):
        d = int(t.rec[r])
        a, b = d & 0xFFFFFFF, (d >> 28) & 0xFFFFFFF
        typ, P0, P1 = (d >> 56) & 15, (d >> 60) & 3, d >> 62
        comps = [(P0, P1)] if typ == 0 else REC_COMPS[typ]
        assert t.rec_moff[r + 1] - t.rec_moff[r] == len(comps)
        for ca, cb in comps:
            pa.append(a if ca else b)
            Pa.append(ca if ca else cb)
            pb.append(b if (ca and cb) else 0)
            Pb.append(cb if ca else 0)
            p.append(float(t.rec_p[r]))
    return (np.array(pa, dtype=np.int64), np.array(Pa, dtype=np.uint32), np.array(pb, dtype=np.int64),
            np.array(Pb, dtype=np.uint32), np.array(p))


def symptoms(t, snap, band, mech):
    """[M, w] uint64 symptom words of every mechanism."""
    pa, Pa, pb, Pb, _ = mech
    S = np.zeros((len(pa), t.words), dtype=np.uint64)
    for j in range(t.words):
        lo, hi = band[j]
        ina = (pa >= lo) & (pa < hi)
        inb = (pb >= lo) & (pb < hi) & (Pb != 0)
        va = _sel2(Pa, snap[j, pa, 0], snap[j, pa, 1])
        vb = _sel2(Pb, snap[j, pb, 0], snap[j, pb, 1])
        S[:, j] = np.where(ina, va, U64(0)) ^ np.where(inb, vb, U64(0))
    return S


def compile_tape(t):
    """{targets tuple: p} -- the DEM the GPU pipeline must produce for tape ``t``."""
    snap, band = walk(t)
    mech = expand(t)
    S = symptoms(t, snap, band, mech)
    prob = mech[4]
    if S.shape[0] == 0:
        return {}
    uniq, inv = np.unique(S, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    p = np.full(uniq.shape[0], -1.0)
    for m in range(t.num_mechanisms):
        g = inv[m]
        q = float(prob[m])
        p[g] = q if p[g] < 0 else p[g] * (1 - q) + q * (1 - p[g])
    out = {}
    for g in range(uniq.shape[0]):
        ts = []
        for j in range(t.words):
            v = int(uniq[g, j])
            while v:
                b = (v & -v).bit_length() - 1
                ts.append(64 * j + b)
                v &= v - 1
        if ts:
            out[tuple(ts)] = p[g]
    return out
