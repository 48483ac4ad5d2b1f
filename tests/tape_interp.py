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


def walk(t):
    """Returns (snap [w, npoints, 2] uint64, band [w, 2])."""
    w, qpad, nE = t.words, t.qpad, t.num_epochs
    snap = np.zeros((w, max(1, t.num_points), 2), dtype=np.uint64)
    band = np.zeros((w, 2), dtype=np.int64)
    opc_all = (t.ops & U64(0xFF)).astype(np.uint32)
    sub_all = ((t.ops >> U64(8)) & U64(0xFF)).astype(np.uint32)
    arg_all = (t.ops >> U64(32)).astype(np.int64)
    for j in range(w):
        e0 = int(t.inj_lo[j])
        if e0 == NONE or e0 >= nE:
            continue
        elast = int(t.inj_hi[j])
        X = np.zeros(qpad, dtype=np.uint64)
        Z = np.zeros(qpad, dtype=np.uint64)
        last = np.zeros(qpad, dtype=np.uint64)
        acc = np.zeros(qpad, dtype=np.uint64)
        e = e0
        while True:
            pX, pZ = X.copy(), Z.copy()
            anynz = bool(np.any(X | Z))
            if (not anynz and e > elast) or e >= nE:
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
                jlo = 64 * j
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
                m = opc == OP_SNAP
                if m.any():
                    snap[j, arg[m], 0] = X[m]
                    snap[j, arg[m], 1] = Z[m]
                m = opc == OP_SNAPD
                if m.any():
                    snap[j, arg[m], 0] = last[m]
                    snap[j, arg[m], 1] = 0
            e += 1
        band[j] = (int(t.ep_ptoff[e0]), int(t.ep_ptoff[min(e, nE)]))
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
