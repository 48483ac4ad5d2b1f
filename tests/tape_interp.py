"""CPU interpreter of the lowered device tape (test infrastructure).

Executes ``greenpeas_gb300.Tape`` exactly as the walk kernel does -- per
64-bit word, epoch by epoch, two-qubit Cliffords reading the partner rows
published at the epoch barrier, stopping once all rows are zero after the
word's last measurement -- then merges mechanisms the way the merge kernel
does.  It checks the host lowering against the oracle without a GPU.
"""

from __future__ import annotations

import numpy as np

OP_NOP, OP_C1, OP_C2, OP_R, OP_M, OP_MR, OP_SNAP, OP_SNAPD = range(8)
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
                m = (opc == OP_R) | (opc == OP_MR)
                X[m] = 0
                Z[m] = 0
                for q in np.nonzero((opc == OP_M) | (opc == OP_MR))[0]:
                    meas = int(arg[q])
                    inj = 0
                    for b in t.meas_bits[t.meas_off[meas]:t.meas_off[meas + 1]]:
                        if int(b) >> 6 == j:
                            inj |= 1 << (int(b) & 63)
                    inj = U64(inj)
                    if sub[q] != 1:
                        X[q] ^= inj
                    if sub[q] != 0:
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


def symptoms(t, snap, band):
    """[M, w] uint64 symptom words of every mechanism."""
    d = t.desc
    pa = (d & U64(0x3FFFFFFF)).astype(np.int64)
    Pa = ((d >> U64(30)) & U64(3)).astype(np.uint32)
    pb = ((d >> U64(32)) & U64(0x3FFFFFFF)).astype(np.int64)
    Pb = (d >> U64(62)).astype(np.uint32)
    S = np.zeros((t.num_mechanisms, t.words), dtype=np.uint64)
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
    S = symptoms(t, snap, band)
    uniq, inv = np.unique(S, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    p = np.full(uniq.shape[0], -1.0)
    for m in range(t.num_mechanisms):
        g = inv[m]
        q = float(t.prob[m])
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
