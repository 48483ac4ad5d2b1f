"""The allocation-free merge entry point against the allocating compile (needs a GPU).

gpc_merge_mechanisms_static serves callers that cannot allocate device memory
(another runtime owns the memory pool, or the memory budget is fixed up
front).  It gets the raw mechanisms of a circuit -- computed here on the CPU
by interpreting the lowered tape -- in device buffers the test owns, and must
produce the same DEM as gpc_compile (symptoms equal, probabilities within
1e-12 relative), twice in a row on the same static scratch.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from greenpeas_gb300 import _native
from tape_interp import expand, symptoms, walk

pytestmark = pytest.mark.gpu

STRIDE = 32


def _raw_mechanisms(text):
    t = gp.Tape(text)
    snap, band = walk(t)
    mech = expand(t)
    S = symptoms(t, snap, band, mech)
    n = S.shape[0]
    tn = np.zeros(n, dtype=np.uint32)
    tl = np.zeros((n, STRIDE), dtype=np.uint32)
    for m in range(n):
        ts = []
        for j in range(t.words):
            v = int(S[m, j])
            while v:
                b = (v & -v).bit_length() - 1
                ts.append(64 * j + b)
                v &= v - 1
        assert len(ts) <= STRIDE
        tn[m] = len(ts)
        tl[m, :len(ts)] = ts
    return tn, tl, mech[4]


def test_static_merge_matches_compile_twice():
    import torch

    text = gp.SurfaceCode(5).get_memory(5, 1e-3, noise="uniform")
    expected = dict(gp.get_driver(text).compile(text).errors())
    tn, tl, p = _raw_mechanisms(text)
    n = len(tn)
    dev = torch.device("cuda", 0)
    d_tn = torch.from_numpy(tn.view(np.int32)).to(dev)
    d_tl = torch.from_numpy(tl.reshape(-1).view(np.int32)).to(dev)
    d_p = torch.from_numpy(p).to(dev)
    cap = int(tn.sum())
    L = _native.lib()
    for _ in range(2):
        out_p = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
        out_off = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        out_tg = torch.zeros(cap, dtype=torch.int32, device=dev)
        result = torch.zeros(4, dtype=torch.int32, device=dev)
        st = L.gpc_merge_mechanisms_static(
            ctypes.c_void_p(d_tn.data_ptr()), ctypes.c_void_p(d_tl.data_ptr()), STRIDE,
            ctypes.c_void_p(d_p.data_ptr()), n, ctypes.c_void_p(out_p.data_ptr()),
            ctypes.c_void_p(out_off.data_ptr()), ctypes.c_void_p(out_tg.data_ptr()), cap,
            ctypes.c_void_p(result.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0
        torch.cuda.synchronize()
        groups, ntg, flags, _ = (int(x) for x in result.cpu())
        assert flags == 0
        offs = out_off.cpu().numpy()[: groups + 1]
        tg = out_tg.cpu().numpy()[:ntg]
        probs = out_p.cpu().numpy()[:groups]
        got = {tuple(int(x) for x in tg[offs[i]:offs[i + 1]]): float(probs[i]) for i in range(groups)}
        assert len(got) == groups
        compare_errors(got, expected, rel=1e-12)


def test_static_merge_rejects_too_many_mechanisms():
    L = _native.lib()
    null = ctypes.c_void_p(0)
    st = L.gpc_merge_mechanisms_static(null, null, 1, null, (1 << 16) + 1, null, null, null, 0, null, null)
    assert st == -8  # GPC_ERR_CAPACITY, checked before any device work


def _static_call(tn, tl_rows, p, stride, cap, pad=16):
    """Runs the allocation-free merge on small hand-made lists.

    The target buffer carries `pad` sentinel entries past `cap`, and the row
    buffer one spare row past the last mechanism, so a write past the
    capacity or a read past a row shows up as a changed sentinel or a fault
    the bounds of the buffers would not hide.  Returns (result, targets).
    """
    import torch

    dev = torch.device("cuda", 0)
    n = len(tn)
    rows = np.zeros((n + 1, stride), dtype=np.uint32)
    for m, r in enumerate(tl_rows):
        rows[m, : min(len(r), stride)] = r[:stride]
    d_tn = torch.from_numpy(np.asarray(tn, dtype=np.uint32).view(np.int32)).to(dev)
    d_tl = torch.from_numpy(rows.reshape(-1).view(np.int32)).to(dev)
    d_p = torch.tensor(p, dtype=torch.float64, device=dev)
    out_p = torch.zeros(n, dtype=torch.float64, device=dev)
    out_off = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    out_tg = torch.full((cap + pad,), -7, dtype=torch.int32, device=dev)
    result = torch.zeros(4, dtype=torch.int32, device=dev)
    st = _native.lib().gpc_merge_mechanisms_static(
        ctypes.c_void_p(d_tn.data_ptr()), ctypes.c_void_p(d_tl.data_ptr()), stride,
        ctypes.c_void_p(d_p.data_ptr()), n, ctypes.c_void_p(out_p.data_ptr()),
        ctypes.c_void_p(out_off.data_ptr()), ctypes.c_void_p(out_tg.data_ptr()), cap,
        ctypes.c_void_p(result.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    return [int(x) for x in result.cpu()], out_tg.cpu().numpy()


def test_static_merge_reports_a_small_target_buffer():
    # 6 mechanisms, 5 distinct symptoms with 14 targets in all; room for 9
    lists = [[1, 2, 3], [4, 5], [1, 2, 3], [6, 7, 8, 9], [10, 11], [12, 13, 14]]
    tn = [len(r) for r in lists]
    res, tg = _static_call(tn, lists, [1e-3] * 6, 4, cap=9)
    assert res[2] & 8
    assert res[1] == 14  # the count the caller would need
    assert (tg[9:] == -7).all(), "written past out_target_cap"


def test_static_merge_reports_a_list_longer_than_the_stride():
    # mechanism 0 claims stride + 1 targets (not the last row); mechanism 2 is
    # not ascending
    lists = [[1, 2, 3, 4], [5, 6], [9, 7], [8]]
    tn = [5, 2, 2, 1]
    res, tg = _static_call(tn, lists, [1e-3] * 4, 4, cap=16)
    assert res[2] & 64
    assert (tg[16:] == -7).all(), "written past out_target_cap"
    assert res[1] <= 16

