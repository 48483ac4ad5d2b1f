"""Host lowering (libgpc.so, no GPU) checked by interpreting the tape on the CPU."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, compare_errors, flatten_repeats, load_canonical_dem, repetition_with_repeat, to_named
from greenpeas_gb300 import BBCode, SurfaceCode, Tape
from greenpeas_gb300._native import GpcError
from oracle import oracle as O
from tape_interp import compile_tape

SMALL = [
    "R 0\nX_ERROR(0.1) 0\nM 0\nDETECTOR rec[-1]\n",
    "R 0 1\nX_ERROR(0.2) 0\nCX 0 1\nM 0 1\nDETECTOR rec[-1]\nDETECTOR rec[-2]\n",
    "R 0 1 2\nH 0\nDEPOLARIZE1(0.01) 0 1 2\nCZ 0 1\nCY 1 2\nS 2\nDEPOLARIZE2(0.02) 0 2\n"
    "SWAP 0 1\nSQRT_X 0\nMX(0.03) 0\nMY 1\nMR 2\nDETECTOR rec[-1]\nDETECTOR rec[-2] rec[-3]\n"
    "OBSERVABLE_INCLUDE(1) rec[-2]\n",
    "RX 0\nRY 1\nPAULI_CHANNEL_1(0.01,0.02,0.03) 0 1\nE(0.05) X0 Z1\nC_XYZ 0\nH_YZ 1\nXCX 0 1\nXCZ 1 0\n"
    "M 0 1\nDETECTOR rec[-1]\nDETECTOR rec[-2]\n",
    "REPEAT 3 {\nR 0 1\nDEPOLARIZE1(0.001) 0 1\nCX 0 1 1 0\nM(0.01) 0 1\nDETECTOR rec[-1]\n}\n",
]


def _oracle(text, level=2):
    r = O.compile_text(text, level)
    return {t: p for t, p in r.errors()}


@pytest.mark.parametrize("text", SMALL)
def test_small_circuits_match_oracle(text):
    compare_errors(compile_tape(Tape(text)), _oracle(text))


@pytest.mark.parametrize("d", [3, 5])
@pytest.mark.parametrize("level", [0, 1, 2])
def test_surface_golden(d, level):
    text = SurfaceCode(d).get_memory(d, 1e-3)
    t = Tape(text, level)
    got = {to_named(k, t.num_detectors): p for k, p in compile_tape(t).items()}
    compare_errors(got, load_canonical_dem(GOLDEN / "dems" / f"surface{d}_L{level}.dem"))


def test_bb6_uniform_matches_oracle():
    text = BBCode(6).get_memory(6, 1e-3, noise="uniform")
    compare_errors(compile_tape(Tape(text)), _oracle(text))


def _tape_arrays(t):
    return {k: v for k, v in vars(t).items()}


def test_large_text_parsed_in_pieces_gives_the_same_tape():
    """Texts of 64 KiB and more are cut at line ends and parsed on several threads; a '{'
    anywhere (here in a comment) makes the parse take the text whole.  Same tape either way."""
    text = BBCode(12).get_memory(12, 1e-3, noise="uniform")
    assert len(text) > 200_000 and "{" not in text
    a, b = _tape_arrays(Tape(text)), _tape_arrays(Tape("# {\n" + text))
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_large_tape_matches_oracle():
    """A text this large is parsed in pieces and its tape scattered and renumbered on several
    threads; interpreted on the CPU, the tape gives the oracle's DEM."""
    text = BBCode(12).get_memory(12, 1e-3, noise="uniform")
    compare_errors(compile_tape(Tape(text)), _oracle(text))


@pytest.mark.parametrize("bad,code", [("FOO 1\n", -3), ("CX 5\n", -2), ("CX rec[-1] 0\n", -3),
                                      ("DEPOLARIZE1(0.9) 0\n", -2), ("OBSERVABLE_INCLUDE(-1) rec[-1]\n", -2),
                                      ("DETECTOR rec[-100000]\n", -2), ("PAULI_CHANNEL_1(0.4, 0.4, 0.4) 0\n", -3)])
def test_large_text_error_in_a_late_piece(bad, code):
    """Errors late in a text long enough to be parsed in pieces and counted in pieces (the
    forward pass on the pool) are reported as the serial lowering reports them."""
    text = BBCode(12).get_memory(12, 1e-3, noise="uniform")
    with pytest.raises(GpcError) as ei:
        Tape(text + bad)
    assert ei.value.status == code
    lines = text.count("\n") + 1
    with pytest.raises(GpcError) as e2:
        Tape(text + bad + text)  # the same error with a long text after it
    assert e2.value.status == code and str(e2.value) == str(ei.value)
    assert "line" not in str(ei.value) or f"line {lines}" in str(ei.value)


def test_repeat_block_gives_the_tape_of_its_flattened_circuit():
    """Every array of the tape -- ops, records, and the records' (tick, class) sources --
    equals that of the circuit with the REPEAT block written out (500 repetitions share
    one stored copy of the block's targets)."""
    text = repetition_with_repeat(500)
    a, b = _tape_arrays(Tape(text)), _tape_arrays(Tape(flatten_repeats(text)))
    assert a["num_ticks"] == 3 * 501 + 1  # 1503 TICKs
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_tape_shapes():
    t = Tape(SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"))
    assert t.num_mechanisms == 1227  # raw mechanisms of the surface d=3 r=3 config
    assert t.qpad % 32 == 0 and len(t.ops) == int(np.sum(t.ep_k)) * t.qpad
    assert t.ep_ptoff[-1] == t.num_points


@pytest.mark.parametrize("bad,code", [("FOO 0\n", -3), ("CX 0\n", -2), ("DEPOLARIZE1(0.9) 0\n", -2),
                                      ("REPEAT 2 {\nH 0\n", -2), ("M 0\nDETECTOR rec[-2]\n", -2),
                                      ("CX rec[-1] 0\n", -3), ("M 0\nDETECTOR rec[-0]\n", -2),
                                      ("M 0\nDETECTOR rec[-1\n", -2), ("M 0\nDETECTOR rec[1]\n", -2),
                                      ("M 0\nDETECTOR rec[-99999999999]\n", -2), ("M 0\nDETECTOR rec[-1]x\n", -2),
                                      ("H 1234567890\n", -8), ("H 0 1x\n", -2)])
def test_rejects_bad_input(bad, code):
    with pytest.raises(GpcError) as ei:
        Tape(bad)
    assert ei.value.status == code


def test_text_reference_passes_utf8_without_copy():
    """The Python layer hands text to the library as (address, length) of its UTF-8 bytes: a str
    through CPython's UTF-8 buffer (non-ASCII text included), bytes as they are."""
    import ctypes
    from greenpeas_gb300.error_analysis import _text_ref
    for text in ["H 0\nM 0\n", "# qubit é中\nH 0\n", b"CX 0 1\n", ""]:
        addr, n, keep = _text_ref(text)
        want = text if isinstance(text, bytes) else text.encode()
        assert n == len(want) and ctypes.string_at(addr, n) == want
    assert _text_ref(None) == (None, 0, None)


@pytest.mark.parametrize("name", ["surface3", "surface5_golden", "bb6"])
@pytest.mark.parametrize("target", [8, 24])
def test_segmented_walk_matches_the_plain_walk(name, target):
    """The walk cut into time segments (the segmented walk kernels' algorithm: first parts walked
    from zero, later segments from entry rows composed through each segment's GF(2) transfer
    matrix and its walk from zero) gives every mechanism the symptom of the uncut walk, at the
    cuts the library plans."""
    from tape_interp import expand, symptoms, walk, walk_segmented

    text = {"surface3": SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"),
            "surface5_golden": SurfaceCode(5).get_memory(5, 1e-3),
            "bb6": BBCode(6).get_memory(6, 1e-3, noise="uniform")}[name]
    t = Tape(text, segment_target=target)
    assert len(t.walk_bounds) > 2, "the plan should cut this walk"
    mech = expand(t)
    a = symptoms(t, *walk(t), mech)
    b = symptoms(t, *walk_segmented(t, t.walk_bounds), mech)
    assert (a == b).all()


def test_walk_segments_cut_only_between_measurements():
    """No planned cut splits a measurement: the first slot of a cut epoch holds no OP_INJ, OP_M or
    OP_SNAPD (the ops that carry bits from the previous op of their slot)."""
    from tape_interp import OP_INJ, OP_M, OP_SNAPD

    t = Tape(BBCode(12).get_memory(12, 1e-3, noise="uniform"), segment_target=12)
    b = t.walk_bounds
    assert b[0] == 0 and b[-1] == t.num_epochs and (np.diff(b) > 0).all()
    assert len(b) > 10
    for e in b[1:-1]:
        first = t.ops[int(t.ep_opoff[e]): int(t.ep_opoff[e]) + t.qpad] & np.uint64(0xFF)
        assert not np.isin(first, [OP_INJ, OP_M, OP_SNAPD]).any()
