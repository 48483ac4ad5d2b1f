"""Incremental lowering of circuit branches (host only, no GPU).

A lowerer keeps the last circuit it lowered and lowers the next one against
it (``gpc_lowerer_*``).  It parses again only the statements that differ and
takes over the time segments they leave alone.  Every tape must equal a full
lowering of the same text with the same backward-pass cuts, byte for byte.
For small circuits, the DEM that the CPU tape interpreter reads off the tape
must also equal the oracle's.
"""

from __future__ import annotations

import random

import numpy as np
import pytest

from conftest import compare_errors, repetition_with_repeat
from greenpeas_gb300 import GpcError, Lowerer
from greenpeas_gb300 import error_analysis as ea
from greenpeas_gb300.codes import BBCode, SurfaceCode
from oracle import oracle as O
from tape_interp import compile_tape

GPC_ERR_INVALID, GPC_ERR_UNSUPPORTED = -1, -3

ARRAYS = ("ops", "ep_opoff", "ep_k", "ep_ptoff", "inj_lo", "inj_hi", "rec", "rec_p", "rec_moff", "rec_src")
SCALARS = ("num_qubits", "qpad", "num_measurements", "num_detectors", "num_observables", "words", "num_epochs",
           "kmax", "num_points", "num_mechanisms", "num_records", "num_ticks")


def assert_same_tape(a, b):
    for f in SCALARS:
        assert getattr(a, f) == getattr(b, f), f
    for f in ARRAYS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def lower_family(texts, oracle: bool = False):
    """Lowers `texts` in order through one incremental lowerer; checks each tape against the full
    lowering with the same cuts (and the DEM against the oracle); returns the lowerings' stats."""
    lw = Lowerer(2, incremental=True)
    out = []
    for text in texts:
        tape = lw.tape(text)
        assert_same_tape(tape, ea.Tape(text, cuts=lw.cuts))
        if oracle:
            compare_errors(compile_tape(tape), dict(O.compile_text(text, 2).errors()), rel=1e-12)
        out.append(lw.stats)
    lw.close()
    return out


def test_basis_switch_branches_take_over_the_unchanged_segments():
    s = SurfaceCode(11)
    switches = ([], [5], [5, 6], [5, 6, 7], [6, 7], [], [9], [9, 10])
    texts = [s.get_memory(11, 1e-3, noise="uniform", switch_rounds=sw) for sw in switches]
    st = lower_family(texts)
    assert not st[0]["incremental"]
    assert all(x["incremental"] for x in st[1:5])
    assert all(x["reused"] >= 1 for x in st[1:5])
    assert all(x["parsed_bytes"] < len(texts[0]) // 4 for x in st[1:5])


def test_added_and_removed_rounds_shift_the_later_segments():
    """Rounds added or removed in the middle renumber every later measurement, detector and tick:
    the segments after them are taken over with their detector bits and sources shifted."""
    s = SurfaceCode(11)
    texts = [s.get_memory(r, 1e-3, noise="uniform") for r in (11, 12, 11, 10, 13)]
    st = lower_family(texts)
    assert all(x["incremental"] and x["reused"] >= 3 for x in st[1:])
    assert st[2]["parsed_bytes"] == 0  # (12 rounds -> 11: a deleted round leaves nothing to parse)


def test_bb_rounds():
    b = BBCode(6)
    texts = [b.get_memory(r, 1e-3, noise="uniform") for r in (6, 7, 6, 5)]
    lower_family(texts)


def test_line_edits():
    base = SurfaceCode(11).get_memory(11, 1e-3, noise="uniform").split("\n")
    rng = random.Random(1)
    cur = list(base)
    texts = ["\n".join(cur)]
    for i in range(10):
        j = rng.randrange(len(cur))
        op = rng.choice(["del", "dup", "p", "comment"])
        if op == "del" and not cur[j].startswith(("DETECTOR", "OBSERVABLE")):
            del cur[j]
        elif op == "dup" and cur[j].startswith(("X_ERROR", "DEPOLARIZE", "TICK", "H ")):
            cur.insert(j, cur[j])
        elif op == "p" and "ERROR(" in cur[j]:
            cur[j] = cur[j].split("(")[0] + "(0.0042)" + cur[j].split(")", 1)[1]
        else:
            cur.insert(j, f"# note {i}")
        texts.append("\n".join(cur))
    st = lower_family(texts)
    assert sum(x["reused"] for x in st[1:]) >= 10


def test_small_branches_match_the_oracle():
    s = SurfaceCode(5)
    texts = [s.get_memory(5, 1e-3, noise="uniform", switch_rounds=sw) for sw in ([], [2], [2, 3], [4])]
    texts += [s.get_memory(r, 1e-3, noise="uniform") for r in (5, 6, 4)]
    lower_family(texts, oracle=True)


def test_repeat_blocks():
    a = repetition_with_repeat(5)
    texts = [a, repetition_with_repeat(6), a.replace("MR 1 3\n", "MR 1 3\nX_ERROR(0.002) 0\n", 1),
             a.replace("X_ERROR(0.001) 0 2 4\nM 0 2 4", "X_ERROR(0.003) 0 2 4\nM 0 2 4"), a]
    lower_family(texts, oracle=True)


def test_same_text_again_takes_over_every_segment():
    text = SurfaceCode(11).get_memory(11, 1e-3, noise="uniform")
    lw = Lowerer(2)
    t1 = lw.tape(text)
    t2 = lw.tape(text)
    st = lw.stats
    assert st["incremental"] and st["reused"] == st["segments"] and st["parsed_bytes"] == 0
    assert_same_tape(t1, t2)


def test_branches_changed_in_several_places():
    """Two branches that differ in rounds far apart: the segments between the changes are kept."""
    s = SurfaceCode(11)
    switches = ([], [1, 9], [2, 8], [0, 5, 10], [1, 9], [3])
    texts = [s.get_memory(11, 1e-3, noise="uniform", switch_rounds=sw) for sw in switches]
    st = lower_family(texts)
    assert all(x["incremental"] for x in st[1:])
    assert st[1]["reused"] >= 2  # (the segments wholly between rounds 1 and 9)
    assert all(x["parsed_bytes"] < len(texts[0]) // 4 for x in st[1:])


def test_unrelated_circuits_are_lowered_whole():
    texts = [SurfaceCode(5).get_memory(5, 1e-3, noise="uniform"), BBCode(6).get_memory(6, 1e-3, noise="uniform"),
             SurfaceCode(5).get_memory(5, 2e-3, noise="uniform")]
    st = lower_family(texts)
    assert not any(x["incremental"] for x in st)


def test_not_incremental():
    s = SurfaceCode(5)
    lw = Lowerer(2, incremental=False)
    for sw in ([], [2]):
        text = s.get_memory(5, 1e-3, noise="uniform", switch_rounds=sw)
        assert_same_tape(lw.tape(text), ea.Tape(text))
        assert not lw.stats["incremental"]


def test_error_in_the_changed_span_is_reported_on_its_line():
    text = SurfaceCode(5).get_memory(5, 1e-3, noise="uniform")
    lines = text.split("\n")
    k = len(lines) // 2
    bad = "\n".join(lines[:k] + ["FOO 1 2"] + lines[k:])
    lw = Lowerer(2)
    lw.tape(text)
    with pytest.raises(GpcError) as e:
        lw.tape(bad)
    assert e.value.status == GPC_ERR_UNSUPPORTED
    assert f"line {k + 1}" in str(e.value)
    # the failed lowering left nothing to lower against: the next one is whole, and right
    text2 = SurfaceCode(5).get_memory(5, 1e-3, noise="uniform", switch_rounds=[1])
    assert_same_tape(lw.tape(text2), ea.Tape(text2, cuts=lw.cuts))
    assert not lw.stats["incremental"]


def test_bad_cuts_are_rejected():
    text = SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    lw = Lowerer(2)
    lw.tape(text)
    nins = int(lw.cuts[0])
    for cuts in ([nins, 5, 5, 0], [nins - 1, 0], [nins, 3], [0]):
        with pytest.raises(GpcError) as e:
            ea.Tape(text, cuts=cuts)
        assert e.value.status == GPC_ERR_INVALID
    # any cuts give the same DEM
    compare_errors(compile_tape(ea.Tape(text, cuts=[nins, nins // 2, nins // 3, 0])),
                   dict(O.compile_text(text, 2).errors()), rel=1e-12)


@pytest.mark.parametrize("seed,eol", [(0, "\n"), (1, "\n"), (2, "\n"), (3, "\r\n"), (4, "")])
def test_random_edits(seed, eol):
    """Random line edits (deleted, duplicated and moved blocks, changed rates, comments, blank
    lines, a REPEAT block around some lines), with LF or CRLF line ends or no final newline:
    each tape equals the full lowering with its cuts."""
    rng = random.Random(seed)
    base = SurfaceCode(7).get_memory(7, 1e-3, noise="uniform").split("\n")
    cur = list(base)
    texts = ["\n".join(cur)]
    for _ in range(40):
        j = rng.randrange(1, len(cur) - 1)
        n = rng.randrange(1, 6)
        op = rng.randrange(7)
        blk = cur[j:j + n]
        safe = not any(x.startswith(("DETECTOR", "OBSERVABLE", "M", "REPEAT", "}")) or "{" in x for x in blk)
        if op == 0 and safe:
            del cur[j:j + n]
        elif op == 1 and safe:
            cur[j:j] = blk
        elif op == 2 and safe:
            k = rng.randrange(1, len(cur) - 1)
            del cur[j:j + n]
            cur[k:k] = blk
        elif op == 3 and "ERROR(" in cur[j]:
            cur[j] = cur[j].split("(")[0] + f"({rng.choice(['0.002', '0.0005', '0.01'])})" + cur[j].split(")", 1)[1]
        elif op == 4:
            cur.insert(j, rng.choice(["", "# c", "   ", "TICK"]))
        elif op == 5 and safe and not any("{" in x or "}" in x for x in cur):
            cur[j:j + n] = ["REPEAT 2 {"] + ["  " + x for x in blk] + ["}"]
        else:
            cur.insert(j, cur[j] if not cur[j].startswith(("DETECTOR", "OBSERVABLE", "M", "REPEAT", "}")) else "# x")
        texts.append("\n".join(cur))
    if eol == "\r\n":
        texts = [t.replace("\n", "\r\n") for t in texts]
    elif eol == "":
        texts = [t.rstrip("\n") for t in texts]
    st = lower_family(texts)
    assert sum(x["incremental"] for x in st) >= 20


@pytest.mark.parametrize("seed", [0, 1])
def test_random_edits_of_unchanged_length(seed):
    """Edits that keep the text's length (a rate's digit changed, lines swapped, targets of a line
    reversed) take the in-step comparison: each tape equals the full lowering with its cuts."""
    rng = random.Random(seed)
    cur = SurfaceCode(7).get_memory(7, 1e-3, noise="uniform").split("\n")
    texts = ["\n".join(cur)]
    for _ in range(40):
        for _ in range(rng.randrange(1, 4)):
            j = rng.randrange(1, len(cur) - 2)
            op = rng.randrange(3)
            if op == 0 and "(0.00" in cur[j]:
                k = cur[j].index("(0.00") + 5
                cur[j] = cur[j][:k] + rng.choice("123456789") + cur[j][k + 1:]
            elif op == 1 and not cur[j].startswith(("DETECTOR", "OBSERVABLE", "M")) \
                    and not cur[j + 1].startswith(("DETECTOR", "OBSERVABLE", "M")):
                cur[j], cur[j + 1] = cur[j + 1], cur[j]
            elif op == 2 and cur[j].startswith(("H ", "R ", "X_ERROR", "DEPOLARIZE1")):
                name, *tg = cur[j].split(" ")
                cur[j] = " ".join([name] + tg[::-1])
        texts.append("\n".join(cur))
    assert len({len(t) for t in texts}) == 1
    st = lower_family(texts)
    assert sum(x["incremental"] for x in st) >= 30


def test_a_lowering_that_fails_after_the_text_compare_leaves_nothing_to_lower_against():
    """A changed statement that parses but fails in the lowering (a lookback beyond the start of
    the circuit): the error is the whole lowering's, and the next circuit is lowered whole."""
    s = SurfaceCode(7)
    base = s.get_memory(7, 1e-3, noise="uniform")
    lines = base.split("\n")
    k = len(lines) // 2
    bad = "\n".join(lines[:k] + ["DETECTOR rec[-100000]"] + lines[k:])
    lw = Lowerer(2)
    lw.tape(base)
    with pytest.raises(GpcError) as e:
        lw.tape(bad)
    with pytest.raises(GpcError) as e_whole:
        ea.Tape(bad)
    assert e.value.status == e_whole.value.status and str(e.value) == str(e_whole.value)
    nxt = s.get_memory(7, 1e-3, noise="uniform", switch_rounds=[3])
    assert_same_tape(lw.tape(nxt), ea.Tape(nxt, cuts=lw.cuts))
    assert not lw.stats["incremental"]
    assert_same_tape(lw.tape(base), ea.Tape(base, cuts=lw.cuts))
    assert lw.stats["incremental"]
