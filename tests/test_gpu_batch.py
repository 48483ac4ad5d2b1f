"""The batched form: many circuits of uneven sizes in one pipeline (needs a GPU).

Every circuit's DEM from the batch must equal its single-circuit compile
(same symptoms, same probabilities bit for bit, same order) and the oracle.
"""

from __future__ import annotations

import pytest

import greenpeas_gb300 as gp
from conftest import compare_errors
from oracle import oracle as O
from test_lowering import SMALL

pytestmark = pytest.mark.gpu


def _mixed():
    circs = [gp.SurfaceCode(d).get_memory(d, 1e-3, noise=nz) for d, nz in
             [(3, "uniform"), (5, "reference"), (7, "uniform"), (3, "reference")]]
    circs += [gp.BBCode(6).get_memory(6, 1e-3, noise="uniform")]
    circs += SMALL
    return circs


def test_batch_matches_single_and_oracle():
    circs = _mixed()
    drv = gp.get_driver(circs[0])
    batch = drv.compile_batch(circs)
    assert len(batch) == len(circs)
    for text, dem in zip(circs, batch):
        single = gp.get_driver(text).compile(text)
        assert dem.canonical() == single.canonical()
        ref = O.compile_text(text, 2)
        assert dem.num_detectors == ref.num_detectors
        compare_errors(dict(dem.errors()), dict(ref.errors()), rel=1e-12)


def test_batch_device_stages_repeat():
    circs = _mixed()[:5]
    drv = gp.get_driver(circs[0])
    drv.prepare_batch(circs)
    drv.run_device()
    first = drv.fetch_batch()
    for _ in range(3):  # later runs come from a captured graph
        drv.run_device()
    again = drv.fetch_batch()
    assert [a == b for a, b in zip(first, again)] == [True] * len(circs)


def test_batch_falls_back_per_circuit():
    """A circuit with a symptom longer than the target lists makes the batch compile one by one."""
    n = 80
    long = "R " + " ".join(map(str, range(n))) + "\nX_ERROR(0.01) 0\n"
    long += "".join(f"CX 0 {q}\n" for q in range(1, n))
    long += "M " + " ".join(map(str, range(n))) + "\n" + "".join(f"DETECTOR rec[-{k}]\n" for k in range(1, n + 1))
    circs = [gp.SurfaceCode(3).get_memory(3, 1e-3), long, SMALL[2]]
    out = gp.get_driver(circs[0]).compile_batch(circs)
    for text, dem in zip(circs, out):
        compare_errors(dict(dem.errors()), dict(O.compile_text(text, 2).errors()), rel=1e-12)


def test_time_varying_switched_batch_matches_oracle():
    """Small slice of the mixed batch workload (per-instruction p, basis-switch rounds) against the oracle."""
    from greenpeas_gb300.workloads import batch_surface
    circs = batch_surface(n=12, seed=5, switch_prob=0.5, distances=(3, 5, 7))
    out = gp.get_driver(circs[0]).compile_batch(circs)
    for text, dem in zip(circs, out):
        ref = O.compile_text(text, 2)
        assert dem.num_detectors == ref.num_detectors
        compare_errors(dict(dem.errors()), dict(ref.errors()), rel=1e-12)


def test_large_batch_in_chunks_matches_single_compiles():
    """32 circuits with more than 8 MiB of text: compile_batch overlaps chunks on two pipelines;
    every DEM equals the circuit's own compile, bit for bit."""
    from greenpeas_gb300.workloads import batch_surface
    circs = batch_surface()[:32]
    assert sum(len(c) for c in circs) > 8 << 20
    drv = gp.get_driver(circs[0])
    out = drv.compile_batch(circs)
    single = gp.get_driver(circs[0])
    for text, dem in zip(circs, out):
        assert dem == single.compile(text)
    again = drv.compile_batch(circs[::-1])  # the pipelines are reused with other chunk sizes
    for a, b in zip(again, out[::-1]):
        assert a == b


def test_autotune_keeps_results_and_picks_a_configuration():
    """The autotuner times each walk configuration on the batch and keeps the fastest; the DEMs
    before and after are identical, and the prepared batch runs in the chosen configuration."""
    circs = _mixed()
    drv = gp.get_driver(circs[0])
    before = drv.compile_batch(circs)
    tune = drv.autotune(circs, reps=2)
    key = ("walk_words", "walk_qpt", "walk_queue")
    assert tuple(tune[k] for k in key) in {tuple(t[k] for k in key) for t in tune["tried"]}
    # five per-class configurations, and the four persistent ones (these circuits fit them)
    assert len(tune["tried"]) == 9 and sum(t["walk_queue"] for t in tune["tried"]) == 4
    assert tune["ms"] == min(t["ms"] for t in tune["tried"])
    drv.run_device()
    assert [a == b for a, b in zip(drv.fetch_batch(), before)] == [True] * len(circs)
    assert [a == b for a, b in zip(drv.compile_batch(circs), before)] == [True] * len(circs)
    gp.tune_cache_clear()  # (the choice is kept for the process: later tests start from the defaults)


def test_autotune_choice_is_kept_for_batches_of_the_same_widths():
    """Autotune keeps its choice for the process, keyed by the batch's bitset widths: a fresh driver
    preparing a batch of the same widths walks in that configuration, a driver with explicit walk
    options keeps its own, and the DEMs do not depend on either."""
    gp.tune_cache_clear()
    circs = _mixed()
    fresh = gp.get_driver(circs[0])
    fresh.prepare_batch(circs)
    assert fresh.walk_config() == {"walk_words": 0, "walk_qpt": 0, "walk_queue": 0}
    ref = fresh.compile_batch(circs)
    tune = gp.get_driver(circs[0]).autotune(circs, reps=1)
    chosen = {k: tune[k] for k in ("walk_words", "walk_qpt", "walk_queue")}
    other = gp.get_driver(circs[0])
    other.prepare_batch(circs[::-1])  # the same widths in another order
    assert other.walk_config() == chosen
    assert [a == b for a, b in zip(other.compile_batch(circs), ref)] == [True] * len(circs)
    explicit = gp.get_driver(circs[0], walk_words=1)
    explicit.prepare_batch(circs)
    assert explicit.walk_config() == {"walk_words": 0, "walk_qpt": 0, "walk_queue": 0}
    narrower = gp.get_driver(circs[0])
    narrower.prepare_batch(circs[:3])  # other widths: nothing kept for them
    assert narrower.walk_config() == {"walk_words": 0, "walk_qpt": 0, "walk_queue": 0}
    gp.tune_cache_clear()


@pytest.mark.parametrize("words,qpt", [(2, 1), (1, 1), (2, 2), (1, 2)])
def test_persistent_walk_matches_class_launches(words, qpt):
    """One persistent walk launch over circuits of every size (CTAs sized for the largest take
    (circuit, word group) items from a queue, longest first) gives the DEMs of the per-class
    launches, bit for bit, and the oracle's."""
    from greenpeas_gb300.workloads import batch_surface
    circs = _mixed() + batch_surface(n=6, seed=3, distances=(3, 9, 15))
    ref = gp.get_driver(circs[0], walk_queue=-1, walk_words=words, walk_qpt=qpt).compile_batch(circs)
    drv = gp.get_driver(circs[0], walk_queue=1, walk_words=words, walk_qpt=qpt)
    out = drv.compile_batch(circs)
    assert [a == b for a, b in zip(out, ref)] == [True] * len(circs)
    drv.prepare_batch(circs)
    for _ in range(3):  # later runs come from a captured graph (the queue counter is reset in it)
        drv.run_device()
    assert [a == b for a, b in zip(drv.fetch_batch(), ref)] == [True] * len(circs)
    for text, dem in list(zip(circs, out))[:len(_mixed())]:
        compare_errors(dict(dem.errors()), dict(O.compile_text(text, 2).errors()), rel=1e-12)


def test_persistent_walk_with_the_largest_batch_circuit():
    """The persistent launch sized for a d = 21 surface circuit (881 qubits, 896 threads) walks
    d = 3 circuits with most of its warps idle; DEMs equal the per-class launches'."""
    from greenpeas_gb300.workloads import batch_surface
    circs = batch_surface(n=1, seed=7, distances=(21,)) + batch_surface(n=3, seed=8, distances=(3,))
    ref = gp.get_driver(circs[0], walk_queue=-1).compile_batch(circs)
    out = gp.get_driver(circs[0], walk_queue=1).compile_batch(circs)
    assert [a == b for a, b in zip(out, ref)] == [True] * len(circs)


@pytest.mark.parametrize("heap_results", [False, True])
def test_held_batches_keep_their_dems(heap_results):
    """A batch's DEMs view their arrays in a shared page-locked result block, which goes back to the
    page-locked pool when the last of them is freed (heap_results: the DEMs own heap copies
    instead).  Every held DEM stays equal to its circuit's own compile while later batches are
    compiled and earlier ones freed."""
    circs = _mixed()
    drv = gp.get_driver(circs[0], heap_results=heap_results)
    single = [gp.get_driver(t).compile(t) for t in circs]
    held = [drv.compile_batch(circs[k % 3:] + circs[:k % 3]) for k in range(10)]
    for k, out in enumerate(held):
        for dem, ref in zip(out, single[k % 3:] + single[:k % 3]):
            assert dem == ref
    del held[1:4]  # their blocks return to the pool
    more = [drv.compile_batch(circs) for _ in range(3)]
    for out in more:
        for dem, ref in zip(out, single):
            assert dem == ref
    text = next(str(d) for d in held[0])  # the text form reads the viewed arrays
    assert text.startswith("error(") or text == ""


def test_host_timings_cover_prepare_and_fetch():
    circs = _mixed()[:5]
    drv = gp.get_driver(circs[0])
    drv.compile_batch(circs)
    t = drv.last_host_timings()
    assert set(t) == {"lower", "layout", "stage", "wait", "d2h", "split"}
    assert all(v >= 0 for v in t.values()) and t["lower"] > 0



def test_walk_queue_option_selects_the_launch_form():
    """walk_queue=1 prepares the persistent walk (one launch), walk_queue=-1 one launch per
    thread-count class; the autotuner's choice is what the driver then prepares."""
    from greenpeas_gb300.workloads import batch_surface
    circs = batch_surface(n=6, seed=3, distances=(3, 9, 15))
    forms = {}
    for q in (1, -1):
        drv = gp.get_driver(circs[0], walk_queue=q)
        drv.prepare_batch(circs)
        forms[q] = drv.walk_form()
    assert forms[1] == {"launches": 1, "persistent": True}, forms
    classes = len({gp.Tape(c).qpad for c in circs})  # one launch per distinct qubit-slot count
    assert forms[-1] == {"launches": classes, "persistent": False}, forms
    drv = gp.get_driver(circs[0])
    tune = drv.autotune(circs, reps=1)
    assert drv.walk_form()["persistent"] == bool(tune["walk_queue"])
    gp.tune_cache_clear()
