"""CUDA path parity against the CPU FP64 oracle and the reference golden DEMs (needs a GPU).

Comparison rule: symptom sets bit-exact, merged probabilities within 1e-12
relative, same detector / observable counts.
"""

from __future__ import annotations

import numpy as np
import pytest

import greenpeas_gb300 as gp
from conftest import GOLDEN, compare_errors, load_canonical_dem, to_named
from oracle import oracle as O
from test_lowering import SMALL

pytestmark = pytest.mark.gpu
REL = 1e-12


def _check(dem, text, level=2):
    ref = O.compile_text(text, level)
    assert dem.num_detectors == ref.num_detectors and dem.num_observables == ref.num_observables
    compare_errors(dict(dem.errors()), dict(ref.errors()), rel=REL)


@pytest.mark.parametrize("text", SMALL)
def test_small(text):
    _check(gp.get_driver(text).compile(text), text)


@pytest.mark.parametrize("d", [3, 5])
@pytest.mark.parametrize("level", [0, 1, 2])
def test_reference_golden(d, level):
    """python/tests/test_error_analysis.py:27-45 on the GPU path."""
    text = gp.SurfaceCode(d).get_memory(d, 1e-3)
    dem = gp.get_driver(text, gp.CorrelationLevel(level)).compile_detector_error_model(text)
    got = {n: p for n, p in dem.named_errors()}
    compare_errors(got, load_canonical_dem(GOLDEN / "dems" / f"surface{d}_L{level}.dem"), rel=REL)


@pytest.mark.parametrize("level", [0, 1, 2])
def test_driver_reuse(level):
    """python/tests/test_error_analysis.py:48-59: a d5-sized driver compiles d3."""
    d5 = gp.SurfaceCode(5).get_memory(5, 1e-3)
    d3 = gp.SurfaceCode(3).get_memory(3, 1e-3)
    drv = gp.get_driver(d5, gp.CorrelationLevel(level))
    dem = drv.compile(d3)
    got = {n: p for n, p in dem.named_errors()}
    compare_errors(got, load_canonical_dem(GOLDEN / "dems" / f"surface3_L{level}.dem"), rel=REL)
    # and back to the larger circuit, then the no-argument overload
    _check(drv.compile(d5), d5, level)
    _check(drv.compile(), d5, level)


@pytest.mark.parametrize("code,d", [("surface", 7), ("bb", 6), ("bb", 12)])
@pytest.mark.parametrize("noise", ["uniform", "reference"])
def test_codes(code, d, noise):
    c = gp.SurfaceCode(d) if code == "surface" else gp.BBCode(d)
    text = c.get_memory(d, 1e-3, noise=noise)
    _check(gp.get_driver(text).compile(text), text)


def test_deterministic():
    text = gp.BBCode(6).get_memory(6, 1e-3, noise="uniform")
    drv = gp.get_driver(text)
    a, b = drv.compile(text), drv.compile(text)
    assert a == b  # same order, same bits


@pytest.mark.parametrize("bits", [8, 16, 64])
def test_global_sort_path(bits):
    """The global onesweep path (taken when a bucket overflows).  With few sorted key bits, runs of
    different symptoms interleave; the merge must detect them and re-sort on all 128 bits."""
    text = gp.SurfaceCode(5).get_memory(5, 1e-3, noise="uniform")
    _check(gp.get_driver(text, sort_bits=bits, global_sort=True).compile(text), text)


def test_repeated_symptom_overflows_bucket():
    """More copies of one symptom than a bucket CTA holds: falls back to the global sort."""
    text = "R 0 1\n" + "X_ERROR(0.0001) 0\nTICK\n" * 3000 + "CX 0 1\nM 0 1\nDETECTOR rec[-1]\nDETECTOR rec[-2]\n"
    _check(gp.get_driver(text).compile(text), text)


@pytest.mark.parametrize("copies", [129, 200, 250])
def test_large_bucket_cta_path(copies):
    """A symptom repeated more often than one warp merges (128) but within a bucket's slots (256):
    the bucket goes to the CTA kernel, whose runs cross its warps' 32-position chunks."""
    text = "R 0 1 2\n" + "X_ERROR(0.001) 0\nTICK\n" * copies + "DEPOLARIZE1(0.01) 1 2\n"
    text += "CX 0 1\nM 0 1 2\nDETECTOR rec[-1]\nDETECTOR rec[-2]\nDETECTOR rec[-3]\n"
    _check(gp.get_driver(text).compile(text), text)


def test_bucket_and_global_paths_agree():
    text = gp.BBCode(6).get_memory(6, 1e-3, noise="uniform")
    a = gp.get_driver(text).compile(text)
    b = gp.get_driver(text, global_sort=True).compile(text)
    # the bucket path folds runs as a tree, the global path left to right: a few ulps apart
    assert a.canonical() == b.canonical() or a.approx_equals(b, rtol=1e-13)


def test_empty_and_noiseless():
    for text in ["R 0\nM 0\nDETECTOR rec[-1]\n", "TICK\n", "R 0\nZ_ERROR(0.1) 0\nM 0\nDETECTOR rec[-1]\n"]:
        dem = gp.get_driver(text).compile(text)
        assert dem.num_errors == 0


def test_device_stages_and_timings():
    """Stage times need stage timing on for the run (its events live in another captured graph);
    the DEM does not depend on it."""
    text = gp.BBCode(6).get_memory(6, 1e-3, noise="uniform")
    drv = gp.get_driver(text)
    drv.prepare(text)
    drv.run_device()
    with pytest.raises(gp.GpcError):
        drv.last_timings()
    drv.set_stage_timing(True)
    for _ in range(3):  # the third run replays the captured graph with the events
        drv.run_device()
        t = drv.last_timings()
        assert t["total"] > 0 and all(v >= 0 for v in t.values())
    dem = drv.fetch()
    _check(dem, text)
    drv.set_stage_timing(False)
    for _ in range(3):
        drv.run_device()
    assert drv.fetch() == dem


@pytest.mark.parametrize("n", [80, 300])
def test_long_symptoms(n):
    """Symptoms of 80 and 300 targets spread over several 64-bit words, one of them repeated (merged
    after the full-symptom check): past the default target-list stride (32) the driver widens the
    lists and runs again, past 256 targets it merges from the snapshots (the global path; a batch
    holding such a circuit compiles circuit by circuit); alone and in a batch."""
    text = "R " + " ".join(map(str, range(n))) + "\nX_ERROR(0.01) 0\nX_ERROR(0.02) 0\nTICK\n"
    text += "".join(f"CX 0 {q}\n" for q in range(1, n))
    text += "DEPOLARIZE1(0.001) " + " ".join(map(str, range(n))) + "\n"
    text += "M " + " ".join(map(str, range(n))) + "\n" + "".join(f"DETECTOR rec[-{k}]\n" for k in range(1, n + 1))
    _check(gp.get_driver(text).compile(text), text)
    small = gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")
    for dem, t in zip(gp.get_driver(text).compile_batch([small, text, small]), [small, text, small]):
        _check(dem, t)


@pytest.mark.parametrize("heap_results", [False, True])
def test_many_live_dems(heap_results):
    """A single compile copies its result straight into a pinned DEM while at most four of those
    are alive; a caller holding more (or a driver with heap_results) gets DEMs filled through the
    staging buffer.  Every DEM stays intact while others are made and freed."""
    texts = [gp.BBCode(6).get_memory(6, 1e-3, noise="uniform"), gp.SurfaceCode(5).get_memory(5, 1e-3, noise="uniform")]
    drv = gp.get_driver(texts[0], heap_results=heap_results)
    refs = [drv.compile(t).canonical() for t in texts]
    held = [drv.compile(texts[i % 2]) for i in range(9)]
    for i, dem in enumerate(held):
        assert dem.canonical() == refs[i % 2]
    del held[::2]  # freed DEMs return to the cache, are reused by the next compiles
    more = [drv.compile(texts[i % 2]) for i in range(6)]
    for i, dem in enumerate(held):
        assert dem.canonical() == refs[(2 * i + 1) % 2]
    for i, dem in enumerate(more):
        assert dem.canonical() == refs[i % 2]
    _check(more[0], texts[0])


def test_driver_reuse_from_large_to_small_circuits():
    """One driver compiling circuits of falling size (its arena holds the previous circuit's data)
    gives exactly what fresh drivers give."""
    from greenpeas_gb300.workloads import batch_surface
    circs = [gp.SurfaceCode(9).get_memory(9, 1e-3, noise="uniform")]
    circs += batch_surface(n=10, seed=3, switch_prob=0.3, distances=(3, 5, 7))
    drv = gp.get_driver(circs[0])
    for text in circs:
        drv.prepare(text)
        drv.run_device()
        drv.run_device()  # the second run comes from a captured graph
        assert drv.fetch() == gp.get_driver(text).compile(text)


@pytest.mark.parametrize("name", ["iceberg_surface_4_static_circl", "iceberg_surface_4_adaptive_circl",
                                  "iceberg_surface_6_static_circl", "iceberg_surface_6_adaptive_circl",
                                  "iceberg_surface_6_static_pheno", "iceberg_surface_6_adaptive_pheno"])
def test_concatenated_fixture_circuits(name):
    """The reference's iceberg + surface circuits, static and adaptive outer-check schedules."""
    from test_iceberg import load, noisy
    text = noisy(load(name))
    _check(gp.get_driver(text).compile(text), text)


def test_device_dem_arrays_without_copy():
    torch = pytest.importorskip("torch")
    circs = [gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform"), gp.BBCode(6).get_memory(2, 2e-3, noise="uniform")]
    drv = gp.get_driver(circs[0])
    dem = drv.compile(circs[0])
    p, off, tg = drv.device_dem()
    assert p.is_cuda and np.array_equal(p.cpu().numpy(), dem.probs)
    assert np.array_equal(off.cpu().numpy().astype(np.uint32), dem.offsets)
    assert np.array_equal(tg.cpu().numpy().astype(np.uint32), dem.targets)
    drv.prepare_batch(circs)
    drv.run_device()
    host = drv.fetch_batch()
    for i, d in enumerate(host):
        p, off, tg = drv.device_dem(i)
        o = off.cpu().numpy().astype(np.int64)
        assert np.array_equal(p.cpu().numpy(), d.probs)
        assert np.array_equal(o - o[0], d.offsets.astype(np.int64))
        assert np.array_equal(tg.cpu().numpy()[o[0]:o[-1]].astype(np.uint32), d.targets)


def test_more_than_1024_qubits():
    """Two qubits per walk thread; the packed slot count need not split into whole warps."""
    # the first round count whose packed slot count leaves a partial warp (1,184 slots: 592 threads;
    # the packing follows the circuit's op sequences, so which round counts qualify can change)
    text = next(c for c in (gp.SurfaceCode(23).get_memory(r, 1e-3, noise="uniform") for r in (8, 3, 1, 2, 4, 5, 6, 7))
                if (gp.Tape(c).qpad // 2) % 32 != 0)
    t = gp.Tape(text)
    assert t.num_qubits > 1024 and (t.qpad // 2) % 32 != 0
    _check(gp.get_driver(text).compile(text), text)
    out = gp.get_driver(text).compile_batch([text, gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")])
    _check(out[0], text)
