"""Benchmark: DEM compiles per second on one GB300 (plain method, BB [[144,12,12]] memory).

Workload (the plain large configuration): bivariate-bicycle [[144,12,12]]
code, l=12, m=6, A=x^3+y+y^2, B=y^3+x+x^2, 12 rounds of syndrome extraction,
uniform circuit-level depolarizing noise p=1e-3 (DEPOLARIZE2 after each CNOT,
DEPOLARIZE1 on data before each round, X_ERROR after resets and before
measurements).  The circuit is generated here (synthetic, seeded by nothing:
it is deterministic).

Lines printed (one JSON line on rank 0):
  value  -- DEM compiles/s with the tape resident in HBM: one step is one run
            of the kernel pipeline (walk, keys, bucket partition, merge),
            timed with CUDA events on the driver's stream; the L2 is flushed
            between steps (a 512 MiB write, outside the timed window).
  e2e    -- the same metric through the C ABI from host text to host DEM
            arrays (parse + lowering + H2D + kernels + D2H), wall clock.
  roofline, cpu_baseline, clocks, gpu_launches, batch, grad, branches, serve -- see main().

``--impl reference`` times the CPU FP64 oracle (a restatement of the
reference's algorithm; the reference itself has no CPU path) for the same
workload in its fastest CPU configuration: one single-threaded process per
host core, each compiling the workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DEM compiles/s (plain method, one circuit per compile)"
UNIT = "DEM/s"
WORKLOAD = "bb_144_12_12_r12_uniform_p1e-3"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
# kernels of one run of the pipeline on one circuit: key-block table, walk, keys,
# warp grouping, large-bucket grouping, scan, emit (the segmented walk is two launches)
KERNELS_PER_RUN = 7
# DRAM bytes (read + write) of the walk on the headline workload, from ncu captures (cold cache:
# the tape is read once from DRAM, the word walks re-read it from L2): the plain walk launch
# (profiles/headline_bb12_kernels.txt) and the two launches of the segmented walk
# (profiles/headline_bb12_segmented_walk.txt).
WALK_DRAM_BYTES_PLAIN = 1_245_440
WALK_DRAM_BYTES_PER_RUN = 1_147_904 + 1_919_488


def workload_text() -> str:
    from greenpeas_gb300.codes import BBCode
    return BBCode(12).get_memory(rounds=12, p=1e-3, noise="uniform")


def config(extra=None) -> dict:
    c = {"workload": WORKLOAD, "code": "bivariate-bicycle [[144,12,12]] l=12 m=6", "rounds": 12, "p": 1e-3,
         "noise": "uniform circuit-level", "correlation_level": "L2", "circuits_per_compile": 1,
         "l2": "flushed between timed steps (512 MiB write)", "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons in a background process."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> tuple:
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


_worker_text = None


def _oracle_init(text: str) -> None:
    global _worker_text
    _worker_text = text
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    O.lib()


def _oracle_one(_=None) -> int:
    """One single-threaded oracle compile of the worker's workload."""
    from oracle import oracle as O
    O.time_compile(_worker_text, 2, 1)
    return 1


def _oracle_rate(args) -> tuple:
    """Single-threaded oracle compiles for a time budget (one process of the per-core figure)."""
    text, budget = args
    _oracle_init(text)
    _oracle_one()
    n, t0 = 0, time.perf_counter()
    while True:
        _oracle_one()
        n += 1
        el = time.perf_counter() - t0
        if el > budget:
            return n, el


def run_reference(args, rank: int, world: int) -> None:
    """The CPU arm: the CPU FP64 oracle (the reference has no CPU implementation of this path) as
    the fastest CPU configuration measured -- one single-threaded process per host core, each
    compiling the workload (independent circuits, as a request stream gives them).  One step is
    one compile on every core; W warm-up steps, then K timed."""
    if rank != 0:
        return
    import multiprocessing as mp
    text = workload_text()
    cores = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(cores, initializer=_oracle_init, initargs=(text,)) as pool:
        for _ in range(max(1, args.warmup)):
            pool.map(_oracle_one, range(cores), chunksize=1)
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            pool.map(_oracle_one, range(cores), chunksize=1)
            t.append(time.perf_counter() - t0)
    total = sum(t)
    v = cores * args.steps / total
    sample = (f"{args.steps} steps of one compile of the workload on each of {cores} single-threaded processes "
              f"(one per host core) after {max(1, args.warmup)} warm-up steps; the CPU FP64 oracle")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 bitsets, f64 probabilities",
            "data": "synthetic (generated circuit)", "config": config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(text: str, budget_s: float = 10.0) -> dict:
    """The oracle on the host cores: one single-threaded process per core (the headline figure:
    the fastest CPU configuration), all threads on one compile, and one thread."""
    import multiprocessing as mp
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    # processes are spawned, never forked after CUDA use
    with mp.get_context("spawn").Pool(threads) as pool:
        res = pool.map(_oracle_rate, [(text, budget_s / 2)] * threads)
    per_core = sum(k / t for k, t in res)
    O.time_compile(text, 2, threads)
    n, t0 = 0, time.perf_counter()
    while True:
        O.time_compile(text, 2, threads)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s / 4 or n >= 400:
            break
    n1, t1 = 0, time.perf_counter()
    while True:
        O.time_compile(text, 2, 1)
        n1 += 1
        el1 = time.perf_counter() - t1
        if el1 > budget_s / 4 or n1 >= 100:
            break
    return {"value": per_core, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sum(k for k, _ in res)} compiles of the workload, one single-threaded CPU FP64 oracle "
                      f"process per host core, {budget_s / 2:.1f} s each",
            "all_threads_one_compile": {"value": n / el, "unit": UNIT, "threads": threads,
                                        "sample": f"{n} compiles in {el:.1f} s"},
            "single_thread": {"value": n1 / el1, "unit": UNIT, "sample": f"{n1} compiles in {el1:.1f} s on one thread"}}


def dem_arrays_equal(a, b) -> bool:
    import numpy as np
    return (a.num_detectors == b.num_detectors and np.array_equal(a.offsets, b.offsets)
            and np.array_equal(a.targets, b.targets) and np.array_equal(a.probs, b.probs))


def batched_leg(gp, torch, local: int, flush, steps: int, warmup: int, circuits: int = 256, walk_queue: int = 0,
                device_only: bool = False) -> dict:
    """Mixed-size batch: one batched pipeline vs the plain per-circuit path on the same circuits.

    Device rates time only the kernel pipelines (CUDA events on the driver's
    stream, L2 flushed before each); e2e rates run host text to host arrays.
    ``device_only`` times the batched pipeline alone (for profiling);
    ``circuits`` takes the first circuits of the batch.
    """
    from greenpeas_gb300.workloads import batch_surface
    texts = batch_surface()[:circuits]
    n = len(texts)
    dev = torch.device("cuda", local)
    if device_only:
        # walk_queue: 1 persistent walk launch, -1 per-class launches, 0 the default
        bdrv = gp.get_driver(texts[0], device=local, walk_queue=walk_queue)
        bext = torch.cuda.ExternalStream(bdrv.stream, device=dev)
        bdrv.prepare_batch(texts)
        for _ in range(warmup):
            bdrv.run_device()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(bext):
            for i in range(steps):
                flush.fill_(float(i))
                ev[i][0].record(bext)
                bdrv.run_device()
                ev[i][1].record(bext)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        bdrv.fetch_batch()
        return {"circuits": n, "ms_per_batch": ms, "value": n / (ms / 1e3), "unit": UNIT, "device_only": True}
    # plain: one circuit per compile, the same driver reused
    plain = gp.get_driver(texts[0], device=local)
    ext = torch.cuda.ExternalStream(plain.stream, device=dev)
    singles = []
    plain_ms = 0.0
    for t in texts:
        plain.prepare(t)
        plain.run_device()  # warm
        plain.run_device()  # the second run of a launch shape captures it as a CUDA graph (host work)
        with torch.cuda.stream(ext):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            plain.run_device()
            e1.record(ext)
        e1.synchronize()
        plain_ms += e0.elapsed_time(e1)
        singles.append(plain.fetch())
    # plain end to end
    t0 = time.perf_counter()
    for t in texts:
        plain.compile(t)
    plain_e2e_s = time.perf_counter() - t0
    raw = sum(d.num_raw_mechanisms for d in singles)
    merged = sum(d.num_errors for d in singles)
    plain_fallbacks = plain.fallback_counts()
    del plain

    bdrv = gp.get_driver(texts[0], device=local)
    bext = torch.cuda.ExternalStream(bdrv.stream, device=dev)
    tuning = bdrv.autotune(texts, reps=2)  # walk configuration of this driver's batches (the DEMs do not depend on it)
    bdrv.prepare_batch(texts)
    for _ in range(warmup):
        bdrv.run_device()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(bext):
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(bext)
            bdrv.run_device()
            ev[i][1].record(bext)
    torch.cuda.synchronize()
    batch_ms = [a.elapsed_time(b) for a, b in ev]
    # stage times and algorithmic bytes of one batched run of the whole batch (L2 flushed first)
    bdrv.set_stage_timing(True)  # (events between the stages: in this run only)
    with torch.cuda.stream(bext):
        flush.fill_(0.5)
    bdrv.run_device()
    st = bdrv.last_timings()
    bdrv.set_stage_timing(False)
    tr = bdrv.last_traffic()
    outs = bdrv.fetch_batch()
    ok = len(outs) == n and all(dem_arrays_equal(a, b) for a, b in zip(outs, singles))
    if not ok:
        raise SystemExit("bench: batched DEMs differ from the plain per-circuit DEMs")
    e2e_outs = bdrv.compile_batch(texts)  # warm the end-to-end path
    if not all(dem_arrays_equal(a, b) for a, b in zip(e2e_outs, singles)):
        raise SystemExit("bench: end-to-end batched DEMs differ from the plain per-circuit DEMs")
    del e2e_outs
    h2d_b = d2h_b = 0
    t0 = time.perf_counter()
    e2e_steps = max(3, min(steps, 10))
    for _ in range(e2e_steps):
        bdrv.compile_batch(texts)
    batch_e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d_b, d2h_b = bdrv.last_io_bytes()
    bmean = sum(batch_ms) / len(batch_ms)
    peak, peak_kind = peaks()
    stages = {"walk": "walk", "key": "key", "sort": "bucket", "merge": "merge"}
    roof = {k: {"ms": st[k], "algorithmic_bytes": tr[v], "achieved": tr[v] / (st[k] / 1e3) / 1e9,
                "frac": tr[v] / (st[k] / 1e3) / 1e9 / peak} for k, v in stages.items()}
    plain_rate = n / (plain_ms / 1e3)
    batch_rate = n / (bmean / 1e3)
    return {
        "workload": "surface_batch256_seed0_d3-21_logp1e-4..1e-2_switch0.1",
        "circuits": n, "raw_mechanisms": raw, "merged_mechanisms": merged,
        "batched": {"value": batch_rate, "unit": UNIT, "ms_per_batch": bmean, "steps": steps,
                    "mechanisms_per_s": {"raw": batch_rate * raw / n, "merged": batch_rate * merged / n},
                    "e2e": {"value": n / batch_e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d_b,
                            "d2h_bytes_per_step": d2h_b}},
        "plain": {"value": plain_rate, "unit": UNIT, "ms_total": plain_ms,
                  "mechanisms_per_s": {"raw": plain_rate * raw / n, "merged": plain_rate * merged / n},
                  "e2e": {"value": n / plain_e2e_s, "unit": UNIT}},
        "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": peak_kind, "stages": roof,
                     "note": "walk bytes: each word's band of the tape (re-read from L2 across words) + snapshots"},
        "fallbacks": {"batched": bdrv.fallback_counts(), "plain": plain_fallbacks},
        "speedup_device": batch_rate / plain_rate,
        "speedup_e2e": plain_e2e_s / batch_e2e_s,
        "tuning": tuning,
        "bit_exact_vs_plain": ok,
    }


def plain_leg(gp, torch, local: int, flush, text: str, steps: int, warmup: int, e2e_steps: int) -> dict:
    """One circuit per compile.  Device rate: CUDA events around each run of the kernel pipeline
    on the driver's stream (tape resident in HBM, L2 flushed before each run, outside the
    events); e2e: host text to host DEM arrays through the C ABI, wall clock."""
    drv = gp.get_driver(text, device=local)
    ext = torch.cuda.ExternalStream(drv.stream, device=torch.device("cuda", local))
    ref_dem = drv.compile(text)  # also checks the run completes
    sizes = drv.last_sizes()
    drv.prepare(text)
    for _ in range(warmup):
        drv.run_device()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(ext):
        for i in range(steps):
            flush.fill_(float(i))  # evict the tape and scratch from L2 (not timed)
            ev[i][0].record(ext)
            drv.run_device()
            ev[i][1].record(ext)
    torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    # per-stage times: events between the stages, in runs of their own (the timed runs above
    # have none: an event node between two kernels of the captured graph costs microseconds)
    stage = {"walk": 0.0, "key": 0.0, "sort": 0.0, "merge": 0.0, "total": 0.0}
    nstage = min(20, steps)
    drv.set_stage_timing(True)
    drv.run_device()
    for i in range(nstage):
        with torch.cuda.stream(ext):
            flush.fill_(float(i))
        drv.run_device()
        t = drv.last_timings()
        for k in stage:
            stage[k] += t[k] / nstage
    drv.set_stage_timing(False)
    dem_dev = drv.fetch()
    traffic = drv.last_traffic()
    for _ in range(warmup):
        drv.compile(text)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dem = drv.compile(text)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    h2d, d2h = drv.last_io_bytes()
    host, nhost = {}, min(10, e2e_steps)
    for _ in range(nhost):  # host phases of a compile, after the timed loop
        drv.compile(text)
        for k, v in drv.last_host_timings().items():
            host[k] = host.get(k, 0.0) + v / nhost
    if dem_dev.canonical() != ref_dem.canonical() or dem.canonical() != ref_dem.canonical():
        raise SystemExit("bench: results changed between runs")
    return {"drv": drv, "step_ms": step_ms, "dev_ms": sum(step_ms), "stage": stage, "traffic": traffic,
            "sizes": sizes, "merged": ref_dem.num_errors, "e2e_s": e2e_s, "e2e_steps": e2e_steps, "h2d": h2d,
            "d2h": d2h, "walk_plan": drv.walk_segments(), "fallbacks": drv.fallback_counts(), "host_ms": host}


# The plain-method configurations beside the headline: surface d = 3 (3 rounds), [[72,12,6]]
# (6 rounds), [[288,12,18]] (18 rounds), uniform circuit-level noise p = 1e-3.
SWEEP = (("surface_d3_r3_uniform_p1e-3", lambda gp: gp.SurfaceCode(3).get_memory(3, 1e-3, noise="uniform")),
         ("bb_72_12_6_r6_uniform_p1e-3", lambda gp: gp.BBCode(6).get_memory(6, 1e-3, noise="uniform")),
         ("bb_288_12_18_r18_uniform_p1e-3", lambda gp: gp.BBCode(18).get_memory(18, 1e-3, noise="uniform")))
NOMINAL_HBM_GBS = 8000.0


def sweep_entry(r: dict) -> dict:
    peak, kind = peaks()
    n = len(r["step_ms"])
    v = n / (r["dev_ms"] / 1e3)
    walk_gbs = r["traffic"]["walk"] / (r["stage"]["walk"] / 1e3) / 1e9
    return {"value": v, "unit": UNIT, "ms_per_step": r["dev_ms"] / n,
            "e2e": {"value": r["e2e_steps"] / r["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "mechanisms_per_s": {"raw": v * r["sizes"]["raw"], "merged": v * r["merged"]},
            "raw_mechanisms": r["sizes"]["raw"], "merged_mechanisms": r["merged"], "words": r["sizes"]["words"],
            "epochs": r["sizes"]["epochs"], "stage_ms": r["stage"], "walk_segments": r["walk_plan"],
            "walk_roofline": {"algorithmic_bytes": r["traffic"]["walk"], "ms": r["stage"]["walk"],
                              "achieved": walk_gbs, "unit": "GB/s", "frac_of_measured": walk_gbs / peak,
                              "peak_measured": peak, "peak_source": kind,
                              "frac_of_nominal_8tbs": walk_gbs / NOMINAL_HBM_GBS},
            "fallbacks": r["fallbacks"]}


def _incremental_family(gp, local: int, texts: list, reps: int) -> dict:
    """One family compiled by a driver that lowers each circuit whole and by an incremental one."""
    out = {"circuits": len(texts)}
    for mode in (False, True):  # one host thread, lowering only
        lw = gp.Lowerer(2, incremental=mode)
        for t in texts[:4]:
            lw.lower(t)
        reused = segs = parsed = 0
        t0 = time.perf_counter()
        for t in texts:
            lw.lower(t)
            st = lw.stats
            reused += st["reused"]
            segs += st["segments"]
            parsed += st["parsed_bytes"]
        dt = time.perf_counter() - t0
        lw.close()
        out["lowering_" + ("incremental" if mode else "whole")] = {
            "ms_per_circuit": 1e3 * dt / len(texts), "segments_reused": reused / max(segs, 1),
            "text_parsed": parsed / sum(len(t) for t in texts), "threads": 1}
    # both drivers and both servers stay up and are timed in turn, twice each (whole, incremental,
    # incremental, whole), so that neither side sees only a cold or only a warm machine
    from greenpeas_gb300.serving import Server, replay
    dems, bt, st = {}, {False: [], True: []}, {False: [], True: []}
    drv = {m: gp.get_driver(texts[0], device=local, incremental=m) for m in (False, True)}
    for m in (False, True):
        drv[m].compile_batch(texts)  # warm: buffers sized, graphs captured, lowering state kept
    for order in ((False, True), (True, False)):
        for m in order:
            t0 = time.perf_counter()
            for _ in range(reps):
                dems[m] = drv[m].compile_batch(texts)
            bt[m].append((time.perf_counter() - t0) / reps)
    host = {m: drv[m].last_host_timings() for m in (False, True)}
    del drv
    # (the batches' DEMs hold page-locked result blocks: compared, then let go before serving)
    out["same_order"] = all(dem_arrays_equal(a, b) for a, b in zip(dems[False], dems[True]))
    out["same_dems"] = all(a.canonical() == b.canonical() for a, b in zip(dems[False][:8], dems[True][:8]))
    del dems
    # served as bursts of requests (4 workers x 16, 13 lowering threads: lowering bounds the server)
    srv = {m: Server(slots=4, max_batch=16, incremental=m) for m in (False, True)}
    try:
        for m in (False, True):
            replay(srv[m], [(0.0, t) for t in texts[:128]])  # warm: workers' buffers, page-locked blocks
        for order in ((False, True), (True, False)):
            for m in order:
                st[m].append(replay(srv[m], [(0.0, t) for _ in range(reps) for t in texts])["dems_per_s"])
    finally:
        for m in (False, True):
            srv[m].close()
    for m in (False, True):
        ms = 1e3 * sum(bt[m]) / len(bt[m])
        out["incremental" if m else "whole"] = {
            "batch_e2e": {"value": len(texts) / (ms / 1e3), "unit": UNIT, "ms_per_batch": ms,
                          "runs_ms": [1e3 * x for x in bt[m]]},
            "serve_burst": {"value": sum(st[m]) / len(st[m]), "unit": UNIT, "requests": reps * len(texts),
                            "runs": st[m]},
            "host_ms_last_batch": host[m]}
    out["speedup"] = {k: out["incremental"][k]["value"] / out["whole"][k]["value"] for k in ("batch_e2e", "serve_burst")}
    out["speedup"]["lowering"] = out["lowering_whole"]["ms_per_circuit"] / out["lowering_incremental"]["ms_per_circuit"]
    return out


def branches_leg(gp, local: int, n: int = 256, reps: int = 4) -> dict:
    """Incremental lowering on two families of one circuit (BB [[144,12,12]] r=12, ``workloads``):
    256 distinct basis-switch branches, and 256 noise what-if variants (one noise instruction's rate
    changed per variant).  Each is compiled end to end (host text in, DEM arrays out) in batches of
    256 and as bursts of 1,024 server requests, lowering each circuit whole and lowering it against
    the previous one of the same host thread; host lowering alone (one thread, ``Lowerer``) is
    timed beside them, with the share of time segments taken over and of text parsed again.  The
    DEMs of both batch drivers are compared."""
    from greenpeas_gb300.workloads import branches, noise_variants
    return {"basis_switch_branches": dict(workload="bb_144_12_12_r12_uniform_p1e-3, basis-switch branches (seed 5)",
                                          **_incremental_family(gp, local, branches(n), reps)),
            "noise_variants": dict(workload="bb_144_12_12_r12_uniform_p1e-3, one noise rate changed (seed 6)",
                                   **_incremental_family(gp, local, noise_variants(n), reps))}


def batch_workload_texts(circuits: int) -> list:
    from greenpeas_gb300.workloads import batch_surface
    return batch_surface()[:circuits]


def serving_leg(gp, requests: int, cap_requests: int, slots: int, max_batch: int, plain_every: int = 10,
                batch_texts=None, batch_plain_e2e=None) -> dict:
    """Continuous batching: capacity (a burst of requests queued at once), then a Poisson trace at 80% of it.

    Mix (seed 2): half rotated surface-code memory with d uniform in {5..25},
    half bivariate-bicycle memory drawn from [[72,12,6]], [[144,12,12]],
    [[288,12,18]], rounds = d, uniform noise with p log-uniform in [1e-4,
    1e-2]; 120 GiB device-memory admission budget.  Latency is submit ->
    result, host text to host DEM arrays."""
    from greenpeas_gb300.serving import Server, replay
    from greenpeas_gb300.workloads import ServingMix
    mix = ServingMix(seed=2)

    def materialise(reqs):  # request texts built before the timed replay (the harness is not measured)
        return [(t, f()) for t, f in reqs]

    cap_reqs = materialise(mix.requests(cap_requests, 0.0))
    on_batch = None
    with Server(slots=slots, max_batch=max_batch, hbm_budget=120 << 30) as srv:
        # warm every worker and the page-locked pool its tapes and results come from (not timed)
        replay(srv, materialise(mix.requests(8 * slots * max_batch, 0.0)))
        cap = replay(srv, cap_reqs)
        rate = 0.8 * cap["dems_per_s"]
        tr = replay(srv, materialise(mix.requests(requests, rate)))
        if batch_texts:
            # the mixed-size batch workload served as requests (repeated to a
            # burst of >= 1,024), against the plain path on the same circuits
            reps = max(1, -(-1024 // len(batch_texts)))
            bc = replay(srv, [(0.0, t) for _ in range(reps) for t in batch_texts])
            on_batch = {"requests": bc["requests"], "dems_per_s": bc["dems_per_s"],
                        "plain_e2e_dems_per_s": batch_plain_e2e,
                        "speedup_vs_plain_e2e": bc["dems_per_s"] / batch_plain_e2e if batch_plain_e2e else None}
        fallbacks = srv.fallback_counts()
    # the plain per-circuit path on the same mix: one driver, one circuit per
    # compile, over every `plain_every`-th request of the capacity burst (a
    # sample of the same size distribution)
    texts = [t for _, t in cap_reqs[::plain_every]]
    drv = gp.get_driver(texts[0])
    drv.compile(texts[0])
    t0 = time.perf_counter()
    for t in texts:
        drv.compile(t)
    plain = len(texts) / (time.perf_counter() - t0)
    return {
        "workload": "serving_mix_seed2_surface5-25_bb72-288_logp1e-4..1e-2", "slots": slots, "max_batch": max_batch,
        "hbm_budget_bytes": 120 << 30,
        "capacity": {"requests": cap["requests"], "dems_per_s": cap["dems_per_s"]},
        "trace": {"requests": tr["requests"], "offered_per_s": rate, "dems_per_s": tr["dems_per_s"],
                  "p50_ms": tr["p50_ms"], "p99_ms": tr["p99_ms"], "mean_ms": tr["mean_ms"], "max_ms": tr["max_ms"],
                  "batches": tr["stats"]["batches"], "budget_peak_bytes": tr["stats"]["budget_peak"]},
        "plain_e2e_dems_per_s": plain, "plain_sample": f"every {plain_every}th request of the capacity burst "
                                                          f"({len(texts)})",
        "speedup_capacity_vs_plain_e2e": cap["dems_per_s"] / plain,
        "on_batch_workload": on_batch,
        "fallbacks": fallbacks,
    }


def grad_leg(gp, torch, reps: int = 20, fd_entries: int = 16) -> dict:
    """Noise-rate gradients of the [[144,12,12]] memory (12 rounds): rates [num_ticks, 4] log-uniform in
    [5e-4, 2e-3] (seed 1), loss sum_k w_k log p_k with w_k ~ N(0,1) keyed by the canonical symptom."""
    import math
    import numpy as np
    from greenpeas_gb300 import noise as N
    from greenpeas_gb300.autograd import NoiseRateDEM
    tmpl = gp.BBCode(12).get_memory(12, 1e-3, noise="uniform")
    model = NoiseRateDEM(tmpl)
    rates = N.sample_rates(model.num_ticks, 5e-4, 2e-3, 1)
    noise = torch.tensor(rates, dtype=torch.float64, device="cuda", requires_grad=True)
    p = model(noise)
    dem = model.last_dem()
    w_np = N.symptom_weights(dem.offsets, dem.targets, seed=1)
    w = torch.tensor(w_np, device="cuda")
    fwd, bwd = [], []
    for _ in range(reps):
        noise.grad = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p = model(noise)
        loss = (w * torch.log(p)).sum()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss.backward()
        torch.cuda.synchronize()
        fwd.append(t1 - t0)
        bwd.append(time.perf_counter() - t1)
    g = noise.grad.detach().cpu().numpy()

    def L(r):
        with torch.no_grad():
            q = model(torch.tensor(r, dtype=torch.float64, device="cuda")).cpu().numpy()
        return math.fsum(w_np * np.log(q))

    rng = np.random.default_rng(1)
    live = np.argwhere(g != 0)
    worst = 0.0
    h = 1e-7
    for i, j in live[rng.choice(len(live), min(fd_entries, len(live)), replace=False)]:
        rp, rm = rates.copy(), rates.copy()
        rp[i, j] += h
        rm[i, j] -= h
        fd = (L(rp) - L(rm)) / (2 * h)
        worst = max(worst, abs(fd - g[i, j]) / abs(g[i, j]))
    fwd.sort()
    bwd.sort()
    return {"workload": "bb_144_12_12_r12_rates_seed1_logp5e-4..2e-3", "num_ticks": model.num_ticks,
            "merged_mechanisms": int(dem.num_errors), "forward_ms": 1e3 * fwd[len(fwd) // 2],
            "backward_ms": 1e3 * bwd[len(bwd) // 2], "fd_entries": int(min(fd_entries, len(live))), "fd_h": h,
            "fd_max_rel_err": worst, "dtype": "f64"}


def global_sort_leg(gp, torch, local: int, flush, args) -> dict:
    """One circuit compiled on the global merge path (every mechanism's key through the onesweep
    radix sort, merged from the snapshots: the path a bucket overflow or a symptom over 256
    targets takes), device-resident runs timed by CUDA events, L2 flushed before each."""
    make = {"bb18": lambda: gp.BBCode(18).get_memory(18, 1e-3, noise="uniform"),
            "s21": lambda: gp.SurfaceCode(21).get_memory(21, 1e-3, noise="uniform"),
            "s25": lambda: gp.SurfaceCode(25).get_memory(25, 1e-3, noise="uniform")}[args.global_sort]
    text = make()
    drv = gp.get_driver(text, device=local, global_sort=True)
    ref = drv.compile(text)
    ext = torch.cuda.ExternalStream(drv.stream, device=torch.device("cuda", local))
    drv.prepare(text)
    for _ in range(max(1, args.warmup)):
        drv.run_device()
    torch.cuda.synchronize()
    ms = []
    for i in range(max(1, args.steps)):
        with torch.cuda.stream(ext):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            drv.run_device()
            e1.record(ext)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    drv.set_stage_timing(True)
    drv.run_device()
    st = drv.last_timings()
    if drv.fetch() != ref:
        raise SystemExit("bench: global-path runs changed the DEM")
    sizes = drv.last_sizes()
    return {"circuit": args.global_sort, "raw_mechanisms": sizes["raw"], "merged": ref.num_errors,
            "ms_median": sorted(ms)[len(ms) // 2], "stage_ms": st}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the mixed-size batch leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the headline single-circuit leg (profiling)")
    ap.add_argument("--batch-device-only", action="store_true", help="batch leg: time the batched pipeline alone")
    ap.add_argument("--batch-circuits", type=int, default=256)
    ap.add_argument("--walk-queue", type=int, default=0, choices=(-1, 0, 1),
                    help="batch leg with --batch-device-only: 1 one persistent walk launch, -1 per-class launches")
    ap.add_argument("--global-sort", choices=("bb18", "s21", "s25"), default=None,
                    help="profiling: one circuit on the global (onesweep sort) merge path, timed alone")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-grad", action="store_true", help="skip the noise-rate gradient leg")
    ap.add_argument("--no-branches", action="store_true", help="skip the incremental-lowering leg")
    ap.add_argument("--no-sweep", action="store_true", help="skip the plain-method configuration sweep")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-batch", type=int, default=16)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.warmup < 3:
        args.warmup = 3

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import greenpeas_gb300 as gp

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    if args.global_sort:  # profiling runs: the global merge path (sort kernels) on one circuit
        if rank == 0:
            print(json.dumps({"profiling": True, "global_sort": global_sort_leg(gp, torch, local, flush, args)}), flush=True)
        return
    if args.no_plain:  # profiling runs: the batch leg alone
        out = {"profiling": True}
        if not args.no_batch:
            out["batch"] = batched_leg(gp, torch, local, flush, steps=max(3, min(args.steps, 10)), warmup=args.warmup,
                                       circuits=args.batch_circuits, walk_queue=args.walk_queue,
                                       device_only=args.batch_device_only)
        if not args.no_branches:
            try:
                out["branches"] = branches_leg(gp, local)
            except Exception as e:
                out["branches"] = {"error": f"{type(e).__name__}: {e}"}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return
    text = workload_text()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(local) as clocks:
        r = plain_leg(gp, torch, local, flush, text, args.steps, args.warmup, args.steps)
    barrier()
    dev_ms, e2e_s = r["dev_ms"], r["e2e_s"]
    if dist is not None:
        tt = torch.tensor([dev_ms, e2e_s], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dev_ms, e2e_s = float(tt[0]), float(tt[1])
    if rank != 0:
        dist.destroy_process_group()
        return
    stage, traffic, sizes = r["stage"], r["traffic"], r["sizes"]
    value = world * args.steps / (dev_ms / 1e3)
    e2e = world * args.steps / e2e_s
    ms_sorted = sorted(r["step_ms"])
    p50 = ms_sorted[len(ms_sorted) // 2]
    p99 = ms_sorted[min(len(ms_sorted) - 1, int(0.99 * len(ms_sorted)))]
    # roofline of the dominant stage (HBM-bound integer/bitset work)
    names = {"walk": "walk", "key": "key", "sort": "bucket", "merge": "merge"}
    dom = max(("walk", "key", "sort", "merge"), key=lambda k: stage[k])
    achieved = traffic[names[dom]] / (stage[dom] / 1e3) / 1e9
    peak, peak_kind = peaks()
    # Whole pipeline, two byte counts: the bytes this design's kernels must move
    # (sparse symptoms: snapshots and target lists), and the fixed formulas of a
    # dense-symptom pipeline (8w bytes per raw mechanism written and re-read,
    # 16-byte keys + 4-byte permutation through an 8-pass radix sort):
    # B = 8wM + 24M + T  +  2*8*20*M  +  28M + 8wM + C(8w + 8), T = tape bytes (the H2D).
    M, w, C = sizes["raw"], sizes["words"], r["merged"]
    dense = (8 * w * M + 24 * M + r["h2d"]) + 2 * 8 * 20 * M + (28 * M + 8 * w * M + C * (8 * w + 8))
    stored = sum(traffic.values())
    pipe_s = stage["total"] / 1e3
    pipeline = {"ms": stage["total"], "algorithmic_bytes_stored": stored, "achieved_stored": stored / pipe_s / 1e9,
                "algorithmic_bytes_dense": dense, "achieved_dense": dense / pipe_s / 1e9,
                "frac_dense": dense / pipe_s / 1e9 / peak}
    plan = r["walk_plan"]
    walk_launches = 2 if plan["segments"] else 1
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 bitsets, f64 probabilities", "data": "synthetic (generated circuit)",
        "config": config({"raw_mechanisms": sizes["raw"], "merged_mechanisms": C,
                          "qubits": sizes["qubits"], "words": sizes["words"], "epochs": sizes["epochs"],
                          "snapshot_points": sizes["points"]}),
        "mechanisms_per_s": {"raw": value * sizes["raw"], "merged": value * C},
        "latency_ms": {"p50": p50, "p99": p99, "e2e_mean": 1e3 * e2e_s / args.steps,
                       "e2e_host_phases": {k: round(v, 4) for k, v in r["host_ms"].items()}},
        "stage_ms": stage,
        "walk_segments": plan,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "frac_of_nominal_8tbs": achieved / NOMINAL_HBM_GBS,
                     "algorithmic_bytes": traffic[names[dom]],
                     "traffic": (WALK_DRAM_BYTES_PER_RUN if plan["segments"] else WALK_DRAM_BYTES_PLAIN)
                     if dom == "walk" else None,
                     "note": "latency-bound: word walks cut into time segments walked side by side",
                     "pipeline": pipeline},
        "fallbacks": r["fallbacks"],
        # key-block table, walk launch(es), keys, warp grouping, large-bucket grouping, scan, emit
        "gpu_launches": (KERNELS_PER_RUN - 1 + walk_launches) * args.steps,
        "clocks": clocks.summary(),
    }
    del r
    if world == 1 and not args.no_sweep:
        sweep = {}
        for name, make in SWEEP:
            sweep[name] = sweep_entry(plain_leg(gp, torch, local, flush, make(gp), min(args.steps, 30),
                                                args.warmup, min(args.steps, 20)))
        sweep["bb_144_12_12_r12_uniform_p1e-3"] = {"value": value, "e2e": line["e2e"],
                                                   "note": "the headline line above"}
        line["plain_sweep"] = sweep
    # the other forms and the CPU baseline are single-GPU measurements (a multi-GPU
    # run reports the replicated headline only)
    if not args.no_batch and world == 1:
        line["batch"] = batched_leg(gp, torch, local, flush, steps=max(3, min(args.steps, 10)),
                                    warmup=args.warmup, circuits=args.batch_circuits, walk_queue=args.walk_queue,
                                    device_only=args.batch_device_only)
    if not args.no_grad and world == 1:
        line["grad"] = grad_leg(gp, torch, fd_entries=64)
    if not args.no_serve and world == 1:
        # capacity from a burst long enough that filling and draining the
        # pipeline is a small part of it (1,000 requests: ~0.2 s, 5-15% low)
        bl = line.get("batch") or {}
        line["serve"] = serving_leg(gp, args.serve_requests, max(200, min(3000, args.serve_requests // 3)),
                                    args.serve_slots, args.serve_batch,
                                    batch_texts=batch_workload_texts(args.batch_circuits) if bl.get("plain") else None,
                                    batch_plain_e2e=bl.get("plain", {}).get("e2e", {}).get("value"))
    if not args.no_branches and world == 1:  # (after serving: its page-locked blocks are of other sizes)
        try:
            line["branches"] = branches_leg(gp, local)
        except Exception as e:  # an auxiliary leg: its failure is reported in the line, not fatal to it
            line["branches"] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(text)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
