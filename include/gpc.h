/* gpc.h -- C ABI of the GB300 detector-error-model compiler.
 *
 * This is the drop-in boundary for GreenPeas' DEM-compilation path.  Each
 * entry point names the reference interface it replaces:
 *
 *   gpc_get_driver          <- greenpeas.get_driver(circuit, correlation_level)
 *                              (source/QEC/ErrorAnalysis/ErrorAnalysis.pybind.cu:72-78,
 *                               getDriver 26-41, Driver::fromStimCircuit
 *                               QEC/ErrorAnalysis/Driver.hpp:216-218)
 *   gpc_compile             <- Driver.compile_detector_error_model(circuit) and its
 *                              no-argument overload
 *                              (ErrorAnalysis.pybind.cu:56-70; Driver.hpp:199-211)
 *   gpc_dem_*               <- the stim::DetectorErrorModel the reference builds in
 *                              Driver::getDetectorErrorModel (Driver.hpp:166-194):
 *                              one error per merged symptom, target index
 *                              >= num_detectors is observable (index - num_detectors)
 *   gpc_driver_destroy      <- destruction of the pybind-owned Driver variant
 *
 * Circuits are passed as stim circuit text and DEMs come back as arrays (or
 * stim DEM text), so no C++ or Python object crosses the boundary.
 *
 * Conventions: every function returns a gpc_status (0 = success, < 0 =
 * error) and never throws; gpc_last_error() gives a thread-local message for
 * the most recent failure on the calling thread.  A driver owns one CUDA
 * stream and its device buffers; different drivers may be used from
 * different threads concurrently, one driver may not.  A driver's buffers
 * grow when a larger circuit is compiled (the reference throws instead).
 */
#ifndef GPC_H
#define GPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t gpc_status;

enum {
  GPC_OK = 0,
  GPC_ERR_INVALID = -1,     /* bad argument (null pointer, bad level, ...) */
  GPC_ERR_PARSE = -2,       /* circuit text does not parse */
  GPC_ERR_UNSUPPORTED = -3, /* instruction outside the supported gate set */
  GPC_ERR_CUDA = -4,        /* CUDA runtime error or no device */
  GPC_ERR_OOM = -5,         /* device or host allocation failed */
  GPC_ERR_COLLISION = -6,   /* two different symptoms share a 128-bit key */
  GPC_ERR_TIMEOUT = -7,     /* a bounded device wait gave up */
  GPC_ERR_CAPACITY = -8     /* a size limit of the library was exceeded */
};

/* Correlation levels, as greenpeas.CorrelationLevel (Mixer.hpp:13-20). */
enum { GPC_L0 = 0, GPC_L1 = 1, GPC_L2 = 2 };

typedef struct gpc_driver gpc_driver;
typedef struct gpc_dem gpc_dem;

typedef struct gpc_options {
  int32_t device;      /* CUDA device ordinal (default 0) */
  int32_t sort_bits;   /* global path only: key bits sorted before the merge (0 = 64) */
  int32_t global_sort; /* 1: always take the global sort path (tests); 0: buckets first */
  int32_t walk_qpt;    /* qubits per thread of the walk (1,2,3,4,6,8,12,16; 0 = chosen per circuit) */
  int32_t bucket_mean; /* target mechanisms per merge bucket (8..128; 0 = default) */
  int32_t walk_words;  /* detector words per walk CTA (1, 2; 0 = two in batches, one for a single circuit) */
  int32_t key_split;   /* one circuit: key the detector words beside the observables' walk (0 = when it pays, -1 = never) */
  int32_t walk_queue;  /* batches: 1 = one persistent walk launch (resident CTAs take (circuit, word group) items
                          from a queue, longest first), -1 = one launch per thread-count class,
                          0 = classes unless gpc_autotune chose the persistent launch */
  int32_t walk_segment; /* one circuit: cut the walk into time segments walked side by side, composed
                           through their GF(2) transfer maps (0 = when it pays, -1 = never, > 0 = always,
                           about this many cost units per segment: an epoch costs its slots + 2) */
  int32_t wait_limit_us; /* global path: a decoupled look-back wait gives up after this many microseconds
                            and the compile fails with GPC_ERR_TIMEOUT (0 = 200,000) */
  int32_t test_hold_tile; /* tests of the bounded waits: the next this-many global-path runs keep the
                             first radix tile's counts unpublished, so the waits after it run out
                             (0 = never) */
  int32_t test_fail_alloc; /* tests of the allocation failure path: the driver's k-th device allocation
                              (counting from its creation) fails once with GPC_ERR_OOM (0 = never) */
  int32_t heap_results;    /* 1: DEM arrays are heap copies out of a staging buffer; 0: the device copies
                              them into page-locked memory the DEM keeps (a single circuit's own arrays, a
                              batch's shared result block), while a 4 GiB page-locked pool reaches */
  int32_t incremental;     /* 1: in batches, each host thread lowers a circuit against the previous one it
                              lowered (branches of one circuit): only the statements that differ are parsed
                              again, and only the time segments they change are scheduled again (see
                              gpc_lowerer_create); the DEMs are the same.  A single circuit is still lowered
                              whole (on all host threads, which is faster for one circuit).  0: every
                              circuit is lowered whole */
} gpc_options;

/* Parses `stim_text` (length `len`), sizes device buffers for it and returns
 * a driver bound to `correlation_level`.  `options` may be NULL. */
gpc_status gpc_get_driver(const char *stim_text, size_t len, int32_t correlation_level,
                          const gpc_options *options, gpc_driver **out);

/* Compiles a circuit to a DEM.  With `stim_text` == NULL the driver's
 * current (last parsed) circuit is compiled again, like the reference's
 * no-argument overload.  The result is owned by the caller. */
gpc_status gpc_compile(gpc_driver *driver, const char *stim_text, size_t len, gpc_dem **out);

/* Compiles `n` circuits in one batched pipeline: the circuits are lowered on
 * host threads, uploaded with one copy, walked by one launch per thread-count
 * class (classes run concurrently), keyed, bucketed and merged by single
 * launches over the whole batch (buckets are numbered circuit by circuit, so
 * each circuit's output is contiguous).  outs[i] receives circuit i's DEM.
 * Batches whose merge needs a fallback are compiled circuit by circuit.  A
 * large batch (32 circuits and 8 MiB of text or more) runs as up to four
 * chunks alternating between the driver and a second pipeline it owns, so
 * one chunk's host work overlaps another's device work; the DEMs are the
 * same, and the driver's device arrays (gpc_device_dem) then hold one chunk
 * only -- gpc_prepare_batch + gpc_run_device give a whole batch's. */
gpc_status gpc_compile_batch(gpc_driver *driver, const char *const *texts, const size_t *lens,
                             int32_t n, gpc_dem **outs);

/* ---- autotuning (batched form) ------------------------------------------
 * Times the batched pipeline of circuits texts[0..n) (n >= 2) under each walk
 * configuration the kernels offer -- detector words per walk CTA (1, 2) x
 * qubits per walk thread (1, 2, 4; a choice that does not fit a circuit's
 * slot count falls back to the default for that circuit) x one launch per
 * thread-count class or one persistent launch (queue; only where the
 * largest circuit fits its block and shared memory) -- best of `reps` runs
 * each by CUDA events on the driver's stream, and keeps the fastest for the
 * driver's later batches (single circuits keep their defaults; explicit
 * walk_words / walk_qpt / walk_queue options take precedence).  The DEMs do
 * not depend on the choice.  On return the circuits are prepared in the
 * chosen configuration (gpc_run_device runs them). */
typedef struct gpc_tuning_entry {
  int32_t walk_words, walk_qpt, walk_queue;
  float ms; /* pipeline time, best of the repetitions */
} gpc_tuning_entry;
typedef struct gpc_tuning {
  int32_t walk_words, walk_qpt, walk_queue; /* the chosen configuration */
  float ms;
  int32_t num_tried;
  gpc_tuning_entry tried[12];
} gpc_tuning;
gpc_status gpc_autotune(gpc_driver *driver, const char *const *texts, const size_t *lens, int32_t n,
                        int32_t reps, gpc_tuning *out);

/* Merged mechanisms as CSR arrays owned by the DEM: error i has targets
 * targets[offsets[i] .. offsets[i+1]) (ascending) and probability probs[i]. */
gpc_status gpc_dem_arrays(const gpc_dem *dem, const uint32_t **offsets, const uint32_t **targets,
                          const double **probs, uint32_t *num_errors);

/* Circuit counts of the compiled DEM. */
gpc_status gpc_dem_info(const gpc_dem *dem, uint32_t *num_detectors, uint32_t *num_observables,
                        uint64_t *num_raw_mechanisms);

/* stim DEM text ("error(p) D0 D3 L0" lines); the buffer is owned by the DEM. */
gpc_status gpc_dem_text(const gpc_dem *dem, const char **text, size_t *len);

void gpc_dem_free(gpc_dem *dem);
void gpc_driver_destroy(gpc_driver *driver);

/* Thread-local message of the last failure on this thread ("" if none). */
const char *gpc_last_error(void);

/* ---- device-resident stages (benchmarking and serving) -------------------
 * gpc_prepare parses and uploads a circuit; gpc_run_device runs the kernel
 * pipeline on the uploaded tape with results left on the device;
 * gpc_fetch copies the last device result into a new DEM.  gpc_compile is
 * gpc_prepare + gpc_run_device + gpc_fetch. */
gpc_status gpc_prepare(gpc_driver *driver, const char *stim_text, size_t len);
gpc_status gpc_run_device(gpc_driver *driver);
gpc_status gpc_fetch(gpc_driver *driver, gpc_dem **out);
/* Batched forms of gpc_prepare / gpc_fetch (gpc_run_device runs either). */
gpc_status gpc_prepare_batch(gpc_driver *driver, const char *const *texts, const size_t *lens, int32_t n);
gpc_status gpc_fetch_batch(gpc_driver *driver, gpc_dem **outs, int32_t n);

/* ---- device-resident DEM for GPU consumers --------------------------------
 * Replaces the text round trip of Driver::getDetectorErrorModel
 * (Driver.hpp:166-194) for decoders on the same GPU: device pointers to
 * circuit `circuit`'s merged mechanisms of the last run (0 for a single
 * circuit; a batch index after gpc_prepare_batch + gpc_run_device), no copy.
 * probs[num_errors]; offsets[num_errors + 1] are positions in `targets` (the
 * run's whole target array), so error e has targets
 * targets[offsets[e] .. offsets[e+1]); *targets_end = offsets[num_errors].
 * Valid until the driver's next prepare, run or compile.  A batch that fell
 * back to circuit-by-circuit compiles has no device arrays
 * (GPC_ERR_UNSUPPORTED). */
gpc_status gpc_device_dem(gpc_driver *driver, int32_t circuit, const double **probs, const uint32_t **offsets,
                          const uint32_t **targets, uint32_t *num_errors, uint32_t *targets_end);

/* ---- noise-rate gradients (differentiation form) ------------------------
 * No counterpart in the reference (GreenPeas computes DEMs only).  A circuit
 * is prepared as a template: each noise instruction's rate is read from a
 * device FP64 tensor noise[num_ticks][4] instead of its text argument.  The
 * tick of an instruction is the number of TICKs before it; classes: 0
 * DEPOLARIZE2, 1 DEPOLARIZE1, 2 measurement flip (X/Y/Z_ERROR on a qubit
 * whose last operation was not a reset, or a measurement's flip argument),
 * 3 reset flip (X/Y/Z_ERROR on a qubit whose last operation was a reset).
 * The template's noise instructions need non-zero text arguments (a zero
 * rate creates no mechanisms); PAULI_CHANNEL_1 and E keep their text rates.
 * All pointers below are device pointers; `stream` is the caller's CUDA
 * stream (cudaStream_t): the driver's work is ordered after the caller's
 * prior work on it, and the caller's later work after the driver's.
 *   gpc_param_prepare  parse and upload the template; *num_ticks = TICKs + 1
 *   gpc_param_forward  merged mechanisms for noise[] (then gpc_fetch gives
 *                      the DEM: symptoms and probabilities, host arrays)
 *   gpc_param_probs    the merged probabilities of the last forward
 *                      (*num_errors of them, DEM order) into probs[]
 *   gpc_param_backward grad_noise[num_ticks * 4] = dL/dnoise from
 *                      grad_probs[*num_errors] = dL/dp of each merged
 *                      mechanism (FP64 adjoint of the XOR-merge and of the
 *                      channel splits; deterministic).  Returns after the
 *                      gradient is written. */
gpc_status gpc_param_prepare(gpc_driver *driver, const char *stim_text, size_t len, uint32_t *num_ticks);
gpc_status gpc_param_forward(gpc_driver *driver, const double *noise, void *stream, uint32_t *num_errors);
gpc_status gpc_param_probs(gpc_driver *driver, double *probs, void *stream);
gpc_status gpc_param_backward(gpc_driver *driver, const double *grad_probs, double *grad_noise, void *stream);

/* ---- serving: continuous batching of compile requests --------------------
 * No counterpart in the reference (its Driver compiles one circuit per call,
 * Driver.hpp:199-211).  Requests are lowered (parsed and scheduled into a
 * tape) on `lower_threads` host threads as they arrive.  A server owns
 * `slots` workers, each with a resident driver (stream + device buffers kept
 * between requests).  A free worker takes every lowered request up to
 * max_batch, admits the device
 * bytes its buffers must grow by against hbm_budget (waiting, after giving
 * back its own buffers, until enough is free; a request that alone exceeds
 * the budget fails with GPC_ERR_CAPACITY), and compiles them in one batched
 * pipeline.  Workers run concurrently, so batches overlap on the device.
 * Each DEM equals the one gpc_compile gives for the same circuit alone.
 *   gpc_server_submit  queue a circuit (thread-safe); returns a ticket
 *   gpc_server_wait    wait up to timeout_s for a ticket (GPC_ERR_TIMEOUT if
 *                      not done; the ticket stays valid); on completion the
 *                      ticket is consumed and *latency_s is submit -> done
 *   gpc_server_stats   requests completed, batches run, budget bytes held
 *                      now and at peak */
typedef struct gpc_server gpc_server;
typedef struct gpc_server_options {
  int32_t device;
  int32_t correlation_level; /* 0, 1, 2 */
  uint32_t slots;            /* workers (resident drivers), default 4 */
  uint32_t max_batch;        /* circuits per batch, default 16 */
  uint64_t hbm_budget;       /* device bytes all workers' buffers may hold, default 120 GiB */
  uint32_t lower_threads;    /* host threads lowering requests as they arrive (0 = the cores left after one per
                                slot, plus one: workers sleep while their batch runs) */
  uint32_t incremental;      /* 1: each lowering thread lowers a request against the previous one it lowered
                                (as gpc_options.incremental) */
  uint32_t reserved[2];
} gpc_server_options;
gpc_status gpc_server_create(const gpc_server_options *options, gpc_server **out);
gpc_status gpc_server_submit(gpc_server *server, const char *stim_text, size_t len, uint64_t *ticket);
gpc_status gpc_server_wait(gpc_server *server, uint64_t ticket, double timeout_s, gpc_dem **out, double *latency_s);
gpc_status gpc_server_stats(gpc_server *server, uint64_t *completed, uint64_t *batches, uint64_t *budget_used,
                            uint64_t *budget_peak);
/* Fallbacks taken by a server's workers, summed (as gpc_fallback_counts). */
gpc_status gpc_server_fallback_counts(gpc_server *server, uint64_t *counts5);
void gpc_server_destroy(gpc_server *server);

/* The driver's CUDA stream (a cudaStream_t), for callers that time it. */
void *gpc_driver_stream(gpc_driver *driver);

/* Stage timing (no counterpart in the reference): with `on` != 0 the
 * pipeline records CUDA events between its stages on the driver's stream
 * (off by default: in a captured graph each event node between two kernels
 * adds a few microseconds to the run). */
gpc_status gpc_set_stage_timing(gpc_driver *driver, int32_t on);

/* Kernel timing of the last gpc_run_device, in milliseconds (CUDA events on
 * the driver's stream): [0] walk, [1] key, [2] sort, [3] merge, [4] total.
 * GPC_ERR_INVALID unless stage timing was on for that run. */
gpc_status gpc_last_timings(gpc_driver *driver, float *ms5);

/* Host wall-clock phases of the driver's last prepare and fetch, in
 * milliseconds (no counterpart in the reference): [0] parse + lower (0 when
 * the prepared tapes were reused), [1] layout and device buffer growth, [2]
 * staging of the inputs into pinned memory, [3] waiting for the pipeline and
 * its result sizes, [4] device-to-host copies of the DEM arrays, [5] splitting
 * them into per-circuit DEMs.  After a gpc_compile_batch that ran in chunks,
 * each phase summed over the chunks. */
gpc_status gpc_last_host_timings(gpc_driver *driver, double *ms6);

/* Walk configuration of the driver's batches (no counterpart in the
 * reference): detector words per walk CTA, qubits per walk thread and the
 * persistent launch (0: the defaults).  gpc_autotune sets it and also keeps
 * it for the process, keyed by the bitset widths of the batch it tuned (the
 * set of its circuits' walk slot counts and word counts rounded up to a
 * power of two); a batch prepared on a driver without explicit walk options
 * that has not tuned itself takes the configuration kept for its widths. */
gpc_status gpc_walk_config(gpc_driver *driver, int32_t *words, int32_t *qpt, int32_t *queue);
/* Forgets every kept walk configuration. */
void gpc_tune_cache_clear(void);

/* Walk launches of the prepared circuits (no counterpart in the reference):
 * `launches` per run (one per thread-count class, or 1), `persistent` 1 when
 * the batch walks in one persistent launch off its work queue. */
gpc_status gpc_walk_form(gpc_driver *driver, int32_t *launches, int32_t *persistent);

/* How often this driver (and the second pipeline of its chunked batches)
 * left the fast path since it was created (no counterpart in the reference):
 * counts5[0] batches compiled circuit by circuit instead (a circuit needed
 * one of the fallbacks below), [1] runs merged through the global radix sort
 * (a symptom repeated more often than a bucket's 256 slots), [2] reruns with
 * wider target lists (a symptom longer than the list stride), [3] full
 * 128-bit re-sorts on the global path, [4] reruns of scan + emit after the
 * target buffer grew. */
gpc_status gpc_fallback_counts(gpc_driver *driver, uint64_t *counts5);

/* Device allocations and frees of this driver's own buffers since its
 * creation (no counterpart in the reference's API; its tests count the
 * allocations of a host storage policy, tests/Helpers/CountingStorage.hpp:9-51).
 * A driver compiling circuits no larger than the largest it has seen
 * allocates nothing. */
gpc_status gpc_alloc_counts(gpc_driver *driver, uint64_t *device_allocs, uint64_t *device_frees);

/* Segmented walk of the prepared single circuit (no counterpart in the
 * reference): `segments` the time segments its walk is cut into (0: not
 * segmented), `items_first` the CTAs of the first launch (first parts of the
 * words, their walks of later segments from zero rows, the transfer-matrix
 * columns) and `items_rest` those of the second (each later segment of a
 * word, from its composed entry rows). */
gpc_status gpc_walk_segments(gpc_driver *driver, uint32_t *segments, uint32_t *items_first,
                             uint32_t *items_rest);

/* Algorithmic bytes moved by each stage of the last run, counted from its
 * sizes: [0] walk (tape read + snapshots written), [1] key (records + snapshot
 * reads + keys, descriptors, target lists and bucket slots written), [2]
 * bucket grouping (slots read, lists compared, group records written), [3]
 * scan + emit (group records and head lists read, DEM written). */
gpc_status gpc_last_traffic(gpc_driver *driver, double *bytes4);

/* Bytes copied host -> device by the last gpc_prepare (the tape) and device ->
 * host by the last gpc_fetch (the DEM arrays and the result flags). */
gpc_status gpc_last_io_bytes(gpc_driver *driver, uint64_t *h2d, uint64_t *d2h);

/* Sizes of the last prepared circuit: raw mechanisms, snapshot points,
 * epochs, words per bitset, qubits. */
gpc_status gpc_last_sizes(gpc_driver *driver, uint64_t *raw, uint64_t *points, uint32_t *epochs,
                          uint32_t *words, uint32_t *qubits);

/* ---- merging without allocation -------------------------------------------
 * No counterpart in the reference: GreenPeas always allocates its workspaces
 * (Driver.hpp:69-76).  This entry point is for callers that cannot allocate
 * device memory -- for example code running while another runtime owns the
 * device's memory pool, or a decoder loop whose memory is reserved up front
 * and must not grow or synchronise the device in an allocation.
 *
 * Merges n raw error mechanisms into a DEM on `stream` (a cudaStream_t, NULL
 * for the default stream) on the current device.  All pointers are device
 * memory the caller owns:
 *   num_targets[n], targets[n * stride] (ascending target indices of
 *   mechanism i at targets[i*stride ...]; stride a multiple of 4 and
 *   targets 16-byte aligned), probs[n]  -- inputs;
 *   out_probs[n], out_offsets[n + 1], out_targets[out_target_cap]  -- the
 *   merged DEM, as gpc_dem_arrays; result[4] = {errors, targets, flags, 0},
 *   flags != 0 means the output is not valid (1 timeout, 2 hash collision,
 *   8 out_target_cap too small: nothing is written past it, 16 more than
 *   1024 mechanisms fell into one of the 1024 key buckets (for example one
 *   symptom repeated over 1024 times; that bucket's errors are missing),
 *   64 a target list is longer than stride (it is read cut to stride) or
 *   not ascending).
 * Empty symptoms are dropped; equal symptoms are merged with
 * p <- p1(1-p2) + p2(1-p1).
 *
 * It calls no allocator: all scratch lives in a static device array of about
 * 2.3 MiB that every GPU loading the library keeps until exit, which limits n
 * to 65,536 and n * stride to 2^32 - 1 (GPC_ERR_CAPACITY above either).
 * Every call on a device shares that array, so calls that overlap on the GPU
 * race: serialise them.  The
 * first call on each device looks up the array's device address (make it
 * before any stream capture).  Returns once the work is queued. */
gpc_status gpc_merge_mechanisms_static(const uint32_t *num_targets, const uint32_t *targets, uint32_t stride,
                                       const double *probs, uint32_t n, double *out_probs,
                                       uint32_t *out_offsets, uint32_t *out_targets, uint32_t out_target_cap,
                                       uint32_t *result, void *stream);

/* ---- tape inspection (host only, no GPU needed) ---------------------------
 * Lowers a circuit to the device tick tape without compiling it, for tools
 * and tests that check the lowering.  Arrays are owned by the tape. */
typedef struct gpc_tape gpc_tape;
typedef struct gpc_tape_view {
  uint32_t num_qubits, qpad, num_measurements, num_detectors, num_observables, words;
  uint32_t num_epochs, kmax, num_points, num_mechanisms, num_records;
  uint64_t num_ops;
  const uint64_t *ops;        /* epoch-major; epoch e is ep_k[e] slots x qpad ops */
  const uint32_t *ep_opoff;   /* [num_epochs] */
  const uint32_t *ep_k;       /* [num_epochs] */
  const uint32_t *ep_ptoff;   /* [num_epochs + 1] */
  const uint32_t *inj_lo;     /* [words] */
  const uint32_t *inj_hi;     /* [words] */
  const uint64_t *rec;        /* [num_records] noise records */
  const double *rec_p;        /* [num_records] */
  const uint32_t *rec_moff;   /* [num_records + 1] first mechanism of each record */
  const uint32_t *rec_src;    /* [num_records] tick * 4 + class, 0xFFFFFFFF: no source */
  uint32_t num_ticks;         /* TICK instructions + 1 */
} gpc_tape_view;

/* The tape a compile lowers the circuit to. */
gpc_status gpc_tape_lower(const char *stim_text, size_t len, int32_t correlation_level, gpc_tape **out);
gpc_status gpc_tape_get_view(const gpc_tape *tape, gpc_tape_view *view);
/* The epoch boundaries a single-circuit compile cuts its walk at, for a
 * segment cost of `target` (slots + 2 per epoch): bounds[0] = 0 < ... <
 * bounds[n-1] = num_epochs, written when n <= cap (GPC_ERR_CAPACITY
 * otherwise; n is always set). */
gpc_status gpc_tape_walk_segments(const gpc_tape *tape, uint32_t target, uint32_t *bounds, uint32_t cap,
                                  uint32_t *n);
void gpc_tape_free(gpc_tape *tape);
/* Thread-local message of the last gpc_tape_lower (or gpc_tape_lower_cuts,
 * gpc_lowerer_lower) failure. */
const char *gpc_tape_last_error(void);
/* The tape of a lowering whose backward pass is cut at `cuts` (instruction
 * indices of the flattened circuit, descending from its instruction count to
 * 0) instead of by its default segment size. */
gpc_status gpc_tape_lower_cuts(const char *stim_text, size_t len, int32_t correlation_level, const uint64_t *cuts,
                               uint32_t ncuts, gpc_tape **out);

/* Incremental lowering (no counterpart in the reference; host only).  A
 * lowerer keeps the last circuit it lowered.  With `incremental` != 0 it
 * lowers the next circuit against it: the statements between the two texts'
 * longest common prefix and suffix (whole top-level statements) are parsed
 * again and spliced between the kept ones; the backward pass keeps the
 * previous cuts outside that span, and a time segment over unchanged
 * statements is taken over, not scheduled again, when its measurements'
 * detector bits and its noise targets' sources equal the previous ones up
 * to one shift each (a span that adds rounds shifts the detectors and ticks
 * after it).  The tape equals gpc_tape_lower_cuts of the same text with the
 * same cuts, byte for byte.  A changed span over more than half of the text
 * is lowered whole.
 *   gpc_lowerer_lower  the tape of a circuit (owned by the caller), lowered on
 *                      the calling thread
 *   gpc_lowerer_stats  the last lowering: whether it was incremental, its
 *                      segments, those taken over, the text bytes parsed;
 *                      and its cuts (written when *ncuts <= cap)
 * A lowerer is used by one thread at a time; lowerers are independent. */
typedef struct gpc_lowerer gpc_lowerer;
typedef struct gpc_lower_stats {
  uint32_t incremental, segments, reused, reserved;
  uint64_t parsed_bytes;
} gpc_lower_stats;
gpc_status gpc_lowerer_create(int32_t correlation_level, int32_t incremental, gpc_lowerer **out);
gpc_status gpc_lowerer_lower(gpc_lowerer *lowerer, const char *stim_text, size_t len, gpc_tape **out);
gpc_status gpc_lowerer_stats(const gpc_lowerer *lowerer, gpc_lower_stats *stats, uint64_t *cuts, uint32_t cap,
                             uint32_t *ncuts);
void gpc_lowerer_free(gpc_lowerer *lowerer);

#ifdef __cplusplus
}
#endif

#endif /* GPC_H */
