/* semb_gb300.h - C ABI of the GB300 CMP/CRS semblance search and stack.
 *
 * The reference (cuplgb/IPDPS-CRS-CMP-code) has no library: each of its programs
 * is one main() that reads an SU file, searches, and writes SU files.  This ABI
 * exposes the same path as four steps a foreign-function caller can bind with
 * plain pointers and sizes:
 *
 *   ingest   semb_survey_load / semb_survey_view      <- su_gather + linearize
 *   setup    semb_plan_create / semb_plan_upload      <- parameter grid, per-trace
 *                                                        geometry, neighbour lists
 *   search   semb_plan_run                            <- per-CDP semblance loop,
 *                                                        argmax and stack
 *   output   semb_plan_download / semb_survey_write   <- result arrays, SU writer
 *
 * Conventions: every function returns an int status (SEMB_OK = 0) instead of
 * exiting the process as the reference's LOG(FAIL) does (CMP/OpenMP/src/log.cpp:
 * 44-46); semb_last_error() gives a message for the calling thread.  Host buffers
 * belong to the caller.  A plan owns its device memory and one CUDA stream; plans
 * are not shared between threads.  Nothing here falls back to the CPU: without a
 * usable GPU, semb_plan_create fails with SEMB_E_NODEV.
 *
 * libsemb_gb300_checked.so exports the same ABI with bounds-checked search kernels:
 * every item that reads a staged sample window is tested against the window the
 * planner staged for its trace, and a violation makes semb_plan_run return
 * SEMB_E_BOUNDS with the first offending CDP, t0 and trace in the message (the
 * production library clamps such an address to the buffer instead).
 */
#ifndef SEMB_GB300_H
#define SEMB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEMB_ABI_VERSION 9

/* Search-kernel variant slots of semb_plan_autotune / semb_plan_set_variant. */
#define SEMB_MAX_VARIANTS 34

/* Aperture buckets of a batched plan's work queue (semb_plan_buckets). */
#define SEMB_MAX_BUCKETS 4

/* Methods. */
enum { SEMB_CMP = 0, SEMB_CRS = 1 };

/* Search forms.
 *  SEMB_PLAIN_F32 : FP32 throughout, the reference's arithmetic order (no fused
 *                   multiply-add, IEEE sqrt/div); results match the reference's
 *                   single-precision OpenMP build.
 *  SEMB_BATCHED   : persistent kernel over an aperture-sorted work queue, traces
 *                   stored as FP16/BF16 with a per-trace FP32 scale (or FP32),
 *                   FP32 interpolation and sums with compensated energy sums,
 *                   top-4 candidates kept per (CDP, t0) and re-evaluated in FP64
 *                   where the best two are closer than `repick_gap`. */
enum { SEMB_PLAIN_F32 = 0, SEMB_BATCHED = 1 };
enum { SEMB_STORE_F32 = 0, SEMB_STORE_F16 = 1, SEMB_STORE_BF16 = 2 };
enum { SEMB_REPICK_OFF = 0, SEMB_REPICK_NEAR_TIES = 1, SEMB_REPICK_ALWAYS = 2 };
/* CRS midpoint displacement.  SEMB_DM_SIGNED has no counterpart in the reference,
 * whose CRS operator uses the unsigned distance |dm| (CRS/OpenMP/src/main.cpp:198-204):
 * dm = (mx - mx0) cos(azimuth) + (my - my0) sin(azimuth), dm^2 = dm * dm. */
enum { SEMB_DM_ABS = 0, SEMB_DM_SIGNED = 1 };

/* Status codes. */
enum {
  SEMB_OK = 0,
  SEMB_E_ARG = 1,       /* invalid argument or parameter */
  SEMB_E_IO = 2,        /* file could not be opened, read or written */
  SEMB_E_FORMAT = 3,    /* malformed SU data (truncated trace, mixed ns, ...) */
  SEMB_E_WINDOW = 4,    /* semblance window 2*tau/dt+1 above the method's maximum */
  SEMB_E_NOMEM = 5,     /* host or device allocation failed */
  SEMB_E_CUDA = 6,      /* a CUDA call failed */
  SEMB_E_TIMEOUT = 7,   /* a bounded device-side wait gave up */
  SEMB_E_STATE = 8,     /* call out of order (e.g. run before upload) */
  SEMB_E_NODEV = 9,     /* no usable CUDA device */
  SEMB_E_BOUNDS = 10    /* checked build only: an item's sample window left the
                           window staged for its trace (see libsemb_gb300_checked) */
};

/* Search parameters, with the meaning of the reference's command-line flags
 * (CMP/OpenMP/src/main.cpp:57-74, CRS/OpenMP/src/main.cpp:67-98).  Numbers are the
 * values the reference's parser produces: for CMP the flags are read with stof,
 * so pass values already rounded to float; for CRS with stod.  c0/c1 are in s^2/m^2
 * (the library applies the reference's 1e6 scale); tau in seconds. */
typedef struct semb_params {
  int32_t method;        /* SEMB_CMP | SEMB_CRS */
  int32_t mode;          /* SEMB_PLAIN_F32 | SEMB_BATCHED */
  double a0, a1;         /* CRS only: -a0 -a1 */
  double b0, b1;         /* CRS only: -b0 -b1 */
  double c0, c1;         /* -c0 -c1 */
  int32_t na, nb, nc;    /* -na -nb (CRS only) -nc */
  int32_t aph;           /* -aph: half-offset aperture (m), applied at ingest */
  int32_t apm;           /* -apm: midpoint aperture (m), CRS only */
  int32_t storage;       /* SEMB_STORE_*, batched form only */
  double tau;            /* -tau: half window (s) */
  double azimuth;        /* -azimuth (deg), counterclockwise from +x.  With
                            dm_mode SEMB_DM_ABS (the reference's operator, which
                            never reads it) it has no effect. */
  int32_t repick;        /* SEMB_REPICK_*, batched form only */
  float repick_gap;      /* near-tie threshold on semblance (batched form) */
  int32_t dm_mode;       /* CRS midpoint displacement: SEMB_DM_ABS (|dm|, as the
                            reference) or SEMB_DM_SIGNED (dm projected on the
                            azimuth direction, so A sees its sign) */
  int32_t attrs;         /* batched form: 1 keeps the extra attribute outputs of
                            semb_plan_download_attrs (second-best candidate, FP64
                            error of the pick); 0 (default) does not */
  int32_t ngen;          /* CRS, plain form: > 0 runs CRS-DE (-ngen of the reference's
                            crs-ocl-de) instead of the grid search: differential
                            evolution of na*nb*nc individuals (<= 256) for ngen
                            generations; 0 (default) is the grid search */
} semb_params;

/* Fill `p` with the defaults for `method` (grid fields zero, batched FP16 with
 * near-tie re-pick at gap 1e-4).  Replaces nothing in the reference. */
void semb_params_init(semb_params* p, int32_t method);

/* A linearized gather: what su_gather::linearize hands to the search
 * (CRS/OpenMP/src/su_gather.cpp:94-127), with 64-bit counts.  Traces of one CDP
 * are contiguous; cdp_end[i] is the inclusive prefix count of traces up to CDP i
 * (the reference's ntraces_by_cdp_id).  Header integers are the raw SU fields. */
typedef struct semb_gather_view {
  int32_t ncdps;
  int32_t ns;            /* samples per trace */
  int32_t dt_us;         /* SU dt of the first trace of the first CDP (microseconds) */
  int32_t reserved;
  int64_t ntraces;
  const int64_t* cdp_end;    /* [ncdps] */
  const int32_t* cdp;        /* [ncdps] cdp header value of each CDP (may be NULL) */
  const int32_t* gx;         /* [ntraces] */
  const int32_t* gy;
  const int32_t* sx;
  const int32_t* sy;
  const int32_t* scalco;
  const float* samples;      /* [ntraces * ns], trace-major */
} semb_gather_view;

/* ---- ingest (host) ---------------------------------------------------------- */

typedef struct semb_survey semb_survey;

/* Read an SU file and group it as the reference does: traces whose half-offset
 * exceeds aph are dropped, traces are grouped by their cdp header in ascending
 * order, keeping file order inside a CDP (CRS/OpenMP/src/su_gather.cpp:33-65);
 * for SEMB_CMP the CDPs are then ordered by decreasing fold with the reference's
 * std::sort (CMP/OpenMP/src/su_gather.cpp:68).  Replaces su_gather::su_gather. */
int semb_survey_load(const char* path, int32_t method, int32_t aph, semb_survey** out);

/* Same, from SU bytes already in memory (headers and samples interleaved exactly
 * as in a file). */
int semb_survey_from_bytes(const void* su_bytes, int64_t nbytes, int32_t method, int32_t aph,
                           semb_survey** out);

/* Borrow the survey's linearized arrays (valid until semb_survey_free).
 * Replaces su_gather::linearize (CRS/OpenMP/src/su_gather.cpp:94-127). */
int semb_survey_view(const semb_survey* s, semb_gather_view* out);

/* Write the reference's output files into out_dir: cmp.{c,coher,stack}.su or
 * crs.{a,b,c,coher,stack}.su, one trace per CDP in the survey's CDP order, each
 * with a copy of the CDP's first trace header; in the parameter files (c, a, b)
 * offset is 0 and sx=gx, sy=gy hold the integer midpoint, in the coherence and
 * stack files the header is unchanged (CRS/OpenMP/src/main.cpp:331-359).  ctr/str/stk are
 * [ncdps * ns] as returned by semb_plan_download. */
int semb_survey_write(const semb_survey* s, const semb_params* p, const int32_t* ctr,
                      const float* str, const float* stk, const char* out_dir);

/* Write one extra attribute file out_dir/name: one trace per CDP in the survey's
 * CDP order with the CDP's first trace header unchanged (as the coherence file) and
 * the ns samples data[i * ns ...].  For the attribute grids of
 * semb_plan_download_attrs (e.g. "crs.coher2.su", "crs.err64.su"); an aperture map
 * is a per-CDP count spread over ns samples.  No counterpart in the reference. */
int semb_survey_write_attr(const semb_survey* s, const char* name, const float* data, const char* out_dir);

/* The CRS output files from explicit parameter values (CRS-DE): crs.{a,b,c,coher,
 * stack}.su as semb_survey_write writes them, with a/b/c [ncdps * ns] taken as given. */
int semb_survey_write_abc(const semb_survey* s, const float* a, const float* b, const float* c, const float* str,
                          const float* stk, const char* out_dir);

void semb_survey_free(semb_survey* s);

/* ---- search (device) -------------------------------------------------------- */

typedef struct semb_plan semb_plan;

/* Validate parameters and create a plan on CUDA device `device` (its own stream).
 * Replaces the set-up in main (CMP/OpenMP/src/main.cpp:67-110,
 * CRS/OpenMP/src/main.cpp:84-138) and the reference CUDA device wrapper
 * (CMP/CUDA/src/cuda.cpp:139-175). */
int semb_plan_create(const semb_params* p, int32_t device, semb_plan** out);

/* Copy a gather to the device and build everything the search reads: the FP32
 * (and, batched, FP16/BF16 + scale) trace store, per-trace half-offsets and
 * midpoints, the per-CDP neighbour lists within apm (CRS), the per-CDP aperture
 * index lists with |dm|, dm^2, h per entry, the candidate grid and the work queue.
 * Replaces CMP/OpenMP/src/main.cpp:118-143 and CRS/OpenMP/src/main.cpp:154-204,
 * 289-317 (and the reference CUDA kernels init_c, init_half, init_par, init_mid,
 * compute_points_for_gather: CMP/CUDA/src/main.cu:61-83, CRS/CUDA/src/main.cu:61-150).
 * Synchronous: on return the caller's buffers may be reused. */
int semb_plan_upload(semb_plan* plan, const semb_gather_view* g);

/* Search every CDP of the uploaded gather and keep, per (CDP, t0), the picked
 * candidate index, its semblance and its stack on the device.  Replaces the
 * per-CDP loop (CMP/OpenMP/src/main.cpp:146-236, CRS/OpenMP/src/main.cpp:207-320)
 * and the CUDA kernels compute_semblances + redux_semblances
 * (CMP/CUDA/src/main.cu:87-173, CRS/CUDA/src/main.cu:154-264).  Synchronous. */
int semb_plan_run(semb_plan* plan);

/* Upload and search in one call, streamed (batched grid search): the gather's CDPs
 * are cut into nchunks (1..64) contiguous chunks of about equal trace counts; the
 * traces of each chunk are copied to the device while the search of the chunks
 * whose apertures have landed runs, so the host-to-device transfer overlaps the
 * search.  Results as semb_plan_upload + semb_plan_run (same queue per chunk, longest
 * aperture first); the plan is then uploaded as by semb_plan_upload.  Synchronous;
 * the gather's memory must stay valid until it returns.  No counterpart in the
 * reference, which reads, copies and searches CDP by CDP. */
int semb_plan_stream(semb_plan* plan, const semb_gather_view* gather, int32_t nchunks);

/* Copy the results to host arrays of ncdps*ns elements, CDP-major in the gather's
 * CDP order: ctr = picked candidate index (CMP: -1 when no candidate has positive
 * semblance; CRS: linear index ia*nb*nc + ib*nc + ic), str = semblance, stk = stack.
 * These are the reference's ctr/str/stk arrays (CRS/OpenMP/src/main.cpp:126-128). */
int semb_plan_download(semb_plan* plan, int32_t* ctr, float* str, float* stk);

/* Extra attributes of the last run (any pointer may be NULL):
 *   sem2, idx2 [ncdps * ns]  second-best candidate: the best candidate other than the
 *                            pick, by single-precision semblance (0 and -1 where
 *                            there is none); batched form with attrs = 1
 *   err64 [ncdps * ns]       |single-precision semblance - FP64 semblance| of the
 *                            pick where the FP64 re-pick evaluated it, -1 elsewhere
 *                            (every (CDP, t0) with repick = SEMB_REPICK_ALWAYS);
 *                            batched form with attrs = 1
 *   aperture [ncdps]         aperture traces of each CDP (its fold for CMP); any form
 * SEMB_E_STATE when an attribute of the batched form is asked of a plan without it.
 * No counterpart in the reference. */
int semb_plan_download_attrs(semb_plan* plan, float* sem2, int32_t* idx2, float* err64, int32_t* aperture);

/* CRS-DE results of the last run: the picked A, B, C per (CDP, t0) (C in s^2/m^2);
 * semblance and stack come from semb_plan_download, whose ctr is -1 for CRS-DE (the
 * pick is not a grid index).  SEMB_E_STATE for a grid-search plan.  Replaces the
 * result arrays of crs-ocl-de (README.md:86-106). */
int semb_plan_download_abc(semb_plan* plan, float* a, float* b, float* c);

/* Copy the device-built neighbour lists (CRS): off[ncdps+1], list[off[ncdps]]
 * (pass list = NULL to query the size in *n_out).  The lists are those of
 * su_gather::su_gather (CRS/OpenMP/src/su_gather.cpp:70-87). */
int semb_plan_neighbours(semb_plan* plan, int32_t* off, int32_t* list, int64_t* n_out);

/* Neighbour lists with no device allocation.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc while they run: a pipeline whose device
 * memory belongs to another allocator (a framework's caching pool, buffers
 * registered with a communication library), or a real-time loop that forbids
 * allocation after start-up.  The caller passes device pointers: the first trace's
 * gx, gy, sx, sy and scalco of each of ncdps CDPs (inputs) and off[ncdps+1] and
 * list[capacity] (outputs, the same lists semb_plan_neighbours returns for a plan).
 * Scratch lives in one fixed array inside this library, 2.5 MB on every GPU that
 * loads it, kept until the process exits, so ncdps is limited to 131072 (larger is
 * SEMB_E_ARG).  The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current and keeps it for later calls, so
 * make that first call before any stream capture; a cudaDeviceReset voids the kept
 * address, and the entry point must not be used after one.  The call enqueues on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) and synchronizes it
 * to return the list length in *n_list; if that exceeds capacity the lists are
 * truncated and SEMB_E_ARG is returned (with *n_list set).  The search is all
 * pairs, 2 x ncdps^2 distance tests (count, then fill): about 3.4e10 at the limit.
 * All calls share the scratch: calls that overlap on the GPU (other threads, other
 * streams) race and must be serialized by the caller. */
int semb_neighbours_noalloc(const int32_t* gx, const int32_t* gy, const int32_t* sx, const int32_t* sy,
                            const int32_t* scalco, int32_t ncdps, int32_t apm, int32_t* off, int32_t* list,
                            int64_t capacity, int64_t* n_list, void* stream);

typedef struct semb_stats {
  double ms_search;       /* device time of the last run's semblance kernel(s);
                             0 when the run was a graph replay */
  double ms_repick;       /* device time of the last run's FP64 re-pick kernel;
                             0 when the run was a graph replay */
  double ms_total;        /* device time of the whole last run */
  double ms_upload;       /* device time of the last upload (copies + binning) */
  int64_t evals;          /* (CDP, t0, candidate) semblance evaluations per run */
  int64_t trace_evals;    /* evals x aperture traces (the reference's "semblance-traces") */
  int64_t repicked;       /* (CDP, t0) pairs re-evaluated in FP64 by the last run */
  int64_t kernel_launches;/* kernels launched by the last run */
  int32_t window;         /* w = 2*tau+1 */
  int32_t max_aperture;   /* largest aperture (traces) */
  int32_t ncdps, ns, ncand;
  int32_t grid_ctas;      /* CTAs of the main search launch */
  int32_t ctas_per_sm;    /* resident CTAs per SM of the main search kernel */
  int32_t sms;
  int32_t variant;        /* search-kernel variant in use (see semb_plan_autotune) */
} semb_stats;

int semb_plan_stats(const semb_plan* plan, semb_stats* out);

/* Time each variant of the search kernel available for this plan's window
 * (candidates per thread x CTA size x resident CTAs per SM x staging layout x
 * candidate layout) on a strided sample of the plan's own work queue and keep the fastest
 * for later runs.  *chosen gets the variant, ms_of_variant[0..SEMB_MAX_VARIANTS-1]
 * (optional) the
 * sample times (-1: no such variant).
 * No counterpart in the reference, which has one fixed launch shape
 * (CRS/CUDA/src/main.cu:45-51, 439). */
int semb_plan_autotune(semb_plan* plan, int32_t* chosen, double* ms_of_variant);

/* The aperture buckets of the plan's work queue: a batched plan splits its CDPs,
 * sorted by aperture size, at 1024, 384 and 128 aperture traces (merging buckets
 * too small to fill the GPU), and searches each bucket with its own launch and its
 * own kernel variant; semb_plan_autotune tunes each bucket on a sample of its own
 * tasks and merges neighbours that chose the same variant.  The plain form has one
 * bucket.  Arrays have SEMB_MAX_BUCKETS entries (any may be NULL): aperture range
 * [ap_lo, ap_hi], tasks (CDP x 32-sample t0 blocks) and variant of each bucket.
 * No counterpart in the reference. */
int semb_plan_buckets(const semb_plan* plan, int32_t* nbuckets, int32_t* ap_lo, int32_t* ap_hi,
                      int32_t* ntasks, int32_t* variant);

/* Use search-kernel variant `variant` (0..SEMB_MAX_VARIANTS-1) for later runs; SEMB_E_ARG when this
 * plan's window and form have no such variant.  No counterpart in the reference. */
int semb_plan_set_variant(semb_plan* plan, int32_t variant);

/* Batched form: stage at most max_samples window samples per chunk in shared memory
 * (0, the default: as much as the kernel variant's resident CTAs per SM leave).
 * Applies to the variants built with a global-memory path (16-18), whose stages may
 * be smaller than a trace (at least 512 samples by default): a trace whose window is
 * larger than the stage is read from the FP32 store in global memory instead, with
 * the staged path's arithmetic (with SEMB_STORE_F32 the results differ only by the
 * order of FP32 sums).  The other variants always stage whole windows.  Smaller
 * stages let more CTAs share an SM.  Takes effect at once on an uploaded plan.  No
 * counterpart in the reference. */
int semb_plan_set_staging(semb_plan* plan, int32_t max_samples);

/* Batched grid search in chunks of cdps_per_chunk contiguous CDPs (0, the default:
 * the whole survey at once).  semb_plan_run then searches the chunks one after the
 * other; each chunk's work (the CRS t0 = 0 stacks, one search launch per run of
 * aperture buckets on the same kernel variant, the FP64 re-pick of its samples) is
 * captured as a CUDA graph on the chunk's first run and replayed on later runs.
 * Results equal the unchunked run's.  No counterpart in the reference, which
 * searches CDP by CDP (CRS/CUDA/src/main.cu:420-450). */
int semb_plan_set_chunks(semb_plan* plan, int32_t cdps_per_chunk);

/* Device time of each chunk of the last chunked run: *nchunks gets the number of
 * chunks and ms[0..min(max, nchunks)-1] their milliseconds (0 chunks after an
 * unchunked run). */
int semb_plan_chunk_times(const semb_plan* plan, int32_t max, double* ms, int32_t* nchunks);

/* Capture the search (work-queue reset + kernels) in a CUDA graph and replay it on
 * later semb_plan_run calls (batched form).  on = 0 goes back to direct launches. */
int semb_plan_use_graph(semb_plan* plan, int32_t on);

int semb_plan_destroy(semb_plan* plan);

/* ---- helpers ---------------------------------------------------------------- */

/* Page-locked host memory for input/output buffers (cudaMallocHost). */
int semb_host_alloc(size_t bytes, void** out);
int semb_host_free(void* p);

/* Diagnostic with no counterpart in the reference: measured FP32 fused-multiply-
 * add throughput of `device` in TFLOP/s (2 flops per FMA), the denominator of the
 * search kernels' roofline, which are bound by FP32 issue rather than HBM. */
int semb_probe_fp32(int32_t device, double* tflops);

/* Diagnostic with no counterpart in the reference: runs the bounded barrier wait
 * the search kernels use for their bulk copies on a barrier that nothing
 * completes, with a limit of limit_us microseconds, and sets *timed_out to 1 when
 * the wait gave up (as it must) -- the failure path that turns a lost copy into
 * SEMB_E_TIMEOUT instead of a hung GPU, exercised without a fault. */
int semb_selftest_wait(int32_t device, int64_t limit_us, int32_t* timed_out);

/* Number of visible CUDA devices (0 when none); never fails. */
int32_t semb_device_count(void);

const char* semb_strerror(int code);
const char* semb_last_error(void);
int32_t semb_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SEMB_GB300_H */
