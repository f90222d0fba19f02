// semb_plan: device state and the C ABI of the search (see include/semb_gb300.h).
//
// Device data layout (all in HBM, built once per upload):
//   samples    FP32 [ntraces][pitch], pitch = ns rounded up to 8 (16-byte rows)
//   samples16  FP16/BF16 [ntraces][pitch] + scale[ntraces]   (batched form)
//   ap_off     int64 [ncdps+1]; ap_tr int32, ap_geo float4 (|dm|, dm^2, h, -),
//              ap_geo64 (double |dm|, dm^2, h) per aperture entry
//   cand       float4 [npass*cpp]: candidates in search order (C-major for CRS)
//   tasks      int2 (cdp, t0_start), sorted by decreasing aperture
//   outputs    ctr/str/stk [ncdps][ns]; top-4 [ncdps][ns][4] (batched form)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "common.h"
#include "pipe_kernel.cuh"
#include "plan_kernels.cuh"
#include "semb_kernels.cuh"

namespace semb {

// Launchers of the search kernel instantiations (kernels_*.cu).
int launch_search(int method, int form, int w, int variant, const KParams& P, int nwarps, int grid, size_t smem,
                  cudaStream_t st);
int search_variant(int method, int form, int w, int variant, int* rc, int* minb, int* brun, int* nt, int* pipe,
                   int* lay, int* glob = nullptr, int* z0 = nullptr);
constexpr int kVariantSlots = SEMB_MAX_VARIANTS;
constexpr int kMaxBuckets = SEMB_MAX_BUCKETS;
// aperture split points of the work queue (traces): buckets > 1024, 385-1024,
// 129-384 and <= 128 aperture traces
constexpr int kBucketSplits = 3;
constexpr int kBucketAp[kBucketSplits] = {1024, 384, 128};
static_assert(kBucketSplits + 1 <= kMaxBuckets, "bucket table");
int search_occupancy(int method, int form, int w, int variant, int nwarps, size_t smem, int* ctas_per_sm);
int default_variant(int method, int form, int w, int nb);
int fallback_variant(int method, int form, int w, int nb);
int grid_neighbours(int ncdps, const float* d_fmx, const float* d_fmy, int apm, int64_t* d_off, int32_t** d_list,
                    int64_t* n_out, cudaStream_t st);
// CDP count from which the CRS neighbour lists come from the grid search
constexpr int kGridNeighbours = 2048;
// smallest automatic staging capacity of the batched form (samples per chunk)
constexpr int kMinStage = 512;
int launch_stt00(int w, int cdp0, int cdp1, const KParams& P, float a, float b, float c, float* out, cudaStream_t st);
int launch_repick(int w, const RepickParams& R, cudaStream_t st);
int launch_crs_de(int w, const DeParams& R, cudaStream_t st);

}  // namespace semb

using namespace semb;

namespace {

// One search-kernel configuration: a variant with its candidate table, per-pass
// parameter bounds, staging capacity, shared memory and residency.
struct KernelCfg {
  int variant = -1, rc = 0, minb = 0, nwarps = 0, cpp = 0, npass = 0, cap = 0, occ = 0;
  size_t smem = 0;
  float4* d_cand = nullptr;
  float* d_pass_bounds = nullptr;
  int2* d_pass_c = nullptr;   // Z0 variants: per pass its first C index and C-index count
};

// A contiguous range of the aperture-sorted work queue, searched by one launch
// with its own configuration.
struct Bucket {
  int begin = 0, end = 0;     // tasks [begin, end)
  int ap_lo = 0, ap_hi = 0;   // aperture traces of its CDPs
  int64_t work = 0;           // sum of aperture traces over its tasks
  KernelCfg cfg;
};

}  // namespace

struct semb_plan {
  semb_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;   // upload: the trace copy and store build
  cudaEvent_t copy_done = nullptr;
  int sms = 0;
  bool uploaded = false;

  int ncdps = 0, ns = 0, dt_us = 0;
  int64_t ntraces = 0, pitch = 0, nap = 0;
  float dt = 0.f, idt = 0.f;
  double dt64 = 0.0, idt64 = 0.0;
  int tau = 0, w = 1;
  int ncand = 0;
  int ntasks = 0, max_ap = 0;
  int64_t n_nbr = 0;
  float cand0_a = 0.f, cand0_b = 0.f, cand0_c = 0.f;
  // candidate grid kept on the host for re-configuration
  std::vector<float> ga, gb, gc;
  std::vector<double> g64;
  std::vector<int> order;

  // device buffers
  float* d_samples = nullptr;
  float* d_ingest = nullptr;   // staging of the linear trace copies (copy_traces)
  uint16_t* d_samples16 = nullptr;
  float* d_scale = nullptr;
  unsigned char* d_setup = nullptr;   // upload scratch arena (Scratch)
  int64_t* d_ap_off = nullptr;
  int2* d_z0r = nullptr;      // CRS: each CDP's own traces in its aperture list (first, count)
  float* d_cvals = nullptr;   // CRS: the C value of each C index in sample units
  int32_t* d_ap_tr = nullptr;
  float4* d_ap_geo = nullptr;
  Geo64* d_ap_geo64 = nullptr;
  int64_t* d_nbr_off = nullptr;
  int32_t* d_nbr = nullptr;
  double* d_cand64 = nullptr;
  int2* d_tasks = nullptr;
  int* d_counter = nullptr;   // work-queue heads, one per bucket
  // aperture buckets of the work queue (batched form; one bucket in the plain form)
  std::vector<Bucket> buckets;
  int32_t* d_ctr = nullptr;
  float* d_str = nullptr;
  float* d_stk = nullptr;
  float* d_stt00 = nullptr;
  float* d_top_sem = nullptr;
  int32_t* d_top_idx = nullptr;
  float* d_top_stk = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_repicked = nullptr;
  // extra attributes (batched form with attrs = 1)
  float* d_sem2 = nullptr;
  int32_t* d_idx2 = nullptr;
  float* d_err64 = nullptr;
  std::vector<int32_t> aperture;   // aperture traces per CDP (host copy)
  // CRS-DE (ngen > 0): the single-precision grid and the picked parameters
  float* d_grid = nullptr;
  float* d_de_a = nullptr;
  float* d_de_b = nullptr;
  float* d_de_c = nullptr;

  // streamed upload (semb_plan_stream): CDP chunks whose traces are copied while
  // the search of earlier chunks runs
  int nchunks = 0;
  std::vector<int> chunk_cdp;    // [nchunks+1] CDP boundaries
  std::vector<int> chunk_task;   // [nchunks+1] boundaries in the task queue
  std::vector<int> chunk_need;   // the last chunk whose traces chunk k's apertures read
  std::vector<cudaEvent_t> chunk_done;
  int* d_chunk_counter = nullptr;

  // bytes held by each buffer that a later upload of the same size reuses
  std::unordered_map<const void*, size_t> caps;

  cudaEvent_t ev[6] = {};
  bool use_graph = false;
  cudaGraphExec_t graph = nullptr;
  int stage_cap = 0;   // batched form: most staged samples per chunk (0: as shared memory allows)
  // chunked runs (semb_plan_set_chunks): contiguous CDP chunks searched one after the
  // other, each chunk's work (CRS t0 = 0 stacks, search launches per aperture bucket,
  // FP64 re-pick) captured once as a CUDA graph and replayed on later runs
  struct RunChunk {
    int cdp0 = 0, cdp1 = 0;
    std::vector<int> bucket_begin;   // [nbuckets + 1] task ranges in d_chunk_tasks
    cudaGraphExec_t graph = nullptr;
  };
  int chunk_cdps = 0;
  bool chunks_dirty = true;
  std::vector<RunChunk> run_chunks;
  int2* d_chunk_tasks = nullptr;
  std::vector<cudaEvent_t> chunk_ev;
  std::vector<double> chunk_ms;
  semb_stats stats{};
};

namespace {

template <typename T>
int dev_alloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (e != cudaSuccess)
    return fail(SEMB_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
  return SEMB_OK;
}

// Set-up scratch of an upload: consecutive 256-byte-aligned arrays carved from one
// device arena that the plan keeps for the next upload (no allocation or free, and so
// no device-wide synchronisation, when the survey's size repeats).
constexpr size_t scratch_bytes(size_t bytes) { return ((bytes > 0 ? bytes : 1) + 255) & ~(size_t)255; }

struct Scratch {
  unsigned char* base = nullptr;
  size_t used = 0, cap = 0;
  template <typename T>
  int alloc(T** p, size_t n) {
    const size_t b = scratch_bytes(n * sizeof(T));
    if (used + b > cap) return fail(SEMB_E_ARG, "upload scratch of %zu bytes exceeded", cap);
    *p = reinterpret_cast<T*>(base + used);
    used += b;
    return SEMB_OK;
  }
};

template <typename T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

void free_cfg(KernelCfg& c) {
  dev_free(c.d_cand);
  dev_free(c.d_pass_bounds);
  dev_free(c.d_pass_c);
  c.variant = -1;
}

void drop_graph(semb_plan* pl) {
  if (pl->graph) cudaGraphExecDestroy(pl->graph);
  pl->graph = nullptr;
  for (auto& c : pl->run_chunks)
    if (c.graph) cudaGraphExecDestroy(c.graph);
  pl->run_chunks.clear();
  pl->chunks_dirty = true;
}

// Device buffer *p of n elements, kept from the previous upload when it is large
// enough (re-uploads of a survey of the same size then allocate nothing).
template <typename T>
int dev_reuse(semb_plan* pl, T** p, size_t n) {
  const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  auto it = pl->caps.find(p);
  if (*p && it != pl->caps.end() && it->second >= bytes) return SEMB_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  pl->caps.erase(p);
  SEMB_TRY(dev_alloc(p, n));
  pl->caps[p] = bytes;
  return SEMB_OK;
}

// Free the plan's data; with keep_reusable the buffers dev_reuse manages stay.
void free_data(semb_plan* pl, bool keep_reusable = false) {
  auto release = [&](auto& ptr) {
    if (keep_reusable && pl->caps.count(&ptr)) return;
    pl->caps.erase(&ptr);
    dev_free(ptr);
  };
  release(pl->d_samples);
  release(pl->d_ingest);
  release(pl->d_samples16);
  release(pl->d_scale);
  release(pl->d_setup);
  release(pl->d_ap_off);
  release(pl->d_z0r);
  release(pl->d_cvals);
  release(pl->d_ap_tr);
  release(pl->d_ap_geo);
  release(pl->d_ap_geo64);
  release(pl->d_nbr_off);
  release(pl->d_nbr);
  for (Bucket& b : pl->buckets) free_cfg(b.cfg);
  pl->buckets.clear();
  release(pl->d_cand64);
  release(pl->d_tasks);
  release(pl->d_ctr);
  release(pl->d_str);
  release(pl->d_stk);
  release(pl->d_stt00);
  release(pl->d_top_sem);
  release(pl->d_top_idx);
  release(pl->d_top_stk);
  release(pl->d_sem2);
  release(pl->d_idx2);
  release(pl->d_err64);
  release(pl->d_grid);
  release(pl->d_de_a);
  release(pl->d_de_b);
  release(pl->d_de_c);
  drop_graph(pl);
  release(pl->d_chunk_tasks);
  pl->uploaded = false;
}

int check_params(const semb_params* p) {
  if (!p) return fail(SEMB_E_ARG, "null params");
  if (p->method != SEMB_CMP && p->method != SEMB_CRS) return fail(SEMB_E_ARG, "unknown method %d", p->method);
  if (p->mode != SEMB_PLAIN_F32 && p->mode != SEMB_BATCHED) return fail(SEMB_E_ARG, "unknown mode %d", p->mode);
  if (p->nc <= 0) return fail(SEMB_E_ARG, "nc must be positive");
  if (p->method == SEMB_CRS && (p->na <= 0 || p->nb <= 0)) return fail(SEMB_E_ARG, "na and nb must be positive");
  const int64_t ncand = p->method == SEMB_CMP ? (int64_t)p->nc : (int64_t)p->na * p->nb * p->nc;
  if (ncand > (1 << 24)) return fail(SEMB_E_ARG, "candidate grid of %lld is too large", (long long)ncand);
  if (p->storage < SEMB_STORE_F32 || p->storage > SEMB_STORE_BF16) return fail(SEMB_E_ARG, "unknown storage");
  if (p->repick < 0 || p->repick > 2) return fail(SEMB_E_ARG, "unknown repick mode");
  if (p->dm_mode != SEMB_DM_ABS && p->dm_mode != SEMB_DM_SIGNED) return fail(SEMB_E_ARG, "unknown dm_mode");
  if (p->attrs != 0 && p->attrs != 1) return fail(SEMB_E_ARG, "attrs must be 0 or 1");
  if (p->ngen < 0) return fail(SEMB_E_ARG, "ngen must be >= 0");
  if (p->ngen > 0 && (p->method != SEMB_CRS || p->mode != SEMB_PLAIN_F32))
    return fail(SEMB_E_ARG, "CRS-DE (ngen > 0) is a CRS search of the plain form");
  if (p->ngen > 0 && ncand > 256) return fail(SEMB_E_ARG, "CRS-DE population na*nb*nc = %lld above 256",
                                              (long long)ncand);
  if (!std::isfinite(p->azimuth)) return fail(SEMB_E_ARG, "azimuth must be finite");
  if (!(p->tau >= 0.0) || !std::isfinite(p->tau)) return fail(SEMB_E_ARG, "tau must be a non-negative number");
  return SEMB_OK;
}

// Reference parameter grids.  Single precision: the reference's float build
// (CMP/OpenMP/src/main.cpp:88,119-122; CRS/OpenMP/src/main.cpp:112-116,155-160
// with real = float); double precision: its double build.  `volatile` keeps each
// operation rounded on its own whatever the host compiler's contraction rules.
void grid_f32(const semb_params& p, std::vector<float>& a, std::vector<float>& b, std::vector<float>& c) {
  if (p.method == SEMB_CMP) {
    const int nc = p.nc;
    const float c0 = (float)(p.c0 * kFactor), c1 = (float)(p.c1 * kFactor);
    volatile float diff = c1 - c0;
    const float inc = diff * (1.0f / (float)nc);
    a.assign(nc, 0.f);
    b.assign(nc, 0.f);
    c.resize(nc);
    for (int i = 0; i < nc; ++i) {
      volatile float prod = inc * (float)i;
      c[i] = c0 + prod;
    }
  } else {
    const int na = p.na, nb = p.nb, nc = p.nc, n = na * nb * nc;
    const float a0 = (float)p.a0, a1 = (float)p.a1, b0 = (float)p.b0, b1 = (float)p.b1;
    const float c0 = (float)(p.c0 * kFactor), c1 = (float)(p.c1 * kFactor);
    volatile float da = a1 - a0, db = b1 - b0, dc = c1 - c0;
    const float inc_a = (float)((double)da * (1.0 / (double)(float)na));
    const float inc_b = (float)((double)db * (1.0 / (double)(float)nb));
    const float inc_c = (float)((double)dc * (1.0 / (double)(float)nc));
    a.resize(n);
    b.resize(n);
    c.resize(n);
    for (int i = 0; i < n; ++i) {
      volatile float pa = inc_a * (float)(i / (nc * nb));
      volatile float pb = inc_b * (float)((i / nc) % nb);
      volatile float pc = inc_c * (float)(i % nc);
      a[i] = a0 + pa;
      b[i] = b0 + pb;
      c[i] = c0 + pc;
    }
  }
}

void grid_f64(const semb_params& p, std::vector<double>& abc) {
  if (p.method == SEMB_CMP) {
    const int nc = p.nc;
    const double c0 = p.c0 * kFactor, c1 = p.c1 * kFactor;
    const double inc = (c1 - c0) * (1.0 / (double)nc);
    abc.assign(3 * (size_t)nc, 0.0);
    for (int i = 0; i < nc; ++i) {
      volatile double prod = inc * (double)i;
      abc[3 * i + 2] = c0 + prod;
    }
  } else {
    const int na = p.na, nb = p.nb, nc = p.nc, n = na * nb * nc;
    const double a0 = p.a0, b0 = p.b0, c0 = p.c0 * kFactor;
    const double inc_a = (p.a1 - a0) * (1.0 / (double)na);
    const double inc_b = (p.b1 - b0) * (1.0 / (double)nb);
    const double inc_c = (p.c1 * kFactor - c0) * (1.0 / (double)nc);
    abc.resize(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      volatile double pa = inc_a * (double)(i / (nc * nb));
      volatile double pb = inc_b * (double)((i / nc) % nb);
      volatile double pc = inc_c * (double)(i % nc);
      abc[3 * (size_t)i] = a0 + pa;
      abc[3 * (size_t)i + 1] = b0 + pb;
      abc[3 * (size_t)i + 2] = c0 + pc;
    }
  }
}

// Launch configuration of search-kernel variant v into `out`: candidates per pass
// (warps x RC), the search-order candidate table padded to whole passes, per-pass
// parameter bounds, the staging capacity (as large as the variant's resident CTAs
// per SM allow, never less than one whole trace), shared memory and occupancy.
// Whether the variant fits is checked before `out` changes.
int build_cfg(semb_plan* pl, int v, KernelCfg& out) {
  const semb_params& p = pl->p;
  const int form = p.mode == SEMB_PLAIN_F32 ? FORM_PLAIN : FORM_FAST;
  int rc = 0, minb = 0, brun = 0, nt = 0, pipe = 0, lay = 0, glob = 0, z0 = 0;
  if (!search_variant(p.method, form, pl->w, v, &rc, &minb, &brun, &nt, &pipe, &lay, &glob, &z0))
    return fail(SEMB_E_WINDOW, "no search kernel variant %d for w = %d", v, pl->w);
  if (lay == LAY_FT && pl->ns > kMaxNsFT)
    return fail(SEMB_E_ARG, "variant %d (pre-offset values) is for ns <= %d", v, kMaxNsFT);
  // LAY_X3 stages fixed planes: a whole trace and the zero block must fit one plane
  if (lay == LAY_X3 && (int64_t)pl->pitch + 16 > kXPlane - kZeroSlots)
    return fail(SEMB_E_ARG, "variant %d (sample and difference planes) is for ns <= %d", v,
                kXPlane - kZeroSlots - 24);
  const int ncand = pl->ncand;
  // search order; a negative slot -1-g marks padding that repeats candidate g.
  // B-run variants pad each (A, C) group's run of nb B values to a multiple of RC
  // so that every thread's RC candidates share A and C.
  std::vector<int> slots;
  if (brun && p.method == SEMB_CRS) {
    const int nbp = (p.nb + rc - 1) / rc * rc;
    slots.reserve((size_t)p.na * p.nc * nbp);
    for (int g0 = 0; g0 < ncand; g0 += p.nb)
      for (int k = 0; k < nbp; ++k) slots.push_back(k < p.nb ? pl->order[g0 + k] : -1 - pl->order[g0 + p.nb - 1]);
  } else {
    slots = pl->order;
  }
  const int nslots = (int)slots.size();
  // the most warps whose padding stays within 1% of the slots, else the least padding
  int best_nw = nt / 32, best_tot = INT32_MAX;
  for (int nw = nt / 32; nw >= 4; --nw) {
    const int per = nw * rc;
    const int tot = ((nslots + per - 1) / per) * per;
    if ((int64_t)tot * 100 <= (int64_t)nslots * 101) {
      best_tot = tot;
      best_nw = nw;
      break;
    }
    if (tot < best_tot) {
      best_tot = tot;
      best_nw = nw;
    }
  }
  const int cpp = best_nw * rc;
  const int npass = (nslots + cpp - 1) / cpp;
  // Z0 variants: each pass's C indices (C is outermost in the search order, so they are
  // consecutive); a pass may span at most kZ0C of them
  std::vector<int2> pass_c;
  if (z0) {
    if (p.method != SEMB_CRS || !pl->d_z0r || !pl->d_cvals)
      return fail(SEMB_E_ARG, "variant %d (shared central traces) is for CRS plans", v);
    for (int q = 0; q < npass; ++q) {
      int lo = INT32_MAX, hi = -1;
      for (int k = q * cpp; k < std::min(nslots, (q + 1) * cpp); ++k) {
        const int sv = slots[k];
        const int ic = (sv >= 0 ? sv : -1 - sv) % p.nc;
        lo = std::min(lo, ic);
        hi = std::max(hi, ic);
      }
      if (hi < lo) lo = hi = 0;
      if (hi - lo + 1 > kZ0C)
        return fail(SEMB_E_ARG, "variant %d (shared central traces): a pass spans %d C values (at most %d)", v,
                    hi - lo + 1, kZ0C);
      pass_c.push_back(make_int2(lo, hi - lo + 1));
    }
  }

  // staging capacity, shared memory and residency, checked before the plan's
  // device state changes (a variant that does not fit leaves the plan as it was)
  // Variants without the global path (glob = 0, every plain variant) stage whole
  // windows always (capacity >= one trace).  A batched variant with it reads a window
  // larger than its staging capacity from the FP32 store in global memory
  // (kGlobalEntry), so its stages need not hold a whole trace: the capacity is what
  // the variant's resident CTAs per SM leave, at least kMinStage samples (or the
  // plan's stage_cap, which also bounds it from above).
  const bool small_stages = form == FORM_FAST && glob;
  const int store = (form == FORM_FAST) ? p.storage : SEMB_STORE_F32;
  const size_t budget = (227 * 1024) / minb - 1024;
  int cap = form == FORM_PLAIN ? 32768 : 8192;
  if (form == FORM_FAST && pl->stage_cap > 0) cap = std::min(cap, pl->stage_cap);
  auto smem_of = [&](int cp) {
    return pipe ? pipe_layout(rc, cp, store, nt, lay, z0).total : smem_layout(form, rc, cp, store, nt, lay).total;
  };
  if (lay == LAY_X3) cap = std::min(cap, kXPlane - kZeroSlots);
  while (cap > 64 && smem_of(cap) > budget) cap -= 64;
  int min_cap = (int)pl->pitch + 16;
  if (small_stages) min_cap = std::min(min_cap, pl->stage_cap > 0 ? pl->stage_cap : kMinStage);
  if (cap < min_cap) cap = (min_cap + 63) & ~63;
  const size_t smem = smem_of(cap);
  if (smem > 227 * 1024) return fail(SEMB_E_ARG, "ns %d too large for the staging buffer", pl->ns);
  int occ = 0;
  SEMB_TRY(search_occupancy(p.method, form, pl->w, v, best_nw, smem, &occ));
  if (occ <= 0) return fail(SEMB_E_CUDA, "search kernel cannot be resident with %zu bytes", smem);

  const int npad = npass * cpp;
  std::vector<float4> cand(npad);
  std::vector<float> bounds((size_t)npass * 8, 0.f);
  const double s1 = pl->idt64, s2 = pl->idt64 * pl->idt64;
  for (int k = 0; k < npad; ++k) {
    // padding slots repeat a real candidate's parameters (so the pass bounds are
    // unchanged) with grid index -1: they are evaluated but never picked
    const int sv = slots[std::min(k, nslots - 1)];
    const bool pad = k >= nslots || sv < 0;
    const int gi = sv >= 0 ? sv : -1 - sv;
    float4 c;
    if (form == FORM_PLAIN) {
      c = make_float4(pl->ga[gi], pl->gb[gi], pl->gc[gi], 0.f);
    } else {
      c = make_float4((float)(pl->g64[3 * (size_t)gi] * s1), (float)(pl->g64[3 * (size_t)gi + 1] * s2),
                      (float)(pl->g64[3 * (size_t)gi + 2] * s2), 0.f);
    }
    int32_t gbits = pad ? -1 : gi;
    std::memcpy(&c.w, &gbits, 4);
    cand[k] = c;
    float* bp = &bounds[(size_t)(k / cpp) * 8];
    if (k % cpp == 0) {
      bp[0] = bp[1] = pl->ga[gi];
      bp[2] = bp[3] = pl->gb[gi];
      bp[4] = bp[5] = pl->gc[gi];
    } else {
      bp[0] = std::min(bp[0], pl->ga[gi]);
      bp[1] = std::max(bp[1], pl->ga[gi]);
      bp[2] = std::min(bp[2], pl->gb[gi]);
      bp[3] = std::max(bp[3], pl->gb[gi]);
      bp[4] = std::min(bp[4], pl->gc[gi]);
      bp[5] = std::max(bp[5], pl->gc[gi]);
    }
  }
  KernelCfg c;
  if (dev_alloc(&c.d_cand, npad) != SEMB_OK || dev_alloc(&c.d_pass_bounds, bounds.size()) != SEMB_OK ||
      (z0 && dev_alloc(&c.d_pass_c, pass_c.size()) != SEMB_OK)) {
    free_cfg(c);
    return fail(SEMB_E_NOMEM, "candidate table of %d entries", npad);
  }
  cudaError_t e = cudaMemcpyAsync(c.d_cand, cand.data(), npad * sizeof(float4), cudaMemcpyHostToDevice, pl->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c.d_pass_bounds, bounds.data(), bounds.size() * 4, cudaMemcpyHostToDevice, pl->stream);
  if (e == cudaSuccess && z0)
    e = cudaMemcpyAsync(c.d_pass_c, pass_c.data(), pass_c.size() * sizeof(int2), cudaMemcpyHostToDevice, pl->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(pl->stream);
  if (e != cudaSuccess) {
    free_cfg(c);
    SEMB_CUDA(e);
  }
  c.variant = v;
  c.rc = rc;
  c.minb = minb;
  c.nwarps = best_nw;
  c.cpp = cpp;
  c.npass = npass;
  c.cap = cap;
  c.smem = smem;
  c.occ = occ;
  free_cfg(out);
  out = c;
  drop_graph(pl);
  return SEMB_OK;
}

int bucket_grid(const semb_plan* pl, const Bucket& b) {
  const int n = b.end - b.begin;
  return pl->p.mode == SEMB_PLAIN_F32 ? n : std::min(n, pl->sms * b.cfg.occ);
}

// The bucket that holds most of the search work (its variant is the one reported).
const Bucket& main_bucket(const semb_plan* pl) {
  size_t best = 0;
  for (size_t i = 1; i < pl->buckets.size(); ++i)
    if (pl->buckets[i].work > pl->buckets[best].work) best = i;
  return pl->buckets[best];
}

void refresh_stats(semb_plan* pl) {
  const Bucket& b = main_bucket(pl);
  pl->stats.grid_ctas = bucket_grid(pl, b);
  pl->stats.ctas_per_sm = b.cfg.occ;
  pl->stats.variant = b.cfg.variant;
}

// Variant v for every bucket.  A variant fits all buckets or none (the fit depends
// on the plan's traces only), so a failure leaves the plan unchanged.
int set_all(semb_plan* pl, int v) {
  for (Bucket& b : pl->buckets) SEMB_TRY(build_cfg(pl, v, b.cfg));
  refresh_stats(pl);
  return SEMB_OK;
}

}  // namespace

extern "C" {

int32_t semb_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int semb_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(SEMB_E_ARG, "null argument");
  *out = nullptr;
  SEMB_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
  return SEMB_OK;
}

int semb_host_free(void* p) {
  if (p) SEMB_CUDA(cudaFreeHost(p));
  return SEMB_OK;
}

int semb_plan_create(const semb_params* p, int32_t device, semb_plan** out) {
  if (!out) return fail(SEMB_E_ARG, "null argument");
  *out = nullptr;
  SEMB_TRY(check_params(p));
  if (semb_device_count() <= device || device < 0)
    return fail(SEMB_E_NODEV, "CUDA device %d is not available", device);
  SEMB_CUDA(cudaSetDevice(device));
  semb_plan* pl = new (std::nothrow) semb_plan();
  if (!pl) return fail(SEMB_E_NOMEM, "out of host memory");
  pl->p = *p;
  pl->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pl->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->copy_done, cudaEventDisableTiming);
  for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&pl->ev[i]);
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_status, kStatusWords * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_counter, kMaxBuckets * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_repicked, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    semb_plan_destroy(pl);
    return fail(SEMB_E_CUDA, "plan set-up failed: %s", cudaGetErrorString(e));
  }
  if (prop.major < 10) {
    semb_plan_destroy(pl);
    return fail(SEMB_E_NODEV, "device %d is sm_%d%d; this library is built for sm_103a", device, prop.major,
                prop.minor);
  }
  pl->sms = prop.multiProcessorCount;
  *out = pl;
  return SEMB_OK;
}

int semb_plan_destroy(semb_plan* pl) {
  if (!pl) return SEMB_OK;
  cudaSetDevice(pl->device);
  if (pl->stream) cudaStreamSynchronize(pl->stream);
  free_data(pl);
  dev_free(pl->d_status);
  dev_free(pl->d_counter);
  dev_free(pl->d_repicked);
  for (auto& ev : pl->ev)
    if (ev) cudaEventDestroy(ev);
  if (pl->copy_stream) cudaStreamSynchronize(pl->copy_stream);
  for (cudaEvent_t e : pl->chunk_done) cudaEventDestroy(e);
  for (cudaEvent_t e : pl->chunk_ev) cudaEventDestroy(e);
  dev_free(pl->d_chunk_counter);
  if (pl->copy_done) cudaEventDestroy(pl->copy_done);
  if (pl->copy_stream) cudaStreamDestroy(pl->copy_stream);
  if (pl->stream) cudaStreamDestroy(pl->stream);
  delete pl;
  return SEMB_OK;
}

namespace {
int upload_impl(semb_plan* pl, const semb_gather_view* g, int nchunks);
int enqueue_streamed(semb_plan* pl, const semb_gather_view* g);
int enqueue_repick(semb_plan* pl, cudaStream_t st, int cdp0, int cdp1, bool reset_count);
}  // namespace

int semb_plan_upload(semb_plan* pl, const semb_gather_view* g) { return upload_impl(pl, g, 0); }

int semb_plan_stream(semb_plan* pl, const semb_gather_view* g, int32_t nchunks) {
  if (!pl || !g) return fail(SEMB_E_ARG, "null argument");
  if (pl->p.mode != SEMB_BATCHED || pl->p.ngen > 0)
    return fail(SEMB_E_ARG, "the streamed search is the batched form's grid search");
  if (nchunks < 1 || nchunks > 64) return fail(SEMB_E_ARG, "nchunks must be in 1..64");
  // the chunk copies, queued by the upload, read the caller's buffer until they end:
  // every exit waits for them
  struct CopyJoin {
    cudaStream_t s;
    ~CopyJoin() { cudaStreamSynchronize(s); }
  } join{pl->copy_stream};
  SEMB_TRY(upload_impl(pl, g, nchunks));
  return enqueue_streamed(pl, g);
}

}  // extern "C"

namespace {

// Traces [t0, t1) of the gather into the device stores on stream cs: linear copies of
// up to kIngestBytes of the caller's trace-major samples into a staging buffer (the
// copy engine's fastest form), each followed by k_ingest_rows, which lays the rows out
// at the plan's pitch with their zero padding and builds the 16-bit batched store.
constexpr int64_t kIngestBytes = (int64_t)1 << 30;

int copy_traces(semb_plan* pl, const semb_gather_view* g, int64_t t0, int64_t t1, cudaStream_t cs) {
  const int64_t n = t1 - t0;
  if (n <= 0) return SEMB_OK;
  const int64_t row_bytes = (int64_t)g->ns * (int64_t)sizeof(float);
  const int64_t per = std::max<int64_t>(1, kIngestBytes / row_bytes);
  // one size for every call of an upload (the streamed run copies chunk after chunk)
  SEMB_TRY(dev_reuse(pl, &pl->d_ingest, (size_t)std::min(pl->ntraces, per) * g->ns));
  const bool s16 = pl->p.mode == SEMB_BATCHED && pl->p.storage != SEMB_STORE_F32;
  for (int64_t r0 = t0; r0 < t1; r0 += per) {
    const int64_t r1 = std::min(t1, r0 + per);
    SEMB_CUDA(cudaMemcpyAsync(pl->d_ingest, g->samples + r0 * g->ns, (size_t)((r1 - r0) * row_bytes),
                              cudaMemcpyHostToDevice, cs));
    k_ingest_rows<<<(int)std::min<int64_t>(r1 - r0, 65535), 256, 0, cs>>>(
        r1 - r0, g->ns, pl->pitch, pl->p.storage, pl->d_ingest, pl->d_samples + r0 * pl->pitch,
        s16 ? pl->d_samples16 + r0 * pl->pitch : nullptr, s16 ? pl->d_scale + r0 : nullptr);
    SEMB_CUDA(cudaGetLastError());
  }
  return SEMB_OK;
}

// Streamed upload: the traces of CDP chunks k0 .. k1-1 (pl->chunk_cdp) into the device
// stores on stream cs, each chunk followed by its chunk_done event.
int copy_chunks(semb_plan* pl, const semb_gather_view* g, int k0, int k1, cudaStream_t cs) {
  for (int k = k0; k < k1; ++k) {
    const int c0 = pl->chunk_cdp[k], c1 = pl->chunk_cdp[k + 1];
    const int64_t t0 = c0 > 0 ? g->cdp_end[c0 - 1] : 0, t1 = c1 > 0 ? g->cdp_end[c1 - 1] : 0;
    SEMB_TRY(copy_traces(pl, g, t0, t1, cs));
    SEMB_CUDA(cudaEventRecord(pl->chunk_done[k], cs));
  }
  return SEMB_OK;
}

// streamed upload: chunks whose copies start before the set-up
constexpr int kEarlyChunks = 2;

int upload_impl(semb_plan* pl, const semb_gather_view* g, int nchunks) {
  if (!pl || !g) return fail(SEMB_E_ARG, "null argument");
  const semb_params& p = pl->p;
  if (g->ncdps <= 0 || g->ns <= 0 || g->ntraces <= 0 || !g->cdp_end || !g->gx || !g->gy || !g->sx || !g->sy ||
      !g->scalco || !g->samples)
    return fail(SEMB_E_ARG, "empty or incomplete gather");
  if (g->ns > 65535) return fail(SEMB_E_ARG, "ns %d exceeds the SU limit", g->ns);
  if (g->dt_us <= 0) return fail(SEMB_E_ARG, "dt must be positive");
  if (g->ntraces >= (int64_t)1 << 31) return fail(SEMB_E_ARG, "more than 2^31 traces");
  int64_t prev = 0;
  for (int i = 0; i < g->ncdps; ++i) {
    if (g->cdp_end[i] <= prev) return fail(SEMB_E_ARG, "CDP %d has no traces (cdp_end must increase)", i);
    prev = g->cdp_end[i];
  }
  if (prev != g->ntraces) return fail(SEMB_E_ARG, "cdp_end[ncdps-1] must equal ntraces");

  SEMB_CUDA(cudaSetDevice(pl->device));
  free_data(pl, true);
  cudaStream_t st = pl->stream;
  pl->ncdps = g->ncdps;
  pl->ns = g->ns;
  pl->dt_us = g->dt_us;
  pl->ntraces = g->ntraces;
  pl->pitch = ((g->ns + 7) & ~7) + 8;   // >= 8 zero samples after each trace

  // time sampling (CMP/OpenMP/src/main.cpp:107-110, CRS/OpenMP/src/main.cpp:135-138)
  {
    volatile float dt = (float)g->dt_us;
    dt = dt / 1000000.0f;
    const float idt = 1.0f / dt;
    const float itau = (float)p.tau;
    volatile float prod = itau * idt;
    const int tau = (int)prod > 0 ? (int)prod : 0;
    pl->dt = dt;
    pl->idt = idt;
    pl->tau = tau;
    pl->w = 2 * tau + 1;
    pl->dt64 = (double)g->dt_us / 1000000.0f;
    pl->idt64 = 1.0f / pl->dt64;
  }
  const int maxw = p.method == SEMB_CMP ? kMaxWCmp : kMaxWCrs;
  if (pl->w > maxw)
    return fail(SEMB_E_WINDOW, "semblance window w = %d exceeds the maximum %d of this method", pl->w, maxw);

  cudaEventRecord(pl->ev[4], st);
  // trace store
  const int64_t ntr = g->ntraces;
  // the traces go on the copy stream, overlapped with the geometry and aperture
  // set-up on the plan's stream: the pitched store (zero padding, rows copied by one
  // 2-D transfer) and, batched, the 16-bit store built from it on the device
  cudaStream_t cs = pl->copy_stream;
  struct CopyJoin {   // every exit waits for the copies, which read the caller's buffer
    cudaStream_t s;   // (streamed: semb_plan_stream waits for them after the search)
    ~CopyJoin() {
      if (s) cudaStreamSynchronize(s);
    }
  } copy_join{nchunks == 0 ? cs : nullptr};
  SEMB_CUDA(cudaStreamWaitEvent(cs, pl->ev[4], 0));
  SEMB_TRY(dev_reuse(pl, &pl->d_samples, (size_t)ntr * pl->pitch));
  if (p.mode == SEMB_BATCHED && p.storage != SEMB_STORE_F32) {
    SEMB_TRY(dev_reuse(pl, &pl->d_samples16, (size_t)ntr * pl->pitch));
    SEMB_TRY(dev_reuse(pl, &pl->d_scale, ntr));
  }
  if (nchunks == 0) SEMB_TRY(copy_traces(pl, g, 0, ntr, cs));
  SEMB_CUDA(cudaEventRecord(pl->copy_done, cs));
  pl->nchunks = nchunks;
  // header fields and CDP ranges (scratch for the set-up kernels)
  int32_t *d_gx, *d_gy, *d_sx, *d_sy, *d_sc;
  int64_t* d_cdp_end;
  float *d_h32, *d_mx32, *d_my32, *d_fmx, *d_fmy;
  double *d_h64, *d_mx64, *d_my64;
  int32_t* d_cnt32;
  int64_t* d_cnt64;
  Scratch scratch;
  {
    const size_t ncd = (size_t)g->ncdps, nt = (size_t)ntr;
    scratch.cap = 8 * scratch_bytes(nt * 4) + 3 * scratch_bytes(nt * 8) + 3 * scratch_bytes(ncd * 4) +
                  2 * scratch_bytes(ncd * 8);
    SEMB_TRY(dev_reuse(pl, &pl->d_setup, scratch.cap));
    scratch.base = pl->d_setup;
  }
  SEMB_TRY(scratch.alloc(&d_gx, ntr));
  SEMB_TRY(scratch.alloc(&d_gy, ntr));
  SEMB_TRY(scratch.alloc(&d_sx, ntr));
  SEMB_TRY(scratch.alloc(&d_sy, ntr));
  SEMB_TRY(scratch.alloc(&d_sc, ntr));
  SEMB_TRY(scratch.alloc(&d_cdp_end, g->ncdps));
  SEMB_TRY(scratch.alloc(&d_h32, ntr));
  SEMB_TRY(scratch.alloc(&d_mx32, ntr));
  SEMB_TRY(scratch.alloc(&d_my32, ntr));
  SEMB_TRY(scratch.alloc(&d_h64, ntr));
  SEMB_TRY(scratch.alloc(&d_mx64, ntr));
  SEMB_TRY(scratch.alloc(&d_my64, ntr));
  SEMB_TRY(scratch.alloc(&d_fmx, g->ncdps));
  SEMB_TRY(scratch.alloc(&d_fmy, g->ncdps));
  SEMB_TRY(scratch.alloc(&d_cnt32, g->ncdps));
  SEMB_TRY(scratch.alloc(&d_cnt64, g->ncdps));
  SEMB_CUDA(cudaMemcpyAsync(d_gx, g->gx, ntr * 4, cudaMemcpyHostToDevice, st));
  SEMB_CUDA(cudaMemcpyAsync(d_gy, g->gy, ntr * 4, cudaMemcpyHostToDevice, st));
  SEMB_CUDA(cudaMemcpyAsync(d_sx, g->sx, ntr * 4, cudaMemcpyHostToDevice, st));
  SEMB_CUDA(cudaMemcpyAsync(d_sy, g->sy, ntr * 4, cudaMemcpyHostToDevice, st));
  SEMB_CUDA(cudaMemcpyAsync(d_sc, g->scalco, ntr * 4, cudaMemcpyHostToDevice, st));
  SEMB_CUDA(cudaMemcpyAsync(d_cdp_end, g->cdp_end, g->ncdps * 8, cudaMemcpyHostToDevice, st));
  if (nchunks > 0) {
    // streamed: CDP chunks of about equal trace counts in gather order.  The first
    // chunks' copies are queued now, behind the header fields that the set-up needs
    // first, so that they run during the set-up below; the others at the end of the
    // set-up, after its own small copies, and during the search of the chunks before
    // them.  chunk_done[k] marks chunk k's traces in place.
    pl->chunk_cdp.assign(1, 0);
    for (int k = 1; k < nchunks; ++k) {
      const int64_t target = g->ntraces * k / nchunks;
      int c = pl->chunk_cdp.back();
      while (c < g->ncdps && g->cdp_end[c] <= target) ++c;
      pl->chunk_cdp.push_back(std::max(c, pl->chunk_cdp.back()));
    }
    pl->chunk_cdp.push_back(g->ncdps);
    while ((int)pl->chunk_done.size() < nchunks) {
      cudaEvent_t e;
      SEMB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      pl->chunk_done.push_back(e);
    }
    SEMB_TRY(copy_chunks(pl, g, 0, std::min(nchunks, kEarlyChunks), cs));
  }

  const int tgrid = (int)std::min<int64_t>((ntr + 255) / 256, 65535);
  k_trace_geometry<<<tgrid, 256, 0, st>>>(ntr, d_gx, d_gy, d_sx, d_sy, d_sc, d_h32, d_mx32, d_my32, d_h64, d_mx64,
                                          d_my64);
  SEMB_CUDA(cudaGetLastError());

  // neighbour lists: CRS from midpoints within apm, CMP the CDP itself
  const int nc_blocks = (g->ncdps + 255) / 256;
  SEMB_TRY(dev_reuse(pl, &pl->d_nbr_off, g->ncdps + 1));
  if (p.method == SEMB_CRS) {
    k_cdp_midpoints<<<nc_blocks, 256, 0, st>>>(g->ncdps, d_cdp_end, d_gx, d_gy, d_sx, d_sy, d_sc, d_fmx, d_fmy);
    if (g->ncdps >= kGridNeighbours) {
      // large surveys: grid cells + sorts, O(n log n); the same lists
      SEMB_TRY(grid_neighbours(g->ncdps, d_fmx, d_fmy, p.apm, pl->d_nbr_off, &pl->d_nbr, &pl->n_nbr, st));
    } else {
      const float lim = (float)((int32_t)p.apm * (int32_t)p.apm);
      k_neighbours<<<nc_blocks, 256, 0, st>>>(g->ncdps, d_fmx, d_fmy, lim, d_cnt32, nullptr, nullptr);
      k_scan_exclusive<int32_t><<<1, 1024, 0, st>>>(g->ncdps, d_cnt32, pl->d_nbr_off);
      SEMB_CUDA(cudaMemcpyAsync(&pl->n_nbr, pl->d_nbr_off + g->ncdps, 8, cudaMemcpyDeviceToHost, st));
      SEMB_CUDA(cudaStreamSynchronize(st));
      SEMB_TRY(dev_alloc(&pl->d_nbr, (size_t)pl->n_nbr));
      k_neighbours<<<nc_blocks, 256, 0, st>>>(g->ncdps, d_fmx, d_fmy, lim, nullptr, pl->d_nbr_off, pl->d_nbr);
    }
  } else {
    std::vector<int64_t> off(g->ncdps + 1);
    std::vector<int32_t> lst(g->ncdps);
    for (int i = 0; i <= g->ncdps; ++i) off[i] = i;
    std::iota(lst.begin(), lst.end(), 0);
    pl->n_nbr = g->ncdps;
    SEMB_TRY(dev_reuse(pl, &pl->d_nbr, g->ncdps));
    SEMB_CUDA(cudaMemcpyAsync(pl->d_nbr_off, off.data(), off.size() * 8, cudaMemcpyHostToDevice, st));
    SEMB_CUDA(cudaMemcpyAsync(pl->d_nbr, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice, st));
    SEMB_CUDA(cudaStreamSynchronize(st));
  }
  SEMB_CUDA(cudaGetLastError());

  // aperture lists
  SEMB_TRY(dev_reuse(pl, &pl->d_ap_off, g->ncdps + 1));
  k_aperture_count<<<nc_blocks, 256, 0, st>>>(g->ncdps, pl->d_nbr_off, pl->d_nbr, d_cdp_end, d_cnt64);
  k_scan_exclusive<int64_t><<<1, 1024, 0, st>>>(g->ncdps, d_cnt64, pl->d_ap_off);
  std::vector<int64_t> ap_off(g->ncdps + 1);
  SEMB_CUDA(cudaMemcpyAsync(ap_off.data(), pl->d_ap_off, ap_off.size() * 8, cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  pl->nap = ap_off[g->ncdps];
  SEMB_TRY(dev_reuse(pl, &pl->d_ap_tr, pl->nap));
  SEMB_TRY(dev_reuse(pl, &pl->d_ap_geo, pl->nap));
  SEMB_TRY(dev_reuse(pl, &pl->d_ap_geo64, pl->nap));
  // azimuth direction for the signed midpoint displacement (SEMB_DM_SIGNED)
  const double az = p.azimuth * 3.14159265358979323846 / 180.0;
  const double cos_d = std::cos(az), sin_d = std::sin(az);
  k_aperture_fill<<<(g->ncdps + 7) / 8, 256, 0, st>>>(g->ncdps, p.method, pl->d_nbr_off, pl->d_nbr, d_cdp_end,
                                                       pl->d_ap_off, d_h32, d_mx32, d_my32, d_h64, d_mx64, d_my64,
                                                       pl->d_ap_tr, pl->d_ap_geo, pl->d_ap_geo64,
                                                       p.dm_mode == SEMB_DM_SIGNED ? 1 : 0, (float)cos_d,
                                                       (float)sin_d, cos_d, sin_d);
  SEMB_CUDA(cudaGetLastError());
  if (p.method == SEMB_CRS) {
    SEMB_TRY(dev_reuse(pl, &pl->d_z0r, g->ncdps));
    k_central_range<<<nc_blocks, 256, 0, st>>>(g->ncdps, pl->d_nbr_off, pl->d_nbr, d_cdp_end, pl->d_z0r);
    SEMB_CUDA(cudaGetLastError());
  }
  int max_ap = 0;
  for (int i = 0; i < g->ncdps; ++i) max_ap = std::max<int64_t>(max_ap, ap_off[i + 1] - ap_off[i]);
  pl->max_ap = max_ap;

  // candidate grid and search order
  grid_f32(p, pl->ga, pl->gb, pl->gc);
  grid_f64(p, pl->g64);
  const int ncand = (int)pl->gc.size();
  pl->ncand = ncand;
  pl->cand0_a = pl->ga[0];
  pl->cand0_b = pl->gb[0];
  pl->cand0_c = pl->gc[0];
  pl->order.resize(ncand);
  if (p.method == SEMB_CMP) {
    std::iota(pl->order.begin(), pl->order.end(), 0);
  } else {
    // C outermost, then A, then B: a pass spans few C values, which dominate the
    // spread of traveltimes, so its staged windows stay narrow.
    int q = 0;
    for (int ic = 0; ic < p.nc; ++ic)
      for (int ia = 0; ia < p.na; ++ia)
        for (int ib = 0; ib < p.nb; ++ib) pl->order[q++] = ia * p.nb * p.nc + ib * p.nc + ic;
  }
  const int form = p.mode == SEMB_PLAIN_F32 ? FORM_PLAIN : FORM_FAST;
  SEMB_TRY(dev_reuse(pl, &pl->d_cand64, pl->g64.size()));
  SEMB_CUDA(cudaMemcpyAsync(pl->d_cand64, pl->g64.data(), pl->g64.size() * 8, cudaMemcpyHostToDevice, st));
  if (p.method == SEMB_CRS) {
    // the C value of C index ic in sample units, as the candidate table holds it (grid
    // index ic: A and B at their first values)
    std::vector<float> cv(p.nc);
    for (int ic = 0; ic < p.nc; ++ic) cv[ic] = (float)(pl->g64[3 * (size_t)ic + 2] * (pl->idt64 * pl->idt64));
    SEMB_TRY(dev_reuse(pl, &pl->d_cvals, cv.size()));
    SEMB_CUDA(cudaMemcpyAsync(pl->d_cvals, cv.data(), cv.size() * 4, cudaMemcpyHostToDevice, st));
    SEMB_CUDA(cudaStreamSynchronize(st));   // cv is a host temporary
  }

  // work queue: (cdp, t0 block), largest aperture first (longest-processing-time order)
  const int nblk = (g->ns + kTB - 1) / kTB;
  std::vector<int> cdp_order(g->ncdps);
  std::iota(cdp_order.begin(), cdp_order.end(), 0);
  std::stable_sort(cdp_order.begin(), cdp_order.end(), [&](int x, int y) {
    return ap_off[x + 1] - ap_off[x] > ap_off[y + 1] - ap_off[y];
  });
  const int64_t ntasks = (int64_t)g->ncdps * nblk;
  if (ntasks >= INT32_MAX) return fail(SEMB_E_ARG, "too many tasks");
  std::vector<int2> tasks((size_t)ntasks);
  size_t q = 0;
  if (nchunks == 0) {
    for (int c : cdp_order)
      for (int b = 0; b < nblk; ++b) tasks[q++] = make_int2(c, b * kTB);
  } else {
    // streamed: each chunk's tasks longest aperture first; chunk k's search waits for
    // the copies of the last chunk its apertures read (chunk_need)
    std::vector<int> chunk_of(g->ncdps);
    for (int k = 0; k < nchunks; ++k)
      for (int c = pl->chunk_cdp[k]; c < pl->chunk_cdp[k + 1]; ++c) chunk_of[c] = k;
    std::vector<int64_t> noff(g->ncdps + 1);
    std::vector<int32_t> nlist((size_t)std::max<int64_t>(pl->n_nbr, 1));
    SEMB_CUDA(cudaMemcpyAsync(noff.data(), pl->d_nbr_off, noff.size() * 8, cudaMemcpyDeviceToHost, st));
    SEMB_CUDA(cudaMemcpyAsync(nlist.data(), pl->d_nbr, (size_t)pl->n_nbr * 4, cudaMemcpyDeviceToHost, st));
    SEMB_CUDA(cudaStreamSynchronize(st));
    pl->chunk_need.assign(nchunks, 0);
    pl->chunk_task.assign(1, 0);
    for (int k = 0; k < nchunks; ++k) {
      int need = k;
      std::vector<int> cs_k;
      for (int c = pl->chunk_cdp[k]; c < pl->chunk_cdp[k + 1]; ++c) {
        cs_k.push_back(c);
        for (int64_t e = noff[c]; e < noff[c + 1]; ++e) need = std::max(need, chunk_of[nlist[e]]);
      }
      pl->chunk_need[k] = need;
      std::stable_sort(cs_k.begin(), cs_k.end(), [&](int x, int y) {
        return ap_off[x + 1] - ap_off[x] > ap_off[y + 1] - ap_off[y];
      });
      for (int c : cs_k)
        for (int b = 0; b < nblk; ++b) tasks[q++] = make_int2(c, b * kTB);
      pl->chunk_task.push_back((int)q);
    }
  }
  pl->ntasks = (int)ntasks;
  SEMB_TRY(dev_reuse(pl, &pl->d_tasks, tasks.size()));
  SEMB_CUDA(cudaMemcpyAsync(pl->d_tasks, tasks.data(), tasks.size() * sizeof(int2), cudaMemcpyHostToDevice, st));

  // aperture buckets (batched form): contiguous ranges of the sorted queue split at
  // kBucketAp traces, each with its own variant (neighbours on the same variant
  // share a launch); a bucket too small to fill the GPU a few times over joins its
  // larger neighbour
  {
    auto ap_of = [&](size_t t) { return (int)(ap_off[tasks[t].x + 1] - ap_off[tasks[t].x]); };
    std::vector<Bucket> bs;
    size_t t = 0;
    const size_t nt = tasks.size();
    const int nsplit = form == FORM_FAST && nchunks == 0 ? kBucketSplits : 0;
    for (int k = 0; k <= nsplit && t < nt; ++k) {
      const int lo = k < nsplit ? kBucketAp[k] : INT32_MIN;   // bucket k holds apertures > lo
      Bucket b;
      b.begin = (int)t;
      while (t < nt && ap_of(t) > lo) ++t;
      if (k == nsplit) t = nt;
      b.end = (int)t;
      if (b.end > b.begin) bs.push_back(b);
    }
    if (bs.empty()) bs.push_back(Bucket{});
    for (size_t i = 0; i + 1 < bs.size();) {
      const int small = std::max(1, pl->sms * 8);
      if (bs[i].end - bs[i].begin < small || bs[i + 1].end - bs[i + 1].begin < small) {
        bs[i].end = bs[i + 1].end;
        bs.erase(bs.begin() + (long)i + 1);
      } else {
        ++i;
      }
    }
    for (Bucket& b : bs) {
      b.ap_hi = b.end > b.begin ? ap_of(b.begin) : 0;
      b.ap_lo = b.end > b.begin ? ap_of(b.end - 1) : 0;
      for (int i = b.begin; i < b.end; ++i) b.work += ap_of(i);
    }
    pl->buckets = bs;
  }

  // outputs
  const size_t nout = (size_t)g->ncdps * g->ns;
  SEMB_TRY(dev_reuse(pl, &pl->d_ctr, nout));
  SEMB_TRY(dev_reuse(pl, &pl->d_str, nout));
  SEMB_TRY(dev_reuse(pl, &pl->d_stk, nout));
  SEMB_TRY(dev_reuse(pl, &pl->d_stt00, g->ncdps));
  SEMB_CUDA(cudaMemsetAsync(pl->d_stt00, 0, g->ncdps * sizeof(float), st));
  if (form == FORM_FAST) {
    SEMB_TRY(dev_reuse(pl, &pl->d_top_sem, nout * kTopK));
    SEMB_TRY(dev_reuse(pl, &pl->d_top_idx, nout * kTopK));
    SEMB_TRY(dev_reuse(pl, &pl->d_top_stk, nout * kTopK));
    if (p.attrs) {
      SEMB_TRY(dev_alloc(&pl->d_sem2, nout));
      SEMB_TRY(dev_alloc(&pl->d_idx2, nout));
      SEMB_TRY(dev_alloc(&pl->d_err64, nout));
    }
  }
  if (p.ngen > 0) {
    std::vector<float> grid(3 * (size_t)pl->ncand);
    for (int i = 0; i < pl->ncand; ++i) {
      grid[3 * (size_t)i] = pl->ga[i];
      grid[3 * (size_t)i + 1] = pl->gb[i];
      grid[3 * (size_t)i + 2] = pl->gc[i];
    }
    SEMB_TRY(dev_alloc(&pl->d_grid, grid.size()));
    SEMB_CUDA(cudaMemcpyAsync(pl->d_grid, grid.data(), grid.size() * 4, cudaMemcpyHostToDevice, st));
    SEMB_CUDA(cudaStreamSynchronize(st));
    SEMB_TRY(dev_alloc(&pl->d_de_a, nout));
    SEMB_TRY(dev_alloc(&pl->d_de_b, nout));
    SEMB_TRY(dev_alloc(&pl->d_de_c, nout));
  }
  pl->aperture.resize(g->ncdps);
  for (int i = 0; i < g->ncdps; ++i) pl->aperture[i] = (int32_t)(ap_off[i + 1] - ap_off[i]);

  // the default variant of this method and window; variant 0 where it does not fit
  if (set_all(pl, default_variant(p.method, form, pl->w, p.nb)) != SEMB_OK &&
      set_all(pl, fallback_variant(p.method, form, pl->w, p.nb)) != SEMB_OK)
    SEMB_TRY(set_all(pl, 0));
  // streamed: the other chunks' copies, after the set-up's own small copies
  if (nchunks > kEarlyChunks) SEMB_TRY(copy_chunks(pl, g, kEarlyChunks, nchunks, cs));
  SEMB_CUDA(cudaStreamWaitEvent(st, pl->copy_done, 0));   // the stores are complete for the run
  cudaEventRecord(pl->ev[5], st);
  SEMB_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, pl->ev[4], pl->ev[5]);

  std::memset(&pl->stats, 0, sizeof(pl->stats));
  pl->stats.ms_upload = ms;
  pl->stats.window = pl->w;
  pl->stats.max_aperture = pl->max_ap;
  pl->stats.ncdps = pl->ncdps;
  pl->stats.ns = pl->ns;
  pl->stats.ncand = pl->ncand;
  pl->stats.evals = (int64_t)pl->ncdps * pl->ns * pl->ncand;
  pl->stats.trace_evals = pl->nap * (int64_t)pl->ns * pl->ncand;
  refresh_stats(pl);
  pl->stats.sms = pl->sms;
  pl->uploaded = true;
  return SEMB_OK;
}

// Kernel parameters for configuration `cfg` over tasks[0, ntasks) with work-queue
// head `counter`.
KParams make_kparams_cfg(semb_plan* pl, const KernelCfg& cfg, const int2* tasks, int ntasks, int* counter) {
  KParams P{};
  P.samples = pl->d_samples;
  P.samples16 = pl->d_samples16;
  P.scale = pl->d_scale;
  P.pitch = pl->pitch;
  P.storage = (pl->p.mode == SEMB_BATCHED) ? pl->p.storage : SEMB_STORE_F32;
  P.ap_off = pl->d_ap_off;
  P.ap_tr = pl->d_ap_tr;
  P.ap_geo = pl->d_ap_geo;
  P.cand = cfg.d_cand;
  P.pass_bounds = cfg.d_pass_bounds;
  P.z0r = pl->d_z0r;
  P.cvals = pl->d_cvals;
  P.pass_c = cfg.d_pass_c;
  P.nc_grid = pl->p.nc;
  P.npass = cfg.npass;
  P.cpp = cfg.cpp;
  P.tasks = tasks;
  P.ntasks = ntasks;
  P.counter = counter;
  P.ns = pl->ns;
  P.tau = pl->tau;
  P.dt = pl->dt;
  P.idt = pl->idt;
  P.cap = cfg.cap;
  P.ctr = pl->d_ctr;
  P.str = pl->d_str;
  P.stk = pl->d_stk;
  P.stt00 = pl->d_stt00;
  P.top_sem = pl->d_top_sem;
  P.top_idx = pl->d_top_idx;
  P.top_stk = pl->d_top_stk;
  P.status = pl->d_status;
  return P;
}

KParams make_kparams(semb_plan* pl, int bucket) {
  const Bucket& b = pl->buckets[bucket];
  return make_kparams_cfg(pl, b.cfg, pl->d_tasks + b.begin, b.end - b.begin, pl->d_counter + bucket);
}

// Enqueue one whole search on the plan's stream (no synchronization).
int enqueue_run(semb_plan* pl, bool timed) {
  cudaStream_t st = pl->stream;
  const semb_params& p = pl->p;
  const int form = p.mode == SEMB_PLAIN_F32 ? FORM_PLAIN : FORM_FAST;
  KParams P = make_kparams(pl, 0);
  int launches = 0;
  if (timed) SEMB_CUDA(cudaEventRecord(pl->ev[0], st));
  if (pl->ns < 2 * pl->tau + 2) {
    // no trace can hold a whole window: every item is out of range
    SEMB_CUDA(cudaMemsetAsync(pl->d_str, 0, (size_t)pl->ncdps * pl->ns * 4, st));
    SEMB_CUDA(cudaMemsetAsync(pl->d_stk, 0, (size_t)pl->ncdps * pl->ns * 4, st));
    SEMB_CUDA(cudaMemsetAsync(pl->d_ctr, p.method == SEMB_CMP ? 0xff : 0, (size_t)pl->ncdps * pl->ns * 4, st));
    if (timed) {
      SEMB_CUDA(cudaEventRecord(pl->ev[1], st));
      SEMB_CUDA(cudaEventRecord(pl->ev[2], st));
      SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
    }
    pl->stats.kernel_launches = 0;
    return SEMB_OK;
  }
  if (p.method == SEMB_CRS) {
    SEMB_TRY(launch_stt00(pl->w, 0, pl->ncdps, P, pl->cand0_a, pl->cand0_b, pl->cand0_c, pl->d_stt00, st));
    ++launches;
  }
  if (p.ngen > 0) {
    // CRS-DE: differential evolution per (CDP, t0) instead of the grid search
    DeParams D{};
    D.samples = pl->d_samples;
    D.pitch = pl->pitch;
    D.ap_off = pl->d_ap_off;
    D.ap_tr = pl->d_ap_tr;
    D.ap_geo = pl->d_ap_geo;
    D.grid = pl->d_grid;
    D.lo[0] = (float)p.a0;
    D.lo[1] = (float)p.b0;
    D.lo[2] = (float)(p.c0 * kFactor);
    D.hi[0] = (float)p.a1;
    D.hi[1] = (float)p.b1;
    D.hi[2] = (float)(p.c1 * kFactor);
    D.np = pl->ncand;
    D.ngen = p.ngen;
    D.ncdps = pl->ncdps;
    D.ns = pl->ns;
    D.tau = pl->tau;
    D.dt = pl->dt;
    D.idt = pl->idt;
    D.stt00 = pl->d_stt00;
    D.a = pl->d_de_a;
    D.b = pl->d_de_b;
    D.c = pl->d_de_c;
    D.str = pl->d_str;
    D.stk = pl->d_stk;
    SEMB_CUDA(cudaMemsetAsync(pl->d_ctr, 0xff, (size_t)pl->ncdps * pl->ns * 4, st));
    if (timed) SEMB_CUDA(cudaEventRecord(pl->ev[1], st));
    SEMB_TRY(launch_crs_de(pl->w, D, st));
    ++launches;
    if (timed) {
      SEMB_CUDA(cudaEventRecord(pl->ev[2], st));
      SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
    }
    pl->stats.kernel_launches = launches;
    return SEMB_OK;
  }
  if (form == FORM_FAST) SEMB_CUDA(cudaMemsetAsync(pl->d_counter, 0, kMaxBuckets * sizeof(int), st));
  if (timed) SEMB_CUDA(cudaEventRecord(pl->ev[1], st));
  // neighbouring buckets on the same variant (same launch configuration) run as one
  // launch over their tasks, longest aperture first, on the first one's queue head
  for (int i = 0; i < (int)pl->buckets.size();) {
    int j = i + 1;
    while (j < (int)pl->buckets.size() && pl->buckets[j].cfg.variant == pl->buckets[i].cfg.variant) ++j;
    Bucket run = pl->buckets[i];
    run.end = pl->buckets[j - 1].end;
    if (run.end > run.begin) {
      const KParams Pb = make_kparams_cfg(pl, run.cfg, pl->d_tasks + run.begin, run.end - run.begin, pl->d_counter + i);
      SEMB_TRY(launch_search(p.method, form, pl->w, run.cfg.variant, Pb, run.cfg.nwarps, bucket_grid(pl, run),
                             run.cfg.smem, st));
      ++launches;
    }
    i = j;
  }
  if (timed) SEMB_CUDA(cudaEventRecord(pl->ev[2], st));
  if (form == FORM_FAST) {
    SEMB_TRY(enqueue_repick(pl, st, 0, pl->ncdps, true));
    ++launches;
  }
  if (timed) SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
  pl->stats.kernel_launches = launches;
  return SEMB_OK;
}

// The FP64 near-tie re-pick of the batched form over CDPs [cdp0, cdp1) (every CDP
// by default), on stream st; reset_count clears the re-picked-items counter first.
int enqueue_repick(semb_plan* pl, cudaStream_t st, int cdp0, int cdp1, bool reset_count) {
  const semb_params& p = pl->p;
  {
    RepickParams R{};
    R.top_sem = pl->d_top_sem;
    R.top_idx = pl->d_top_idx;
    R.top_stk = pl->d_top_stk;
    R.samples = pl->d_samples;
    R.pitch = pl->pitch;
    R.ap_off = pl->d_ap_off;
    R.ap_tr = pl->d_ap_tr;
    R.ap_geo64 = pl->d_ap_geo64;
    R.cand64 = pl->d_cand64;
    R.stt00 = pl->d_stt00;
    R.ncdps = pl->ncdps;
    R.ns = pl->ns;
    R.tau = pl->tau;
    R.method = p.method;
    R.mode = p.repick;
    R.ncand = pl->ncand;
    R.dt = pl->dt64;
    R.idt = pl->idt64;
    R.gap = p.repick_gap;
    R.ctr = pl->d_ctr;
    R.str = pl->d_str;
    R.stk = pl->d_stk;
    R.repicked = pl->d_repicked;
    R.sem2 = pl->d_sem2;
    R.idx2 = pl->d_idx2;
    R.err64 = pl->d_err64;
    R.item0 = (int64_t)cdp0 * pl->ns;
    R.item_end = (int64_t)cdp1 * pl->ns;
    if (reset_count) SEMB_CUDA(cudaMemsetAsync(pl->d_repicked, 0, sizeof(unsigned long long), st));
    SEMB_TRY(launch_repick(pl->w, R, st));
  }
  return SEMB_OK;
}

// Streamed search (semb_plan_stream): the traces of chunk k are copied on the copy
// stream while the plan's stream searches the chunks whose apertures have landed;
// then the CRS t0 = 0 stacks and the re-pick.  Synchronous, like semb_plan_run.
int enqueue_streamed(semb_plan* pl, const semb_gather_view* g) {
  cudaStream_t st = pl->stream, cs = pl->copy_stream;
  const semb_params& p = pl->p;
  struct CopyJoin {
    cudaStream_t s;
    ~CopyJoin() { cudaStreamSynchronize(s); }
  } join{cs};
  const int nk = pl->nchunks;
  (void)g;   // the chunk copies were queued by the upload (upload_impl)
  SEMB_TRY(dev_reuse(pl, &pl->d_chunk_counter, nk));
  SEMB_CUDA(cudaMemsetAsync(pl->d_status, 0, kStatusWords * sizeof(int), st));
  SEMB_CUDA(cudaMemsetAsync(pl->d_chunk_counter, 0, nk * sizeof(int), st));
  SEMB_CUDA(cudaEventRecord(pl->ev[0], st));
  const Bucket& b = pl->buckets[0];
  const int form = FORM_FAST;
  int launches = 0;
  for (int k = 0; k < nk; ++k) {
    const int n = pl->chunk_task[k + 1] - pl->chunk_task[k];
    if (n == 0) continue;
    SEMB_CUDA(cudaStreamWaitEvent(st, pl->chunk_done[pl->chunk_need[k]], 0));
    const KParams P = make_kparams_cfg(pl, b.cfg, pl->d_tasks + pl->chunk_task[k], n, pl->d_chunk_counter + k);
    SEMB_TRY(launch_search(p.method, form, pl->w, b.cfg.variant, P, b.cfg.nwarps, std::min(n, pl->sms * b.cfg.occ),
                           b.cfg.smem, st));
    ++launches;
  }
  SEMB_CUDA(cudaStreamWaitEvent(st, pl->chunk_done[nk - 1], 0));
  if (p.method == SEMB_CRS) {
    const KParams P = make_kparams(pl, 0);
    SEMB_TRY(launch_stt00(pl->w, 0, pl->ncdps, P, pl->cand0_a, pl->cand0_b, pl->cand0_c, pl->d_stt00, st));
    ++launches;
  }
  SEMB_TRY(enqueue_repick(pl, st, 0, pl->ncdps, true));
  ++launches;
  SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  int status_words[kStatusWords] = {};
  unsigned long long rep = 0;
  SEMB_CUDA(cudaMemcpy(status_words, pl->d_status, sizeof(status_words), cudaMemcpyDeviceToHost));
  const int status = status_words[0];
  SEMB_CUDA(cudaMemcpy(&rep, pl->d_repicked, sizeof(rep), cudaMemcpyDeviceToHost));
  float ms = 0.f;
  SEMB_CUDA(cudaEventElapsedTime(&ms, pl->ev[0], pl->ev[3]));
  pl->stats.ms_search = 0.f;
  pl->stats.ms_repick = 0.f;
  pl->stats.ms_total = ms;
  pl->stats.repicked = (int64_t)rep;
  pl->stats.kernel_launches = launches;
  if (status & ST_TIMEOUT) return fail(SEMB_E_TIMEOUT, "a staging wait in the search kernel timed out");
  if (status & ST_BOUNDS)
    return fail(SEMB_E_BOUNDS, "checked build: an item's window left its staged window (CDP %d, t0 %d, trace %d)",
                status_words[1], status_words[2], status_words[3]);
  if (status) return fail(SEMB_E_CUDA, "search kernel reported status %d", status);
  return SEMB_OK;
}

// Kernels one chunk launches (the same count its graph holds).
int count_chunk_launches(const semb_plan* pl, const semb_plan::RunChunk& ch, int* n) {
  *n = (pl->p.method == SEMB_CRS ? 1 : 0) + 1;
  const int nb = (int)pl->buckets.size();
  for (int i = 0; i < nb;) {
    int j = i + 1;
    while (j < nb && pl->buckets[j].cfg.variant == pl->buckets[i].cfg.variant) ++j;
    if (ch.bucket_begin[j] > ch.bucket_begin[i]) ++*n;
    i = j;
  }
  return SEMB_OK;
}

// The tasks of every run chunk (semb_plan_set_chunks): per chunk its CDPs by
// decreasing aperture, split at the plan's aperture buckets so that each bucket's
// tasks run with that bucket's kernel variant.
int build_run_chunks(semb_plan* pl) {
  drop_graph(pl);
  dev_free(pl->d_chunk_tasks);
  const int nb = (int)pl->buckets.size();
  const int nblk = (pl->ns + kTB - 1) / kTB;
  auto bucket_of = [&](int ap) {
    for (int b = 0; b < nb; ++b)
      if (ap >= pl->buckets[b].ap_lo) return b;
    return nb - 1;
  };
  std::vector<int2> tasks;
  tasks.reserve((size_t)pl->ncdps * nblk);
  for (int c0 = 0; c0 < pl->ncdps; c0 += pl->chunk_cdps) {
    semb_plan::RunChunk ch;
    ch.cdp0 = c0;
    ch.cdp1 = std::min(pl->ncdps, c0 + pl->chunk_cdps);
    std::vector<int> cdps(ch.cdp1 - ch.cdp0);
    std::iota(cdps.begin(), cdps.end(), ch.cdp0);
    std::stable_sort(cdps.begin(), cdps.end(), [&](int x, int y) { return pl->aperture[x] > pl->aperture[y]; });
    ch.bucket_begin.assign(nb + 1, 0);
    size_t q = 0;
    for (int b = 0; b < nb; ++b) {
      ch.bucket_begin[b] = (int)tasks.size();
      while (q < cdps.size() && bucket_of(pl->aperture[cdps[q]]) == b) {
        for (int k = 0; k < nblk; ++k) tasks.push_back(make_int2(cdps[q], k * kTB));
        ++q;
      }
    }
    ch.bucket_begin[nb] = (int)tasks.size();
    if (q != cdps.size()) return fail(SEMB_E_STATE, "aperture buckets do not cover chunk %d", (int)pl->run_chunks.size());
    pl->run_chunks.push_back(std::move(ch));
  }
  SEMB_TRY(dev_alloc(&pl->d_chunk_tasks, tasks.size()));
  SEMB_CUDA(cudaMemcpy(pl->d_chunk_tasks, tasks.data(), tasks.size() * sizeof(int2), cudaMemcpyHostToDevice));
  const size_t nev = pl->run_chunks.size() + 1;
  while (pl->chunk_ev.size() < nev) {
    cudaEvent_t e;
    SEMB_CUDA(cudaEventCreate(&e));
    pl->chunk_ev.push_back(e);
  }
  pl->chunks_dirty = false;
  return SEMB_OK;
}

// One chunk's work on the plan's stream: CRS t0 = 0 stacks of its CDPs, the search
// of its tasks (one launch per run of buckets on the same variant), the re-pick of
// its (CDP, t0) items.
int enqueue_chunk(semb_plan* pl, const semb_plan::RunChunk& ch, int* launches) {
  cudaStream_t st = pl->stream;
  const semb_params& p = pl->p;
  SEMB_CUDA(cudaMemsetAsync(pl->d_counter, 0, kMaxBuckets * sizeof(int), st));
  if (p.method == SEMB_CRS) {
    const KParams P = make_kparams(pl, 0);
    SEMB_TRY(launch_stt00(pl->w, ch.cdp0, ch.cdp1, P, pl->cand0_a, pl->cand0_b, pl->cand0_c, pl->d_stt00, st));
    ++*launches;
  }
  const int nb = (int)pl->buckets.size();
  for (int i = 0; i < nb;) {
    int j = i + 1;
    while (j < nb && pl->buckets[j].cfg.variant == pl->buckets[i].cfg.variant) ++j;
    const int t0 = ch.bucket_begin[i], n = ch.bucket_begin[j] - t0;
    if (n > 0) {
      const KernelCfg& cfg = pl->buckets[i].cfg;
      const KParams P = make_kparams_cfg(pl, cfg, pl->d_chunk_tasks + t0, n, pl->d_counter + i);
      SEMB_TRY(launch_search(p.method, FORM_FAST, pl->w, cfg.variant, P, cfg.nwarps, std::min(n, pl->sms * cfg.occ),
                             cfg.smem, st));
      ++*launches;
    }
    i = j;
  }
  SEMB_TRY(enqueue_repick(pl, st, ch.cdp0, ch.cdp1, false));
  ++*launches;
  return SEMB_OK;
}

// A whole search in chunks (semb_plan_run with chunks set): each chunk's graph,
// captured on its first run, replayed in order; per-chunk device times kept.
int run_chunked(semb_plan* pl) {
  cudaStream_t st = pl->stream;
  if (pl->chunks_dirty) SEMB_TRY(build_run_chunks(pl));
  SEMB_CUDA(cudaMemsetAsync(pl->d_repicked, 0, sizeof(unsigned long long), st));
  int launches = 0;
  const int nk = (int)pl->run_chunks.size();
  SEMB_CUDA(cudaEventRecord(pl->ev[0], st));
  SEMB_CUDA(cudaEventRecord(pl->chunk_ev[0], st));
  for (int k = 0; k < nk; ++k) {
    semb_plan::RunChunk& ch = pl->run_chunks[k];
    int n = 0;
    if (!ch.graph) {
      cudaGraph_t graph;
      SEMB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_chunk(pl, ch, &n);
      const cudaError_t e = cudaStreamEndCapture(st, &graph);
      if (rc != SEMB_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
      }
      SEMB_CUDA(e);
      const cudaError_t ei = cudaGraphInstantiate(&ch.graph, graph, 0);
      cudaGraphDestroy(graph);
      SEMB_CUDA(ei);
    } else {
      // the launch count of a replayed chunk: buckets on distinct variants with tasks
      SEMB_TRY(count_chunk_launches(pl, ch, &n));
    }
    launches += n;
    SEMB_CUDA(cudaGraphLaunch(ch.graph, st));
    SEMB_CUDA(cudaEventRecord(pl->chunk_ev[k + 1], st));
  }
  SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
  pl->stats.kernel_launches = launches;
  return SEMB_OK;
}

}  // namespace

extern "C" {

int semb_plan_set_chunks(semb_plan* pl, int32_t cdps_per_chunk) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (cdps_per_chunk < 0) return fail(SEMB_E_ARG, "cdps_per_chunk must be >= 0");
  if (cdps_per_chunk > 0 && (pl->p.mode != SEMB_BATCHED || pl->p.ngen > 0))
    return fail(SEMB_E_ARG, "chunked runs are the batched form's grid search");
  SEMB_CUDA(cudaSetDevice(pl->device));
  pl->chunk_cdps = cdps_per_chunk;
  drop_graph(pl);
  return SEMB_OK;
}

int semb_plan_chunk_times(const semb_plan* pl, int32_t max, double* ms, int32_t* nchunks) {
  if (!pl || !nchunks) return fail(SEMB_E_ARG, "null argument");
  *nchunks = (int32_t)pl->chunk_ms.size();
  for (int i = 0; ms && i < std::min<int>(max, (int)pl->chunk_ms.size()); ++i) ms[i] = pl->chunk_ms[i];
  return SEMB_OK;
}

int semb_plan_set_staging(semb_plan* pl, int32_t max_samples) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (max_samples != 0 && max_samples < 64) return fail(SEMB_E_ARG, "staging capacity %d below 64", max_samples);
  pl->stage_cap = max_samples;
  if (!pl->uploaded) return SEMB_OK;
  SEMB_CUDA(cudaSetDevice(pl->device));
  for (Bucket& b : pl->buckets) SEMB_TRY(build_cfg(pl, b.cfg.variant, b.cfg));
  refresh_stats(pl);
  return SEMB_OK;
}

int semb_plan_use_graph(semb_plan* pl, int32_t on) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  pl->use_graph = on != 0;
  if (!pl->use_graph && pl->graph) {
    cudaGraphExecDestroy(pl->graph);
    pl->graph = nullptr;
  }
  return SEMB_OK;
}

int semb_plan_run(semb_plan* pl) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_run before semb_plan_upload");
  SEMB_CUDA(cudaSetDevice(pl->device));
  cudaStream_t st = pl->stream;
  SEMB_CUDA(cudaMemsetAsync(pl->d_status, 0, kStatusWords * sizeof(int), st));
  const bool chunked = pl->chunk_cdps > 0 && pl->p.mode == SEMB_BATCHED && pl->p.ngen == 0 &&
                       pl->ns >= 2 * pl->tau + 2;
  pl->chunk_ms.clear();
  if (chunked) {
    SEMB_TRY(run_chunked(pl));
  } else if (pl->use_graph) {
    if (!pl->graph) {
      cudaGraph_t graph;
      SEMB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_run(pl, false);
      cudaError_t e = cudaStreamEndCapture(st, &graph);
      if (rc != SEMB_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
      }
      SEMB_CUDA(e);
      e = cudaGraphInstantiate(&pl->graph, graph, 0);
      cudaGraphDestroy(graph);
      SEMB_CUDA(e);
    }
    SEMB_CUDA(cudaEventRecord(pl->ev[0], st));
    SEMB_CUDA(cudaGraphLaunch(pl->graph, st));
    SEMB_CUDA(cudaEventRecord(pl->ev[3], st));
  } else {
    SEMB_TRY(enqueue_run(pl, true));
  }
  SEMB_CUDA(cudaStreamSynchronize(st));
  int status_words[kStatusWords] = {};
  unsigned long long rep = 0;
  SEMB_CUDA(cudaMemcpy(status_words, pl->d_status, sizeof(status_words), cudaMemcpyDeviceToHost));
  const int status = status_words[0];
  if (pl->p.mode == SEMB_BATCHED)
    SEMB_CUDA(cudaMemcpy(&rep, pl->d_repicked, sizeof(rep), cudaMemcpyDeviceToHost));
  // graph replays are timed as a whole; the per-kernel split needs direct launches
  float a = 0.f, b = 0.f, c = 0.f;
  if (chunked) {
    for (size_t k = 0; k < pl->run_chunks.size(); ++k) {
      float m = 0.f;
      SEMB_CUDA(cudaEventElapsedTime(&m, pl->chunk_ev[k], pl->chunk_ev[k + 1]));
      pl->chunk_ms.push_back(m);
    }
  } else if (!pl->use_graph) {
    SEMB_CUDA(cudaEventElapsedTime(&a, pl->ev[1], pl->ev[2]));
    SEMB_CUDA(cudaEventElapsedTime(&b, pl->ev[2], pl->ev[3]));
  }
  SEMB_CUDA(cudaEventElapsedTime(&c, pl->ev[0], pl->ev[3]));
  pl->stats.ms_search = a;
  pl->stats.ms_repick = b;
  pl->stats.ms_total = c;
  pl->stats.repicked = (int64_t)rep;
  if (status & ST_TIMEOUT) return fail(SEMB_E_TIMEOUT, "a staging wait in the search kernel timed out");
  if (status & ST_BOUNDS)
    return fail(SEMB_E_BOUNDS, "checked build: an item's window left its staged window (CDP %d, t0 %d, trace %d)",
                status_words[1], status_words[2], status_words[3]);
  if (status) return fail(SEMB_E_CUDA, "search kernel reported status %d", status);
  return SEMB_OK;
}

int semb_plan_download(semb_plan* pl, int32_t* ctr, float* str, float* stk) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_download before semb_plan_upload");
  SEMB_CUDA(cudaSetDevice(pl->device));
  const size_t n = (size_t)pl->ncdps * pl->ns;
  cudaStream_t st = pl->stream;
  if (ctr) SEMB_CUDA(cudaMemcpyAsync(ctr, pl->d_ctr, n * 4, cudaMemcpyDeviceToHost, st));
  if (str) SEMB_CUDA(cudaMemcpyAsync(str, pl->d_str, n * 4, cudaMemcpyDeviceToHost, st));
  if (stk) SEMB_CUDA(cudaMemcpyAsync(stk, pl->d_stk, n * 4, cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  return SEMB_OK;
}

int semb_plan_download_attrs(semb_plan* pl, float* sem2, int32_t* idx2, float* err64, int32_t* aperture) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_download_attrs before semb_plan_upload");
  if ((sem2 || idx2 || err64) && !pl->d_sem2)
    return fail(SEMB_E_STATE, "second-best and FP64-error attributes need the batched form with attrs = 1");
  SEMB_CUDA(cudaSetDevice(pl->device));
  const size_t n = (size_t)pl->ncdps * pl->ns;
  cudaStream_t st = pl->stream;
  if (sem2) SEMB_CUDA(cudaMemcpyAsync(sem2, pl->d_sem2, n * 4, cudaMemcpyDeviceToHost, st));
  if (idx2) SEMB_CUDA(cudaMemcpyAsync(idx2, pl->d_idx2, n * 4, cudaMemcpyDeviceToHost, st));
  if (err64) SEMB_CUDA(cudaMemcpyAsync(err64, pl->d_err64, n * 4, cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  if (aperture) std::memcpy(aperture, pl->aperture.data(), pl->aperture.size() * sizeof(int32_t));
  return SEMB_OK;
}

int semb_plan_download_abc(semb_plan* pl, float* a, float* b, float* c) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_download_abc before semb_plan_upload");
  if (!pl->d_de_a) return fail(SEMB_E_STATE, "explicit A, B, C are the results of CRS-DE (ngen > 0)");
  SEMB_CUDA(cudaSetDevice(pl->device));
  const size_t n = (size_t)pl->ncdps * pl->ns;
  cudaStream_t st = pl->stream;
  if (a) SEMB_CUDA(cudaMemcpyAsync(a, pl->d_de_a, n * 4, cudaMemcpyDeviceToHost, st));
  if (b) SEMB_CUDA(cudaMemcpyAsync(b, pl->d_de_b, n * 4, cudaMemcpyDeviceToHost, st));
  if (c) SEMB_CUDA(cudaMemcpyAsync(c, pl->d_de_c, n * 4, cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  return SEMB_OK;
}

int semb_plan_neighbours(semb_plan* pl, int32_t* off, int32_t* list, int64_t* n_out) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_neighbours before semb_plan_upload");
  SEMB_CUDA(cudaSetDevice(pl->device));
  if (n_out) *n_out = pl->n_nbr;
  if (off && pl->n_nbr > INT32_MAX)
    return fail(SEMB_E_ARG, "%lld neighbour pairs do not fit 32-bit offsets", (long long)pl->n_nbr);
  if (off) {
    std::vector<int64_t> o(pl->ncdps + 1);
    SEMB_CUDA(cudaMemcpy(o.data(), pl->d_nbr_off, o.size() * 8, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < o.size(); ++i) off[i] = (int32_t)o[i];
  }
  if (list) SEMB_CUDA(cudaMemcpy(list, pl->d_nbr, (size_t)pl->n_nbr * 4, cudaMemcpyDeviceToHost));
  return SEMB_OK;
}

int semb_plan_set_variant(semb_plan* pl, int32_t variant) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_set_variant before semb_plan_upload");
  SEMB_CUDA(cudaSetDevice(pl->device));
  const int form = pl->p.mode == SEMB_PLAIN_F32 ? FORM_PLAIN : FORM_FAST;
  int rc = 0, minb = 0, brun = 0, nt = 0;
  if (!search_variant(pl->p.method, form, pl->w, variant, &rc, &minb, &brun, &nt, nullptr, nullptr))
    return fail(SEMB_E_ARG, "no search kernel variant %d for this plan", variant);
  return set_all(pl, variant);
}

int semb_plan_autotune(semb_plan* pl, int32_t* chosen, double* ms_of_variant) {
  if (!pl) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_autotune before semb_plan_upload");
  SEMB_CUDA(cudaSetDevice(pl->device));
  const semb_params& p = pl->p;
  const int form = p.mode == SEMB_PLAIN_F32 ? FORM_PLAIN : FORM_FAST;
  cudaStream_t st = pl->stream;
  std::vector<int2> all(pl->ntasks);
  SEMB_CUDA(cudaMemcpy(all.data(), pl->d_tasks, all.size() * sizeof(int2), cudaMemcpyDeviceToHost));
  const int smax = std::max(1, pl->sms * 8);
  int2* d_sample = nullptr;
  SEMB_TRY(dev_alloc(&d_sample, smax));
  struct Free {
    int2* p;
    KernelCfg trial;
    ~Free() {
      cudaFree(p);
      free_cfg(trial);
    }
  } guard{d_sample, {}};
  std::vector<double> total(kVariantSlots, 0.0);
  std::vector<char> fits(kVariantSlots, 1);
  for (Bucket& b : pl->buckets) {
    const int n = b.end - b.begin;
    if (n == 0) continue;
    // a strided sample of the bucket's (aperture-sorted) tasks
    const int S = std::min(n, smax);
    std::vector<int2> sample(S);
    for (int i = 0; i < S; ++i) sample[i] = all[b.begin + (int64_t)i * n / S];
    SEMB_CUDA(cudaMemcpy(d_sample, sample.data(), S * sizeof(int2), cudaMemcpyHostToDevice));
    int best = -1;
    double best_ms = 1e300;
    for (int v = 0; v < kVariantSlots; ++v) {
      int rc = 0, minb = 0, brun = 0, nt = 0;
      // a variant with no kernel for this window, or whose staging does not fit
      // this plan's traces, is skipped
      if (!fits[v] || !search_variant(p.method, form, pl->w, v, &rc, &minb, &brun, &nt, nullptr, nullptr) ||
          build_cfg(pl, v, guard.trial) != SEMB_OK) {
        fits[v] = 0;
        continue;
      }
      const KParams P = make_kparams_cfg(pl, guard.trial, d_sample, S, pl->d_counter);
      const int grid = form == FORM_PLAIN ? S : std::min(S, pl->sms * guard.trial.occ);
      float ms = 1e30f;
      for (int rep = 0; rep < 3; ++rep) {
        SEMB_CUDA(cudaMemsetAsync(pl->d_counter, 0, sizeof(int), st));
        SEMB_CUDA(cudaEventRecord(pl->ev[4], st));
        SEMB_TRY(launch_search(p.method, form, pl->w, v, P, guard.trial.nwarps, grid, guard.trial.smem, st));
        SEMB_CUDA(cudaEventRecord(pl->ev[5], st));
        SEMB_CUDA(cudaStreamSynchronize(st));
        float t = 0.f;
        SEMB_CUDA(cudaEventElapsedTime(&t, pl->ev[4], pl->ev[5]));
        if (rep > 0) ms = std::min(ms, t);   // the first launch is a warm-up
      }
      total[v] += ms;
      if (ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    if (best < 0) return fail(SEMB_E_WINDOW, "no search kernel for w = %d", pl->w);
    SEMB_TRY(build_cfg(pl, best, b.cfg));
  }
  // neighbouring buckets that chose the same variant become one launch
  for (size_t i = 0; i + 1 < pl->buckets.size();) {
    Bucket& a = pl->buckets[i];
    Bucket& c = pl->buckets[i + 1];
    if (a.cfg.variant == c.cfg.variant) {
      a.end = c.end;
      a.ap_lo = c.ap_lo;
      a.work += c.work;
      free_cfg(c.cfg);
      pl->buckets.erase(pl->buckets.begin() + (long)i + 1);
    } else {
      ++i;
    }
  }
  drop_graph(pl);
  refresh_stats(pl);
  if (ms_of_variant)
    for (int v = 0; v < kVariantSlots; ++v) ms_of_variant[v] = fits[v] ? total[v] : -1.0;
  if (chosen) *chosen = main_bucket(pl).cfg.variant;
  return SEMB_OK;
}

int semb_plan_buckets(const semb_plan* pl, int32_t* nbuckets, int32_t* ap_lo, int32_t* ap_hi, int32_t* ntasks,
                      int32_t* variant) {
  if (!pl || !nbuckets) return fail(SEMB_E_ARG, "null argument");
  if (!pl->uploaded) return fail(SEMB_E_STATE, "semb_plan_buckets before semb_plan_upload");
  const int n = (int)pl->buckets.size();
  *nbuckets = n;
  for (int i = 0; i < n; ++i) {
    const Bucket& b = pl->buckets[i];
    if (ap_lo) ap_lo[i] = b.ap_lo;
    if (ap_hi) ap_hi[i] = b.ap_hi;
    if (ntasks) ntasks[i] = b.end - b.begin;
    if (variant) variant[i] = b.cfg.variant;
  }
  return SEMB_OK;
}

int semb_plan_stats(const semb_plan* pl, semb_stats* out) {
  if (!pl || !out) return fail(SEMB_E_ARG, "null argument");
  *out = pl->stats;
  return SEMB_OK;
}

}  // extern "C"
