// Fused CMP/CRS semblance search kernels for sm_103a.
//
// One CTA works on one task: a CDP and a block of 32 consecutive output samples t0
// (lane l of every warp owns t0 = t0_start + l).  The CTA walks the candidate grid
// in passes; in a pass, warp w owns RC candidates, so each thread carries RC
// (t0, candidate) items whose partial sums live in registers.  The CDP's aperture
// traces are streamed through shared memory in chunks: warp 0 works out, for every
// trace of the next chunk, the sample window that any item of this pass can touch
// (from the pass's parameter bounds and the task's t0 range) and stages exactly
// those windows, so every staged sample is reused by all items of the pass.
// Semblance, stack and the per-t0 argmax are fused: the pick is reduced in
// registers and then across warps through shared memory, and only ctr/str/stk (or,
// in the fast form, the per-t0 top-4 list) leave the SM.
//
// Reference semantics (per item (t0, candidate), CMP/OpenMP/src/main.cpp:149-204,
// CRS/OpenMP/src/main.cpp:209-267):
//   CMP  t = sqrt((dt*t0)^2 + c*h) * idt
//   CRS  t = (dt*t0 + a*|dm|)^2 + b*dm^2 + c*h;  t = t < 0 ? -1 : sqrt(t);  t *= idt
//   it = (int)t, x = t - it; the trace is in range iff it-tau >= 0 && it+tau+1 < ns;
//   for j < w: v = (s[it-tau+j+1] - s[it-tau+j]) * x + s[it-tau+j],
//   num_j += v, den += v^2, lin += v, M++; out of range: err++.
//   valid iff den > 1e-13 && M > 0 && err < 2: sem = sum_j num_j^2 / (den*M),
//   stk = lin / (w*M); invalid: sem = stk = -1 (CMP) or 0 (CRS).
//   Argmax per t0 (CMP main.cpp:207-222, CRS main.cpp:270-285): the first
//   candidate (lowest index) with the largest semblance, which must exceed 0.
//
// Items carry no branch: an out-of-range trace reads a block of zeros kept at the
// end of the staging buffer with interpolation weight 0, so it adds exactly +0 to
// the sums, and only M counts it out.  The RC items of a thread are then straight-
// line code the compiler can interleave.
//
// Two forms share the structure:
//   PLAIN  FP32 with the reference's operation order: every multiply and add is
//          rounded separately (__fmul_rn/__fadd_rn: no contraction), IEEE sqrt
//          and division, the same `lin` accumulator; staged by 1-D bulk copies
//          (TMA) of the FP32 trace store.  Bit-compatible with the reference's
//          single-precision build.
//   FAST   traces stored as FP16/BF16 (+ FP32 scale) or FP32, staged as FP32
//          16-byte entries (s_k, s_k+1, s_k+2, s_k+3), one per sample, so that the
//          w+1 samples of a window are ceil((w+1)/4) vector loads (w = 3: one
//          LDS.128, 16 bytes; w = 5: LDS.128 + LDS.64, 24 bytes);
//          FP32 arithmetic with fused multiply-adds and hardware sqrt, traveltimes
//          in sample units (candidates pre-scaled by idt), the stack taken from
//          sum_j num_j, and the energy accumulated per chunk and folded into a
//          Kahan-compensated total; keeps the top-4 candidates per t0 for the
//          FP64 re-pick.  With BRUN (CRS), the plan lays the candidates out so that
//          each thread's RC candidates are consecutive B values of one (A, C) pair,
//          and the A and C terms of the traveltime are computed once per trace.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace semb {

enum { METHOD_CMP = 0, METHOD_CRS = 1 };
enum { FORM_PLAIN = 0, FORM_FAST = 1 };
enum { STORE_F32 = 0, STORE_F16 = 1, STORE_BF16 = 2 };

constexpr int kTB = 32;          // t0 samples per task (one per lane)
constexpr int kMaxChunk = 128;   // aperture traces staged per chunk
constexpr int kMargin = 2;       // extra samples on each side of a staged window
constexpr int kTopK = 4;
constexpr int kZeroSlots = 16;   // zero block after the staging buffer (floats or entries)
// Entry offset (ChunkMeta::geo[].w) of a trace whose window does not fit the staging
// buffer (batched form): its items read the FP32 store in global memory instead, and
// ChunkMeta::raw holds its trace index.
constexpr int kGlobalEntry = INT32_MIN;
constexpr int kMaxThreads = 256; // CTA size limit of the search kernel (variants use 128 or 256)
constexpr uint64_t kWaitNs = 2000000000ull;  // bounded mbarrier wait (2 s), then error

// Device status words: [0] bits, [1..3] the first bounds violation of a checked build
// (CDP, t0, trace).
enum { ST_TIMEOUT = 1, ST_BAD_ARG = 2, ST_BOUNDS = 4 };
constexpr int kStatusWords = 4;

// Checked build (compiled with -DSEMB_CHECKED=1 into libsemb_gb300_checked.so): every
// item that reads a staged window is tested against the window its trace was staged
// with, the property the planner's bounds guarantee (the unchecked kernels rely on it
// and only clamp addresses to the buffer as a guard).  A violation sets ST_BOUNDS and
// records the first offender; the address stays clamped, so nothing outside the
// buffer is read and the search runs to its end.
#ifndef SEMB_CHECKED
#define SEMB_CHECKED 0
#endif

struct KParams {
  // trace store, [ntr][pitch]; pitch is a multiple of 8 elements with at least 8
  // zero elements after the last sample of each trace
  const float* samples;         // FP32
  const uint16_t* samples16;    // FP16 or BF16 bit patterns (fast form)
  const float* scale;           // per-trace scale of samples16
  int64_t pitch;
  int storage;                  // STORE_*
  // aperture lists: entries ap_off[c] .. ap_off[c+1]-1 of CDP c
  const int64_t* ap_off;
  const int32_t* ap_tr;         // trace index of each entry
  const float4* ap_geo;         // (|dm|, dm^2, h, 0) per entry, FP32
  // candidates in search order, padded to npass*cpp; .w holds the grid index bits
  // (-1 in padding slots)
  const float4* cand;
  const float* pass_bounds;     // [npass][8]: amin amax bmin bmax cmin cmax (raw units)
  int npass;
  int cpp;                      // candidates per pass = warps * RC
  // tasks (cdp, t0_start)
  const int2* tasks;
  int ntasks;
  int* counter;                 // work-queue head (fast form)
  // sampling
  int ns;
  int tau;
  float dt, idt;
  int cap;                      // staging capacity: floats (plain) or 16-byte entries (fast)
  // outputs [ncdps][ns]
  int32_t* ctr;
  float* str;
  float* stk;
  const float* stt00;           // CRS: stack of item (t0=0, candidate 0) per CDP
  float* top_sem;               // fast form: [ncdps][ns][4]
  int32_t* top_idx;
  float* top_stk;
  int* status;
  // CRS, variants that share the central CDP's traces over A and B (Z0): per CDP the
  // (first entry, count) of its own traces in its aperture list, relative to ap_off;
  // the C value of each C index in sample units; per pass its first C index and the
  // number of C indices it spans (at most kZ0C)
  const int2* z0r;
  const float* cvals;
  const int2* pass_c;
  int nc_grid;
};

// Z0 variants: the most C indices one pass may span, and the pass slots of the central
// traces' sums (a slot is zeroed again at the start of the fourth pass after, when every
// warp has finalized the pass that used it)
constexpr int kZ0C = 4;
constexpr int kZ0Slots = 4;

// ---------------------------------------------------------------------------
// small PTX helpers (mbarrier + bulk copy)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// 1-D bulk copy global -> shared (TMA), completion counted on `bar` in bytes.
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float sqrt_fast(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float half_bits_to_float(uint32_t b) {
  return __half2float(__ushort_as_half(static_cast<unsigned short>(b)));
}

// Checked build: the window samples idx .. idx + W of an item must lie inside the
// staged window [off, off + len) of its entry (src = (trace, lo, len, off), buffer
// units); the first violation is recorded with its CDP, t0 and trace.
static __device__ __noinline__ void report_window(int* status, int idx, int W, int4 src, int cdp, int t0) {
  if (idx >= src.w && idx + W <= src.w + src.z - 1) return;
  if ((atomicOr(status, ST_BOUNDS) & ST_BOUNDS) == 0) {
    status[1] = cdp;
    status[2] = t0;
    status[3] = src.x;
  }
}

// Pick order: larger semblance first; equal semblance -> lower grid index first.
__device__ __forceinline__ bool better(float s, int i, float bs, int bi) {
  return s > bs || (s == bs && i < bi);
}

// ---------------------------------------------------------------------------
// staging plan: warp 0 sizes and stages the next chunk of aperture entries.

// staging layouts of the fast form (one 16-byte entry per window sample k)
constexpr int LAY_QUAD = 0;   // (s_k, s_k+1, s_k+2, s_k+3)
constexpr int LAY_SD = 1;     // (s_k, s_k+1 - s_k, s_k+1, s_k+2 - s_k+1)
constexpr int LAY_P2 = 2;     // (s_k, s_k+2, s_k+1, s_k+3)
constexpr int LAY_PD = 3;     // w = 3: (s_k, s_k+2, s_k+1 - s_k, s_k+3 - s_k+2)
// The same staged entries as LAY_P2 / LAY_PD; the items form the two interpolated
// samples of a pair with scalar FMAs into one register pair instead of a packed
// FP32x2 FMA, whose weight operand (x, x) costs register moves per item.
constexpr int LAY_P2S = 4;
constexpr int LAY_PDS = 5;
// w = 3, pipelined kernel only: values pre-offset by their window's integer sample,
// F_k,j = s_k+j - (k + tau) d_k+j with d_m = s_m+1 - s_m, so that an item at
// traveltime t (samples) interpolates v_j = F_k,j + t d_k+j with no weight t - floor(t):
// a 16-byte entry (F_k,0, F_k,2, d_k, d_k+2) and an 8-byte side entry (F_k,1, d_k+1)
// per window start k, 24 bytes per sample.  The pre-offset costs precision in
// proportion to the sample index (about ns x 2^-24 of |d|), so plans use it for
// ns <= 8192 only.
constexpr int LAY_FT = 6;
constexpr int kMaxNsFT = 8192;
// w = 5: the packed value/difference entry (s_k, s_k+2, d_k, d_k+2) of LAY_PD and an
// 8-byte side entry (s_k, d_k) per sample, d_m = s_m+1 - s_m.  An item whose window
// starts at k reads entry k and side entry k+4: 24 bytes, i.e. six shared-memory
// wavefronts per warp instead of the eight of two 16-byte entries (LAY_P2), and
// the pairs (0, 2) and (1, 3) need no differences formed from two loaded values
// but (s_2, s_4) - (s_1, s_3).  LAY_PD5S forms the interpolated pairs with scalar
// FMAs (no (x, x) operand).
constexpr int LAY_PD5 = 7;
constexpr int LAY_PD5S = 8;
// w = 3, pipelined kernel only: two planes of floats per stage, the samples s_k and
// their differences d_k = s_k+1 - s_k, the difference plane kXPlane floats after the
// sample plane.  An item reads s_k, s_k+2, d_k, d_k+2 with four 32-bit loads (four
// shared-memory wavefronts per warp, as one 16-byte entry), and two items of a
// thread share every FP32x2 instruction: lane .x holds item 2p, lane .y item 2p+1,
// so the window arithmetic is packed throughout and needs no (x, x) operand.
constexpr int LAY_X3 = 9;
constexpr int kXPlane = 4096;

// layout of the staged entries of an accumulation layout
__host__ __device__ constexpr int stage_lay(int lay) {
  return lay == LAY_P2S ? LAY_P2 : lay == LAY_PDS ? LAY_PD : lay == LAY_PD5S ? LAY_PD5 : lay;
}

// layouts with an 8-byte side entry per sample after the main entries
__host__ __device__ constexpr bool lay_has_side(int lay) {
  return stage_lay(lay) == LAY_FT || stage_lay(lay) == LAY_PD5;
}

// bytes of one staged entry (the address stride of an item's window), and of one
// staged sample with its side entry (LAY_FT, LAY_PD5) or its difference (LAY_X3)
__host__ __device__ constexpr int lay_entry_bytes(int lay) { return lay == LAY_X3 ? 4 : 16; }
__host__ __device__ constexpr int lay_stage_bytes(int lay) { return lay_has_side(lay) ? 24 : lay == LAY_X3 ? 8 : 16; }

struct ChunkMeta {
  float4 geo[kMaxChunk];   // (|dm|, dm^2, h, soff as int bits)
  float scale[kMaxChunk];  // fast form: per-trace scale of the 16-bit store
  int raw[kMaxChunk];      // fast form: start of the entry's raw window (samples):
                           // its buffer offset + 8 x its rank in aperture order;
                           // the trace index for a kGlobalEntry entry
  int n;                   // entries in this chunk
  int n_in;                // fast form: entries on which every item of the pass is in
                           // range, in slots [0, n_in); the others fill slots
                           // [kMaxChunk - (n - n_in), kMaxChunk).  Plain form: n_in = n
  int consumed;            // aperture traces the chunk covers (entries + skipped)
  int bytes;               // bytes staged (TMA form)
};

constexpr size_t kMetaBytes = ((sizeof(ChunkMeta) + 127) / 128) * 128;

// Slot of the i-th entry (0 <= i < n) of a chunk: the in-range entries first, then
// the others from the top of the table.
__device__ __forceinline__ int entry_slot(const ChunkMeta* m, int i) {
  return i < m->n_in ? i : kMaxChunk - m->n + i;
}

// Shared-memory layout of the search kernel (bytes), shared by host and device:
//   [0, 64)   two mbarriers and control words
//   meta[2]   chunk metadata (the fast form alternates two chunks)
//   src[2]    per-entry copy descriptors (trace, first sample, length, offset)
//   top-K     per-thread running picks [3][K][nt]
//   kahan     fast form: per-item compensated energy totals [2][RC][nt]
//   buf       staging buffer: cap floats (plain) or cap 16-byte quads (fast),
//             followed by kZeroSlots zeroed slots read by out-of-range items;
//             layouts with side entries (LAY_PD5) then hold cap + kZeroSlots
//             8-byte side entries, the last kZeroSlots zeroed
//   raw[2]    fast form: the raw windows of two chunks as stored in HBM
//             (16-bit or FP32), cap + 8*kMaxChunk samples each
struct SmemLayout {
  size_t meta, src, tops, kahan, buf, raw0, raw1, total;
};

__host__ __device__ inline size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }

__host__ __device__ inline SmemLayout smem_layout(int form, int rc, int cap, int storage, int nt, int lay) {
  const int K = form == 1 ? 4 : 1;
  SmemLayout L;
  L.meta = 64;
  L.src = L.meta + 2 * kMetaBytes;
  L.tops = L.src + 2 * kMaxChunk * sizeof(int4);
  L.kahan = L.tops + align128(3 * (size_t)K * nt * 4);
  L.buf = L.kahan + (form == 1 ? 2 * (size_t)rc * nt * 4 : 0);
  const size_t unit = form == 1 ? (size_t)lay_stage_bytes(lay) : 4;
  const size_t raw_end = L.buf + align128(((size_t)cap + kZeroSlots) * unit);
  if (form == 1) {
    const size_t rb = align128(((size_t)cap + 8 * kMaxChunk) * (storage == 0 ? 4 : 2));
    L.raw0 = raw_end;
    L.raw1 = raw_end + rb;
    L.total = raw_end + 2 * rb;
  } else {
    L.raw0 = L.raw1 = raw_end;
    L.total = raw_end;
  }
  return L;
}

// Sample window [lo, hi] of one trace that items of a pass can read, for t0 in
// [T_lo, T_hi] (seconds) and parameters within the pass bounds.  Returns false
// when no item can be in range: then the trace is left out of the chunk, which is
// exact, because an out-of-range trace only counts in err = N_ap - M.
template <int METHOD>
__device__ __forceinline__ bool trace_window(const float* pb, float4 g, float T_lo, float T_hi, float idt,
                                             int tau, int ns, int& lo, int& hi, bool& inrange) {
  inrange = false;
  float t2min, t2max;
  if (METHOD == METHOD_CMP) {
    // t^2 = t0^2 + c*h, h >= 0
    t2min = T_lo * T_lo + fminf(pb[4] * g.z, pb[5] * g.z);
    t2max = T_hi * T_hi + fmaxf(pb[4] * g.z, pb[5] * g.z);
  } else {
    // t^2 = (t0 + a*m)^2 + b*m2 + c*h with m2, h >= 0; m >= 0, or signed along the
    // azimuth
    const float am0 = pb[0] * g.x, am1 = pb[1] * g.x;
    float ulo = T_lo + fminf(am0, am1), uhi = T_hi + fmaxf(am0, am1);
    float u2lo = (ulo <= 0.f && uhi >= 0.f) ? 0.f : fminf(ulo * ulo, uhi * uhi);
    float u2hi = fmaxf(ulo * ulo, uhi * uhi);
    t2min = u2lo + pb[2] * g.y + pb[4] * g.z;
    t2max = u2hi + pb[3] * g.y + pb[5] * g.z;
  }
  // relative slack for rounding differences between this bound and the items
  t2min -= fabsf(t2min) * 1e-5f;
  t2max += fabsf(t2max) * 1e-5f;
  if (!(t2max >= 0.f)) {
    // every item has a negative t^2 (or the bound is not finite): nothing in range
    if (t2max < 0.f) return false;
    lo = 0;
    hi = ns - 1;
    return true;
  }
  float smin = t2min > 0.f ? sqrtf(t2min) * idt : 0.f;
  float smax = sqrtf(t2max) * idt;
  smin = fminf(smin, (float)ns + 8.f);
  smax = fminf(smax, (float)ns + 8.f);
  // in range for sure: tau <= it <= ns - tau - 2 for every item, with one sample of slack
  inrange = t2min > 0.f && smin >= (float)(tau + 1) && smax <= (float)(ns - tau - 3);
  // out of range for sure (t < tau or t >= ns - tau - 1 for every item, again with a
  // sample of slack): the trace adds nothing but its out-of-range count
  if (smax < (float)(tau - 1) || smin > (float)(ns - tau)) return false;
  lo = (int)smin - tau - kMargin;
  hi = (int)smax + tau + 1 + kMargin;
  lo = max(lo, 0);
  hi = min(hi, ns - 1);
  return lo <= hi;
}

// Warp 0: choose the entries of the next chunk starting at ap_pos and record, per
// entry, its geometry, its buffer offset (minus the window start, so that an item
// indexes with it - tau directly) and its source window (trace, first sample,
// length, offset) in `src`.  Aperture traces on which no item can be in range are
// consumed without an entry.  meta->n counts entries, meta->consumed the aperture
// traces the chunk covers.  Fast form: entries on which every item is in range go
// to the front slots, the others to the back (entry_slot).  Windows are aligned to ALIGN samples: 4 for FP32 bulk
// copies (16 bytes), 8 for the fast form's raw windows.  Buffer units: floats
// (plain) or one 16-byte entry per sample (fast).
template <int METHOD, int FORM>
__device__ void plan_chunk(const KParams& P, const float* pb, int64_t ap_pos, int64_t ap_end, float T_lo,
                           float T_hi, ChunkMeta* meta, int4* src, int64_t skip_b = 0, int64_t skip_e = 0) {
  const int lane = threadIdx.x & 31;
  constexpr int ALIGN = (FORM == FORM_PLAIN) ? 4 : 8;
  int base = 0;       // buffer units used
  int n_in = 0;       // entries in the in-range part (front)
  int n_out = 0;      // other entries (back)
  int consumed = 0;   // aperture traces covered
  while (n_in + n_out + 32 <= kMaxChunk) {
    const int64_t k = ap_pos + consumed + lane;
    const bool have = k < ap_end;
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
    int lo = 0, hi = -1;
    int len = 0;
    bool inr = false, keep = false;
    int tr = 0;
    float sc = 1.0f;
    bool glob = false;
    if (have) {
      g = P.ap_geo[k];
      keep = trace_window<METHOD>(pb, g, T_lo, T_hi, P.idt, P.tau, P.ns, lo, hi, inr);
      // a trace of the central CDP at zero midpoint distance whose sums the pass shares
      // over A and B (Z0 variants) is left out
      if (k >= skip_b && k < skip_e && g.x == 0.f) keep = false;
      if (keep) {
        tr = P.ap_tr[k];
        if (FORM == FORM_FAST && P.storage != STORE_F32) sc = __ldg(P.scale + tr);
        lo &= ~(ALIGN - 1);
        hi |= (ALIGN - 1);
        len = hi - lo + 1;
        // batched form: a window larger than the whole buffer is not staged; its
        // items read the FP32 store (the partly-in-range section checks each item)
        if (FORM == FORM_FAST && len > P.cap) {
          glob = true;
          len = 0;
        }
      }
    }
    // inclusive scan of the kept windows' lengths over the warp
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    // the first kept trace that does not fit ends the chunk
    const unsigned over = __ballot_sync(0xffffffffu, keep && base + incl > P.cap);
    const int stop = over ? __ffs(over) - 1 : 32;
    // the plain form keeps every entry in aperture order at the front
    const bool take = keep && lane < stop;
    const bool front = FORM == FORM_PLAIN || (inr && !glob);
    const unsigned fr = __ballot_sync(0xffffffffu, take && front);
    const unsigned bk = __ballot_sync(0xffffffffu, take && !front);
    if (take) {
      const unsigned below = (1u << lane) - 1u;
      const int e = front ? n_in + __popc(fr & below) : kMaxChunk - 1 - (n_out + __popc(bk & below));
      const int off = base + incl - len;
      const int rank = n_in + n_out + __popc((fr | bk) & below);   // in aperture order
      g.w = __int_as_float(glob ? kGlobalEntry : off - lo);
      meta->geo[e] = g;
      meta->scale[e] = sc;
      meta->raw[e] = glob ? tr : off + 8 * rank;
      src[e] = make_int4(tr, lo, len, off);   // len 0: nothing to copy or convert
    }
    const int nhave = __popc(__ballot_sync(0xffffffffu, have));
    base += stop > 0 ? __shfl_sync(0xffffffffu, incl, stop - 1) : 0;
    n_in += __popc(fr);
    n_out += __popc(bk);
    consumed += min(stop, nhave);
    if (stop < 32 || nhave < 32) break;
  }
  if (lane == 0) {
    meta->n = n_in + n_out;
    meta->n_in = n_in;
    meta->consumed = consumed;
    meta->bytes = base * 4;
  }
  __syncwarp();
}

// Warp 0, after plan_chunk (plain form): announce the chunk's bytes on the
// barrier, then start one bulk copy per staged window.
__device__ __forceinline__ void issue_chunk_copies(const KParams& P, ChunkMeta* meta, const int4* src, float* buf,
                                                   uint64_t* bar) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)meta->bytes);
  __syncwarp();
  const int n = meta->n;
  for (int i = lane; i < n; i += 32) {
    const int4 si = src[entry_slot(meta, i)];
    if (si.z > 0) bulk_g2s(buf + si.w, P.samples + (int64_t)si.x * P.pitch + si.y, (uint32_t)si.z * 4u, bar);
  }
}

// Fast form, warp 0 after plan_chunk: start one bulk copy (TMA) per staged window
// of the raw store into `raw`, each window plus the 8 samples after it (the quads
// of the last samples read 3 past the window).  The k-th entry in aperture order
// lands at raw offset off + 8k samples (meta->raw), so windows never overlap.  The barrier is told the total bytes first.
__device__ __forceinline__ void issue_raw(const KParams& P, const ChunkMeta* meta, const int4* src,
                                          unsigned char* raw, uint64_t* bar) {
  const int lane = threadIdx.x & 31;
  const int n = meta->n;
  const uint32_t unit = P.storage == STORE_F32 ? 4u : 2u;
  uint32_t bytes = 0;
  for (int i = lane; i < n; i += 32) {
    const int4 si = src[entry_slot(meta, i)];
    if (si.z > 0) bytes += (uint32_t)(si.z + 8) * unit;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
  if (lane == 0) mbar_arrive_expect_tx(bar, bytes);
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    const int e = entry_slot(meta, i);
    const int4 si = src[e];
    if (si.z <= 0) continue;
    const int64_t at = (int64_t)si.x * P.pitch + si.y;
    const void* g = P.storage == STORE_F32 ? (const void*)(P.samples + at) : (const void*)(P.samples16 + at);
    bulk_g2s(raw + (size_t)meta->raw[e] * unit, g, (uint32_t)(si.z + 8) * unit, bar);
  }
}

// Fast form, all warps: turn the landed raw windows into 16-byte entries, one per
// sample k: (s_k, s_k+1, s_k+2, s_k+3) ("quads", LAY_QUAD), (s_k, s_k+1 - s_k,
// s_k+1, s_k+2 - s_k+1) ("value/difference pairs", LAY_SD) or (s_k, s_k+2, s_k+1,
// s_k+3) ("packed pairs", LAY_P2).  Lane l builds entry k0 + l, so
// the warp's 16-byte stores cover consecutive addresses (no bank conflicts).
template <int LAY>
__device__ __forceinline__ void convert_chunk(const KParams& P, const ChunkMeta* meta, const int4* src,
                                              const unsigned char* raw, float4* bufq, int first_warp = 0) {
  const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int warp = ((threadIdx.x >> 5) + nwarps - first_warp) % nwarps;   // rank from first_warp on
  const int n = meta->n;
  for (int i = warp; i < n; i += nwarps) {
    const int e = entry_slot(meta, i);
    const int4 si = src[e];   // (trace, lo, len, off)
    if (si.z <= 0) continue;
    float4* dst = bufq + (size_t)si.w * (lay_entry_bytes(LAY) / 16);
    const int roff = meta->raw[e];
    const float sc = P.storage == STORE_F32 ? 1.0f : meta->scale[e];
    const float* r32 = reinterpret_cast<const float*>(raw) + roff;
    const uint16_t* r16 = reinterpret_cast<const uint16_t*>(raw) + roff;
    const bool f16 = P.storage == STORE_F16;
    if constexpr (LAY == LAY_X3) {
      // the sample and difference planes
      float* S = reinterpret_cast<float*>(bufq) + si.w;
      for (int k = lane; k < si.z; k += 32) {
        float v[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (P.storage == STORE_F32) {
            v[u] = r32[k + u];
          } else {
            const uint32_t b = r16[k + u];
            v[u] = (f16 ? half_bits_to_float(b) : __uint_as_float(b << 16)) * sc;
          }
        }
        S[k] = v[0];
        S[kXPlane + k] = v[1] - v[0];
      }
      continue;
    }
    if constexpr (stage_lay(LAY) == LAY_FT) {
      // values pre-offset by the window's integer sample (absolute index lo + k + tau)
      float2* side = reinterpret_cast<float2*>(bufq + P.cap + kZeroSlots) + si.w;
      for (int k = lane; k < si.z; k += 32) {
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (P.storage == STORE_F32) {
            v[u] = r32[k + u];
          } else {
            const uint32_t b = r16[k + u];
            v[u] = (f16 ? half_bits_to_float(b) : __uint_as_float(b << 16)) * sc;
          }
        }
        const float it = (float)(si.y + k + P.tau);
        const float d0 = v[1] - v[0], d1 = v[2] - v[1], d2 = v[3] - v[2];
        dst[k] = make_float4(fmaf(-it, d0, v[0]), fmaf(-it, d2, v[2]), d0, d2);
        side[k] = make_float2(fmaf(-it, d1, v[1]), d1);
      }
      continue;
    }
    for (int k = lane; k < si.z; k += 32) {
      float v[4];
#pragma unroll
      for (int u = 0; u < (LAY == LAY_SD ? 3 : 4); ++u) {
        if (P.storage == STORE_F32) {
          v[u] = r32[k + u];
        } else {
          const uint32_t b = r16[k + u];
          v[u] = (f16 ? half_bits_to_float(b) : __uint_as_float(b << 16)) * sc;
        }
      }
      constexpr int SL = stage_lay(LAY);
      dst[k] = SL == LAY_SD   ? make_float4(v[0], v[1] - v[0], v[1], v[2] - v[1])
               : SL == LAY_P2 ? make_float4(v[0], v[2], v[1], v[3])
               : (SL == LAY_PD || SL == LAY_PD5) ? make_float4(v[0], v[2], v[1] - v[0], v[3] - v[2])
                                                 : make_float4(v[0], v[1], v[2], v[3]);
      if constexpr (SL == LAY_PD5) {
        // side entry (s_k, d_k), after the main entries and their zero block
        reinterpret_cast<float2*>(bufq + P.cap + kZeroSlots)[si.w + k] = make_float2(v[0], v[1] - v[0]);
      }
    }
  }
}

// Bounded wait on a barrier phase; false when it did not complete within limit_ns.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t_start = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t_start > limit_ns) return false;
  }
  return true;
}

// Shared-memory vector loads at a 32-bit shared address.
__device__ __forceinline__ float4 lds128(uint32_t a) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}

__device__ __forceinline__ float lds32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
  return v;
}

__device__ __forceinline__ float2 lds64(uint32_t a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}

// Samples s[0..W] of a window starting at entry address `a` (quad layout).
template <int W>
__device__ __forceinline__ void load_window(uint32_t a, float (&sv)[W + 1]) {
#pragma unroll
  for (int i = 0; i < (W + 1) / 4; ++i) {
    const float4 q = lds128(a + 64u * i);
    sv[4 * i] = q.x;
    sv[4 * i + 1] = q.y;
    sv[4 * i + 2] = q.z;
    sv[4 * i + 3] = q.w;
  }
  if ((W + 1) % 4 == 2) {
    const float2 q = lds64(a + 64u * ((W + 1) / 4));
    sv[W - 1] = q.x;
    sv[W] = q.y;
  }
}

// ---------------------------------------------------------------------------
// item state

template <int W>
struct PlainAcc {
  float num[W];
  float den, lin;
  int M;
};

// Fast form: sums of one item.  den_c is the energy of the current chunk; the
// Kahan-compensated total and its compensation live in shared memory
// (kahan_hi/lo).  add(a, x) folds in the window at entry address a with
// interpolation weight x, in the staging layout LAY.
template <int W, int LAY>
struct FastAcc {
  float num[W];
  float den_c;
  int M;

  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int j = 0; j < W; ++j) num[j] = 0.f;
    den_c = 0.f;
    M = 0;
  }
  __device__ __forceinline__ void add(uint32_t a, float x) {
    if constexpr (LAY == LAY_SD) {
      // entries (s_k, d_k, s_k+1, d_k+1): v_j = s_j + x * d_j
#pragma unroll
      for (int p = 0; p < W / 2; ++p) {
        const float4 ev = lds128(a + 32u * p);
        const float v0 = fmaf(ev.y, x, ev.x);
        const float v1 = fmaf(ev.w, x, ev.z);
        num[2 * p] += v0;
        num[2 * p + 1] += v1;
        den_c = fmaf(v0, v0, den_c);
        den_c = fmaf(v1, v1, den_c);
      }
      if (W & 1) {
        const float2 ev = lds64(a + 16u * (W - 1));
        const float v = fmaf(ev.y, x, ev.x);
        num[W - 1] += v;
        den_c = fmaf(v, v, den_c);
      }
    } else {
      float sv[W + 1];
      load_window<W>(a, sv);
#pragma unroll
      for (int j = 0; j < W; ++j) {
        const float v = fmaf(sv[j + 1] - sv[j], x, sv[j]);
        num[j] += v;
        den_c = fmaf(v, v, den_c);
      }
    }
  }
  // the same arithmetic on the window samples sv[0..W] of the FP32 store, for a
  // trace whose window was not staged (the staged entries hold the same values)
  __device__ __forceinline__ void add_samples(const float* sv, float x) {
#pragma unroll
    for (int j = 0; j < W; ++j) {
      const float v = fmaf(sv[j + 1] - sv[j], x, sv[j]);
      num[j] += v;
      den_c = fmaf(v, v, den_c);
    }
  }
  __device__ __forceinline__ float take_energy() {
    const float e = den_c;
    den_c = 0.f;
    return e;
  }
  __device__ __forceinline__ void sums(float& acsq, float& lin) const {
    acsq = 0.f;
    lin = 0.f;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      acsq = fmaf(num[j], num[j], acsq);
      lin += num[j];
    }
  }
};

// Packed layout: entry k = (s_k, s_k+2, s_k+1, s_k+3), so that window samples j
// and j+2 of an item are one FP32x2 operation: (v_j, v_j+2) = lo + x * (hi - lo)
// with lo = (s_j, s_j+2), hi = (s_j+1, s_j+3).  Window samples 4q..4q+3 use
// entries k+4q (pairs (4q, 4q+2)) and k+4q+2 (pairs (4q+1, 4q+3)); the one
// sample left over (W is odd) is done in scalar arithmetic.
template <int W, bool SV>
struct P2Acc {
  static constexpr int NP = (W - 1) / 2 > 0 ? (W - 1) / 2 : 1;
  float2 np[NP];   // packed sums (num_j, num_j+2)
  float ns;        // sum of the unpaired window sample
  float2 den2;     // energy of the current chunk, two partial sums
  int M;

  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int i = 0; i < NP; ++i) np[i] = make_float2(0.f, 0.f);
    ns = 0.f;
    den2 = make_float2(0.f, 0.f);
    M = 0;
  }
  __device__ __forceinline__ void pair(int i, float2 lo, float2 hi, float2 xx) {
    const float2 d = __ffma2_rn(lo, make_float2(-1.f, -1.f), hi);   // hi - lo, exact as a subtraction
    const float2 v = SV ? make_float2(fmaf(d.x, xx.x, lo.x), fmaf(d.y, xx.x, lo.y)) : __ffma2_rn(d, xx, lo);
    np[i] = __fadd2_rn(np[i], v);
    den2 = __ffma2_rn(v, v, den2);
  }
  __device__ __forceinline__ void single(float s0, float s1, float x) {
    const float v = fmaf(s1 - s0, x, s0);
    ns += v;
    den2.x = fmaf(v, v, den2.x);
  }
  __device__ __forceinline__ void add(uint32_t a, float x) {
    const float2 xx = make_float2(x, x);
    float4 B = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; 4 * q < W; ++q) {
      const int j0 = 4 * q;
      if (j0 + 1 == W && q > 0) {
        // last sample j0 = W-1: s_j0 and s_j0+1 are in the previous group's entry k+j0-2
        single(B.y, B.w, x);
        break;
      }
      const float4 A = lds128(a + 64u * q);   // (s_j0, s_j0+2, s_j0+1, s_j0+3)
      if (j0 + 2 < W) pair(2 * q, make_float2(A.x, A.y), make_float2(A.z, A.w), xx);
      if (j0 + 3 < W) {
        B = lds128(a + 64u * q + 32u);        // (s_j0+2, s_j0+4, s_j0+3, s_j0+5)
        pair(2 * q + 1, make_float2(A.z, A.w), make_float2(B.x, B.y), xx);
      } else if (j0 + 3 == W) {
        single(A.z, A.y, x);                  // sample j0+1: s_j0+1, s_j0+2
      } else if (j0 + 1 == W) {
        single(A.x, A.z, x);                  // W = 1
      }
    }
  }
  // add() on window samples sv[0..W] of the FP32 store (sv zero past W)
  __device__ __forceinline__ void add_samples(const float* sv, float x) {
    const float2 xx = make_float2(x, x);
    float4 B = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; 4 * q < W; ++q) {
      const int j0 = 4 * q;
      if (j0 + 1 == W && q > 0) {
        single(B.y, B.w, x);
        break;
      }
      const float4 A = make_float4(sv[j0], sv[j0 + 2], sv[j0 + 1], sv[j0 + 3]);
      if (j0 + 2 < W) pair(2 * q, make_float2(A.x, A.y), make_float2(A.z, A.w), xx);
      if (j0 + 3 < W) {
        B = make_float4(sv[j0 + 2], sv[j0 + 4], sv[j0 + 3], sv[j0 + 5]);
        pair(2 * q + 1, make_float2(A.z, A.w), make_float2(B.x, B.y), xx);
      } else if (j0 + 3 == W) {
        single(A.z, A.y, x);
      } else if (j0 + 1 == W) {
        single(A.x, A.z, x);
      }
    }
  }
  __device__ __forceinline__ float take_energy() {
    const float e = den2.x + den2.y;
    den2 = make_float2(0.f, 0.f);
    return e;
  }
  __device__ __forceinline__ void sums(float& acsq, float& lin) const {
    acsq = fmaf(ns, ns, 0.f);
    lin = ns;
#pragma unroll
    for (int i = 0; i < (W - 1) / 2; ++i) {
      acsq = fmaf(np[i].x, np[i].x, acsq);
      acsq = fmaf(np[i].y, np[i].y, acsq);
      lin += np[i].x + np[i].y;
    }
  }
};

template <int W>
struct FastAcc<W, LAY_P2> : P2Acc<W, false> {};
template <int W>
struct FastAcc<W, LAY_P2S> : P2Acc<W, true> {};

// Packed values with their differences (w = 3): entry k = (s_k, s_k+2, d_k, d_k+2),
// d_j = s_j+1 - s_j.  Window samples 0 and 2 are one FP32x2 FMA without forming the
// differences; sample 1 takes s_1 = s_0 + d_0 (within a rounding of the stored value)
// and d_1 = s_2 - s_1.
template <int W, bool SV>
struct PDAcc {
  static_assert(W == 3, "the packed value/difference layout is for w = 3");
  float2 np;     // (num_0, num_2)
  float ns;      // num_1
  float2 den2;   // energy of the current chunk, two partial sums
  int M;

  __device__ __forceinline__ void reset() {
    np = make_float2(0.f, 0.f);
    ns = 0.f;
    den2 = make_float2(0.f, 0.f);
    M = 0;
  }
  __device__ __forceinline__ void add(uint32_t a, float x) { acc(lds128(a), x); }
  // window numerators computed elsewhere (the central traces' sums of a Z0 kernel)
  __device__ __forceinline__ void add_sums(float n0, float n1, float n2) {
    np = __fadd2_rn(np, make_float2(n0, n2));
    ns += n1;
  }
  // add() on window samples sv[0..3] of the FP32 store
  __device__ __forceinline__ void add_samples(const float* sv, float x) {
    acc(make_float4(sv[0], sv[2], sv[1] - sv[0], sv[3] - sv[2]), x);
  }
  __device__ __forceinline__ void acc(const float4 A, float x) {   // A = (s_0, s_2, d_0, d_2)
    const float2 v = SV ? make_float2(fmaf(A.z, x, A.x), fmaf(A.w, x, A.y))
                        : __ffma2_rn(make_float2(A.z, A.w), make_float2(x, x), make_float2(A.x, A.y));
    np = __fadd2_rn(np, v);
    den2 = __ffma2_rn(v, v, den2);
    const float s1 = A.x + A.z;
    const float v1 = fmaf(A.y - s1, x, s1);
    ns += v1;
    den2.x = fmaf(v1, v1, den2.x);
  }
  __device__ __forceinline__ float take_energy() {
    const float e = den2.x + den2.y;
    den2 = make_float2(0.f, 0.f);
    return e;
  }
  __device__ __forceinline__ void sums(float& acsq, float& lin) const {
    acsq = fmaf(np.x, np.x, fmaf(np.y, np.y, ns * ns));
    lin = np.x + np.y + ns;
  }
};

template <int W>
struct FastAcc<W, LAY_PD> : PDAcc<W, false> {};
template <int W>
struct FastAcc<W, LAY_PDS> : PDAcc<W, true> {};

// w = 5 with side entries (LAY_PD5): the window at main entry address a, A = (s_0,
// s_2, d_0, d_2), and side entry address b of entry k+4, B = (s_4, d_4).  Window
// samples (0, 2) interpolate straight from A; (s_1, s_3) = (s_0, s_2) + (d_0, d_2)
// (within a rounding of the stored values), (d_1, d_3) = (s_2 - s_1, s_4 - s_3);
// sample 4 from B.
template <int W, bool SV>
struct PD5Acc {
  static_assert(W == 5, "the side-entry layout is for w = 5");
  float2 np02, np13;   // (num_0, num_2), (num_1, num_3)
  float ns;            // num_4
  float2 den2;         // energy of the current chunk, two partial sums
  int M;

  __device__ __forceinline__ void reset() {
    np02 = np13 = make_float2(0.f, 0.f);
    ns = 0.f;
    den2 = make_float2(0.f, 0.f);
    M = 0;
  }
  __device__ __forceinline__ void add_side(uint32_t a, uint32_t b, float x) { acc(lds128(a), lds64(b), x); }
  // the same sums from window samples sv[0..5] of the FP32 store
  __device__ __forceinline__ void add_samples(const float* sv, float x) {
    acc(make_float4(sv[0], sv[2], sv[1] - sv[0], sv[3] - sv[2]), make_float2(sv[4], sv[5] - sv[4]), x);
  }
  __device__ __forceinline__ void acc(const float4 A, const float2 B, float x) {
    const float2 v02 = SV ? make_float2(fmaf(A.z, x, A.x), fmaf(A.w, x, A.y))
                          : __ffma2_rn(make_float2(A.z, A.w), make_float2(x, x), make_float2(A.x, A.y));
    const float2 s13 = __fadd2_rn(make_float2(A.x, A.y), make_float2(A.z, A.w));
    const float2 d13 = make_float2(A.y - s13.x, B.x - s13.y);
    const float2 v13 = SV ? make_float2(fmaf(d13.x, x, s13.x), fmaf(d13.y, x, s13.y))
                          : __ffma2_rn(d13, make_float2(x, x), s13);
    const float v4 = fmaf(B.y, x, B.x);
    np02 = __fadd2_rn(np02, v02);
    np13 = __fadd2_rn(np13, v13);
    ns += v4;
    den2 = __ffma2_rn(v02, v02, den2);
    den2 = __ffma2_rn(v13, v13, den2);
    den2.x = fmaf(v4, v4, den2.x);
  }
  __device__ __forceinline__ float take_energy() {
    const float e = den2.x + den2.y;
    den2 = make_float2(0.f, 0.f);
    return e;
  }
  __device__ __forceinline__ void sums(float& acsq, float& lin) const {
    acsq = fmaf(np02.x, np02.x, fmaf(np02.y, np02.y, fmaf(np13.x, np13.x, fmaf(np13.y, np13.y, ns * ns))));
    lin = np02.x + np02.y + np13.x + np13.y + ns;
  }
};

template <int W>
struct FastAcc<W, LAY_PD5> : PD5Acc<W, false> {};
template <int W>
struct FastAcc<W, LAY_PD5S> : PD5Acc<W, true> {};

// Pre-offset values (LAY_FT, w = 3): the window at main entry address a and side
// entry address b, interpolated at traveltime t (samples): v_j = F_j + t d_j.
template <int W>
struct FastAcc<W, LAY_FT> {
  static_assert(W == 3, "the pre-offset layout is for w = 3");
  float2 np;     // (num_0, num_2)
  float ns;      // num_1
  float2 den2;   // energy of the current chunk, two partial sums
  int M;

  __device__ __forceinline__ void reset() {
    np = make_float2(0.f, 0.f);
    ns = 0.f;
    den2 = make_float2(0.f, 0.f);
    M = 0;
  }
  __device__ __forceinline__ void add_ft(uint32_t a, uint32_t b, float t) {
    const float4 A = lds128(a);   // (F_0, F_2, d_0, d_2)
    const float2 B = lds64(b);    // (F_1, d_1)
    const float2 v = make_float2(fmaf(A.z, t, A.x), fmaf(A.w, t, A.y));
    const float v1 = fmaf(B.y, t, B.x);
    np = __fadd2_rn(np, v);
    den2 = __ffma2_rn(v, v, den2);
    ns += v1;
    den2.x = fmaf(v1, v1, den2.x);
  }
  // the same sums from window samples sv[0..3] at weight x (a path the variants of
  // this layout do not take: they stage every window)
  __device__ __forceinline__ void add_samples(const float* sv, float x) {
    const float v0 = fmaf(sv[1] - sv[0], x, sv[0]), v1 = fmaf(sv[2] - sv[1], x, sv[1]);
    const float v2 = fmaf(sv[3] - sv[2], x, sv[2]);
    np = __fadd2_rn(np, make_float2(v0, v2));
    den2 = __ffma2_rn(make_float2(v0, v2), make_float2(v0, v2), den2);
    ns += v1;
    den2.x = fmaf(v1, v1, den2.x);
  }
  __device__ __forceinline__ float take_energy() {
    const float e = den2.x + den2.y;
    den2 = make_float2(0.f, 0.f);
    return e;
  }
  __device__ __forceinline__ void sums(float& acsq, float& lin) const {
    acsq = fmaf(np.x, np.x, fmaf(np.y, np.y, ns * ns));
    lin = np.x + np.y + ns;
  }
};




// The RC item accumulators of one thread.  For the 16-byte and side-entry layouts
// an array of FastAcc, one per item; set[r] is item r.
template <int W, int LAY, int RC>
struct AccSet {
  FastAcc<W, LAY> a[RC];
  __device__ __forceinline__ FastAcc<W, LAY>& operator[](int r) { return a[r]; }
};

// LAY_X3 (w = 3): the sums of items 2p and 2p+1 share FP32x2 registers, item 2p in
// lane .x and item 2p+1 in lane .y.  add_pair() folds in one trace for both items of
// pair p with packed arithmetic throughout: (s_1, d_1) are rebuilt as s_1 = s_0 + d_0
// and d_1 = s_2 - s_1, as in LAY_PD.  set[r] is a view of item r with the per-item
// interface of FastAcc (scalar arithmetic on its lane), for the partly-in-range traces
// and the odd item of an odd RC.
template <int RC>
struct AccSet<3, LAY_X3, RC> {
  static constexpr int RP = (RC + 1) / 2;
  static constexpr uint32_t kD = 4u * kXPlane;   // bytes from a sample to its difference
  float2 n0[RP], n1[RP], n2[RP], den[RP];
  int Ms[RC];

  struct Item {
    AccSet& s;
    const int r;
    int& M;
    __device__ __forceinline__ float& lanev(float2& v) const { return (r & 1) ? v.y : v.x; }
    __device__ __forceinline__ void reset() const {
      lanev(s.n0[r >> 1]) = 0.f;
      lanev(s.n1[r >> 1]) = 0.f;
      lanev(s.n2[r >> 1]) = 0.f;
      lanev(s.den[r >> 1]) = 0.f;
      M = 0;
    }
    __device__ __forceinline__ void acc(float s0, float s2, float d0, float d2, float x) const {
      const float v0 = fmaf(d0, x, s0), v2 = fmaf(d2, x, s2);
      const float s1 = s0 + d0;
      const float v1 = fmaf(s2 - s1, x, s1);
      float& e = lanev(s.den[r >> 1]);
      lanev(s.n0[r >> 1]) += v0;
      lanev(s.n1[r >> 1]) += v1;
      lanev(s.n2[r >> 1]) += v2;
      e = fmaf(v0, v0, e);
      e = fmaf(v1, v1, e);
      e = fmaf(v2, v2, e);
    }
    // the window at sample address a (sample plane) with weight x
    __device__ __forceinline__ void add(uint32_t a, float x) const {
      acc(lds32(a), lds32(a + 8u), lds32(a + kD), lds32(a + kD + 8u), x);
    }
    __device__ __forceinline__ void add_samples(const float* sv, float x) const {
      acc(sv[0], sv[2], sv[1] - sv[0], sv[3] - sv[2], x);
    }
    __device__ __forceinline__ float take_energy() const {
      float& e = lanev(s.den[r >> 1]);
      const float v = e;
      e = 0.f;
      return v;
    }
    __device__ __forceinline__ void sums(float& acsq, float& lin) const {
      const float a0 = lanev(s.n0[r >> 1]), a1 = lanev(s.n1[r >> 1]), a2 = lanev(s.n2[r >> 1]);
      acsq = fmaf(a0, a0, fmaf(a2, a2, a1 * a1));
      lin = a0 + a1 + a2;
    }
  };
  __device__ __forceinline__ Item operator[](int r) { return Item{*this, r, Ms[r]}; }

  // one trace for items 2p (window at a0) and 2p+1 (at a1), weights x = (x_2p, x_2p+1)
  __device__ __forceinline__ void add_pair(int p, uint32_t a0, uint32_t a1, float2 x) {
    const float2 s0 = make_float2(lds32(a0), lds32(a1));
    const float2 s2 = make_float2(lds32(a0 + 8u), lds32(a1 + 8u));
    const float2 d0 = make_float2(lds32(a0 + kD), lds32(a1 + kD));
    const float2 d2 = make_float2(lds32(a0 + kD + 8u), lds32(a1 + kD + 8u));
    const float2 v0 = __ffma2_rn(d0, x, s0);
    const float2 v2 = __ffma2_rn(d2, x, s2);
    const float2 s1 = __fadd2_rn(s0, d0);
    const float2 d1 = __ffma2_rn(s1, make_float2(-1.f, -1.f), s2);   // s_2 - s_1, exact as a subtraction
    const float2 v1 = __ffma2_rn(d1, x, s1);
    n0[p] = __fadd2_rn(n0[p], v0);
    n1[p] = __fadd2_rn(n1[p], v1);
    n2[p] = __fadd2_rn(n2[p], v2);
    den[p] = __ffma2_rn(v0, v0, den[p]);
    den[p] = __ffma2_rn(v1, v1, den[p]);
    den[p] = __ffma2_rn(v2, v2, den[p]);
  }
};

// Batched form: the items of one thread on a trace whose window was not staged
// (kGlobalEntry): the traveltime as on the staged traces, then the window samples
// from the FP32 store in global memory, checked against the record's ends.
template <int METHOD, bool BRUN, int W, int LAY, int RC, int RP>
__device__ __forceinline__ void global_entry(const KParams& P, int tr, float4 g, float q0, float Tsmp, float T2smp,
                                             unsigned span, const float2 (&ca2)[RP], const float2 (&cb2)[RP],
                                             const float2 (&cc2)[RP], FastAcc<W, LAY> (&fa)[RC]) {
  const float* row = P.samples + (int64_t)tr * P.pitch;
#pragma unroll
  for (int r = 0; r < RC; ++r) {
    const float ca = (r & 1) ? ca2[r >> 1].y : ca2[r >> 1].x;
    const float cb = (r & 1) ? cb2[r >> 1].y : cb2[r >> 1].x;
    const float cc = (r & 1) ? cc2[r >> 1].y : cc2[r >> 1].x;
    float t2;
    if (METHOD == METHOD_CMP) {
      t2 = fmaf(cc, g.z, T2smp);
    } else if (BRUN) {
      t2 = fmaf(cb, g.y, q0);
    } else {
      const float u = fmaf(ca, g.x, Tsmp);
      t2 = fmaf(u, u, fmaf(cb, g.y, cc * g.z));
    }
    const float t = sqrt_fast(t2);   // NaN for t2 < 0: out of range below
    const float y = __fadd_rz(t, 8388608.0f);
    const int rel = __float_as_int(y) - (0x4B000000 + P.tau);   // it - tau
    const bool ok = (unsigned)rel <= span;
    const float x = ok ? t - (y - 8388608.0f) : 0.0f;
    float sv[W + 8];
#pragma unroll
    for (int i = 0; i < W + 8; ++i) sv[i] = (ok && i <= W) ? __ldg(row + rel + i) : 0.f;
    fa[r].add_samples(sv, x);
    fa[r].M += ok ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// The search kernel.

// GLOB: the variant may stage less than a whole trace; windows larger than its
// buffer are read from the FP32 store (kGlobalEntry).  Without it the plan gives
// the variant a buffer that holds any window, and the path is not compiled (it
// costs registers in the partly-in-range loop).
// XP (batched form): the chunk stream runs on across passes and tasks.  While the
// warps compute the last chunk of a pass, warp 0 plans the first chunk of the next
// pass, or, after the last pass, takes the next task from the queue and plans its
// first chunk, so that its copies land during that computation; without XP every
// pass starts by planning its first chunk and waiting for its copies.
template <int METHOD, int FORM, int W, int RC, int MINB, int LAY, bool BRUN, int NT, bool GLOB = false,
          bool XP = false>
__global__ void __launch_bounds__(NT, MINB) semb_search_kernel(KParams P) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const SmemLayout L = smem_layout(FORM, RC, P.cap, P.storage, NT, LAY);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);   // [2]
  int* ctl = reinterpret_cast<int*>(smem_raw + 16);
  ChunkMeta* metas = reinterpret_cast<ChunkMeta*>(smem_raw + L.meta);   // [2], stride kMetaBytes
  int4* srcs = reinterpret_cast<int4*>(smem_raw + L.src);               // [2][kMaxChunk]
  // running top-K per thread, [K][NT] (semblance, grid index, stack)
  constexpr int K = (FORM == FORM_FAST) ? kTopK : 1;
  float* top_s = reinterpret_cast<float*>(smem_raw + L.tops);
  int* top_i = reinterpret_cast<int*>(top_s + K * NT);
  float* top_k = top_s + 2 * K * NT;
  float* kahan_hi = reinterpret_cast<float*>(smem_raw + L.kahan);   // fast form: [RC][NT]
  float* kahan_lo = kahan_hi + RC * NT;
  float* buf = reinterpret_cast<float*>(smem_raw + L.buf);
  float4* bufq = reinterpret_cast<float4*>(buf);
  auto raw_at = [&](int i) { return smem_raw + L.raw0 + (size_t)i * (L.raw1 - L.raw0); };
  const uint32_t bufq_addr = smem_u32(bufq);
  auto meta_at = [&](int i) { return reinterpret_cast<ChunkMeta*>(reinterpret_cast<unsigned char*>(metas) + i * kMetaBytes); };
  ChunkMeta* meta = meta_at(0);
  int4* srcinfo = srcs;
  uint64_t* bar = bars;

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  constexpr float kSent = (METHOD == METHOD_CMP) ? -1.0f : 0.0f;

  // zero block read by out-of-range items
  if (FORM == FORM_PLAIN) {
    if (threadIdx.x < kZeroSlots) buf[P.cap + threadIdx.x] = 0.f;
  } else {
    if (threadIdx.x < kZeroSlots) bufq[P.cap + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lay_has_side(LAY) && threadIdx.x < kZeroSlots)   // the side entries' zero block
      reinterpret_cast<float2*>(bufq + P.cap + kZeroSlots)[P.cap + threadIdx.x] = make_float2(0.f, 0.f);
  }
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;    // plain form: parity of bars[0]
  uint32_t phases = 0;   // fast form: bit i = parity of bars[i]

  int task_iter = 0;
  // XP: the staging state carried from one pass (or task) to the next
  int cur = 0;             // buffer (meta, raw, barrier) of the next chunk
  bool pre = false;        // its first chunk is planned in buffer cur, copies issued
  bool task_pre = false;   // the next task was taken from the queue (ctl[0]); ctl[1]
                           // says whether its first chunk is planned
  for (;;) {
    int task;
    if (FORM == FORM_PLAIN) {
      if (task_iter > 0) break;
      task = blockIdx.x;
    } else {
      if (!(XP && task_pre)) {
        if (threadIdx.x == 0) ctl[0] = atomicAdd(P.counter, 1);
        __syncthreads();
      }
      task = ctl[0];
      pre = XP && task_pre && ctl[1] != 0;
      task_pre = false;
      __syncthreads();
    }
    ++task_iter;
    if (task >= P.ntasks) break;

    const int2 td = P.tasks[task];
    const int cdp = td.x;
    const int t0s = td.y;
    const int t0 = min(t0s + lane, P.ns - 1);
    const int t0hi = min(t0s + kTB - 1, P.ns - 1);
    const int64_t ap_begin = P.ap_off[cdp];
    const int64_t ap_end = P.ap_off[cdp + 1];
    const int napert = (int)(ap_end - ap_begin);
    const float T_lo = P.dt * (float)t0s;
    const float T_hi = P.dt * (float)t0hi;

    // per-thread running pick for this lane's t0: top-K in shared memory, the
    // admission threshold (the K-th entry) in registers
#pragma unroll
    for (int q = 0; q < K; ++q) {
      top_s[q * NT + threadIdx.x] = 0.f;
      top_i[q * NT + threadIdx.x] = 0x7fffffff;
      top_k[q * NT + threadIdx.x] = 0.f;
    }
    float last_s = 0.f;
    int last_i = 0x7fffffff;

    // per-lane time values
    const float Tsec = __fmul_rn(P.dt, (float)t0);            // reference: _t0 = dt * t0
    const float T2sec = __fmul_rn(Tsec, Tsec);                 // CMP: _t0 * _t0
    const float Tsmp = (float)t0;                              // fast form: sample units
    const float T2smp = Tsmp * Tsmp;
    const float2 Tsmp2 = make_float2(Tsmp, Tsmp);
    const float2 T2smp2 = make_float2(T2smp, T2smp);
    const float2 kTwo23x2 = make_float2(8388608.0f, 8388608.0f);
    const float2 kMinusTwo23x2 = make_float2(-8388608.0f, -8388608.0f);
    const float2 kMinusOne2 = make_float2(-1.0f, -1.0f);
    const float tau_lo = (float)P.tau;
    const float tau_hi = (float)(P.ns - P.tau - 1);
    const unsigned span = (unsigned)(P.ns - 2 * P.tau - 2);   // valid iff 0 <= it - tau <= span

    for (int pass = 0; pass < P.npass; ++pass) {
      const float* pb = P.pass_bounds + pass * 8;
      const float4* cand = P.cand + pass * P.cpp + warp * RC;
      // the thread's RC candidates as pairs (items r, r+1) for the packed FP32x2
      // traveltimes; an odd RC repeats its last candidate in the unused half
      constexpr int RP = (RC + 1) / 2;
      float2 ca2[RP], cb2[RP], cc2[RP];
#pragma unroll
      for (int r = 0; r < 2 * RP; ++r) {
        const float4 cv = cand[min(r, RC - 1)];
        if (r & 1) {
          ca2[r >> 1].y = cv.x;
          cb2[r >> 1].y = cv.y;
          cc2[r >> 1].y = cv.z;
        } else {
          ca2[r >> 1].x = cv.x;
          cb2[r >> 1].x = cv.y;
          cc2[r >> 1].x = cv.z;
        }
      }
      auto CA = [&](int r) { return (r & 1) ? ca2[r >> 1].y : ca2[r >> 1].x; };
      auto CB = [&](int r) { return (r & 1) ? cb2[r >> 1].y : cb2[r >> 1].x; };
      auto CC = [&](int r) { return (r & 1) ? cc2[r >> 1].y : cc2[r >> 1].x; };
      PlainAcc<W> pa[FORM == FORM_PLAIN ? RC : 1];
      FastAcc<W, LAY> fa[FORM == FORM_FAST ? RC : 1];
#pragma unroll
      for (int r = 0; r < RC; ++r) {
        if (FORM == FORM_PLAIN) {
#pragma unroll
          for (int j = 0; j < W; ++j) pa[r].num[j] = 0.f;
          pa[r].den = 0.f;
          pa[r].lin = 0.f;
          pa[r].M = 0;
        } else {
          fa[r].reset();
          kahan_hi[r * NT + threadIdx.x] = 0.f;
          kahan_lo[r * NT + threadIdx.x] = 0.f;
        }
      }

      // compute on a staged chunk (meta, n); the fast form then folds the chunk's
      // energy into the Kahan totals
      auto compute_chunk = [&](const ChunkMeta* meta, const int n, const int4* srcc) {
        if (FORM == FORM_PLAIN) {
          for (int e = 0; e < n; ++e) {
            const float4 g = meta->geo[e];
            const int soff = __float_as_int(g.w);
#pragma unroll
            for (int r = 0; r < RC; ++r) {
              float t;
              if (METHOD == METHOD_CMP) {
                t = __fmul_rn(__fsqrt_rn(__fadd_rn(T2sec, __fmul_rn(CC(r), g.z))), P.idt);
              } else {
                t = __fadd_rn(Tsec, __fmul_rn(CA(r), g.x));
                t = __fadd_rn(__fadd_rn(__fmul_rn(t, t), __fmul_rn(CB(r), g.y)), __fmul_rn(CC(r), g.z));
                t = (t < 0.0f) ? -1.0f : __fsqrt_rn(t);
                t = __fmul_rn(t, P.idt);
              }
              const bool ok = (t >= tau_lo) && (t < tau_hi);
              const float y = __fadd_rz(t, 8388608.0f);
              const int it = __float_as_int(y) - 0x4B000000;
              const float x = ok ? __fsub_rn(t, __fsub_rn(y, 8388608.0f)) : 0.0f;
              const unsigned idx = min(ok ? (unsigned)(soff + it - P.tau) : (unsigned)P.cap, (unsigned)P.cap);
              if constexpr (SEMB_CHECKED) {
                if (ok) report_window(P.status, soff + it - P.tau, W, srcc[e], cdp, t0);
              }
              const float* s = buf + idx;
              float s1 = s[0];
#pragma unroll
              for (int j = 0; j < W; ++j) {
                const float s0 = s1;
                s1 = s[j + 1];
                const float v = __fadd_rn(__fmul_rn(__fsub_rn(s1, s0), x), s0);
                pa[r].num[j] = __fadd_rn(pa[r].num[j], v);
                pa[r].den = __fadd_rn(pa[r].den, __fmul_rn(v, v));
                pa[r].lin = __fadd_rn(pa[r].lin, v);
              }
              pa[r].M += ok ? 1 : 0;
            }
          }
        } else {
          const int n_in = meta->n_in;
          const uint32_t top = bufq_addr + 16u * (uint32_t)P.cap;
          // side entries (LAY_PD5): the side entry of window sample W-1 of the item
          // at main entry address a is at a / 2 + side_shift
          const uint32_t side_shift =
              bufq_addr + 16u * (uint32_t)(P.cap + kZeroSlots) + 8u * (uint32_t)(W - 1) - (bufq_addr >> 1);
          // traces on which every item is in range: traveltimes of item pairs in
          // FP32x2, address = bits(t + 2^23) * 16 + base (mod 2^32), clamped to the
          // buffer as a guard
          for (int e = 0; e < n_in; ++e) {
            const float4 g = meta->geo[e];
            const uint32_t base = bufq_addr + 16u * (uint32_t)(__float_as_int(g.w) - P.tau) - 16u * 0x4B000000u;
            const float2 gx2 = make_float2(g.x, g.x), gy2 = make_float2(g.y, g.y), gz2 = make_float2(g.z, g.z);
            // B-run candidates share A and C: (t0 + A|dm|)^2 + C h once per trace
            float2 q02 = make_float2(0.f, 0.f);
            if (BRUN && METHOD == METHOD_CRS) {
              const float u0 = fmaf(CA(0), g.x, Tsmp);
              const float q0 = fmaf(u0, u0, CC(0) * g.z);
              q02 = make_float2(q0, q0);
            }
#pragma unroll
            for (int rp = 0; rp < RP; ++rp) {
              float2 t2;
              if (METHOD == METHOD_CMP) {
                t2 = __ffma2_rn(cc2[rp], gz2, T2smp2);
              } else if (BRUN) {
                t2 = __ffma2_rn(cb2[rp], gy2, q02);
              } else {
                const float2 u = __ffma2_rn(ca2[rp], gx2, Tsmp2);
                t2 = __ffma2_rn(u, u, __ffma2_rn(cb2[rp], gy2, __fmul2_rn(cc2[rp], gz2)));
              }
              const float2 t = make_float2(sqrt_fast(t2.x), sqrt_fast(t2.y));
              const float2 y = __fadd2_rz(t, kTwo23x2);
              const float2 x = __ffma2_rn(__fadd2_rn(y, kMinusTwo23x2), kMinusOne2, t);   // t - floor(t)
              if constexpr (SEMB_CHECKED) {
                const int i0 = __float_as_int(g.w) - P.tau - 0x4B000000;
                report_window(P.status, __float_as_int(y.x) + i0, W, srcc[e], cdp, t0);
                if (2 * rp + 1 < RC) report_window(P.status, __float_as_int(y.y) + i0, W, srcc[e], cdp, t0);
              }
              if constexpr (lay_has_side(LAY)) {
                const uint32_t a0 = min(__float_as_uint(y.x) * 16u + base, top);
                fa[2 * rp].add_side(a0, (a0 >> 1) + side_shift, x.x);
                if (2 * rp + 1 < RC) {
                  const uint32_t a1 = min(__float_as_uint(y.y) * 16u + base, top);
                  fa[2 * rp + 1].add_side(a1, (a1 >> 1) + side_shift, x.y);
                }
              } else {
                fa[2 * rp].add(min(__float_as_uint(y.x) * 16u + base, top), x.x);
                if (2 * rp + 1 < RC) fa[2 * rp + 1].add(min(__float_as_uint(y.y) * 16u + base, top), x.y);
              }
            }
          }
          // the other traces: per-item range checks; an out-of-range item reads the
          // zero block with weight 0 and does not count
          for (int e = kMaxChunk - (n - n_in); e < kMaxChunk; ++e) {
            const float4 g = meta->geo[e];
            const int soff = __float_as_int(g.w);
            float q0 = 0.f;
            if (BRUN && METHOD == METHOD_CRS) {
              const float u0 = fmaf(CA(0), g.x, Tsmp);
              q0 = fmaf(u0, u0, CC(0) * g.z);
            }
            if (GLOB && soff == kGlobalEntry) {
              global_entry<METHOD, BRUN>(P, meta->raw[e], g, q0, Tsmp, T2smp, span, ca2, cb2, cc2, fa);
              continue;
            }
#pragma unroll
            for (int r = 0; r < RC; ++r) {
              float t2;
              if (METHOD == METHOD_CMP) {
                t2 = fmaf(CC(r), g.z, T2smp);
              } else if (BRUN) {
                t2 = fmaf(CB(r), g.y, q0);
              } else {
                const float u = fmaf(CA(r), g.x, Tsmp);
                t2 = fmaf(u, u, fmaf(CB(r), g.y, CC(r) * g.z));
              }
              const float t = sqrt_fast(t2);   // NaN for t2 < 0: out of range below
              const float y = __fadd_rz(t, 8388608.0f);
              const int rel = __float_as_int(y) - (0x4B000000 + P.tau);   // it - tau
              const bool ok = (unsigned)rel <= span;
              const float x = ok ? t - (y - 8388608.0f) : 0.0f;
              const unsigned idx = min(ok ? (unsigned)(soff + rel) : (unsigned)P.cap, (unsigned)P.cap);
              if constexpr (SEMB_CHECKED) {
                if (ok) report_window(P.status, soff + rel, W, srcc[e], cdp, t0);
              }
              if constexpr (lay_has_side(LAY)) {
                const uint32_t a = bufq_addr + 16u * idx;
                fa[r].add_side(a, (a >> 1) + side_shift, x);
              } else {
                fa[r].add(bufq_addr + 16u * idx, x);
              }
              fa[r].M += ok ? 1 : 0;
            }
          }
#pragma unroll
          for (int r = 0; r < RC; ++r) {
            // in-range traces count for every item
            fa[r].M += n_in;
            // Kahan: fold this chunk's energy into the compensated total
            const int o = r * NT + threadIdx.x;
            const float hi = kahan_hi[o], lo = kahan_lo[o];
            const float yv = fa[r].take_energy() - lo;
            const float tv = hi + yv;
            kahan_lo[o] = (tv - hi) - yv;
            kahan_hi[o] = tv;
          }
        }
      };

      if (FORM == FORM_PLAIN) {
        int64_t ap_pos = ap_begin;
        while (ap_pos < ap_end) {
          if (warp == 0) {
            plan_chunk<METHOD, FORM>(P, pb, ap_pos, ap_end, T_lo, T_hi, meta, srcinfo);
            issue_chunk_copies(P, meta, srcinfo, buf, bar);
          }
          __syncthreads();
          const int n = meta->n;
          // wait for the bulk copies of this chunk; give up after kWaitNs
          const bool ok = wait_bar(bar, phase);
          phase ^= 1u;
          if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicOr(P.status, ST_TIMEOUT);
            return;
          }
          const int consumed = meta->consumed;
          compute_chunk(meta, n, srcinfo);
          ap_pos += consumed;
          __syncthreads();   // buffer and meta free for the next chunk
        }
      } else {
        // software pipeline: while all warps compute chunk c from the quad buffer,
        // the raw windows of chunk c+1 land in the other raw buffer by TMA
        if (!XP) cur = 0;
        if (!pre && ap_begin < ap_end) {
          if (warp == 0) {
            plan_chunk<METHOD, FORM>(P, pb, ap_begin, ap_end, T_lo, T_hi, meta_at(cur), srcs + cur * kMaxChunk);
            issue_raw(P, meta_at(cur), srcs + cur * kMaxChunk, raw_at(cur), bars + cur);
          }
          __syncthreads();
        }
        pre = false;
        int64_t ap_pos = ap_begin;
        while (ap_pos < ap_end) {
          ChunkMeta* mc = meta_at(cur);
          const int n = mc->n;
          // every thread observes the copies' completion itself; the timeout vote
          // rides on the barrier after the conversion
          const bool ok = wait_bar(bars + cur, (phases >> cur) & 1u);
          phases ^= 1u << cur;
          if (ok) convert_chunk<LAY>(P, mc, srcs + cur * kMaxChunk, raw_at(cur), bufq);
          if (__syncthreads_or(!ok)) {   // entries ready; raw buffer cur free
            if (threadIdx.x == 0) atomicOr(P.status, ST_TIMEOUT);
            return;
          }
          const int64_t next = ap_pos + mc->consumed;
          const bool last_pass = pass + 1 == P.npass;
          if (warp == 0) {
            ChunkMeta* mn = meta_at(cur ^ 1);
            int4* sn = srcs + (cur ^ 1) * kMaxChunk;
            if (next < ap_end) {
              plan_chunk<METHOD, FORM>(P, pb, next, ap_end, T_lo, T_hi, mn, sn);
              issue_raw(P, mn, sn, raw_at(cur ^ 1), bars + (cur ^ 1));
            } else if (XP && !last_pass) {
              // the first chunk of the next pass of this task
              plan_chunk<METHOD, FORM>(P, pb + 8, ap_begin, ap_end, T_lo, T_hi, mn, sn);
              issue_raw(P, mn, sn, raw_at(cur ^ 1), bars + (cur ^ 1));
            } else if (XP) {
              // the next task and, if it has aperture traces, its first chunk
              int tn = 0;
              if (lane == 0) tn = atomicAdd(P.counter, 1);
              tn = __shfl_sync(0xffffffffu, tn, 0);
              int planned = 0;
              if (tn < P.ntasks) {
                const int2 tdn = P.tasks[tn];
                const int64_t b = P.ap_off[tdn.x], e = P.ap_off[tdn.x + 1];
                if (b < e) {
                  const float tl = P.dt * (float)tdn.y, th = P.dt * (float)min(tdn.y + kTB - 1, P.ns - 1);
                  plan_chunk<METHOD, FORM>(P, P.pass_bounds, b, e, tl, th, mn, sn);
                  issue_raw(P, mn, sn, raw_at(cur ^ 1), bars + (cur ^ 1));
                  planned = 1;
                }
              }
              if (lane == 0) {
                ctl[0] = tn;
                ctl[1] = planned;
              }
            }
          }
          compute_chunk(mc, n, srcs + cur * kMaxChunk);
          __syncthreads();   // quad buffer free; the next chunk's metadata visible
          ap_pos = next;
          cur ^= 1;
          if (XP && next >= ap_end) {
            pre = !last_pass;
            task_pre = last_pass;
          }
        }
      }

      // finalize the pass's items and fold them into this lane's pick
#pragma unroll
      for (int r = 0; r < RC; ++r) {
        float sem, stk;
        if (FORM == FORM_PLAIN) {
          float acsq = 0.f;
#pragma unroll
          for (int j = 0; j < W; ++j) acsq = __fadd_rn(acsq, __fmul_rn(pa[r].num[j], pa[r].num[j]));
          const float mf = (float)pa[r].M;
          const int err = napert - pa[r].M;
          const bool ok = (pa[r].den > kEpsilonF) && (mf > kEpsilonF) && (err < 2);
          sem = ok ? __fdiv_rn(acsq, __fmul_rn(pa[r].den, mf)) : kSent;
          stk = ok ? __fdiv_rn(pa[r].lin, __fmul_rn((float)W, mf)) : kSent;
        } else {
          float acsq, lin;
          fa[r].sums(acsq, lin);
          const float den = kahan_hi[r * NT + threadIdx.x] - kahan_lo[r * NT + threadIdx.x];
          const float mf = (float)fa[r].M;
          const int err = napert - fa[r].M;
          const bool ok = (den > kEpsilonF) && (fa[r].M > 0) && (err < 2);
          sem = ok ? __fdividef(acsq, den * mf) : kSent;
          stk = ok ? __fdividef(lin, (float)W * mf) : kSent;
        }
        const int idx = __float_as_int(cand[r].w);   // -1: padding slot
        if (idx >= 0 && sem > 0.f && better(sem, idx, last_s, last_i)) {
          // sorted insert (descending semblance, ascending index)
          float cs = sem, ck = stk;
          int cidx = idx;
#pragma unroll
          for (int q = 0; q < K; ++q) {
            const int o = q * NT + threadIdx.x;
            const float bs = top_s[o];
            const int bi = top_i[o];
            if (better(cs, cidx, bs, bi)) {
              const float bk = top_k[o];
              top_s[o] = cs;
              top_i[o] = cidx;
              top_k[o] = ck;
              cs = bs;
              cidx = bi;
              ck = bk;
            }
          }
          last_s = top_s[(K - 1) * NT + threadIdx.x];
          last_i = top_i[(K - 1) * NT + threadIdx.x];
        }
      }
    }

    // reduce the picks of all warps for each t0 (lane): warp 0 reads every warp's
    // lists from shared memory
    __syncthreads();
    if (warp == 0) {
      float fs[K], fk[K];
      int fi[K];
#pragma unroll
      for (int q = 0; q < K; ++q) {
        fs[q] = 0.f;
        fi[q] = 0x7fffffff;
        fk[q] = 0.f;
      }
      for (int w2 = 0; w2 < nwarps; ++w2) {
        for (int q2 = 0; q2 < K; ++q2) {
          float cs = top_s[q2 * NT + w2 * 32 + lane];
          int cidx = top_i[q2 * NT + w2 * 32 + lane];
          float ck = top_k[q2 * NT + w2 * 32 + lane];
          if (!(cs > 0.f)) continue;
#pragma unroll
          for (int q = 0; q < K; ++q) {
            if (better(cs, cidx, fs[q], fi[q])) {
              const float ts = fs[q], tk = fk[q];
              const int ti = fi[q];
              fs[q] = cs;
              fi[q] = cidx;
              fk[q] = ck;
              cs = ts;
              cidx = ti;
              ck = tk;
            }
          }
        }
      }
      const int tt = t0s + lane;
      if (tt < P.ns) {
        const int64_t o = (int64_t)cdp * P.ns + tt;
        if (FORM == FORM_PLAIN) {
          if (fs[0] > 0.f) {
            P.ctr[o] = fi[0];
            P.str[o] = fs[0];
            P.stk[o] = fk[0];
          } else {
            // no candidate above 0: CMP ctr -1, stack 0 (CMP main.cpp:219-221);
            // CRS ctr 0 and the stack of item (t0 = 0, candidate 0) (CRS main.cpp:282-284)
            P.ctr[o] = (METHOD == METHOD_CMP) ? -1 : 0;
            P.str[o] = 0.f;
            P.stk[o] = (METHOD == METHOD_CMP) ? 0.f : P.stt00[cdp];
          }
        } else {
#pragma unroll
          for (int q = 0; q < K; ++q) {
            P.top_sem[o * kTopK + q] = fs[q];
            P.top_idx[o * kTopK + q] = fs[q] > 0.f ? fi[q] : -1;
            P.top_stk[o * kTopK + q] = fk[q];
          }
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace semb
