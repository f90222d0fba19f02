// Device-side set-up and post-processing kernels of a plan:
//  * per-trace geometry in the reference's single- and double-precision arithmetic;
//  * per-CDP neighbour lists within apm (CRS) and per-CDP aperture lists;
//  * the 16-bit trace store with a per-trace scale;
//  * the CRS "no pick" stack (item t0 = 0, candidate 0);
//  * the FP64 re-pick of the top-4 candidates per (CDP, t0).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "semb_kernels.cuh"

namespace semb {

struct alignas(32) Geo64 {
  double m, m2, h, pad;
};

// Per-trace geometry.  Single precision follows the reference's float build
// (CRS/OpenMP/src/main.cpp:163-177 with real = float; CMP/OpenMP/src/main.cpp:
// 125-136), double precision its double build; every operation is rounded on its
// own (no contraction).  Outputs: h = half-offset^2 / 1e6, midpoint x/y.
static __global__ void k_trace_geometry(int64_t ntr, const int32_t* __restrict__ gx, const int32_t* __restrict__ gy,
                                 const int32_t* __restrict__ sx, const int32_t* __restrict__ sy,
                                 const int32_t* __restrict__ scalco, float* __restrict__ h32,
                                 float* __restrict__ mx32, float* __restrict__ my32, double* __restrict__ h64,
                                 double* __restrict__ mx64, double* __restrict__ my64) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ntr; i += (int64_t)gridDim.x * blockDim.x) {
    const float gxf = __int2float_rn(gx[i]), gyf = __int2float_rn(gy[i]);
    const float sxf = __int2float_rn(sx[i]), syf = __int2float_rn(sy[i]);
    float s = __int2float_rn(scalco[i]);
    if (-1e-13 < (double)s && (double)s < 1e-13) s = 1.0f;
    else if (s < 0.0f) s = __fdiv_rn(1.0f, s);
    const float hx = __fmul_rn(__fsub_rn(gxf, sxf), s);
    const float hy = __fmul_rn(__fsub_rn(gyf, syf), s);
    const float hh = __fadd_rn(__fmul_rn(hx, hx), __fmul_rn(hy, hy));
    h32[i] = __double2float_rn(__ddiv_rn(__dmul_rn(0.25, (double)hh), 1e6));
    mx32[i] = __fmul_rn(__fmul_rn(__fadd_rn(gxf, sxf), s), 0.5f);
    my32[i] = __fmul_rn(__fmul_rn(__fadd_rn(gyf, syf), s), 0.5f);

    const double gxd = gx[i], gyd = gy[i], sxd = sx[i], syd = sy[i];
    double sd = (double)scalco[i];
    if (-1e-13 < sd && sd < 1e-13) sd = 1.0;
    else if (sd < 0.0) sd = __ddiv_rn(1.0, sd);
    const double hxd = __dmul_rn(__dsub_rn(gxd, sxd), sd);
    const double hyd = __dmul_rn(__dsub_rn(gyd, syd), sd);
    h64[i] = __ddiv_rn(__dmul_rn(0.25, __dadd_rn(__dmul_rn(hxd, hxd), __dmul_rn(hyd, hyd))), 1e6);
    mx64[i] = __dmul_rn(__dmul_rn(__dadd_rn(gxd, sxd), sd), 0.5);
    my64[i] = __dmul_rn(__dmul_rn(__dadd_rn(gyd, syd), sd), 0.5);
  }
}

// Midpoint of each CDP's first trace as su_trace::midpoint_x/y computes it
// (CRS/OpenMP/src/su_trace.cpp:70-80): fscalco() * (gx + sx) * 0.5 in float, with
// the coordinate sum taken in integers.
static __global__ void k_cdp_midpoints(int ncdps, const int64_t* __restrict__ cdp_end, const int32_t* __restrict__ gx,
                                const int32_t* __restrict__ gy, const int32_t* __restrict__ sx,
                                const int32_t* __restrict__ sy, const int32_t* __restrict__ scalco,
                                float* __restrict__ fmx, float* __restrict__ fmy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  const int64_t t = i > 0 ? cdp_end[i - 1] : 0;
  const int sc = scalco[t];
  const float fs = sc == 0 ? 1.0f : (sc > 0 ? (float)sc : __fdiv_rn(1.0f, (float)sc));
  fmx[i] = __fmul_rn(__fmul_rn(fs, __int2float_rn(gx[t] + sx[t])), 0.5f);
  fmy[i] = __fmul_rn(__fmul_rn(fs, __int2float_rn(gy[t] + sy[t])), 0.5f);
}

// Neighbour lists (CRS/OpenMP/src/su_gather.cpp:70-87): CDP j is a neighbour of
// CDP i when dx*dx + dy*dy <= apm*apm in float, dx = mid_j - mid_i.  Thread per i,
// j swept in ascending order through shared-memory tiles, so each list comes out
// in ascending j as in the reference.  Pass 1 counts (off == nullptr), pass 2
// writes at off[i].
static __global__ void k_neighbours(int ncdps, const float* __restrict__ fmx, const float* __restrict__ fmy, float lim,
                             int32_t* __restrict__ count, const int64_t* __restrict__ off,
                             int32_t* __restrict__ list) {
  __shared__ float tx[256], ty[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float xi = i < ncdps ? fmx[i] : 0.f, yi = i < ncdps ? fmy[i] : 0.f;
  int n = 0;
  int64_t o = (off && i < ncdps) ? off[i] : 0;
  for (int j0 = 0; j0 < ncdps; j0 += 256) {
    __syncthreads();
    if (j0 + threadIdx.x < ncdps) {
      tx[threadIdx.x] = fmx[j0 + threadIdx.x];
      ty[threadIdx.x] = fmy[j0 + threadIdx.x];
    }
    __syncthreads();
    if (i < ncdps) {
      const int jn = min(256, ncdps - j0);
      for (int jj = 0; jj < jn; ++jj) {
        const float dx = __fsub_rn(tx[jj], xi);
        const float dy = __fsub_rn(ty[jj], yi);
        if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= lim) {
          if (list) list[o + n] = j0 + jj;
          ++n;
        }
      }
    }
  }
  if (count && i < ncdps) count[i] = n;
}

// Exclusive scan of `in` (int32 or int64 counts) into out[0..n], single block.
template <typename TI>
static __global__ void k_scan_exclusive(int n, const TI* __restrict__ in, int64_t* __restrict__ out) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    int64_t v = i < n ? (int64_t)in[i] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sums[lane] = w;
    }
    __syncthreads();
    const int64_t prefix = carry + (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
    if (i < n) out[i] = prefix;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = prefix + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// Aperture size of each CDP: sum of the folds of its neighbours.
static __global__ void k_aperture_count(int ncdps, const int64_t* __restrict__ nbr_off, const int32_t* __restrict__ nbr,
                                 const int64_t* __restrict__ cdp_end, int64_t* __restrict__ ap_cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  int64_t n = 0;
  for (int64_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
    const int j = nbr[q];
    n += cdp_end[j] - (j > 0 ? cdp_end[j - 1] : 0);
  }
  ap_cnt[i] = n;
}

// Aperture entries of CDP i (one warp per CDP): the traces of its neighbours in
// list order, each trace's |dm|, dm^2 and h relative to the midpoint of CDP i's
// first trace (CRS/OpenMP/src/main.cpp:179-204, 289-317), in float and in double.
// With `signed_dm` (SEMB_DM_SIGNED, no reference counterpart) dm is the midpoint
// displacement projected on the azimuth direction (cos, sin), signed, and dm^2 its
// square.  CMP apertures are the CDP's own traces with dm = 0.
static __global__ void k_aperture_fill(int ncdps, int method, const int64_t* __restrict__ nbr_off,
                                const int32_t* __restrict__ nbr, const int64_t* __restrict__ cdp_end,
                                const int64_t* __restrict__ ap_off, const float* __restrict__ h32,
                                const float* __restrict__ mx32, const float* __restrict__ my32,
                                const double* __restrict__ h64, const double* __restrict__ mx64,
                                const double* __restrict__ my64, int32_t* __restrict__ ap_tr,
                                float4* __restrict__ ap_geo, Geo64* __restrict__ ap_geo64, int signed_dm,
                                float cos_f, float sin_f, double cos_d, double sin_d) {
  const int warps = blockDim.x >> 5;
  const int i = blockIdx.x * warps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= ncdps) return;
  const int64_t first = i > 0 ? cdp_end[i - 1] : 0;
  const float cx = mx32[first], cy = my32[first];
  const double cxd = mx64[first], cyd = my64[first];
  int64_t pos = ap_off[i];
  for (int64_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
    const int j = nbr[q];
    const int64_t t0 = j > 0 ? cdp_end[j - 1] : 0, t1 = cdp_end[j];
    for (int64_t t = t0 + lane; t < t1; t += 32) {
      const int64_t e = pos + (t - t0);
      ap_tr[e] = (int32_t)t;
      if (method == METHOD_CRS && signed_dm) {
        const float dx = __fsub_rn(mx32[t], cx), dy = __fsub_rn(my32[t], cy);
        const float m = __fadd_rn(__fmul_rn(dx, cos_f), __fmul_rn(dy, sin_f));
        ap_geo[e] = make_float4(m, __fmul_rn(m, m), h32[t], 0.f);
        const double dxd = __dsub_rn(mx64[t], cxd), dyd = __dsub_rn(my64[t], cyd);
        const double md = __dadd_rn(__dmul_rn(dxd, cos_d), __dmul_rn(dyd, sin_d));
        ap_geo64[e] = Geo64{md, __dmul_rn(md, md), h64[t], 0.0};
      } else if (method == METHOD_CRS) {
        const float dx = __fsub_rn(mx32[t], cx), dy = __fsub_rn(my32[t], cy);
        const float m2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
        ap_geo[e] = make_float4(__fsqrt_rn(m2), m2, h32[t], 0.f);
        const double dxd = __dsub_rn(mx64[t], cxd), dyd = __dsub_rn(my64[t], cyd);
        const double m2d = __dadd_rn(__dmul_rn(dxd, dxd), __dmul_rn(dyd, dyd));
        ap_geo64[e] = Geo64{__dsqrt_rn(m2d), m2d, h64[t], 0.0};
      } else {
        ap_geo[e] = make_float4(0.f, 0.f, h32[t], 0.f);
        ap_geo64[e] = Geo64{0.0, 0.0, h64[t], 0.0};
      }
    }
    pos += t1 - t0;
  }
}

// CRS: where each CDP's own traces sit in its aperture list (k_aperture_fill appends
// the neighbours' traces in list order, the CDP itself among them): (first entry
// relative to ap_off[i], count).  (0, 0) if the CDP is not in its own list.
static __global__ void k_central_range(int ncdps, const int64_t* __restrict__ nbr_off,
                                       const int32_t* __restrict__ nbr, const int64_t* __restrict__ cdp_end,
                                       int2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  int64_t rel = 0;
  int2 r = make_int2(0, 0);
  for (int64_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
    const int j = nbr[q];
    const int64_t f = cdp_end[j] - (j > 0 ? cdp_end[j - 1] : 0);
    if (j == i) {
      r = make_int2((int)rel, (int)f);
      break;
    }
    rel += f;
  }
  out[i] = r;
}

// Traces copied linearly (ns samples each, back to back, as the caller holds them)
// into the device stores: the FP32 rows at the plan's pitch with their zero padding
// and, for a 16-bit batched store (s16 not null), the FP16/BF16 rows of the samples
// divided by the per-trace scale max|s| / 32768 (1 for an all-zero or non-finite
// trace), with the same padding.  One CTA per trace, grid-stride over traces.
static __global__ void k_ingest_rows(int64_t ntr, int ns, int64_t pitch, int storage, const float* __restrict__ src,
                                     float* __restrict__ s32, uint16_t* __restrict__ s16, float* __restrict__ scale) {
  __shared__ float red[32];
  for (int64_t tr = blockIdx.x; tr < ntr; tr += gridDim.x) {
    const float* row = src + tr * ns;
    float sc = 1.0f;
    if (s16) {
      float m = 0.f;
      for (int k = threadIdx.x; k < ns; k += blockDim.x) m = fmaxf(m, fabsf(row[k]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
      __syncthreads();
      if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) red[0] = v;
      }
      __syncthreads();
      const float mx = red[0];
      sc = (mx > 0.f && isfinite(mx)) ? mx / 32768.0f : 1.0f;
      if (threadIdx.x == 0) scale[tr] = sc;
    }
    for (int k = threadIdx.x; k < pitch; k += blockDim.x) {
      const float v = k < ns ? row[k] : 0.f;
      s32[tr * pitch + k] = v;
      if (s16) {
        const float q = v / sc;
        s16[tr * pitch + k] = storage == STORE_BF16 ? __bfloat16_as_ushort(__float2bfloat16_rn(q))
                                                    : __half_as_ushort(__float2half_rn(q));
      }
    }
    __syncthreads();
  }
}

// CRS stack of item (t0 = 0, candidate 0) per CDP, in the plain FP32 arithmetic of
// the search; the reference reports it as the stack of every t0 where no
// candidate has positive semblance (CRS/OpenMP/src/main.cpp:272-284, stt[max_par]
// with max_par = 0).  One thread per CDP, traces summed in aperture order.
template <int W>
static __global__ void k_crs_stt00(int cdp0, int cdp1, KParams P, float a, float b, float c, float* __restrict__ out) {
  const int cdp = cdp0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (cdp >= cdp1) return;
  const int64_t e0 = P.ap_off[cdp], e1 = P.ap_off[cdp + 1];
  float num[W];
#pragma unroll
  for (int j = 0; j < W; ++j) num[j] = 0.f;
  float den = 0.f, lin = 0.f;
  int M = 0;
  const float tau_lo = (float)P.tau, tau_hi = (float)(P.ns - P.tau - 1);
  const float T = __fmul_rn(P.dt, 0.0f);
  for (int64_t e = e0; e < e1; ++e) {
    const float4 g = P.ap_geo[e];
    float t = __fadd_rn(T, __fmul_rn(a, g.x));
    t = __fadd_rn(__fadd_rn(__fmul_rn(t, t), __fmul_rn(b, g.y)), __fmul_rn(c, g.z));
    t = (t < 0.0f) ? -1.0f : __fsqrt_rn(t);
    t = __fmul_rn(t, P.idt);
    if (t >= tau_lo && t < tau_hi) {
      const float y = __fadd_rz(t, 8388608.0f);
      const int it = __float_as_int(y) - 0x4B000000;
      const float x = __fsub_rn(t, __fsub_rn(y, 8388608.0f));
      const float* s = P.samples + (int64_t)P.ap_tr[e] * P.pitch + (it - P.tau);
      float s1 = s[0];
#pragma unroll
      for (int j = 0; j < W; ++j) {
        const float s0 = s1;
        s1 = s[j + 1];
        const float v = __fadd_rn(__fmul_rn(__fsub_rn(s1, s0), x), s0);
        num[j] = __fadd_rn(num[j], v);
        den = __fadd_rn(den, __fmul_rn(v, v));
        lin = __fadd_rn(lin, v);
      }
      ++M;
    }
  }
  const int err = (int)(e1 - e0) - M;
  const float mf = (float)M;
  const bool ok = (den > kEpsilonF) && (mf > kEpsilonF) && err < 2;
  out[cdp] = ok ? __fdiv_rn(lin, __fmul_rn((float)W, mf)) : 0.0f;
}

// CRS-DE launch parameters (csrc/de.cu)
struct DeParams {
  const float* samples;   // FP32 store [ntr][pitch]
  int64_t pitch;
  const int64_t* ap_off;
  const int32_t* ap_tr;
  const float4* ap_geo;   // (|dm| or signed dm, dm^2, h) in float
  const float* grid;      // [np][3]: the single-precision search grid (C 1e6-scaled)
  float lo[3], hi[3];     // search box
  int np, ngen, ncdps, ns, tau;
  float dt, idt;
  const float* stt00;     // stack of item (t0 = 0, candidate 0) per CDP
  float* a;               // picked parameters per (CDP, t0); C back in s^2/m^2
  float* b;
  float* c;
  float* str;
  float* stk;
};

struct RepickParams {
  const float* top_sem;
  const int32_t* top_idx;
  const float* top_stk;
  const float* samples;        // FP32 store
  int64_t pitch;
  const int64_t* ap_off;
  const int32_t* ap_tr;
  const Geo64* ap_geo64;
  const double* cand64;        // grid order: (a, b, c) x ncand, c in 1e6-scaled units
  const float* stt00;
  int ncdps, ns, tau, method, mode;
  int ncand;                   // candidates of the grid (full re-search of small items)
  int64_t item0, item_end;     // (CDP, t0) items cdp * ns + t0 of this launch
  double dt, idt;
  float gap;
  int32_t* ctr;
  float* str;
  float* stk;
  unsigned long long* repicked;
  // extra attributes (null when the plan does not keep them)
  float* sem2;     // second-best candidate's single-precision semblance
  int32_t* idx2;   // and its grid index (-1: none)
  float* err64;    // |FP32 - FP64 semblance| of the pick where re-evaluated, else -1
};

// Near-tie threshold of an item with `napert` aperture traces: the FP16 store's
// rounding moves a semblance by about 2^-11 / sqrt(napert * w) of its value (random
// rounding errors average over the traces and window samples), so small gathers
// need a wider band than `gap`, which is sized for ~64 traces and up.
__device__ __forceinline__ float repick_band(float gap, int napert) {
  return gap * fmaxf(1.0f, sqrtf(64.0f / (float)max(napert, 1)));
}

// Items with at most this many (aperture trace x candidate) pairs are re-searched
// over every candidate in FP64 when their FP32 top-4 lie within the near-tie band
// (then a candidate outside the top-4 may be the FP64 best).
constexpr int64_t kFullResearch = 16384;

// Semblance and stack of candidate c at sample t0 in FP64 with the reference's
// double-precision arithmetic, operation by operation and trace by trace in
// aperture order (CMP/OpenMP/src/main.cpp:149-204, CRS/OpenMP/src/main.cpp:209-267
// with real = double): every multiply and add rounded on its own.  Returns false
// when the item is invalid (the reference's -1 / 0).
template <int W>
__device__ bool eval_f64_ordered(const RepickParams& R, int64_t e0, int64_t e1, int t0, int c, double& sem,
                                 double& stk) {
  const double pa = R.cand64[3 * (int64_t)c], pb = R.cand64[3 * (int64_t)c + 1], pc = R.cand64[3 * (int64_t)c + 2];
  double num[W], den = 0.0, lin = 0.0, mm = 0.0;
  int err = 0;
#pragma unroll
  for (int j = 0; j < W; ++j) num[j] = 0.0;
  double T = __dmul_rn(R.dt, (double)t0);
  if (R.method == METHOD_CMP) T = __dmul_rn(T, T);
  for (int64_t e = e0; e < e1; ++e) {
    const Geo64 g = R.ap_geo64[e];
    double t;
    if (R.method == METHOD_CMP) {
      t = __dmul_rn(__dsqrt_rn(__dadd_rn(T, __dmul_rn(pc, g.h))), R.idt);
    } else {
      t = __dadd_rn(T, __dmul_rn(pa, g.m));
      t = __dadd_rn(__dadd_rn(__dmul_rn(t, t), __dmul_rn(pb, g.m2)), __dmul_rn(pc, g.h));
      t = t < 0.0 ? -1.0 : __dsqrt_rn(t);
      t = __dmul_rn(t, R.idt);
    }
    // (int)t as the reference; a traveltime outside the int range counts as out of range
    const bool bad = !(t > -2147483648.0 && t < 2147483647.0);
    const int it = bad ? 0 : (int)t;
    const double x = __dsub_rn(t, (double)it);
    if (!bad && it - R.tau >= 0 && it + R.tau + 1 < R.ns) {
      const float* s = R.samples + (int64_t)R.ap_tr[e] * R.pitch + (it - R.tau);
      double s1 = s[0];
#pragma unroll
      for (int j = 0; j < W; ++j) {
        const double s0 = s1;
        s1 = s[j + 1];
        const double v = __dadd_rn(__dmul_rn(__dsub_rn(s1, s0), x), s0);
        num[j] = __dadd_rn(num[j], v);
        den = __dadd_rn(den, __dmul_rn(v, v));
        lin = __dadd_rn(lin, v);
      }
      mm = __dadd_rn(mm, 1.0);
    } else {
      ++err;
    }
  }
  double acsq = 0.0;
#pragma unroll
  for (int j = 0; j < W; ++j) acsq = __dadd_rn(acsq, __dmul_rn(num[j], num[j]));
  if (den > 1e-13 && mm > 1e-13 && err < 2) {
    sem = __ddiv_rn(acsq, __dmul_rn(den, mm));
    stk = __ddiv_rn(lin, __dmul_rn((double)W, mm));
    return true;
  }
  sem = stk = 0.0;
  return false;
}

// The outputs of one (CDP, t0) item: the pick (or the no-pick values of the
// reference: CMP ctr -1, stack 0; CRS ctr 0, the stack of item (t0 = 0, candidate 0))
// and, when kept, the second-best candidate and the FP64 error of the pick.
__device__ __forceinline__ void write_pick(const RepickParams& R, int64_t item, int cdp, bool none, int out_i,
                                           float out_s, float out_k, float err, const float* ts, const int* ti0) {
  if (R.sem2) {
    // the best single-precision candidate other than the pick
    float s2 = 0.f;
    int i2 = -1;
    if (!none) {
#pragma unroll
      for (int q = kTopK - 1; q >= 0; --q)
        if (ti0[q] >= 0 && ts[q] > 0.f && ti0[q] != out_i) {
          s2 = ts[q];
          i2 = ti0[q];
        }
    }
    R.sem2[item] = s2;
    R.idx2[item] = i2;
    R.err64[item] = err;
  }
  if (none) {
    R.ctr[item] = R.method == METHOD_CMP ? -1 : 0;
    R.str[item] = 0.f;
    R.stk[item] = R.method == METHOD_CMP ? 0.f : R.stt00[cdp];
  } else {
    R.ctr[item] = out_i;
    R.str[item] = out_s;
    R.stk[item] = out_k;
  }
}

// One near-tie item, all lanes of the warp: when the best two FP32 candidates are
// closer than the near-tie band (repick_band: `gap`, wider for small apertures), or
// always in mode 2, the top-4 are re-evaluated in FP64 with the reference's
// double-precision arithmetic (CRS/OpenMP/src/main.cpp:209-267 with real = double)
// on the FP32 samples, and the pick follows the FP64 values.  Small items whose
// whole top-4 lies inside the band are re-searched over every candidate instead
// (eval_f64_ordered, one candidate per lane), so that a candidate the FP32 ranking
// put fifth or lower can still win as it does in FP64.
template <int W>
__device__ void repick_item(const RepickParams& R, const int64_t item, const int lane) {
  const int cdp = (int)(item / R.ns);
  const int t0 = (int)(item - (int64_t)cdp * R.ns);
  float ts[kTopK], tk[kTopK];
  int ti[kTopK];
#pragma unroll
  for (int q = 0; q < kTopK; ++q) {
    ts[q] = R.top_sem[item * kTopK + q];
    ti[q] = R.top_idx[item * kTopK + q];
    tk[q] = R.top_stk[item * kTopK + q];
  }
  int ti0[kTopK];   // the list before the candidates out of reach are dropped
#pragma unroll
  for (int q = 0; q < kTopK; ++q) ti0[q] = ti[q];
  const int64_t e0 = R.ap_off[cdp], e1 = R.ap_off[cdp + 1];
  const int napert = (int)(e1 - e0);
  const float band = repick_band(R.gap, napert);
  const bool none = !(ts[0] > 0.f) || ti[0] < 0;
  const bool near_tie = ti[1] >= 0 && ts[1] > 0.f && (ts[0] - ts[1]) < band;
  const bool redo = !none && (R.mode == 2 || (R.mode == 1 && near_tie));
  // the whole top-4 inside the band: the FP64 best may be outside it
  const bool full = redo && ti[kTopK - 1] >= 0 && (ts[0] - ts[kTopK - 1]) < band &&
                    (int64_t)napert * R.ncand <= kFullResearch;
  // candidates that can still win: the best and those within the band of it (all
  // four in mode 2); the others keep their single-precision rank below the best
#pragma unroll
  for (int q = 1; q < kTopK; ++q)
    if (ti[q] >= 0 && !(R.mode == 2 || (ts[0] - ts[q]) < band)) ti[q] = -1;
  int out_i = ti[0];
  float out_s = ts[0], out_k = tk[0];
  float err = -1.f;
  if (full) {
    // every candidate, one per lane, in FP64 in the reference's order; the pick is
    // the reference's: the largest semblance above 0, the lowest index on ties
    double bs = 0.0, bk = 0.0;
    int bi = 0x7fffffff;
    for (int c = lane; c < R.ncand; c += 32) {
      double sem, stk;
      if (eval_f64_ordered<W>(R, e0, e1, t0, c, sem, stk) && sem > bs) {
        bs = sem;
        bi = c;
        bk = stk;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double os = __shfl_xor_sync(0xffffffffu, bs, o);
      const double ok = __shfl_xor_sync(0xffffffffu, bk, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (os > bs || (os == bs && oi < bi)) {
        bs = os;
        bi = oi;
        bk = ok;
      }
    }
    if (bi != 0x7fffffff) {
      out_i = bi;
      out_s = (float)bs;
      out_k = (float)bk;
#pragma unroll
      for (int q = 0; q < kTopK; ++q)
        if (ti0[q] == bi) err = (float)fabs((double)ts[q] - bs);
    }
    if (lane == 0) atomicAdd(R.repicked, 1ull);
  } else if (redo) {
    // sums per candidate; the stack's linear sum is taken as the sum of the window
    // numerators at the end (the same quantity, summed in another order)
    double num[kTopK][W], den[kTopK];
    int M[kTopK];
#pragma unroll
    for (int q = 0; q < kTopK; ++q) {
#pragma unroll
      for (int j = 0; j < W; ++j) num[q][j] = 0.0;
      den[q] = 0.0;
      M[q] = 0;
    }
    double pa[kTopK], pb[kTopK], pc[kTopK];
#pragma unroll
    for (int q = 0; q < kTopK; ++q) {
      const int c = ti[q] >= 0 ? ti[q] : 0;
      pa[q] = R.cand64[3 * (int64_t)c];
      pb[q] = R.cand64[3 * (int64_t)c + 1];
      pc[q] = R.cand64[3 * (int64_t)c + 2];
    }
    const double T = R.dt * (double)t0;
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      const Geo64 g = R.ap_geo64[e];
      const float* row = R.samples + (int64_t)R.ap_tr[e] * R.pitch;
#pragma unroll
      for (int q = 0; q < kTopK; ++q) {
        if (ti[q] < 0) continue;
        double t;
        if (R.method == METHOD_CMP) {
          t = sqrt(T * T + pc[q] * g.h) * R.idt;
        } else {
          t = T + pa[q] * g.m;
          t = t * t + pb[q] * g.m2 + pc[q] * g.h;
          t = t < 0.0 ? -1.0 : sqrt(t);
          t = t * R.idt;
        }
        if (t >= (double)R.tau && t < (double)(R.ns - R.tau - 1)) {
          const int it = (int)t;
          const double x = t - (double)it;
          const float* s = row + (it - R.tau);
          double s1 = s[0];
#pragma unroll
          for (int j = 0; j < W; ++j) {
            const double s0 = s1;
            s1 = s[j + 1];
            const double v = (s1 - s0) * x + s0;
            num[q][j] += v;
            den[q] += v * v;
          }
          ++M[q];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kTopK; ++q) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int j = 0; j < W; ++j) num[q][j] += __shfl_xor_sync(0xffffffffu, num[q][j], o);
        den[q] += __shfl_xor_sync(0xffffffffu, den[q], o);
        M[q] += __shfl_xor_sync(0xffffffffu, M[q], o);
      }
    }
    double bs = 0.0;
    int bi = 0x7fffffff;
    double bk = 0.0;
#pragma unroll
    for (int q = 0; q < kTopK; ++q) {
      if (ti[q] < 0) continue;
      double acsq = 0.0, lin = 0.0;
#pragma unroll
      for (int j = 0; j < W; ++j) {
        acsq += num[q][j] * num[q][j];
        lin += num[q][j];
      }
      const bool ok = den[q] > 1e-13 && M[q] > 0 && (napert - M[q]) < 2;
      const double sem = ok ? acsq / (den[q] * (double)M[q]) : 0.0;
      const double stk = ok ? lin / ((double)W * (double)M[q]) : 0.0;
      if (sem > 0.0 && (sem > bs || (sem == bs && ti[q] < bi))) {
        bs = sem;
        bi = ti[q];
        bk = stk;
      }
    }
    if (bi != 0x7fffffff) {
      out_i = bi;
      out_s = (float)bs;
      out_k = (float)bk;
#pragma unroll
      for (int q = 0; q < kTopK; ++q)
        if (ti0[q] == bi) err = (float)fabs((double)ts[q] - bs);
    }
    if (lane == 0) atomicAdd(R.repicked, 1ull);
  }
  if (lane == 0) write_pick(R, item, cdp, none, out_i, out_s, out_k, err, ts, ti0);
}

// Final pick per (CDP, t0), 32 consecutive items per warp: each lane screens one
// item (no candidate above 0, or no near tie: the FP32 pick stands and the lane writes
// it), then the warp takes the near-tie items one after the other (repick_item), all
// lanes on one item's FP64 evaluation.
template <int W>
static __global__ void k_repick(RepickParams R) {
  const int lane = threadIdx.x & 31;
  const int64_t base = R.item0 + ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32;
  if (base >= R.item_end) return;
  const int64_t item = base + lane;
  bool redo = false;
  if (item < R.item_end) {
    const int cdp = (int)(item / R.ns);
    float ts[kTopK], tk[kTopK];
    int ti[kTopK];
#pragma unroll
    for (int q = 0; q < kTopK; ++q) {
      ts[q] = R.top_sem[item * kTopK + q];
      ti[q] = R.top_idx[item * kTopK + q];
      tk[q] = R.top_stk[item * kTopK + q];
    }
    const int napert = (int)(R.ap_off[cdp + 1] - R.ap_off[cdp]);
    const float band = repick_band(R.gap, napert);
    const bool none = !(ts[0] > 0.f) || ti[0] < 0;
    const bool near_tie = ti[1] >= 0 && ts[1] > 0.f && (ts[0] - ts[1]) < band;
    redo = !none && (R.mode == 2 || (R.mode == 1 && near_tie));
    if (!redo) write_pick(R, item, cdp, none, ti[0], ts[0], tk[0], -1.f, ts, ti);
  }
  unsigned todo = __ballot_sync(0xffffffffu, redo);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    repick_item<W>(R, base + src, lane);
  }
}

}  // namespace semb
