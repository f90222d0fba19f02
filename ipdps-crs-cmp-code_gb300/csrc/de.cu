// CRS-DE on the GPU: the differential-evolution search over (A, B, C) of the
// reference's crs-ocl-de (README.md:86-106; its source is not in the reference).
// One warp per (CDP, t0) evolves a population of NP = na * nb * nc individuals
// started on the search grid, for ngen generations of DE/rand/1/bin (F = 0.5,
// CR = 0.9, trial kept when its semblance is >= the target's, parameters clamped
// to the search box), with counter-based random numbers keyed by (CDP, t0,
// generation, individual, slot), so that a run is reproducible and independent of
// the launch shape.  The population lives in shared memory; lane l owns individuals
// l, l + 32, ...  A semblance evaluation is the plain form's single-precision CRS
// operator (CRS/OpenMP/src/main.cpp:209-267 with real = float, no contraction) over
// the CDP's aperture read from the FP32 trace store, so the search agrees bit for
// bit with the oracle's restatement of the same definition.
#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"
#include "plan_kernels.cuh"

namespace semb {

constexpr int kDeMaxPop = 256;     // NP limit (8 individuals per lane)
constexpr int kDePerLane = kDeMaxPop / 32;
constexpr int kDeWarps = 4;        // warps (items) per CTA


namespace {

__device__ __forceinline__ uint64_t de_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t de_key(int cdp, int t0, int gen, int i, int slot) {
  uint64_t z = de_mix(((uint64_t)(uint32_t)cdp << 32) | (uint32_t)t0);
  z = de_mix(z ^ (((uint64_t)(uint32_t)gen << 32) | (uint32_t)i));
  return de_mix(z ^ (uint64_t)(uint32_t)slot);
}

// r[0..2]: distinct indices, all != i, drawn in turn among those not yet excluded
__device__ __forceinline__ void de_pick3(int cdp, int t0, int gen, int i, int np, int* r) {
  int ex[4] = {i, 0, 0, 0};
  int nex = 1;
  for (int q = 0; q < 3; ++q) {
    int v = (int)(de_key(cdp, t0, gen, i, q) % (uint64_t)(np - nex));
    int sorted[4] = {ex[0], ex[1], ex[2], ex[3]};
    for (int a = 1; a < nex; ++a)
      for (int b = a; b > 0 && sorted[b - 1] > sorted[b]; --b) {
        const int t = sorted[b];
        sorted[b] = sorted[b - 1];
        sorted[b - 1] = t;
      }
    for (int a = 0; a < nex; ++a)
      if (v >= sorted[a]) ++v;
    r[q] = v;
    ex[nex++] = v;
  }
}

// Semblance and stack of up to kDePerLane parameter triples of this lane at t0,
// in single precision with the reference's operation order.
template <int W>
__device__ void de_eval(const DeParams& R, int64_t e0, int64_t e1, float Tsec, const float (*par)[3], int cnt,
                        float* sem, float* stk) {
  float num[kDePerLane][W], den[kDePerLane], lin[kDePerLane];
  int M[kDePerLane], err[kDePerLane];
#pragma unroll
  for (int q = 0; q < kDePerLane; ++q) {
#pragma unroll
    for (int j = 0; j < W; ++j) num[q][j] = 0.f;
    den[q] = 0.f;
    lin[q] = 0.f;
    M[q] = 0;
    err[q] = 0;
  }
  for (int64_t e = e0; e < e1; ++e) {
    const float4 g = __ldg(R.ap_geo + e);
    const float* row = R.samples + (int64_t)__ldg(R.ap_tr + e) * R.pitch;
#pragma unroll
    for (int q = 0; q < kDePerLane; ++q) {
      if (q >= cnt) continue;
      float t = __fadd_rn(Tsec, __fmul_rn(par[q][0], g.x));
      t = __fadd_rn(__fadd_rn(__fmul_rn(t, t), __fmul_rn(par[q][1], g.y)), __fmul_rn(par[q][2], g.z));
      t = (t < 0.0f) ? -1.0f : __fsqrt_rn(t);
      const float ts = __fmul_rn(t, R.idt);
      // (int) truncation; NaN or out of the int range counts as out of range
      const bool fin = ts > -2147483648.0f && ts < 2147483647.0f;
      const int it = fin ? (int)ts : 0;
      const float x = __fsub_rn(ts, (float)it);
      if (fin && it - R.tau >= 0 && it + R.tau + 1 < R.ns) {
        const float* s = row + (it - R.tau);
        float s1 = __ldg(s);
#pragma unroll
        for (int j = 0; j < W; ++j) {
          const float s0 = s1;
          s1 = __ldg(s + j + 1);
          const float v = __fadd_rn(__fmul_rn(__fsub_rn(s1, s0), x), s0);
          num[q][j] = __fadd_rn(num[q][j], v);
          den[q] = __fadd_rn(den[q], __fmul_rn(v, v));
          lin[q] = __fadd_rn(lin[q], v);
        }
        ++M[q];
      } else {
        ++err[q];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kDePerLane; ++q) {
    if (q >= cnt) continue;
    float acsq = 0.f;
#pragma unroll
    for (int j = 0; j < W; ++j) acsq = __fadd_rn(acsq, __fmul_rn(num[q][j], num[q][j]));
    const float mf = (float)M[q];
    const bool ok = (den[q] > kEpsilonF) && (M[q] > 0) && (err[q] < 2);
    sem[q] = ok ? __fdiv_rn(acsq, __fmul_rn(den[q], mf)) : 0.f;
    stk[q] = ok ? __fdiv_rn(lin[q], __fmul_rn((float)W, mf)) : 0.f;
  }
}

template <int W>
__global__ void __launch_bounds__(kDeWarps * 32) k_crs_de(DeParams R) {
  __shared__ float pop[kDeWarps][kDeMaxPop][5];   // a, b, c, sem, stk
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int64_t item = (int64_t)blockIdx.x * kDeWarps + wl;
  if (item >= (int64_t)R.ncdps * R.ns) return;
  const int cdp = (int)(item / R.ns);
  const int t0 = (int)(item - (int64_t)cdp * R.ns);
  const int64_t e0 = R.ap_off[cdp], e1 = R.ap_off[cdp + 1];
  const float Tsec = __fmul_rn(R.dt, (float)t0);
  float (*P)[5] = pop[wl];
  const int np = R.np;
  const int cnt = max(0, min(kDePerLane, (np - lane + 31) / 32));   // individuals of this lane
  float par[kDePerLane][3], sem[kDePerLane], stk[kDePerLane];

  // generation 0: the grid
#pragma unroll
  for (int q = 0; q < kDePerLane; ++q) {
    const int i = lane + 32 * q;
#pragma unroll
    for (int d = 0; d < 3; ++d) par[q][d] = q < cnt ? R.grid[3 * i + d] : 0.f;
  }
  de_eval<W>(R, e0, e1, Tsec, par, cnt, sem, stk);
#pragma unroll
  for (int q = 0; q < kDePerLane; ++q) {
    if (q >= cnt) continue;
    const int i = lane + 32 * q;
    P[i][0] = par[q][0];
    P[i][1] = par[q][1];
    P[i][2] = par[q][2];
    P[i][3] = sem[q];
    P[i][4] = stk[q];
  }
  __syncwarp();

  for (int gen = 1; np >= 4 && gen <= R.ngen; ++gen) {
    // trials from the previous generation's population
#pragma unroll
    for (int q = 0; q < kDePerLane; ++q) {
      if (q >= cnt) continue;
      const int i = lane + 32 * q;
      int r[3];
      de_pick3(cdp, t0, gen, i, np, r);
      const int jrand = (int)(de_key(cdp, t0, gen, i, 3) % 3u);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float u = __fmul_rn((float)(de_key(cdp, t0, gen, i, 4 + d) >> 40), 1.0f / 16777216.0f);
        float v = P[i][d];
        if (u < 0.9f || d == jrand) v = __fadd_rn(P[r[0]][d], __fmul_rn(0.5f, __fsub_rn(P[r[1]][d], P[r[2]][d])));
        v = v < R.lo[d] ? R.lo[d] : (v > R.hi[d] ? R.hi[d] : v);
        par[q][d] = v;
      }
    }
    de_eval<W>(R, e0, e1, Tsec, par, cnt, sem, stk);
    __syncwarp();   // every lane has read the population
#pragma unroll
    for (int q = 0; q < kDePerLane; ++q) {
      if (q >= cnt) continue;
      const int i = lane + 32 * q;
      if (sem[q] >= P[i][3]) {
        P[i][0] = par[q][0];
        P[i][1] = par[q][1];
        P[i][2] = par[q][2];
        P[i][3] = sem[q];
        P[i][4] = stk[q];
      }
    }
    __syncwarp();
  }

  // the best individual (largest semblance, lowest index on ties)
  float bs = 0.f;
  int bi = 0x7fffffff;
  for (int q = 0; q < cnt; ++q) {
    const int i = lane + 32 * q;
    if (P[i][3] > bs) {
      bs = P[i][3];
      bi = i;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float os = __shfl_xor_sync(0xffffffffu, bs, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (os > bs || (os == bs && oi < bi)) {
      bs = os;
      bi = oi;
    }
  }
  if (lane == 0) {
    const int64_t o = item;
    if (bi == 0x7fffffff || !(bs > 0.f)) {
      R.a[o] = R.grid[0];
      R.b[o] = R.grid[1];
      R.c[o] = (float)((double)R.grid[2] / 1e6);
      R.str[o] = 0.f;
      R.stk[o] = R.stt00[cdp];
    } else {
      R.a[o] = P[bi][0];
      R.b[o] = P[bi][1];
      R.c[o] = (float)((double)P[bi][2] / 1e6);
      R.str[o] = bs;
      R.stk[o] = P[bi][4];
    }
  }
}

}  // namespace

int launch_crs_de(int w, const DeParams& R, cudaStream_t st) {
  if (R.np > kDeMaxPop) return fail(SEMB_E_ARG, "CRS-DE population %d above %d", R.np, kDeMaxPop);
  const int64_t items = (int64_t)R.ncdps * R.ns;
  const int grid = (int)((items + kDeWarps - 1) / kDeWarps);
  switch (w) {
    case 1: k_crs_de<1><<<grid, kDeWarps * 32, 0, st>>>(R); break;
    case 3: k_crs_de<3><<<grid, kDeWarps * 32, 0, st>>>(R); break;
    case 5: k_crs_de<5><<<grid, kDeWarps * 32, 0, st>>>(R); break;
    default: return fail(SEMB_E_WINDOW, "no CRS-DE kernel for w = %d", w);
  }
  SEMB_CUDA(cudaGetLastError());
  return SEMB_OK;
}

}  // namespace semb
