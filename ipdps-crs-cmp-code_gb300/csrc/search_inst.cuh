// Instantiation table of the search kernel for one (method, form).  For each
// window width w = 2*tau+1 there are one or more variants (RC candidates per
// thread, MINB resident CTAs per SM of NT threads, staging layout, candidate
// layout): more items per thread give more
// instruction-level parallelism and amortize per-trace work, more CTAs per SM
// give the scheduler more warps to hide barrier and load latency, and smaller
// CTAs let the others fill the cycles one of them spends at a barrier.  The plan's
// autotuner times the variants of its window on a sample of its own tasks and
// keeps the fastest; default_variant() (launch.cu) is where a plan starts.  The value/difference staging
// layout (LAY_SD) saves one FP32 op per window sample for 50% more shared-memory
// bytes per evaluation; the packed layout (LAY_P2) does two window samples per
// FP32x2 instruction, and LAY_PD (w = 3) stores the pair's differences in place of
// the odd samples (its variant unrolls the in-range trace loop by two); LAY_PD5
// (w = 5) adds an 8-byte side entry per sample.  pipe_entry variants use the pipelined
// kernel (semb_pipe_kernel), whose warps hand chunks over through mbarriers instead of
// meeting at CTA barriers; xp_entry variants are the two-barrier kernel with the first
// chunk of each pass staged ahead.  RC values keep the per-item
// register state within 65536 / (256 * MINB) registers without spilling
// (checked with -Xptxas -v).
#pragma once

#include "common.h"
#include "pipe_kernel.cuh"
#include "semb_kernels.cuh"

namespace semb {

struct SearchEntry {
  const void* fn;
  int rc;
  int minb;
  int brun;   // candidates laid out as B runs of RC (CRS)
  int nt;     // threads per CTA
  int pipe;   // 1: semb_pipe_kernel (decoupled staging ring), 0: semb_search_kernel
  int lay;    // staging layout (LAY_*)
  int glob;   // 1: stages may be smaller than a trace (long windows read global memory)
  int z0;     // 1: the central traces' sums are shared over A and B (semb_pipe_kernel Z0)
};

constexpr int kMaxVariants = SEMB_MAX_VARIANTS;

template <int METHOD, int FORM, int W, int RC, int MINB, int LAY = LAY_QUAD, bool BRUN = false, int NT = 256,
          bool GLOB = false, bool XP = false>
SearchEntry entry() {
  return {(const void*)semb_search_kernel<METHOD, FORM, W, RC, MINB, LAY, BRUN, NT, GLOB, XP>, RC, MINB, BRUN ? 1 : 0,
          NT, 0, LAY, GLOB ? 1 : 0, 0};
}

// the two-barrier batched kernel with its chunk stream run on across passes and tasks
template <int METHOD, int FORM, int W, int RC, int MINB, int LAY>
SearchEntry xp_entry() {
  return entry<METHOD, FORM, W, RC, MINB, LAY, false, 256, false, true>();
}

template <int METHOD, int W, int RC, int MINB, int LAY = LAY_P2, bool BRUN = false, int NT = 256, int TU = 1,
          bool GLOB = false, int Z0 = 0>
SearchEntry pipe_entry() {
  return {(const void*)semb_pipe_kernel<METHOD, W, RC, MINB, LAY, BRUN, NT, TU, GLOB, Z0>, RC, MINB, BRUN ? 1 : 0, NT, 1,
          LAY, GLOB ? 1 : 0, Z0 ? 1 : 0};
}

// Plain form: one variant per window.
template <int METHOD, int W>
SearchEntry plain_entry() {
  constexpr int RC = W <= 5 ? 8 : W == 7 ? 6 : W <= 11 ? 4 : W == 13 ? 3 : 2;
  return entry<METHOD, FORM_PLAIN, W, RC, 2>();
}

template <int METHOD, int FORM>
SearchEntry search_entry(int w, int variant) {
  if constexpr (FORM == FORM_PLAIN) {
    if (variant != 0) return {nullptr, 0, 0, 0, 0, 0, 0, 0, 0};
    switch (w) {
      case 1: return plain_entry<METHOD, 1>();
      case 3: return plain_entry<METHOD, 3>();
      case 5: return plain_entry<METHOD, 5>();
#if SEMB_WIDE_WINDOWS
      case 7: return plain_entry<METHOD, 7>();
      case 9: return plain_entry<METHOD, 9>();
      case 11: return plain_entry<METHOD, 11>();
      case 13: return plain_entry<METHOD, 13>();
      case 15: return plain_entry<METHOD, 15>();
#endif
      default: return {nullptr, 0, 0, 0, 0, 0, 0, 0, 0};
    }
  } else {
  // fast form
  switch (w) {
    case 1:
      if (variant == 0) return entry<METHOD, FORM, 1, 8, 2>();
      if (variant == 1) return entry<METHOD, FORM, 1, 4, 3>();
      if (METHOD == METHOD_CRS && variant == 4) return entry<METHOD, FORM, 1, 7, 2, LAY_QUAD, true>();
      if (METHOD == METHOD_CRS && variant == 5) return entry<METHOD, FORM, 1, 8, 2, LAY_QUAD, true>();
      if (variant == 6) return entry<METHOD, FORM, 1, 8, 4, LAY_QUAD, false, 128>();
      if (variant == 11) return pipe_entry<METHOD, 1, 8, 2, LAY_QUAD>();
      if (variant == 12) return pipe_entry<METHOD, 1, 8, 1, LAY_QUAD, false, 512>();
      if (METHOD == METHOD_CRS && variant == 14) return pipe_entry<METHOD, 1, 7, 1, LAY_QUAD, true, 512>();
      break;
    case 3:
      if (variant == 0) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2>();
      if (variant == 1) return entry<METHOD, FORM, 3, 4, 3>();
      if (variant == 2) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 6 : 8), 2>();
      if (variant == 3) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_SD>();
      if (METHOD == METHOD_CRS && variant == 4) return entry<METHOD, FORM, 3, 7, 2, LAY_SD, true>();
      if (METHOD == METHOD_CRS && variant == 5) return entry<METHOD, FORM, 3, 8, 2, LAY_QUAD, true>();
      if (variant == 6) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_QUAD, METHOD == METHOD_CRS, 128>();
      if (variant == 7) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_SD, METHOD == METHOD_CRS, 128>();
      if (variant == 8) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2>();
      if (variant == 9) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_P2, METHOD == METHOD_CRS, 128>();
      if (METHOD == METHOD_CRS && variant == 10) return entry<METHOD, FORM, 3, 8, 2, LAY_P2, true>();
      if (variant == 11) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 6), 2>();
      if (variant == 12) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 6), 1, LAY_P2, false, 512>();
      if (variant == 13) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_PD, METHOD == METHOD_CRS, 512, 2>();
      if (METHOD == METHOD_CRS && variant == 14) return pipe_entry<METHOD, 3, 7, 1, LAY_P2, true, 512>();
      if (variant == 15) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_QUAD, METHOD == METHOD_CRS, 512>();
      // stages smaller than a trace (windows beyond them read from global memory):
      // two 256-thread CTAs per SM, and 640 threads of 6 candidates
      if (variant == 16) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 2, LAY_PD, METHOD == METHOD_CRS, 256, 2, true>();
      if (variant == 17) return pipe_entry<METHOD, 3, 6, 1, LAY_PD, METHOD == METHOD_CRS, 640, 1, true>();
      if (variant == 18) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 2, LAY_P2, METHOD == METHOD_CRS, 256, 1, true>();
      // the packed layouts with the pair's samples formed by scalar FMAs
      if (variant == 19) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_P2S, METHOD == METHOD_CRS, 512>();
      if (variant == 20) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_PDS, METHOD == METHOD_CRS, 512, 2>();
      if (variant == 21) return entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2S>();
      // pre-offset values: no per-item interpolation weight (24 staged bytes per sample)
      if (variant == 22) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_FT, METHOD == METHOD_CRS, 512, 2>();
      if (variant == 23) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_FT, METHOD == METHOD_CRS, 512>();
      // variants 8 and 21 with the first chunk of each pass staged ahead (XP)
      if (variant == 24) return xp_entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2>();
      if (variant == 25) return xp_entry<METHOD, FORM, 3, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2S>();
      // sample and difference planes, two items per FP32x2 instruction
      if (variant == 26) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_X3, METHOD == METHOD_CRS, 512, 2>();
      if (variant == 27) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_X3, METHOD == METHOD_CRS, 512>();
      // variant 13 with 640 threads (20 warps per SM) at whole-trace stages
      if (variant == 28) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_PD, METHOD == METHOD_CRS, 640, 2>();
      if (variant == 29) return pipe_entry<METHOD, 3, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_PD, METHOD == METHOD_CRS, 640>();
      // variant 13 with the central traces' sums shared over A and B (8 or 4 of them
      // added with each planned chunk)
      if constexpr (METHOD == METHOD_CRS) {
        if (variant == 30) return pipe_entry<METHOD, 3, 7, 1, LAY_PD, true, 512, 2, false, 8>();
        if (variant == 31) return pipe_entry<METHOD, 3, 7, 1, LAY_PD, true, 512, 2, false, 4>();
        // B runs of 8 for grids whose nb pads less to a multiple of 8 than of 7 (nb = 31:
        // 32 slots per (A, C) instead of 35): variant 13 with RC = 8 (128 registers, no
        // spills), and the central-trace sharing at 384 threads, where RC = 8 fits in
        // 156 registers (at 512 threads it would spill)
        if (variant == 32) return pipe_entry<METHOD, 3, 8, 1, LAY_PD, true, 512, 2>();
        if (variant == 33) return pipe_entry<METHOD, 3, 8, 1, LAY_PD, true, 384, 2, false, 8>();
      }
      break;
    case 5:
      if (variant == 0) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2>();
      if (variant == 1) return entry<METHOD, FORM, 5, 4, 3>();
      if (variant == 2) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 6 : 4), 2>();
      if (variant == 3) return entry<METHOD, FORM, 5, 6, 2, LAY_SD>();
      if (METHOD == METHOD_CRS && variant == 4) return entry<METHOD, FORM, 5, 7, 2, LAY_QUAD, true>();
      if (METHOD == METHOD_CRS && variant == 5) return entry<METHOD, FORM, 5, 8, 2, LAY_QUAD, true>();
      if (variant == 6) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_QUAD, METHOD == METHOD_CRS, 128>();
      if (variant == 8) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2>();
      if (variant == 9) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_P2, METHOD == METHOD_CRS, 128>();
      if (METHOD == METHOD_CRS && variant == 10) return entry<METHOD, FORM, 5, 8, 2, LAY_P2, true>();
      if (variant == 11) return pipe_entry<METHOD, 5, (METHOD == METHOD_CMP ? 8 : 6), 2>();
      if (variant == 12) return pipe_entry<METHOD, 5, (METHOD == METHOD_CMP ? 8 : 6), 1, LAY_P2, false, 512>();
      if (variant == 13) return pipe_entry<METHOD, 5, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_SD, METHOD == METHOD_CRS, 512>();
      if (METHOD == METHOD_CRS && variant == 14) return pipe_entry<METHOD, 5, 7, 1, LAY_P2, true, 512>();
      if (variant == 15) return pipe_entry<METHOD, 5, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_QUAD, METHOD == METHOD_CRS, 512>();
      // stages smaller than a trace: two 256-thread CTAs per SM
      if (variant == 16) return pipe_entry<METHOD, 5, 7, 2, LAY_P2, METHOD == METHOD_CRS, 256, 1, true>();
      if (variant == 17) return pipe_entry<METHOD, 5, 6, 2, LAY_SD, METHOD == METHOD_CRS, 256, 1, true>();
      if (variant == 18) return pipe_entry<METHOD, 5, 7, 2, LAY_QUAD, METHOD == METHOD_CRS, 256, 1, true>();
      if (variant == 19) return pipe_entry<METHOD, 5, (METHOD == METHOD_CMP ? 8 : 7), 1, LAY_P2S, METHOD == METHOD_CRS, 512>();
      if (variant == 20) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 7), 4, LAY_P2S, METHOD == METHOD_CRS, 128>();
      if (variant == 21) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2S>();
      // packed value/difference entries with side entries: 24 staged bytes per item
      if (variant == 22) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_PD5>();
      if (variant == 23) return entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_PD5S>();
      // variants 21, 22 and 23 with the first chunk of each pass staged ahead (XP)
      if (variant == 24) return xp_entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_P2S>();
      if (variant == 25) return xp_entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_PD5>();
      if (variant == 26) return xp_entry<METHOD, FORM, 5, (METHOD == METHOD_CMP ? 8 : 6), 2, LAY_PD5S>();
      break;
#if SEMB_WIDE_WINDOWS
    case 7: if (variant == 0) return entry<METHOD, FORM, 7, 4, 2>(); break;
    case 9: if (variant == 0) return entry<METHOD, FORM, 9, 4, 2>(); break;
    case 11: if (variant == 0) return entry<METHOD, FORM, 11, 3, 2>(); break;
    case 13: if (variant == 0) return entry<METHOD, FORM, 13, 3, 2>(); break;
    case 15: if (variant == 0) return entry<METHOD, FORM, 15, 2, 2>(); break;
#endif
    default: break;
  }
  return {nullptr, 0, 0, 0, 0, 0, 0, 0, 0};
  }
}

}  // namespace semb
