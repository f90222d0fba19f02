// Instantiation table of the search kernel for one (method, form): one kernel per
// window width w = 2*tau+1, with the number of candidates per thread (RC) chosen
// so that the per-item register state fits two 256-thread CTAs per SM without
// spilling (checked with -Xptxas -v).
#pragma once

#include "common.h"
#include "semb_kernels.cuh"

namespace semb {

struct SearchEntry {
  const void* fn;
  int rc;
};

template <int METHOD, int FORM, int W>
constexpr int rc_for() {
  if (FORM == FORM_PLAIN) return W <= 5 ? 8 : W == 7 ? 6 : W <= 11 ? 4 : W == 13 ? 3 : 2;
  if (METHOD == METHOD_CRS) return W == 1 ? 8 : 6;
  return W <= 5 ? 8 : W <= 9 ? 4 : W <= 13 ? 3 : 2;
}

template <int METHOD, int FORM, int W>
SearchEntry entry() {
  constexpr int RC = rc_for<METHOD, FORM, W>();
  return {(const void*)semb_search_kernel<METHOD, FORM, W, RC>, RC};
}

template <int METHOD, int FORM>
SearchEntry search_entry(int w) {
  switch (w) {
    case 1: return entry<METHOD, FORM, 1>();
    case 3: return entry<METHOD, FORM, 3>();
    case 5: return entry<METHOD, FORM, 5>();
#if SEMB_WIDE_WINDOWS
    case 7: return entry<METHOD, FORM, 7>();
    case 9: return entry<METHOD, FORM, 9>();
    case 11: return entry<METHOD, FORM, 11>();
    case 13: return entry<METHOD, FORM, 13>();
    case 15: return entry<METHOD, FORM, 15>();
#endif
    default: return {nullptr, 0};
  }
}

}  // namespace semb
