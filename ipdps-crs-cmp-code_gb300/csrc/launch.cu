// Kernel lookup and launch helpers shared by the plan.
#include <cuda_runtime.h>

#include "common.h"
#include "plan_kernels.cuh"
#include "search_inst.cuh"

namespace semb {

SearchEntry search_entry_cmp_plain(int w, int variant);
SearchEntry search_entry_cmp_fast(int w, int variant);
SearchEntry search_entry_crs_plain(int w, int variant);
SearchEntry search_entry_crs_fast(int w, int variant);

static SearchEntry lookup(int method, int form, int w, int v) {
  if (method == METHOD_CMP) return form == FORM_PLAIN ? search_entry_cmp_plain(w, v) : search_entry_cmp_fast(w, v);
  return form == FORM_PLAIN ? search_entry_crs_plain(w, v) : search_entry_crs_fast(w, v);
}

int search_variant(int method, int form, int w, int v, int* rc, int* minb, int* brun, int* nt, int* pipe, int* lay,
                   int* glob, int* z0) {
  if (v < 0 || v >= kMaxVariants) return 0;
  SearchEntry e = lookup(method, form, w, v);
  *rc = e.rc;
  *minb = e.minb;
  *brun = e.brun;
  *nt = e.nt;
  if (pipe) *pipe = e.pipe;
  if (lay) *lay = e.lay;
  if (glob) *glob = e.glob;
  if (z0) *z0 = e.z0;
  return e.fn != nullptr;
}

// Candidate slots of one (A, C) group's run of nb B values padded to a multiple of rc.
static int brun_slots(int nb, int rc) { return (std::max(nb, 1) + rc - 1) / rc * rc; }

// Variant a plan starts with (before any autotuning), the fastest measured on GB300
// for the benchmark workloads of each window: for CRS the pipelined B-run kernel
// (packed value/difference staging with a two-way trace unroll and the central traces'
// sums shared over A and B for w = 3, packed pairs otherwise); for CMP the
// two-barrier kernel with packed pairs (w = 3) or packed pairs formed by scalar FMAs
// (w = 5); variant 0 elsewhere.  For CRS with w = 3 the B-run length follows the
// grid's nb: runs of 7 (variant 30, 512 threads) unless nb pads less to a multiple of
// 8 (variant 33, 384 threads; nb = 31 takes 32 slots per (A, C) instead of 35; per
// slot the two run at the same speed).  fallback_variant() is the one to use where the
// default does not fit the plan (a grid whose passes span more C values than the
// central-trace sharing takes).
int default_variant(int method, int form, int w, int nb) {
  if (form != FORM_FAST) return 0;
  if (method == METHOD_CRS && w == 3) return brun_slots(nb, 8) < brun_slots(nb, 7) ? 33 : 30;
  if (method == METHOD_CRS && w <= 5) return 14;
  if (method == METHOD_CMP && w == 3) return 8;
  if (method == METHOD_CMP && w == 5) return 21;
  return 0;
}

int fallback_variant(int method, int form, int w, int nb) {
  if (form == FORM_FAST && method == METHOD_CRS && w == 3) return brun_slots(nb, 8) < brun_slots(nb, 7) ? 32 : 13;
  return 0;
}

int search_occupancy(int method, int form, int w, int v, int nwarps, size_t smem, int* ctas_per_sm) {
  SearchEntry e = lookup(method, form, w, v);
  if (!e.fn) return fail(SEMB_E_WINDOW, "no search kernel for w = %d", w);
  SEMB_CUDA(cudaFuncSetAttribute(e.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SEMB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, e.fn, nwarps * 32, smem));
  return SEMB_OK;
}

int launch_search(int method, int form, int w, int v, const KParams& P, int nwarps, int grid, size_t smem,
                  cudaStream_t st) {
  SearchEntry e = lookup(method, form, w, v);
  if (!e.fn) return fail(SEMB_E_WINDOW, "no search kernel for w = %d", w);
  void* args[] = {const_cast<KParams*>(&P)};
  SEMB_CUDA(cudaLaunchKernel(e.fn, dim3(grid), dim3(nwarps * 32), args, smem, st));
  return SEMB_OK;
}

int launch_stt00(int w, int cdp0, int cdp1, const KParams& P, float a, float b, float c, float* out, cudaStream_t st) {
  const int grid = (cdp1 - cdp0 + 127) / 128;
  if (grid <= 0) return SEMB_OK;
  switch (w) {
    case 1: k_crs_stt00<1><<<grid, 128, 0, st>>>(cdp0, cdp1, P, a, b, c, out); break;
    case 3: k_crs_stt00<3><<<grid, 128, 0, st>>>(cdp0, cdp1, P, a, b, c, out); break;
    case 5: k_crs_stt00<5><<<grid, 128, 0, st>>>(cdp0, cdp1, P, a, b, c, out); break;
    default: return fail(SEMB_E_WINDOW, "no CRS kernel for w = %d", w);
  }
  SEMB_CUDA(cudaGetLastError());
  return SEMB_OK;
}

int launch_repick(int w, const RepickParams& R, cudaStream_t st) {
  const int64_t items = R.item_end - R.item0;
  if (items <= 0) return SEMB_OK;
  const int grid = (int)((items + 255) / 256);   // 32 items per warp, 8 warps per CTA
  switch (w) {
    case 1: k_repick<1><<<grid, 256, 0, st>>>(R); break;
    case 3: k_repick<3><<<grid, 256, 0, st>>>(R); break;
    case 5: k_repick<5><<<grid, 256, 0, st>>>(R); break;
    case 7: k_repick<7><<<grid, 256, 0, st>>>(R); break;
    case 9: k_repick<9><<<grid, 256, 0, st>>>(R); break;
    case 11: k_repick<11><<<grid, 256, 0, st>>>(R); break;
    case 13: k_repick<13><<<grid, 256, 0, st>>>(R); break;
    case 15: k_repick<15><<<grid, 256, 0, st>>>(R); break;
    default: return fail(SEMB_E_WINDOW, "no re-pick kernel for w = %d", w);
  }
  SEMB_CUDA(cudaGetLastError());
  return SEMB_OK;
}

}  // namespace semb
