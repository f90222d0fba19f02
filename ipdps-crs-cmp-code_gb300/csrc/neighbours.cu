// CRS neighbour lists by a uniform grid of cells, O(n log n): the replacement of
// the reference's all-pairs search (CRS/OpenMP/src/su_gather.cpp:70-87) for large
// surveys.  CDP j is a neighbour of CDP i when dx*dx + dy*dy <= apm*apm in float
// with dx = mid_j - mid_i (first-trace midpoints), exactly the reference's test;
// the grid only chooses which pairs are tested:
//
//   1. each CDP's cell (floor(mid / side) in double, side a little above apm, so
//      that every pair the float test can accept lies in neighbouring cells);
//   2. CDPs sorted by cell (radix sort of 64-bit cell keys);
//   3. per CDP, the 3 x 3 neighbouring cells found by binary search, their CDPs
//      tested (count pass, scan, fill pass);
//   4. each list sorted ascending (segmented radix sort), the reference's order.
//
// The result is identical to the all-pairs kernel (k_neighbours).
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <cmath>
#include <cstdint>

#include "common.h"
#include "plan_kernels.cuh"

namespace semb {

namespace {

constexpr int kCellBias = 1 << 30;

__device__ __forceinline__ int cell_of(float v, double inv_side) {
  double c = floor((double)v * inv_side);
  c = fmin(fmax(c, -(double)(kCellBias - 2)), (double)(kCellBias - 2));
  return (int)c;
}

__device__ __forceinline__ unsigned long long cell_key(int cx, int cy) {
  return ((unsigned long long)(unsigned)(cx + kCellBias) << 32) | (unsigned)(cy + kCellBias);
}

__global__ void k_cell_keys(int ncdps, const float* __restrict__ fmx, const float* __restrict__ fmy, double inv_side,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  keys[i] = cell_key(cell_of(fmx[i], inv_side), cell_of(fmy[i], inv_side));
  idx[i] = i;
}

__device__ __forceinline__ int lower_bound_key(const unsigned long long* k, int n, unsigned long long v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (k[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Pass 1 (list == nullptr): count each CDP's neighbours; pass 2: write them at off[i]
// (in cell order; sorted afterwards).
__global__ void k_grid_neighbours(int ncdps, const float* __restrict__ fmx, const float* __restrict__ fmy, float lim,
                                  double inv_side, const unsigned long long* __restrict__ skeys,
                                  const int32_t* __restrict__ sidx, int32_t* __restrict__ count,
                                  const int64_t* __restrict__ off, int32_t* __restrict__ list) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  const float xi = fmx[i], yi = fmy[i];
  const int cx = cell_of(xi, inv_side), cy = cell_of(yi, inv_side);
  int n = 0;
  const int64_t o = off ? off[i] : 0;
  for (int ddx = -1; ddx <= 1; ++ddx) {
    for (int ddy = -1; ddy <= 1; ++ddy) {
      const unsigned long long key = cell_key(cx + ddx, cy + ddy);
      for (int q = lower_bound_key(skeys, ncdps, key); q < ncdps && skeys[q] == key; ++q) {
        const int j = sidx[q];
        const float dx = __fsub_rn(fmx[j], xi);
        const float dy = __fsub_rn(fmy[j], yi);
        if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= lim) {
          if (list) list[o + n] = j;
          ++n;
        }
      }
    }
  }
  if (count) count[i] = n;
}

}  // namespace

// Neighbour lists of ncdps CDPs with first-trace midpoints (fmx, fmy): offsets into
// d_off[ncdps+1] (caller's), the list allocated into *d_list (caller frees), its
// length in *n_out.  Scratch is freed before return.
int grid_neighbours(int ncdps, const float* d_fmx, const float* d_fmy, int apm, int64_t* d_off, int32_t** d_list,
                    int64_t* n_out, cudaStream_t st) {
  *d_list = nullptr;
  *n_out = 0;
  const float lim = (float)((int32_t)apm * (int32_t)apm);
  // a cell side 1/1024 above apm: every pair the float test accepts is at most one
  // cell apart in x and in y (cells are computed in double)
  const double side = (apm > 0 ? (double)apm : 1.0) * (1.0 + 1.0 / 1024.0);
  const double inv_side = 1.0 / side;
  struct Scratch {
    void* p[8] = {};
    ~Scratch() {
      for (void* q : p)
        if (q) cudaFree(q);
    }
  } s;
  unsigned long long *keys = nullptr, *skeys = nullptr;
  int32_t *idx = nullptr, *sidx = nullptr, *cnt = nullptr, *list = nullptr;
  SEMB_CUDA(cudaMalloc(&keys, (size_t)ncdps * 8));
  s.p[0] = keys;
  SEMB_CUDA(cudaMalloc(&skeys, (size_t)ncdps * 8));
  s.p[1] = skeys;
  SEMB_CUDA(cudaMalloc(&idx, (size_t)ncdps * 4));
  s.p[2] = idx;
  SEMB_CUDA(cudaMalloc(&sidx, (size_t)ncdps * 4));
  s.p[3] = sidx;
  SEMB_CUDA(cudaMalloc(&cnt, (size_t)ncdps * 4));
  s.p[4] = cnt;
  const int blocks = (ncdps + 255) / 256;
  k_cell_keys<<<blocks, 256, 0, st>>>(ncdps, d_fmx, d_fmy, inv_side, keys, idx);
  SEMB_CUDA(cudaGetLastError());
  size_t tmp_bytes = 0;
  SEMB_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, skeys, idx, sidx, ncdps, 0, 64, st));
  void* tmp = nullptr;
  SEMB_CUDA(cudaMalloc(&tmp, tmp_bytes > 0 ? tmp_bytes : 1));
  s.p[5] = tmp;
  SEMB_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, skeys, idx, sidx, ncdps, 0, 64, st));
  k_grid_neighbours<<<blocks, 256, 0, st>>>(ncdps, d_fmx, d_fmy, lim, inv_side, skeys, sidx, cnt, nullptr, nullptr);
  SEMB_CUDA(cudaGetLastError());
  k_scan_exclusive<int32_t><<<1, 1024, 0, st>>>(ncdps, cnt, d_off);
  SEMB_CUDA(cudaGetLastError());
  int64_t total = 0;
  SEMB_CUDA(cudaMemcpyAsync(&total, d_off + ncdps, 8, cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  SEMB_CUDA(cudaMalloc(&list, (size_t)(total > 0 ? total : 1) * 4));
  s.p[6] = list;
  k_grid_neighbours<<<blocks, 256, 0, st>>>(ncdps, d_fmx, d_fmy, lim, inv_side, skeys, sidx, nullptr, d_off, list);
  SEMB_CUDA(cudaGetLastError());
  // ascending order within each list, as the reference's j loop
  int32_t* sorted = nullptr;
  SEMB_CUDA(cudaMalloc(&sorted, (size_t)(total > 0 ? total : 1) * 4));
  if (total > 0) {
    size_t seg_bytes = 0;
    SEMB_CUDA(cub::DeviceSegmentedRadixSort::SortKeys(nullptr, seg_bytes, list, sorted, total, ncdps, d_off,
                                                      d_off + 1, 0, 32, st));
    void* seg_tmp = nullptr;
    cudaError_t e = cudaMalloc(&seg_tmp, seg_bytes > 0 ? seg_bytes : 1);
    if (e != cudaSuccess) {
      cudaFree(sorted);
      SEMB_CUDA(e);
    }
    s.p[7] = seg_tmp;
    e = cub::DeviceSegmentedRadixSort::SortKeys(seg_tmp, seg_bytes, list, sorted, total, ncdps, d_off, d_off + 1,
                                                0, 32, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(sorted);
      SEMB_CUDA(e);
    }
  }
  *d_list = sorted;
  *n_out = total;
  return SEMB_OK;
}

}  // namespace semb
