// CRS neighbour lists without any device allocation (semb_neighbours_noalloc).
//
// For callers that cannot allocate device memory while they run: a pipeline whose
// device memory is owned by another allocator (a framework pool, a
// pre-registered communication buffer), or a real-time loop that forbids
// allocation after start-up.  They pass their own device buffers for inputs and
// outputs; the intermediate per-CDP midpoints, counts and offsets live in one
// file-scope __device__ array of fixed size that every GPU loading this library
// holds until the process exits.  The array's device address is looked up once
// per device (the first call on that device, with it current) and kept; a
// cudaDeviceReset voids it.
//
// The search plan builds the same lists (semb_plan_upload), with scratch it
// allocates itself; the arithmetic here is the same: CDP j is a neighbour of CDP i
// when the float distance of their first-trace midpoints is within apm.  The
// search is all pairs (a count pass and a fill pass over ncdps^2 pairs).
#include <cuda_runtime.h>

#include <climits>
#include <mutex>

#include "common.h"
#include "plan_kernels.cuh"

namespace {

// Limit of the no-allocation path and its scratch: per CDP two float midpoints,
// an int32 count and an int64 offset (plus one offset).
constexpr int kNoAllocMaxCdps = 131072;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocMaxCdps * (4 + 4 + 4) + ((size_t)kNoAllocMaxCdps + 1) * 8 + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch on each device, found once per device with
// that device current (the symbol's host-side name is not a device address).
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(void** out) {
  int dev = 0;
  SEMB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return semb::fail(SEMB_E_NODEV, "device %d beyond the supported %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return semb::fail(SEMB_E_CUDA, "cudaGetSymbolAddress of the no-allocation scratch failed on device %d: %s", dev,
                        cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SEMB_OK;
}

// Midpoint of each CDP's first trace (su_trace::midpoint_x/y, CRS/OpenMP/src/
// su_trace.cpp:70-80), from per-CDP first-trace header fields.
__global__ void k_first_midpoints(int ncdps, const int32_t* __restrict__ gx, const int32_t* __restrict__ gy,
                                  const int32_t* __restrict__ sx, const int32_t* __restrict__ sy,
                                  const int32_t* __restrict__ scalco, float* __restrict__ fmx,
                                  float* __restrict__ fmy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncdps) return;
  const int sc = scalco[i];
  const float fs = sc == 0 ? 1.0f : (sc > 0 ? (float)sc : __fdiv_rn(1.0f, (float)sc));
  fmx[i] = __fmul_rn(__fmul_rn(fs, __int2float_rn(gx[i] + sx[i])), 0.5f);
  fmy[i] = __fmul_rn(__fmul_rn(fs, __int2float_rn(gy[i] + sy[i])), 0.5f);
}

// Offsets to the caller's int32 array, and the lists into the caller's buffer
// (entries at or past `capacity` are not written).
__global__ void k_fill_capped(int ncdps, const float* __restrict__ fmx, const float* __restrict__ fmy, float lim,
                              const int64_t* __restrict__ off64, int32_t* __restrict__ off32,
                              int32_t* __restrict__ list, int64_t capacity) {
  __shared__ float tx[256], ty[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float xi = i < ncdps ? fmx[i] : 0.f, yi = i < ncdps ? fmy[i] : 0.f;
  const int64_t o = i < ncdps ? off64[i] : 0;
  if (i < ncdps) off32[i] = (int32_t)o;
  if (i == 0) off32[ncdps] = (int32_t)off64[ncdps];
  int n = 0;
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
          if (o + n < capacity) list[o + n] = j0 + jj;
          ++n;
        }
      }
    }
  }
}

}  // namespace

extern "C" int semb_neighbours_noalloc(const int32_t* gx, const int32_t* gy, const int32_t* sx, const int32_t* sy,
                                       const int32_t* scalco, int32_t ncdps, int32_t apm, int32_t* off,
                                       int32_t* list, int64_t capacity, int64_t* n_list, void* stream) {
  using namespace semb;
  if (!gx || !gy || !sx || !sy || !scalco || !off || !n_list || (!list && capacity > 0) || capacity < 0)
    return fail(SEMB_E_ARG, "null or negative argument");
  if (ncdps <= 0) return fail(SEMB_E_ARG, "ncdps must be positive");
  if (ncdps > kNoAllocMaxCdps)
    return fail(SEMB_E_ARG, "ncdps %d exceeds the no-allocation limit of %d CDPs", ncdps, kNoAllocMaxCdps);
  void* base = nullptr;
  SEMB_TRY(scratch_for_current_device(&base));
  unsigned char* b = static_cast<unsigned char*>(base);
  float* fmx = reinterpret_cast<float*>(b);
  float* fmy = fmx + kNoAllocMaxCdps;
  int32_t* count = reinterpret_cast<int32_t*>(fmy + kNoAllocMaxCdps);
  int64_t* off64 = reinterpret_cast<int64_t*>(b + (((size_t)kNoAllocMaxCdps * 12 + 255) & ~(size_t)255));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float lim = (float)((int32_t)apm * (int32_t)apm);
  const int blocks = (ncdps + 255) / 256;
  // every scratch word read below is written earlier in this call: nothing to clear
  k_first_midpoints<<<blocks, 256, 0, st>>>(ncdps, gx, gy, sx, sy, scalco, fmx, fmy);
  k_neighbours<<<blocks, 256, 0, st>>>(ncdps, fmx, fmy, lim, count, nullptr, nullptr);
  k_scan_exclusive<int32_t><<<1, 1024, 0, st>>>(ncdps, count, off64);
  k_fill_capped<<<blocks, 256, 0, st>>>(ncdps, fmx, fmy, lim, off64, off, list, capacity);
  SEMB_CUDA(cudaGetLastError());
  int64_t total = 0;
  SEMB_CUDA(cudaMemcpyAsync(&total, off64 + ncdps, sizeof(total), cudaMemcpyDeviceToHost, st));
  SEMB_CUDA(cudaStreamSynchronize(st));
  *n_list = total;
  if (total > INT32_MAX) return fail(SEMB_E_ARG, "the lists need %lld entries, beyond int32 offsets", (long long)total);
  if (total > capacity)
    return fail(SEMB_E_ARG, "the lists need %lld entries, the buffer holds %lld", (long long)total,
                (long long)capacity);
  return SEMB_OK;
}
