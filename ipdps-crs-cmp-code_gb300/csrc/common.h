// Shared host-side helpers: status codes with a per-thread message.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>

#include "semb_gb300.h"

namespace semb {

// Records the message for semb_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);

// Reference constants (CMP/OpenMP/src/main.cpp:39-43, CRS/OpenMP/src/main.cpp:39-43).
constexpr double kEpsilon = 1e-13;
// The reference compares a float x with the double 1e-13.  The float nearest 1e-13
// (0x1.c25c26p-44) lies below it and the next float above it, so x > 1e-13 in double
// is exactly x > kEpsilonF in float (no FP64 conversion on the device).
constexpr float kEpsilonF = 1e-13f;
static_assert((double)kEpsilonF < kEpsilon, "kEpsilonF must be the float just below 1e-13");
constexpr double kFactor = 1e6;
constexpr int kMaxWCmp = 16;
constexpr int kMaxWCrs = 5;

}  // namespace semb

#define SEMB_CUDA(call)                                                                           \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return ::semb::fail(e_ == cudaErrorMemoryAllocation ? SEMB_E_NOMEM : SEMB_E_CUDA, "%s: %s (%s:%d)", \
                          #call, cudaGetErrorString(e_), __FILE__, __LINE__);                     \
  } while (0)

#define SEMB_TRY(call)            \
  do {                            \
    int rc_ = (call);             \
    if (rc_ != SEMB_OK) return rc_; \
  } while (0)
