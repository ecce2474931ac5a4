// Shared helpers for the GB300 permutation-inference kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "tfce_gb300.h"

namespace tfgb {

// Per-thread message of the last failure, read by tfce_last_error().
void set_error(const char* fmt, ...);
void clear_error();

// Device-side error codes written into a flag word by the kernels.  Every
// loop that waits on or walks shared state is bounded; hitting a bound sets a
// code here and the kernel carries on to its exit instead of trapping.
enum DevErr : int32_t {
  kDevOk = 0,
  kDevBadIndex = 1,   // adjacency entry outside its segment
  kDevLoopLimit = 2,  // union-find walk / retry limit reached
  kDevTooManySteps = 3,
};

inline int map_dev_err(int32_t e) {
  switch (e) {
    case kDevOk: return TFCE_OK;
    case kDevBadIndex: set_error("adjacency entry outside its segment"); return TFCE_EINVAL;
    case kDevLoopLimit: set_error("union-find iteration limit reached"); return TFCE_ETIMEOUT;
    case kDevTooManySteps: set_error("more thresholds than the sweep supports"); return TFCE_ERANGE;
    default: set_error("unknown device error %d", e); return TFCE_EDEVICE;
  }
}

}  // namespace tfgb

#define TFGB_CUDA(call)                                                            \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      tfgb::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                   \
                      cudaGetErrorString(_e));                                     \
      return (_e == cudaErrorMemoryAllocation) ? TFCE_ENOMEM : TFCE_EDEVICE;       \
    }                                                                              \
  } while (0)

#define TFGB_CHECK_ARG(cond, msg)                                                  \
  do {                                                                             \
    if (!(cond)) {                                                                 \
      tfgb::set_error("invalid argument: %s", msg);                                \
      return TFCE_EINVAL;                                                          \
    }                                                                              \
  } while (0)
