// ps_common.h -- error reporting shared by the C-ABI entry points.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "porescale.h"

namespace ps {

// last error message of the calling host thread
std::string& last_error();

inline int fail(int code, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  last_error() = buf;
  return code;
}

inline int cuda_fail(cudaError_t e, const char* what)
{
  return fail(e == cudaErrorMemoryAllocation ? PS_ERR_NOMEM : PS_ERR_CUDA, "%s: %s (%s)", what,
              cudaGetErrorString(e), cudaGetErrorName(e));
}

}  // namespace ps

#define PS_CUDA(call)                                        \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ps::cuda_fail(e_, #call);  \
  } while (0)
