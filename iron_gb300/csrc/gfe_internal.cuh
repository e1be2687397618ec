// gfe_internal.cuh -- shared host/device helpers of libgfe (status codes, error text, scratch).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/gfe.h"

namespace gfe {

// Record the message of a failure for gfe_last_error() on this host thread and return `code`.
int set_error(int code, const char* fmt, ...);

// Device-resident error word of the current device (lazily allocated once per device), or the
// word this host thread routed its kernels to (gfe_set_thread_error_word).
unsigned* device_error_word();
// The calling thread's override of the error word (nullptr: the per-device word), and its reset.
unsigned* thread_error_word();
void set_thread_error_word(unsigned* w);

// Stream-ordered scratch allocation; returns GFE_ERR_NOMEM with a message on failure.
int scratch_alloc(void** p, size_t bytes, cudaStream_t s, const char* what);
void scratch_free(void* p, cudaStream_t s);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached).
int sm_count();

// Stage timing (gfe_profile_enable): token = stage_begin(...); launch kernels; stage_end(...).
bool profiling();
void* stage_begin(int stage, cudaStream_t s);
void stage_end(int stage, void* token, cudaStream_t s, int launches);

}  // namespace gfe

#define GFE_CUDA_TRY(call)                                                                        \
  do {                                                                                            \
    cudaError_t e__ = (call);                                                                     \
    if (e__ != cudaSuccess)                                                                       \
      return gfe::set_error(GFE_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e__), \
                            __FILE__, __LINE__);                                                  \
  } while (0)

#define GFE_LAUNCH_CHECK(what)                                                                     \
  do {                                                                                             \
    cudaError_t e__ = cudaGetLastError();                                                          \
    if (e__ != cudaSuccess)                                                                        \
      return gfe::set_error(GFE_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e__)); \
  } while (0)

// Device-side error reporting: kernels never trap; they set bits in the error word.
__device__ __forceinline__ void gfe_raise(unsigned* err, unsigned bit) {
  if (err) atomicOr(err, bit);
}
