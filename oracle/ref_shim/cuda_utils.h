/* ORACLE build shim (test infrastructure): stands in for the reference's
 * include/cuda_utils.h when its kernels are compiled to a cubin for use as
 * the traversal checker.  Only device code from those files is ever run; the
 * host wrappers need these names to parse. */
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#define CUDA_CHECK_ERRORS() \
  do {                      \
  } while (0)
namespace at {
namespace cuda {
inline cudaStream_t getCurrentCUDAStream() { return 0; }
}  // namespace cuda
}  // namespace at
