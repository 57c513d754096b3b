// Every device and pinned-host allocation of the library goes through these
// two calls, so that a test can make the k-th allocation fail and check that
// each create path returns RF_ERR_OOM and releases what it had allocated
// (rf_test_fail_alloc; or RF_FAIL_ALLOC=k in the environment at load time).
#pragma once

#include <cstddef>

#include <cuda_runtime.h>

namespace rf {

cudaError_t dev_malloc(void** p, size_t bytes);
cudaError_t host_malloc(void** p, size_t bytes);

}  // namespace rf
