// abi_internal.h -- error reporting shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

struct erlbm_batch_desc;

namespace erlbm {

// Validates a batch description (batch_abi.cu).
int check_desc(const erlbm_batch_desc *d);

// Records the message returned by erlbm_last_error() for this host thread (two %s arguments).
void set_error(const char *fmt, const char *a, const char *b);
// Records a CUDA error and returns ERLBM_E_CUDA.
int cuda_fail(cudaError_t e, const char *where);

}  // namespace erlbm
