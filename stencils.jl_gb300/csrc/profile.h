// profile.h — per-launch CUDA-event timing hooks (see profile.cu).
#pragma once

#include <cuda_runtime.h>

namespace stc {
bool profiling();
// returns a token (nullptr when profiling is off); pass it to prof_end after the launch
void* prof_begin(cudaStream_t s);
void prof_end(void* token, cudaStream_t s, const char* name, double alg_bytes, double updates);
}  // namespace stc
