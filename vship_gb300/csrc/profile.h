// profile.h -- per-kernel instrumentation: an NVTX range around every kernel launch (visible
// to Nsight tools when one is attached, a no-op otherwise), and optional CUDA-event timing (off
// unless enabled by Vship_ProfileSetEnabled): events are recorded on the launching stream
// around each kernel and summed when a report is requested.
#pragma once

#include <cuda_runtime.h>

namespace vship {

bool prof_enabled();
// Returns a token for prof_end; -1 when profiling is off.
int prof_begin(const char* name, cudaStream_t st);
void prof_end(int token, cudaStream_t st);

void prof_range_push(const char* name);
void prof_range_pop();

struct ProfScope {
    int tok;
    cudaStream_t st;
    ProfScope(const char* name, cudaStream_t s) : tok((prof_range_push(name), prof_begin(name, s))), st(s) {}
    ~ProfScope() {
        prof_end(tok, st);
        prof_range_pop();
    }
};

}  // namespace vship
