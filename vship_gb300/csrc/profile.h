// profile.h -- optional per-kernel CUDA-event timing (off unless enabled by
// Vship_ProfileSetEnabled). Events are recorded on the launching stream around each kernel and
// summed when a report is requested.
#pragma once

#include <cuda_runtime.h>

namespace vship {

bool prof_enabled();
// Returns a token for prof_end; -1 when profiling is off.
int prof_begin(const char* name, cudaStream_t st);
void prof_end(int token, cudaStream_t st);

struct ProfScope {
    int tok;
    cudaStream_t st;
    ProfScope(const char* name, cudaStream_t s) : tok(prof_begin(name, s)), st(s) {}
    ~ProfScope() { prof_end(tok, st); }
};

}  // namespace vship
