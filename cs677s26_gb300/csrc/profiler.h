// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each kernel launch while profiling is enabled (vj_profile_enable).
#pragma once

#include <cuda_runtime.h>

namespace vjgb {

bool profiling();
// Returns a slot to pass to prof_end, or -1 when profiling is off.
int prof_begin(const char* name, cudaStream_t s);
void prof_end(int slot, cudaStream_t s);

struct ProfScope {
    int slot;
    cudaStream_t s;
    ProfScope(const char* name, cudaStream_t st) : slot(prof_begin(name, st)), s(st) {}
    ~ProfScope() { prof_end(slot, s); }
};

// Runs the kernel launch expression (the variadic part) bracketed by
// profiling events named `name` on stream `st`.
#define VJ_TIMED_LAUNCH(name, st, ...)      \
    do {                                    \
        ::vjgb::ProfScope vj_ps_(name, st); \
        __VA_ARGS__;                        \
    } while (0)

}  // namespace vjgb
