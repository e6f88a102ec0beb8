// Device-side ordering of the persistent detection kernels of several
// detectors (the serving loop's workers).
#pragma once

#include <mutex>

#include <cuda_runtime.h>

struct vj_detector;

namespace vjgb {

// Each launch through a chain waits on the device for the previous launch
// through it to finish, so cooperative grids that each fill the GPU never
// compete for residency, while the host work and uploads of one detector
// overlap another's kernel.
struct LaunchChain {
    std::mutex mu;
    cudaEvent_t last = nullptr;  // recorded after the latest launch
};

// Routes the detector's launches through `chain` (nullptr: independent).
int detector_set_launch_chain(vj_detector* d, LaunchChain* chain);

}  // namespace vjgb
