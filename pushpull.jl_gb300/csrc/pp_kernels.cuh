// pp_kernels.cuh -- launch descriptors and host-side launchers shared by the .cu files.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pp_common.cuh"

namespace pp {

enum PullOp { kPull = 0, kPullGrad = 1, kPullHess = 2 };
enum PushOp { kPush = 0, kPushGrad = 1 };

// Arguments of one pull-family or push-family launch.  Pointers address the
// first (channel 0, batch 0) element; channel c / batch b slices follow the
// reference layout (src/pushpull_cpu.jl:48, 103, 143, 198, 254).
struct LaunchArgs {
    const float* phi;   // (d1, 3, nb)
    const float* in;    // pull: f0 (d0, nc, nb); push: f1 (d1, nc, nb); push_grad: g1 (d1, 3, nc, nb)
    float* out;         // pull: (d1, ncomp, nc, nb); push: (d0, nc, nb)
    Geometry g;
    BndTable bnd;
};

// pull family: direct gather (one thread per sample voxel, all channels per thread)
cudaError_t launch_pull_direct(int op, const LaunchArgs& a, cudaStream_t s);
// push family: direct scatter with global float atomics
cudaError_t launch_push_direct(int op, const LaunchArgs& a, cudaStream_t s);

// number of SMs of the current device (cached per device)
int sm_count();

}  // namespace pp
