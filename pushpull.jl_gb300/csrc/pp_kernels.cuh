// pp_kernels.cuh -- launch descriptors and host-side launchers shared by the .cu files.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pp_common.cuh"

namespace pp {

// kPullGradDot / kPullHessDot contract the gradient / Hessian of every channel
// with a per-voxel upstream array and sum over channels (the deformation
// cotangents of the reference rrules, src/pushpull_pb.jl:11-51).
// kPullValGrad (internal) evaluates value and gradient in one contraction.
enum PullOp { kPull = 0, kPullGrad = 1, kPullHess = 2, kPullGradDot = 3, kPullHessDot = 4, kPullValGrad = 5 };

// derivative order of the weights an op needs
__host__ __device__ constexpr int op_order(int op) {
    return op == kPull ? 0 : (op == kPullHess || op == kPullHessDot ? 2 : 1);
}
enum PushOp { kPush = 0, kPushGrad = 1 };

// Arguments of one pull-family or push-family launch.  Pointers address the
// first (channel 0, batch 0) element; channel c / batch b slices follow the
// reference layout (src/pushpull_cpu.jl:48, 103, 143, 198, 254).
struct LaunchArgs {
    const float* phi;   // (d1, 3, nb)
    const float* in;    // pull: f0 (d0, nc, nb); push: f1 (d1, nc, nb); push_grad: g1 (d1, 3, nc, nb)
    float* out;         // pull: (d1, ncomp, nc, nb); push: (d0, nc, nb); dot ops: (d1, 3, nb)
    const float* up;    // dot ops: upstream, (d1, nc, nb) for GradDot, (d1, 3, nc, nb) for HessDot;
                        // fused step: the target g, (d1, nc, nb)
    float* out2;        // fused step: deformation cotangent (d1, 3, nb); push: count image or NULL
    double* partial;    // fused step: one loss partial per CTA
    const unsigned* fmax;   // fused step: max |f0| per (channel, batch), float bits
    Geometry g;
    BndTable bnd;
};

// pull family: direct gather (one thread per sample voxel, all channels per thread)
cudaError_t launch_pull_direct(int op, const LaunchArgs& a, cudaStream_t s);
// push family: direct scatter with global float atomics
cudaError_t launch_push_direct(int op, const LaunchArgs& a, cudaStream_t s);

// fused forward + adjoint step, per-voxel variant (one loss partial per CTA into
// a.partial, fused_direct_grid(a).x * .y slots) and the final partial sum
dim3 fused_direct_grid(const LaunchArgs& a);
cudaError_t launch_fused_direct(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_sum_partials(const double* partial, int n, double* out, cudaStream_t s);
// max |f| of each of `planes` contiguous volumes of n voxels into out[planes] (zeroed by the caller)
cudaError_t launch_absmax(const float* f, long long n, int planes, unsigned* out, cudaStream_t s);

// number of SMs of the current device (cached per device)
int sm_count();

}  // namespace pp
