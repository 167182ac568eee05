// FP64 issue throughput of this GPU, measured by the library itself.
//
// The CCD and the PSD projection are bound by FP64 instruction issue, not by
// memory, so their roofline needs the FP64 peak of the part they run on.
// k_fp64_chains runs independent chains of DFMA (or DADD) per thread over a
// full-occupancy grid; the host times it with CUDA events on the legacy
// default stream.  active_lanes < 32 leaves the other lanes of every warp idle, which
// shows whether an FP64 warp instruction costs the FP64 unit the same time
// whatever its active lanes (the issue model the CCD kernels are shaped by).
#include "common.cuh"

namespace rigc {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;

template <int Op>
__global__ void __launch_bounds__(kPeakThreads)
k_fp64_chains(double* __restrict__ out, int iters, int active_lanes, double a, double b)
{
    if ((int)(threadIdx.x & 31) >= active_lanes) return;
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = 1e-3 * (double)(threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) {
            if (Op == 0)
                x[k] = __fma_rn(x[k], a, b);
            else
                x[k] = __dadd_rn(x[k], b);
        }
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s = __dadd_rn(s, x[k]);
    // never true for these inputs; keeps the chains live
    if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace rigc

extern "C" int rigc_fp64_throughput(int32_t op, int32_t active_lanes, int32_t iters,
                                    double* ms, double* warp_instructions, double* lane_flops)
{
    using namespace rigc;
    if ((op != 0 && op != 1) || active_lanes < 1 || active_lanes > 32 || iters < 1 || !ms
        || !warp_instructions || !lane_flops)
        return RIGC_ERR_ARG;
    int dev = 0, sms = 0;
    RIGC_CUDA(cudaGetDevice(&dev));
    RIGC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * (2048 / kPeakThreads);
    double* out = nullptr;
    RIGC_CUDA(cudaMalloc(&out, (size_t)blocks * kPeakThreads * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&](int it) {
        if (op == 0)
            k_fp64_chains<0><<<blocks, kPeakThreads>>>(out, it, active_lanes, 0.999999, 1e-7);
        else
            k_fp64_chains<1><<<blocks, kPeakThreads>>>(out, it, active_lanes, 0.999999, 1e-7);
    };
    RIGC_COUNT_LAUNCH();
    launch(16);  // warm-up
    RIGC_COUNT_LAUNCH();
    cudaEventRecord(e0);
    launch(iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) {
        set_error(RIGC_ERR_CUDA, cudaGetErrorString(err), __FILE__, __LINE__);
        return RIGC_ERR_CUDA;
    }
    const double warps = (double)blocks * (kPeakThreads / 32);
    const double ops = (double)iters * kChains;
    *ms = t;
    *warp_instructions = warps * ops;
    *lane_flops = warps * active_lanes * ops * (op == 0 ? 2.0 : 1.0);
    return RIGC_OK;
}
