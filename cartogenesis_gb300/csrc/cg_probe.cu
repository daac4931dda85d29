// A measurement of this GPU's FP64 rate, for the roofline of the phases the reference computes in
// double (the routing surface, the facet rule, the flat potentials). GB300 issues FP64 at a small
// fraction of its FP32 rate and the driver publishes no figure for it, so the bench measures it.
#include "cg_common.cuh"
#include "cg_internal.h"

namespace cg {
namespace {

constexpr int kChains = 8;     // independent FMA chains per thread, enough to cover the pipe's latency
constexpr int kSteps = 4096;   // FMAs per chain

__global__ void __launch_bounds__(256) k_fp64_fma(double seed, double* __restrict__ sink) {
    double x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = seed + (double)(threadIdx.x + i);
    const double a = 1.0000000001, b = -1e-12;
    for (int s = 0; s < kSteps; ++s) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) x[i] = __fma_rn(x[i], a, b);
    }
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) t += x[i];
    if (t == 12345.678) sink[0] = t;   // never true; keeps the chains alive
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" cg_status cg_probe_fp64_rate(cg_ctx* ctx, double* gflops) {
    if (!ctx || !gflops) return CG_BAD_ARG;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    CG_BUF(double, d_sink, ctx, S_SMALL, 1);
    const int blocks = ctx->num_sms * 8;
    cudaEvent_t a, b;
    CG_CUDA(ctx, cudaEventCreate(&a));
    CG_CUDA(ctx, cudaEventCreate(&b));
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a, ctx->stream);
        CG_LAUNCH(ctx) k_fp64_fma<<<blocks, 256, 0, ctx->stream>>>(1.0 + rep, d_sink);
        cudaEventRecord(b, ctx->stream);
        cudaError_t e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            return cuda_fail(ctx, e, "k_fp64_fma", __FILE__, __LINE__);
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;   // the first launch warms up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double flops = 2.0 * (double)blocks * 256.0 * kChains * kSteps;
    *gflops = flops / (best * 1e-3) / 1e9;
    return CG_OK;
}
