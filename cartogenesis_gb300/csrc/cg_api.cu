// The C ABI (include/cg_erosion.h): context, validation, host<->device staging and the stage's
// round loop. Every phase of a round runs on the device; the host only derives the configuration's
// constants (the reference's `Rates`, `thermalLimits`, `sweepsFor`), sequences launches and reads
// back a few scalars per round.
#include <cmath>
#include <cstdarg>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_params.h"

namespace cg {

cg_status fail(cg_ctx* ctx, cg_status st, const char* fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->error, sizeof(ctx->error), fmt, ap);
        va_end(ap);
    }
    return st;
}

cg_status cuda_fail(cg_ctx* ctx, cudaError_t e, const char* what, const char* file, int line) {
    cg_status st = (e == cudaErrorMemoryAllocation) ? CG_OOM : CG_CUDA;
    return fail(ctx, st, "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
}

void* buf(cg_ctx* ctx, int slot, size_t bytes, cg_status* st) {
    DevBuf& b = ctx->bufs[slot];
    if (bytes == 0) bytes = 16;
    if (b.bytes < bytes) {
        if (b.ptr) cudaFree(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
        cudaError_t e = cudaMalloc(&b.ptr, bytes);
        if (e != cudaSuccess) {
            *st = cuda_fail(ctx, e, "cudaMalloc", __FILE__, __LINE__);
            b.ptr = nullptr;
            return nullptr;
        }
        b.bytes = bytes;
    }
    return b.ptr;
}

void* pinned(cg_ctx* ctx, size_t bytes, cg_status* st) {
    if (ctx->pinned_bytes < bytes) {
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        ctx->pinned = nullptr;
        ctx->pinned_bytes = 0;
        cudaError_t e = cudaMallocHost(&ctx->pinned, bytes);
        if (e != cudaSuccess) {
            *st = cuda_fail(ctx, e, "cudaMallocHost", __FILE__, __LINE__);
            return nullptr;
        }
        ctx->pinned_bytes = bytes;
    }
    return ctx->pinned;
}

cg_status sync(cg_ctx* ctx) {
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}

namespace {

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

cg_status check_grid(cg_ctx* ctx, int W, int H) {
    if (!pow2(W) || !pow2(H)) return fail(ctx, CG_BAD_ARG, "width/height must be powers of two (got %d x %d)", W, H);
    if ((int64_t)W * H > (int64_t)1 << 30) return fail(ctx, CG_BAD_ARG, "grid of %d x %d cells is too large", W, H);
    return CG_OK;
}

cg_status upload(cg_ctx* ctx, void* dst, const void* src, size_t bytes) {
    CG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return CG_OK;
}

cg_status download(cg_ctx* ctx, void* dst, const void* src, size_t bytes) {
    CG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" {

void cg_default_params(cg_erosion_params* p, int32_t width, int32_t height, int64_t seed) {
    default_params(p, width, height, seed);
}

cg_status cg_thermal_limits_for(const cg_erosion_params* p, cg_thermal_limits* limits, int32_t* sweeps) {
    if (!p || !limits || !sweeps) return CG_BAD_ARG;
    *limits = thermal_limits(*p);
    *sweeps = sweeps_for(*p);
    return CG_OK;
}

cg_status cg_create(cg_ctx** out, int32_t device) {
    if (!out) return CG_BAD_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return CG_CUDA;
    if (device < 0 || device >= count) return CG_BAD_ARG;
    cg_ctx* ctx = new cg_ctx();
    ctx->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        cg_destroy(ctx);
        return CG_CUDA;
    }
    *out = ctx;
    return CG_OK;
}

void cg_destroy(cg_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->aux) cudaStreamSynchronize(ctx->aux);
    if (ctx->aux2) cudaStreamSynchronize(ctx->aux2);
    for (auto& b : ctx->bufs)
        if (b.ptr) cudaFree(b.ptr);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->join2) cudaEventDestroy(ctx->join2);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    if (ctx->aux2) cudaStreamDestroy(ctx->aux2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

void cg_cancel(cg_ctx* ctx) {
    if (ctx) ctx->cancel.store(1, std::memory_order_relaxed);
}

const char* cg_last_error(const cg_ctx* ctx) { return ctx ? ctx->error : "no context"; }

void* cg_stream(const cg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int64_t cg_kernel_launches(const cg_ctx* ctx) { return ctx ? (int64_t)ctx->launches : 0; }

cg_status cg_thermal_sweeps(cg_ctx* ctx, int32_t W, int32_t H, const float* in, float* out, cg_thermal_limits lim,
                            int32_t passes, float rate) {
    if (!ctx || !in || !out) return CG_BAD_ARG;
    cg_status st = check_grid(ctx, W, H);
    if (st != CG_OK) return st;
    if (passes < 0) return fail(ctx, CG_BAD_ARG, "negative pass count %d", passes);
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    size_t N = (size_t)W * H;
    CG_BUF(float, d_a, ctx, S_H0, N);
    CG_BUF(float, d_b, ctx, S_H1, N);
    if ((st = upload(ctx, d_a, in, N * sizeof(float))) != CG_OK) return st;
    float* res = d_a;
    if ((st = thermal_error_reset_dev(ctx)) != CG_OK) return st;
    if (passes > 0 && (st = thermal_sweeps_dev(ctx, W, H, d_a, d_b, lim, passes, rate, &res)) != CG_OK) return st;
    if ((st = download(ctx, out, res, N * sizeof(float))) != CG_OK) return st;
    return thermal_error_check(ctx);
}

}  // extern "C"
