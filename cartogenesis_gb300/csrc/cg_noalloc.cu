// The thermal sweeps for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc: a JVM calling through JNI or FFM that
// runs inside a memory-accounted container and hands in buffers it owns, a renderer that owns
// every allocation on its device and only lends buffers for the length of a call, or code
// replaying a CUDA graph captured elsewhere. cg_thermal_sweeps allocates its ping-pong buffer on
// the context; this entry point takes the caller's device input and output and keeps its one
// scratch field in the file-scope array below, so it allocates nothing and needs no context.
//
// The array is sized for grids of up to CG_NOALLOC_MAX_CELLS cells (4 MiB of floats); every GPU
// that loads the library holds it until the process exits. Each CUDA context that runs this code
// loads its own copy of the module, and so its own copy of the array: the runtime resolves the
// array's address in whichever context is current. The address is therefore looked up once per
// context, with that context current, on the first call made in it (so make that first call before
// any stream capture), and cached under the context's unique id. A caller that makes its own
// driver-API context current (a JVM binding or a renderer that owns its device) gets that
// context's array, not the primary context's. Every call shares the array and its contents carry
// over between calls; nothing in it needs to start at zero, because each launch writes every cell
// it later reads. Calls whose work overlaps on the GPU race on the array: serialise them (one
// stream, or events between streams).
#include <cuda.h>

#include <mutex>

#include "cg_common.cuh"
#include "cg_internal.h"

#define CG_NOALLOC_MAX_CELLS (1 << 20)

static __device__ __align__(256) float g_noalloc_scratch[CG_NOALLOC_MAX_CELLS];

namespace {

// The driver's cuCtxGetCurrent and cuCtxGetId, fetched through the runtime so that the library does
// not link libcuda itself (it must load on machines without a driver).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

constexpr int kMaxContexts = 64;
struct ScratchEntry {
    unsigned long long ctx_id;
    float* addr;
};
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_n = 0;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::mutex g_scratch_lock;

// The array's device address in the current context, looked up once per context.
cudaError_t scratch_for_current_context(float** out) {
    // Makes the device's primary context current when the thread has none yet (runtime semantics).
    cudaError_t e = cudaFree(nullptr);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> guard(g_scratch_lock);
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return e != cudaSuccess ? e : cudaErrorNotSupported;
        g_ctx_get_current = (CtxGetCurrentFn)fn;
        fn = nullptr;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return e != cudaSuccess ? e : cudaErrorNotSupported;
        g_ctx_get_id = (CtxGetIdFn)fn;
    }
    CUcontext cu = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&cu) != CUDA_SUCCESS || !cu) return cudaErrorDeviceUninitialized;
    if (g_ctx_get_id(cu, &id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    for (int i = 0; i < g_scratch_n; ++i)
        if (g_scratch[i].ctx_id == id) {
            *out = g_scratch[i].addr;
            return cudaSuccess;
        }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (g_scratch_n < kMaxContexts) g_scratch[g_scratch_n++] = {id, (float*)p};   // else looked up per call
    *out = (float*)p;
    return cudaSuccess;
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Whether the byte ranges [a, a + bytes) and [b, b + bytes) share a byte.
bool overlaps(const void* a, const void* b, size_t bytes) {
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return x < y + bytes && y < x + bytes;
}

}  // namespace

extern "C" cg_status cg_thermal_sweeps_noalloc(const float* heights_in_dev, float* heights_out_dev, int32_t width,
                                               int32_t height, cg_thermal_limits limits, int32_t passes, float rate,
                                               void* stream) {
    if (!heights_in_dev || !heights_out_dev) return CG_BAD_ARG;
    if (!pow2(width) || !pow2(height) || passes < 0) return CG_BAD_ARG;
    if ((int64_t)width * height > CG_NOALLOC_MAX_CELLS) return CG_BAD_ARG;   // beyond the array's size
    cudaStream_t st = (cudaStream_t)stream;
    const size_t N = (size_t)width * height;
    // The first launch writes the output while other CTAs still read the input's halo.
    if (overlaps(heights_in_dev, heights_out_dev, N * sizeof(float))) return CG_BAD_ARG;
    if (passes == 0) {
        return cudaMemcpyAsync(heights_out_dev, heights_in_dev, N * sizeof(float), cudaMemcpyDeviceToDevice, st) ==
                       cudaSuccess
                   ? CG_OK
                   : CG_CUDA;
    }
    float* scratch = nullptr;
    if (scratch_for_current_context(&scratch) != cudaSuccess) return CG_CUDA;
    const cg::ThermalLaunch t = cg::thermal_launch_args(limits, rate);
    // The same launch sequence as cg_thermal_sweeps (two sweeps per launch, one for an odd rest), with the
    // destinations alternating so that the last launch writes the caller's output. The input is
    // only ever read.
    const int launches = cg::thermal_launches(passes);
    const float* src = heights_in_dev;
    int left = passes;
    for (int i = 0; i < launches; ++i) {
        const int k = cg::thermal_step(left);
        float* dst = ((launches - 1 - i) % 2 == 0) ? heights_out_dev : scratch;
        if (cg::thermal_launch(src, dst, width, height, t, k, st) != cudaSuccess) return CG_CUDA;
        left -= k;
        src = dst;
    }
    return CG_OK;
}
