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
// that loads the library holds it until the process exits. Its device address is looked up once
// per device, with that device current, on the first call made on it (so make that first call
// before any stream capture). Every call shares the array and its contents carry over between
// calls; nothing in it needs to start at zero, because each launch writes every cell it later
// reads. Calls whose work overlaps on the GPU race on the array: serialise them (one stream, or
// events between streams).
#include <mutex>

#include "cg_common.cuh"
#include "cg_internal.h"

#define CG_NOALLOC_MAX_CELLS (1 << 20)

static __device__ __align__(256) float g_noalloc_scratch[CG_NOALLOC_MAX_CELLS];

namespace {

constexpr int kMaxDevices = 64;
float* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_lock;

// The array's device address on the current device, looked up once per device.
cudaError_t scratch_for_current_device(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_scratch_lock);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = (float*)p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace

extern "C" cg_status cg_thermal_sweeps_noalloc(const float* heights_in_dev, float* heights_out_dev, int32_t width,
                                               int32_t height, cg_thermal_limits limits, int32_t passes, float rate,
                                               void* stream) {
    if (!heights_in_dev || !heights_out_dev || heights_in_dev == heights_out_dev) return CG_BAD_ARG;
    if (!pow2(width) || !pow2(height) || passes < 0) return CG_BAD_ARG;
    if ((int64_t)width * height > CG_NOALLOC_MAX_CELLS) return CG_BAD_ARG;   // beyond the array's size
    cudaStream_t st = (cudaStream_t)stream;
    const size_t N = (size_t)width * height;
    if (passes == 0) {
        return cudaMemcpyAsync(heights_out_dev, heights_in_dev, N * sizeof(float), cudaMemcpyDeviceToDevice, st) ==
                       cudaSuccess
                   ? CG_OK
                   : CG_CUDA;
    }
    float* scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return CG_CUDA;
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
