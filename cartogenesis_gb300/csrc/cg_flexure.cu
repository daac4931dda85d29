// The plate flexure of profile P3 (Isostasy.Flexure, Isostasy.kt:277-411, over Fft2D, math/Fft.kt;
// HydraulicErosion.kt:707-725, 856-880): at the top of every round, after the uplift, the plate
// answers the whole load the rounds have put on it.
//
// The transform is the reference's own, operation for operation, so that the bend is bit-exact: a
// radix-2 decimation-in-time FFT in double over a grid of W x 2H (the map mirrored about each pole),
// every row and then every column, each butterfly `odd * twiddle` then `even +/- rotated` with the
// twiddles tabulated on the host exactly as the reference tabulates them. The order of the butterflies
// inside a stage does not matter (each writes its own pair), so a line is transformed by one CTA with
// the whole line in shared memory (up to 8192 complex doubles, 128 KB). Columns are transformed as rows
// of the transposed grid (a tiled transpose between the passes keeps every access coalesced); the filter
// is applied in the forward column pass and the inverse's 1 / (W 2H) in the inverse column pass, each
// after the pass's last butterfly, where the reference applies them.
//
// The load's mean is the reference's sequential double sum in cell order (seq_sum_dev, bit for bit).
// Everything else is elementwise or per line.
#include <cmath>
#include <vector>

#include "cg_common.cuh"
#include "cg_internal.h"
#include "cg_params.h"

namespace cg {
namespace {

constexpr int kLineThreads = 512;
constexpr int kMaxLine = 8192;        // W and 2H: one line of complex doubles in a CTA's shared memory
constexpr int kMinLineElems = 2048;   // short lines share a CTA, this many elements at least

int log2_of(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// Isostasy.Flexure's scalars (Isostasy.kt:287-320).
struct FlexConsts {
    double restoring;    // (mantle - fill density) g
    double rigidity;     // E Te^3 / (12 (1 - nu^2))
    double per_across;   // radians per metre per cycle across
    double per_down;     // radians per metre per cycle down (the padded height)
};

FlexConsts flex_consts(const cg_erosion_params& p) {
    const float metres_per_km = 1000.0f;
    FlexConsts k;
    k.restoring = (double)(p.mantle_density - p.deflection_fill_density) * (double)p.gravity;
    const double te = (double)p.elastic_thickness_km * (double)metres_per_km;
    const double e = (double)p.youngs_modulus_gpa * 1e9;
    const double nu = (double)p.poisson_ratio;
    k.rigidity = e * te * te * te / (12.0 * (1.0 - nu * nu));
    const ScaleF sc = scale_of(p);
    k.per_across = 2.0 * M_PI / ((double)p.width * sc.cell_width_km(p.width) * (double)metres_per_km);
    k.per_down = 2.0 * M_PI / ((double)(2 * p.height) * sc.cell_height_km(p.height) * (double)metres_per_km);
    return k;
}

// Fft1D's tables (Fft.kt: cos and sin of 2 pi i / n for i < n / 2), as (cos, sin) pairs.
std::vector<double2> twiddles(int n) {
    std::vector<double2> t((size_t)n / 2);
    for (int i = 0; i < n / 2; ++i) {
        t[(size_t)i].x = std::cos(2.0 * M_PI * (double)i / (double)n);
        t[(size_t)i].y = std::sin(2.0 * M_PI * (double)i / (double)n);
    }
    return t;
}

// The column change the plate answers, in pascals (HydraulicErosion.kt:862-872): float arithmetic in
// the reference's order, with 0 subtracted and added where it has no uplift or no sediment.
__global__ void k_flex_load(const float* __restrict__ work, const float* __restrict__ ref,
                            const float* __restrict__ defl, const float* __restrict__ upl,
                            const float* __restrict__ sed, size_t N, float mpf, float density, float gravity,
                            float* __restrict__ load) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        float column = __fmul_rn(__fsub_rn(work[i], ref[i]), mpf);
        column = __fadd_rn(column, defl[i]);
        column = __fsub_rn(column, upl ? upl[i] : 0.0f);
        column = __fadd_rn(column, sed ? __fmul_rn(sed[i], mpf) : 0.0f);
        load[i] = __fmul_rn(__fmul_rn(column, density), gravity);
    }
}

enum { SRC_GRID = 0, SRC_LOAD = 1 };
enum { POST_NONE = 0, POST_FILTER = 1, POST_SCALE = 2 };

struct LineArgs {
    double2* grid;          // `lines` lines of n complex values, line l at grid + l n
    int n, log2n, lines, per_cta;
    const double2* tw;      // n / 2 (cos, sin)
    int inverse;
    int src;                // SRC_LOAD: line r is map row r (r < H) or 2H - 1 - r, less the mean, imaginary 0
    const float* load;
    const double* mean;
    int post;               // POST_FILTER: line c is column c, element r its padded row
    FlexConsts k;
    int W, H2;
    double scale;           // POST_SCALE
};

// Fft1D.transform over `per_cta` lines, each whole in shared memory: the bit-reversed reordering on
// the way in, then the butterflies stage by stage (Fft.kt:25-96), then the pass's post step.
__global__ void __launch_bounds__(kLineThreads) k_fft_lines(LineArgs a) {
    extern __shared__ double2 sh[];
    const int n = a.n, half_n = n >> 1;
    const int l0 = blockIdx.x * a.per_cta;
    const int elems = a.per_cta * n;
    for (int i = threadIdx.x; i < elems; i += blockDim.x) {
        const int l = i >> a.log2n, j = i & (n - 1);
        const int line = l0 + l;
        double2 v = make_double2(0.0, 0.0);
        if (line < a.lines) {
            if (a.src == SRC_LOAD) {
                const int row = line < a.H2 / 2 ? line : a.H2 - 1 - line;
                v.x = __dsub_rn((double)a.load[(size_t)row * n + j], *a.mean);
            } else {
                v = a.grid[(size_t)line * n + j];
            }
        }
        const int rj = a.log2n > 0 ? (int)(__brev((unsigned)j) >> (32 - a.log2n)) : 0;
        sh[(l << a.log2n) + rj] = v;
    }
    __syncthreads();
    for (int lh = 0; (1 << lh) < n; ++lh) {
        const int half = 1 << lh, tws = n >> (lh + 1);
        for (int b = threadIdx.x; b < a.per_cta * half_n; b += blockDim.x) {
            const int l = b >> (a.log2n - 1), k = b & (half_n - 1);
            const int pair = k & (half - 1);
            const int e = (l << a.log2n) + ((k >> lh) << (lh + 1)) + pair;
            const int o = e + half;
            const double2 t = a.tw[pair * tws];
            const double wr = t.x, wi = a.inverse ? t.y : -t.y;
            const double2 od = sh[o], ev = sh[e];
            const double rr = __dsub_rn(__dmul_rn(od.x, wr), __dmul_rn(od.y, wi));
            const double ri = __dadd_rn(__dmul_rn(od.x, wi), __dmul_rn(od.y, wr));
            sh[e] = make_double2(__dadd_rn(ev.x, rr), __dadd_rn(ev.y, ri));
            sh[o] = make_double2(__dsub_rn(ev.x, rr), __dsub_rn(ev.y, ri));
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < elems; i += blockDim.x) {
        const int l = i >> a.log2n, j = i & (n - 1);
        const int line = l0 + l;
        if (line >= a.lines) continue;
        double2 v = sh[i];
        if (a.post == POST_FILTER) {   // deflectionMetres' response (Isostasy.kt:344-365)
            const int cycles_down = j <= a.H2 / 2 ? j : j - a.H2;
            const double kd = __dmul_rn((double)cycles_down, a.k.per_down);
            const int cycles_across = line <= a.W / 2 ? line : line - a.W;
            const double ka = __dmul_rn((double)cycles_across, a.k.per_across);
            const double k2 = __dadd_rn(__dmul_rn(ka, ka), __dmul_rn(kd, kd));
            if (k2 == 0.0) {
                v = make_double2(0.0, 0.0);
            } else {
                const double response =
                    __ddiv_rn(1.0, __dadd_rn(a.k.restoring, __dmul_rn(__dmul_rn(a.k.rigidity, k2), k2)));
                v = make_double2(__dmul_rn(v.x, response), __dmul_rn(v.y, response));
            }
        } else if (a.post == POST_SCALE) {   // Fft2D.inverse's roundTripScale
            v = make_double2(__dmul_rn(v.x, a.scale), __dmul_rn(v.y, a.scale));
        }
        a.grid[(size_t)line * n + j] = v;
    }
}

// out[c][r] = in[r][c] for an R x C grid of complex doubles, through 32 x 32 tiles.
__global__ void k_transpose(const double2* __restrict__ in, double2* __restrict__ out, int R, int C) {
    __shared__ double2 tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int r = r0 + dy, c = c0 + threadIdx.x;
        if (r < R && c < C) tile[dy][threadIdx.x] = in[(size_t)r * C + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int c = c0 + dy, r = r0 + threadIdx.x;
        if (r < R && c < C) out[(size_t)c * R + r] = tile[threadIdx.x][dy];
    }
}

// The bend read back from the transformed grid (held column-major: W lines of 2H) and applied
// (HydraulicErosion.kt:873-884): surface += (deflection - bend) / metresPerFieldUnit, deflection = bend.
// The deflection is the real part as float, map rows only; through 32 x 32 tiles.
__global__ void k_flex_apply(const double2* __restrict__ t, int W, int H, int H2, float mpf, float* __restrict__ work,
                             float* __restrict__ defl, float* __restrict__ bend_out) {
    __shared__ float tile[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;   // tile: rows r0.., columns c0..
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int c = c0 + dy, r = r0 + threadIdx.x;
        if (r < H && c < W) tile[dy][threadIdx.x] = (float)t[(size_t)c * H2 + r].x;
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int r = r0 + dy, c = c0 + threadIdx.x;
        if (r >= H || c >= W) continue;
        const size_t i = (size_t)r * W + c;
        const float bend = tile[threadIdx.x][dy];
        if (bend_out) {
            bend_out[i] = bend;
        } else {
            work[i] = __fadd_rn(work[i], __fdiv_rn(__fsub_rn(defl[i], bend), mpf));
            defl[i] = bend;
        }
    }
}

cg_status fft_pass(cg_ctx* ctx, LineArgs a, cudaStream_t sm) {
    a.log2n = log2_of(a.n);
    a.per_cta = a.n >= kMinLineElems ? 1 : kMinLineElems / a.n;
    const int ctas = (a.lines + a.per_cta - 1) / a.per_cta;
    const size_t smem = (size_t)a.per_cta * a.n * sizeof(double2);
    CG_LAUNCH(ctx) k_fft_lines<<<ctas, kLineThreads, smem, sm>>>(a);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// deflectionMetres(load, ...) on the device: d_load (W x H floats) to the bend, applied to the surface
// and the running deflection (bend_out null) or written to bend_out.
cg_status flexure_dev(cg_ctx* ctx, const cg_erosion_params& p, const float* d_load, float* d_work, float* d_defl,
                      float* bend_out) {
    const int W = p.width, H = p.height, H2 = 2 * H;
    const size_t N = (size_t)W * H, N2 = (size_t)W * H2;
    cudaStream_t sm = ctx->stream;
    if (!ctx->flex_attr) {
        CG_CUDA(ctx, cudaFuncSetAttribute(k_fft_lines, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(kMaxLine * sizeof(double2))));
        ctx->flex_attr = true;
    }
    // Twiddles, tabulated once per line length.
    CG_BUF(double2, d_tw, ctx, S_FX_TW, (size_t)W / 2 + (size_t)H2 / 2 + 2);
    if (ctx->flex_tw_w != W || ctx->flex_tw_h2 != H2) {
        const std::vector<double2> tw = twiddles(W), th = twiddles(H2);
        CG_CUDA(ctx, cudaMemcpyAsync(d_tw, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice, sm));
        CG_CUDA(ctx, cudaMemcpyAsync(d_tw + W / 2, th.data(), th.size() * sizeof(double2), cudaMemcpyHostToDevice, sm));
        CG_CUDA(ctx, cudaStreamSynchronize(sm));   // the host tables leave scope
        ctx->flex_tw_w = W;
        ctx->flex_tw_h2 = H2;
    }
    CG_BUF(double2, d_a, ctx, S_FX_A, N2);
    CG_BUF(double2, d_b, ctx, S_FX_B, N2);
    CG_BUF(double, d_mean, ctx, S_FX_MEAN, 1);
    const FlexConsts k = flex_consts(p);
    // deflectionMetres' mean (Isostasy.kt:337-339): loadSum += load[c] in cell order, then / cells.
    CG_TRY_ST(seq_sum_dev(ctx, d_load, nullptr, 0, N, (double)N, d_mean, nullptr));
    LineArgs a{};
    a.k = k;
    a.W = W;
    a.H2 = H2;
    // Forward: rows (the mirrored load less its mean), then columns with the filter.
    a.grid = d_a;
    a.n = W;
    a.lines = H2;
    a.tw = d_tw;
    a.inverse = 0;
    a.src = SRC_LOAD;
    a.load = d_load;
    a.mean = d_mean;
    a.post = POST_NONE;
    CG_TRY_ST(fft_pass(ctx, a, sm));
    const dim3 tb(32, 8);
    CG_LAUNCH(ctx) k_transpose<<<dim3((W + 31) / 32, (H2 + 31) / 32), tb, 0, sm>>>(d_a, d_b, H2, W);
    a.grid = d_b;
    a.n = H2;
    a.lines = W;
    a.tw = d_tw + W / 2;
    a.src = SRC_GRID;
    a.post = POST_FILTER;
    CG_TRY_ST(fft_pass(ctx, a, sm));
    // Inverse: rows, then columns, then the round trip's scale.
    CG_LAUNCH(ctx) k_transpose<<<dim3((H2 + 31) / 32, (W + 31) / 32), tb, 0, sm>>>(d_b, d_a, W, H2);
    a.grid = d_a;
    a.n = W;
    a.lines = H2;
    a.tw = d_tw;
    a.inverse = 1;
    a.post = POST_NONE;
    CG_TRY_ST(fft_pass(ctx, a, sm));
    CG_LAUNCH(ctx) k_transpose<<<dim3((W + 31) / 32, (H2 + 31) / 32), tb, 0, sm>>>(d_a, d_b, H2, W);
    a.grid = d_b;
    a.n = H2;
    a.lines = W;
    a.tw = d_tw + W / 2;
    a.post = POST_SCALE;
    a.scale = 1.0 / ((double)W * (double)H2);
    CG_TRY_ST(fft_pass(ctx, a, sm));
    const float mpf = scale_of(p).relief_span();
    CG_LAUNCH(ctx) k_flex_apply<<<dim3((H + 31) / 32, (W + 31) / 32), tb, 0, sm>>>(d_b, W, H, H2, mpf, d_work, d_defl,
                                                                                   bend_out);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

__global__ void k_copy_float(const float* __restrict__ a, float* __restrict__ b, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

}  // namespace

cg_status flexure_check(cg_ctx* ctx, int W, int H) {
    if (W < 2 || W > kMaxLine || 2 * H > kMaxLine)
        return fail(ctx, CG_UNSUPPORTED, "the plate flexure needs width <= %d and height <= %d (got %d x %d)", kMaxLine,
                    kMaxLine / 2, W, H);
    return CG_OK;
}

// HydraulicErosion.kt:707-725: the field before the rounds, no bend yet, no uplift yet.
cg_status flexure_stage_begin_dev(cg_ctx* ctx, const cg_erosion_params& p, const float* d_work, bool uplift) {
    const size_t N = (size_t)p.width * p.height;
    CG_TRY_ST(flexure_check(ctx, p.width, p.height));
    CG_BUF(float, d_ref, ctx, S_FX_REF, N);
    CG_BUF(float, d_defl, ctx, S_FX_DEFL, N);
    CG_LAUNCH(ctx) k_copy_float<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(d_work, d_ref, N);
    CG_CHECK_LAUNCH(ctx);
    CG_CUDA(ctx, cudaMemsetAsync(d_defl, 0, N * sizeof(float), ctx->stream));
    if (uplift) {
        CG_BUF(float, d_upl, ctx, S_FX_UPL, N);
        CG_CUDA(ctx, cudaMemsetAsync(d_upl, 0, N * sizeof(float), ctx->stream));
    }
    return CG_OK;
}

float* flexure_uplifted_dev(cg_ctx* ctx, const cg_erosion_params& p) {
    cg_status st = CG_OK;
    return (float*)buf(ctx, S_FX_UPL, sizeof(float) * (size_t)p.width * p.height, &st);
}

// HydraulicErosion.kt:856-884: the load of everything the rounds have done, its bend, applied.
cg_status flexure_round_dev(cg_ctx* ctx, const cg_erosion_params& p, float* d_work, const float* d_sediment,
                            bool uplift) {
    const size_t N = (size_t)p.width * p.height;
    CG_BUF(float, d_ref, ctx, S_FX_REF, N);
    CG_BUF(float, d_defl, ctx, S_FX_DEFL, N);
    CG_BUF(float, d_load, ctx, S_FX_LOAD, N);
    const float* d_upl = nullptr;
    if (uplift) {
        CG_BUF(float, u, ctx, S_FX_UPL, N);
        d_upl = u;
    }
    const float mpf = scale_of(p).relief_span();
    CG_LAUNCH(ctx) k_flex_load<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(
        d_work, d_ref, d_defl, d_upl, d_sediment, N, mpf, p.continental_crust_density, p.gravity, d_load);
    CG_CHECK_LAUNCH(ctx);
    return flexure_dev(ctx, p, d_load, d_work, d_defl, nullptr);
}

}  // namespace cg

using namespace cg;

extern "C" cg_status cg_flexure_deflection(cg_ctx* ctx, const cg_erosion_params* params, const float* load,
                                           float* deflection, double* rigidity, double* restoring) {
    if (!ctx || !params || !load || !deflection) return CG_BAD_ARG;
    const cg_erosion_params& p = *params;
    if (p.width <= 0 || p.height <= 0 || (p.width & (p.width - 1)) || (p.height & (p.height - 1)))
        return fail(ctx, CG_BAD_ARG, "width/height must be powers of two (got %d x %d)", p.width, p.height);
    CG_TRY_ST(flexure_check(ctx, p.width, p.height));
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->run.active = false;
    const size_t N = (size_t)p.width * p.height;
    CG_BUF(float, d_load, ctx, S_FX_LOAD, N);
    CG_BUF(float, d_out, ctx, S_FX_DEFL, N);
    CG_CUDA(ctx, cudaMemcpyAsync(d_load, load, N * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CG_TRY_ST(flexure_dev(ctx, p, d_load, nullptr, nullptr, d_out));
    CG_CUDA(ctx, cudaMemcpyAsync(deflection, d_out, N * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const FlexConsts k = flex_consts(p);
    if (rigidity) *rigidity = k.rigidity;
    if (restoring) *restoring = k.restoring;
    return CG_OK;
}
