// Device building blocks shared by the phases: an exclusive prefix sum, and connected-component
// labels over an 8-neighbour mask whose root is the component's smallest cell index (the order the
// reference's DFS walks number components in: ascending start cell).
#include "cg_common.cuh"
#include "cg_util.h"

namespace cg {

namespace {

constexpr int SCAN_BLOCK = 1024;

__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out, int* __restrict__ sums, int n) {
    __shared__ int sh[SCAN_BLOCK];
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    int v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
        int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;   // exclusive
    if (threadIdx.x == SCAN_BLOCK - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_add(int* __restrict__ out, const int* __restrict__ offs, int n) {
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}

__device__ __forceinline__ int find_root(int* parent, int a) {
    int p = parent[a];
    while (p != a) {
        int gp = parent[p];
        if (gp != p) parent[a] = gp;   // path halving; a benign race, every write is an ancestor
        a = p;
        p = parent[a];
    }
    return a;
}

__device__ void unite(int* parent, int a, int b) {
    while (true) {
        a = find_root(parent, a);
        b = find_root(parent, b);
        if (a == b) return;
        if (a < b) {
            int t = a;
            a = b;
            b = t;
        }
        // Hook the larger root under the smaller; retry if another thread moved it first.
        int old = atomicCAS(&parent[a], a, b);
        if (old == a) return;
    }
}

__global__ void k_cc_init(const uint8_t* __restrict__ mask, int* __restrict__ parent, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        parent[i] = mask[i] ? (int)i : -1;
}

// Each edge once: east, south-west, south, south-east (x wraps, y stops).
__global__ void k_cc_union(const uint8_t* __restrict__ mask, int* __restrict__ parent, int W, int H) {
    size_t N = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        if (!mask[i]) continue;
        const int row = pdiv((int)i, W), col = pmod((int)i, W);
        int e = row * W + wrap_col(col + 1, W);
        if (mask[e]) unite(parent, (int)i, e);
        if (row + 1 < H) {
            for (int cs = -1; cs <= 1; ++cs) {
                int n = (row + 1) * W + wrap_col(col + cs, W);
                if (mask[n]) unite(parent, (int)i, n);
            }
        }
    }
}

// Point every cell straight at its root. Read-only walks: the only writes are true roots, so a
// concurrent walk through a cell sees either its old ancestor or its root, both on the way up.
// (Path halving here would race: a halving write could replace a root just written with an
// intermediate ancestor.)
__global__ void k_cc_flatten(int* __restrict__ parent, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        int p = parent[i];
        if (p < 0) continue;
        int a = (int)i;
        while (p != a) {
            a = p;
            p = parent[a];
        }
        parent[i] = a;
    }
}

__global__ void k_root_flags(const int* __restrict__ parent, int* __restrict__ flag, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        flag[i] = parent[i] == (int)i ? 1 : 0;
}

__global__ void k_label_from_root(const int* __restrict__ parent, const int* __restrict__ rank,
                                  int* __restrict__ label, size_t N) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        int p = parent[i];
        label[i] = p < 0 ? -1 : rank[p];
    }
}

}  // namespace

cg_status exclusive_scan(cg_ctx* ctx, const int* d_in, int* d_out, int n, int* h_total) {
    if (n <= 0) {
        if (h_total) *h_total = 0;
        return CG_OK;
    }
    // Up to three levels: 2^10 elements per block, 2^10 block sums per second-level block, and a
    // single block over at most 2^10 second-level sums: 2^30 elements.
    int blocks = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    int blocks2 = (blocks + SCAN_BLOCK - 1) / SCAN_BLOCK;
    if (blocks2 > SCAN_BLOCK) return fail(ctx, CG_BAD_ARG, "scan of %d elements is too long", n);
    CG_BUF(int, d_tmp, ctx, S_SCRATCH5, 2 * (size_t)blocks + 2 * (size_t)blocks2 + 4);
    int* d_sums1 = d_tmp;                 // [blocks]
    int* d_offs1 = d_sums1 + blocks;      // [blocks]
    int* d_sums2 = d_offs1 + blocks;      // [blocks2]
    int* d_offs2 = d_sums2 + blocks2;     // [blocks2]
    int* d_total = d_offs2 + blocks2;     // [1]
    CG_LAUNCH(ctx) k_scan_blocks<<<blocks, SCAN_BLOCK, 0, ctx->stream>>>(d_in, d_out, d_sums1, n);
    CG_CHECK_LAUNCH(ctx);
    if (blocks > 1) {
        CG_LAUNCH(ctx) k_scan_blocks<<<blocks2, SCAN_BLOCK, 0, ctx->stream>>>(d_sums1, d_offs1, d_sums2, blocks);
        if (blocks2 > 1) {
            CG_LAUNCH(ctx) k_scan_blocks<<<1, SCAN_BLOCK, 0, ctx->stream>>>(d_sums2, d_offs2, d_total, blocks2);
            CG_LAUNCH(ctx) k_scan_add<<<blocks2, SCAN_BLOCK, 0, ctx->stream>>>(d_offs1, d_offs2, blocks);
        }
        CG_LAUNCH(ctx) k_scan_add<<<blocks, SCAN_BLOCK, 0, ctx->stream>>>(d_out, d_offs1, n);
        CG_CHECK_LAUNCH(ctx);
    }
    if (h_total) {
        int last_in, last_out;
        CG_CUDA(ctx, cudaMemcpyAsync(&last_in, d_in + n - 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(&last_out, d_out + n - 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *h_total = last_in + last_out;
    }
    return CG_OK;
}

cg_status component_labels(cg_ctx* ctx, int W, int H, const uint8_t* d_mask, int* d_root, int* d_label,
                           int* h_count) {
    size_t N = (size_t)W * H;
    int grid = ctx->num_sms * 8;
    CG_LAUNCH(ctx) k_cc_init<<<grid, 256, 0, ctx->stream>>>(d_mask, d_root, N);
    CG_LAUNCH(ctx) k_cc_union<<<grid, 256, 0, ctx->stream>>>(d_mask, d_root, W, H);
    CG_LAUNCH(ctx) k_cc_flatten<<<grid, 256, 0, ctx->stream>>>(d_root, N);
    CG_CHECK_LAUNCH(ctx);
    if (d_label) {
        CG_BUF(int, d_flag, ctx, S_SCRATCH0, N);
        CG_BUF(int, d_rank, ctx, S_SCRATCH1, N);
        CG_LAUNCH(ctx) k_root_flags<<<grid, 256, 0, ctx->stream>>>(d_root, d_flag, N);
        CG_CHECK_LAUNCH(ctx);
        cg_status st = exclusive_scan(ctx, d_flag, d_rank, (int)N, h_count);
        if (st != CG_OK) return st;
        CG_LAUNCH(ctx) k_label_from_root<<<grid, 256, 0, ctx->stream>>>(d_root, d_rank, d_label, N);
        CG_CHECK_LAUNCH(ctx);
    }
    return CG_OK;
}

}  // namespace cg
