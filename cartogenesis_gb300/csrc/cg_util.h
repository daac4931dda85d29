// Shared device building blocks (cg_util.cu).
#pragma once

#include "cg_common.cuh"

namespace cg {

// Exclusive prefix sum of n ints; *h_total (optional, synchronises) receives the sum.
cg_status exclusive_scan(cg_ctx* ctx, const int* d_in, int* d_out, int n, int* h_total);

// 8-neighbour components of d_mask (x wraps, y stops). d_root[i] = the component's smallest cell
// index (-1 outside the mask). If d_label is given, it receives the component's rank among roots in
// ascending index order (-1 outside), and *h_count the number of components.
cg_status component_labels(cg_ctx* ctx, int W, int H, const uint8_t* d_mask, int* d_root, int* d_label,
                           int* h_count);

}  // namespace cg
