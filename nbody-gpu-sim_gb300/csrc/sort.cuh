// sort.cuh -- device-wide scan and stable radix sort (sort.cu).
#pragma once

#include "common.cuh"

namespace nbgb {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;

// Workspace sizes (in uint32 elements).
size_t scan_workspace_elems(int64_t n);
size_t radix_hist_elems(int64_t n);

// out[i] = sum_{j<i} in[j]; in may alias out.  ws: scan_workspace_elems(n).
// total (device pointer, may be null) receives the sum of all n inputs.
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* ws,
                        uint32_t* total, cudaStream_t st);

// Stable LSD radix sort of (keys, vals) on bits [begin_bit, end_bit), 8 bits
// per pass, ping-ponging with the *_alt buffers.  *result_in_alt tells which
// pair holds the result.  hist: radix_hist_elems(n); scan_ws:
// scan_workspace_elems(radix_hist_elems(n)).  A look-back wait that runs
// out of iterations sets kErrWaitTimeout in *err (may be null).
template <typename K>
void radix_sort_pairs(K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                      int begin_bit, int end_bit, uint32_t* hist, uint32_t* scan_ws,
                      cudaStream_t st, bool* result_in_alt, uint32_t* err = nullptr);

}  // namespace nbgb
