// sort.cu -- device-wide exclusive scan and stable LSD radix sort (K3).
//
// Replaces thrust::sort_by_key (src/cuda/force_barnes_hut.cu:324-328) and
// thrust::exclusive_scan (src/cuda/force_spatial_hash.cu:292-294).  The sort
// is stable (equal keys keep their input order), which is the order Thrust's
// radix sort produces for primitive keys, so (key, value) outputs compare
// bit-exactly with the reference.
//
// Radix pass (8-bit digit, tiles of kSortTile items):
//   1. digit histogram per tile -> hist[digit * n_tiles + tile]
//   2. exclusive scan of hist (digit-major) -> global offset per (digit, tile)
//   3. scatter: each tile ranks its items stably (warp match + per-warp digit
//      counts in shared memory, rounds in input order) and writes them to
//      offset + rank.
#include "common.cuh"
#include "kernels.cuh"
#include "sort.cuh"

namespace nbgb {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;  // per thread
constexpr int kScanChunk = kScanThreads * kScanItems;

// ---------------------------------------------------------------- scan --
__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, int64_t n,
                                   uint32_t* __restrict__ block_sums) {
  __shared__ uint32_t s[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  uint32_t acc = 0;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) acc += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += s[w];
    block_sums[blockIdx.x] = t;
  }
}

// Exclusive scan of `n` values by one block (n up to a few hundred thousand).
__global__ void scan_single_block_kernel(uint32_t* __restrict__ data, int64_t n,
                                         uint32_t* __restrict__ total) {
  __shared__ uint32_t s_carry;
  __shared__ uint32_t s_warp[32];
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t base = 0; base < n; base += blockDim.x) {
    int64_t i = base + threadIdx.x;
    uint32_t v = (i < n) ? data[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = (lane < nw) ? s_warp[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = (warp > 0) ? s_warp[warp - 1] : 0u;
    uint32_t carry = s_carry;
    if (i < n) data[i] = carry + warp_prefix + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = carry + warp_prefix + x;
    __syncthreads();
  }
  if (total && threadIdx.x == 0) *total = s_carry;
}

__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, int64_t n,
                                  const uint32_t* __restrict__ block_offsets,
                                  uint32_t* __restrict__ out) {
  __shared__ uint32_t s_vals[kScanChunk];
  __shared__ uint32_t s_warp[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  // load the chunk into shared memory (coalesced), each thread then owns
  // kScanItems consecutive items.
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    s_vals[k * kScanThreads + threadIdx.x] = (i < n) ? in[i] : 0u;
  }
  __syncthreads();
  uint32_t local[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    local[k] = sum;
    sum += s_vals[threadIdx.x * kScanItems + k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t wp = 0;
  for (int w = 0; w < warp; ++w) wp += s_warp[w];
  const uint32_t excl = block_offsets[blockIdx.x] + wp + x - sum;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s_vals[threadIdx.x * kScanItems + k] = excl + local[k];
  __syncthreads();
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) out[i] = s_vals[k * kScanThreads + threadIdx.x];
  }
}

size_t scan_workspace_elems(int64_t n) { return (size_t)ceil_div(std::max<int64_t>(n, 1), kScanChunk) + 1; }

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* ws,
                        uint32_t* total, cudaStream_t st) {
  if (n <= 0) return;
  const int64_t nb = ceil_div(n, kScanChunk);
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, ws);
  NBGB_LAUNCH_CHECK();
  scan_single_block_kernel<<<1, 1024, 0, st>>>(ws, nb, total);
  NBGB_LAUNCH_CHECK();
  scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, ws, out);
  NBGB_LAUNCH_CHECK();
}

// ----------------------------------------------------------- radix sort --
template <typename K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift) {
  return (uint32_t)((k >> shift) & (K)0xFF);
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const K* __restrict__ keys,
                                                                  int64_t n, int shift,
                                                                  int64_t n_tiles,
                                                                  uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_h[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) s_h[d] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int k = 0; k < kSortItems; ++k) {
    int64_t i = base + (int64_t)k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&s_h[digit_of(keys[i], shift)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x)
    hist[(int64_t)d * n_tiles + blockIdx.x] = s_h[d];
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, K* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out, int64_t n, int shift, int64_t n_tiles,
    const uint32_t* __restrict__ offsets) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t s_base[256];           // running count per digit (earlier rounds)
  __shared__ uint32_t s_wcnt[kWarps][256];   // per-warp digit counts of this round
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int d = tid; d < 256; d += blockDim.x) {
    s_base[d] = offsets[(int64_t)d * n_tiles + blockIdx.x];
  }
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortItems; ++r) {
    for (int e = tid; e < kWarps * 256; e += blockDim.x) (&s_wcnt[0][0])[e] = 0;
    __syncthreads();
    const int64_t i = base + (int64_t)r * kSortThreads + tid;
    const bool valid = i < n;
    K key = valid ? keys_in[i] : (K)0;
    uint32_t val = valid ? vals_in[i] : 0u;
    const uint32_t d = valid ? digit_of(key, shift) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t wrank = __popc(peers & lt_mask);
    if (valid && wrank == 0) s_wcnt[warp][d] = __popc(peers);
    __syncthreads();
    // exclusive prefix over warps per digit; advance the running base
    for (int dd = tid; dd < 256; dd += blockDim.x) {
      uint32_t run = s_base[dd];
      for (int w = 0; w < kWarps; ++w) {
        uint32_t c = s_wcnt[w][dd];
        s_wcnt[w][dd] = run;
        run += c;
      }
      s_base[dd] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_wcnt[warp][d] + wrank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
  }
}

template <typename K>
void radix_sort_pairs(K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                      int begin_bit, int end_bit, uint32_t* hist, uint32_t* scan_ws,
                      cudaStream_t st, bool* result_in_alt) {
  *result_in_alt = false;
  if (n <= 1) return;
  const int64_t n_tiles = ceil_div(n, kSortTile);
  const int64_t n_hist = 256 * n_tiles;
  K* kin = keys;
  K* kout = keys_alt;
  uint32_t* vin = vals;
  uint32_t* vout = vals_alt;
  bool alt = false;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    radix_hist_kernel<K><<<(unsigned)n_tiles, kSortThreads, 0, st>>>(kin, n, shift, n_tiles, hist);
    NBGB_LAUNCH_CHECK();
    scan_exclusive_u32(hist, hist, n_hist, scan_ws, nullptr, st);
    radix_scatter_kernel<K><<<(unsigned)n_tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, n,
                                                                        shift, n_tiles, hist);
    NBGB_LAUNCH_CHECK();
    std::swap(kin, kout);
    std::swap(vin, vout);
    alt = !alt;
  }
  *result_in_alt = alt;
}

size_t radix_hist_elems(int64_t n) { return (size_t)256 * ceil_div(std::max<int64_t>(n, 1), kSortTile); }

template void radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, int64_t, int,
                                         int, uint32_t*, uint32_t*, cudaStream_t, bool*);
template void radix_sort_pairs<unsigned long long>(unsigned long long*, unsigned long long*,
                                                   uint32_t*, uint32_t*, int64_t, int, int,
                                                   uint32_t*, uint32_t*, cudaStream_t, bool*);

}  // namespace nbgb
