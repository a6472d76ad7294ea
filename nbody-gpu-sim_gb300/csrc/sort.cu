// sort.cu -- device-wide exclusive scan and stable LSD radix sort (K3).
//
// Replaces thrust::sort_by_key (src/cuda/force_barnes_hut.cu:324-328) and
// thrust::exclusive_scan (src/cuda/force_spatial_hash.cu:292-294).  The sort
// is stable (equal keys keep their input order), which is the order Thrust's
// radix sort produces for primitive keys, so (key, value) outputs compare
// bit-exactly with the reference.
//
// Radix sort (8-bit digits, tiles of 4096 items), one kernel per digit:
//   0. one histogram kernel reads the keys once and counts every digit of
//      every pass; its last block turns the counts into each pass's global
//      digit offsets;
//   1. per pass, each CTA takes the next tile (dynamic tile id), ranks its
//      items stably (warp match + per-warp digit counts over rounds in input
//      order), publishes its per-digit counts, obtains the counts of all
//      earlier tiles by decoupled look-back over their published
//      aggregates / inclusive prefixes (every wait bounded), sorts the tile
//      by digit in shared memory and writes it out in digit runs (coalesced).
// Inputs of 2^30 items or more use the three-phase path (per-tile
// histograms, device-wide scan, scatter), 5 launches per pass.
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
static void radix_sort_pairs_3phase(K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                                    int64_t n, int begin_bit, int end_bit, uint32_t* hist,
                                    uint32_t* scan_ws, cudaStream_t st, bool* result_in_alt) {
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

// ------------------------------------------------- one-sweep radix sort --
constexpr int kOSThreads = 256;
constexpr int kOSItems = 16;
constexpr int kOSTile = kOSThreads * kOSItems;
// the workspace (radix_hist_elems) holds one status row per kSortTile keys
static_assert(kOSTile == kSortTile, "one-sweep tile must match the workspace tile");
constexpr int kOSWarps = kOSThreads / 32;
constexpr int kOSWarpItems = kOSTile / kOSWarps;  // consecutive items per warp
constexpr int kOSMaxPasses = 8;
constexpr uint32_t kOSValMask = (1u << 30) - 1u;
constexpr uint32_t kOSAgg = 1u << 30;  // tile aggregate published
constexpr uint32_t kOSInc = 2u << 30;  // inclusive prefix published
constexpr uint32_t kOSSpinLimit = 1u << 22;
constexpr int kOSLookBatch = 4;
// workspace (u32): counts [8][256] | offsets [8][256] | tile counters [8],
// ticket | status [passes][n_tiles][256]
constexpr int kOSCounters = 2 * kOSMaxPasses * 256;
constexpr int kOSHeader = kOSCounters + 256;
constexpr int64_t kOSMaxItems = (int64_t)1 << 30;  // prefixes fit 30 bits

__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* s_w) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  uint32_t wp = 0;
  for (int w = 0; w < warp; ++w) wp += s_w[w];
  __syncthreads();
  return wp + x - v;
}

template <typename K>
__global__ void __launch_bounds__(256) onesweep_hist_kernel(const K* __restrict__ keys, int64_t n,
                                                            int begin_bit, int passes,
                                                            uint32_t* __restrict__ ws) {
  __shared__ uint32_t s_h[kOSMaxPasses][256];
  __shared__ uint32_t s_w[8];
  __shared__ bool s_last;
  for (int e = threadIdx.x; e < kOSMaxPasses * 256; e += blockDim.x) (&s_h[0][0])[e] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const K k = keys[i];
    for (int p = 0; p < passes; ++p) atomicAdd(&s_h[p][digit_of(k, begin_bit + 8 * p)], 1u);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < passes * 256; e += blockDim.x) {
    const uint32_t c = (&s_h[0][0])[e];
    if (c) atomicAdd(&ws[e], c);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&ws[kOSCounters + kOSMaxPasses], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int p = 0; p < passes; ++p) {  // last block: digit offsets of every pass
    const uint32_t c = __ldcg(&ws[p * 256 + threadIdx.x]);
    const uint32_t e = block_excl_scan256(c, s_w);
    ws[kOSMaxPasses * 256 + p * 256 + threadIdx.x] = e;
  }
}

template <typename K>
__global__ void __launch_bounds__(kOSThreads) onesweep_pass_kernel(
    const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
    uint32_t* __restrict__ vout, int64_t n, int shift, int pass, int64_t n_tiles,
    uint32_t* __restrict__ ws, uint32_t* err) {
  extern __shared__ __align__(16) unsigned char os_smem[];
  K* s_keys = reinterpret_cast<K*>(os_smem);                          // [kOSTile]
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + kOSTile);   // [kOSTile]
  uint32_t* s_wh = s_vals + kOSTile;                                  // [kOSWarps][256]
  uint32_t* s_loc = s_wh + kOSWarps * 256;                            // [256]
  long long* s_gb = reinterpret_cast<long long*>(s_loc + 256);        // [256]
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_w[kOSWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(&ws[kOSCounters + pass], 1u);
  for (int e = tid; e < kOSWarps * 256; e += kOSThreads) s_wh[e] = 0;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t wbase = tile * kOSTile + (int64_t)warp * kOSWarpItems;
  K key[kOSItems];
  uint32_t rank[kOSItems];
#pragma unroll
  for (int r = 0; r < kOSItems; ++r) {
    const int64_t i = wbase + r * 32 + lane;
    key[r] = (i < n) ? kin[i] : (K)0;
  }
  // stable rank within the warp's 512 consecutive items
  uint32_t* wh = s_wh + warp * 256;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kOSItems; ++r) {
    const bool valid = wbase + r * 32 + lane < n;
    const uint32_t d = valid ? digit_of(key[r], shift) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (valid && lane == leader) {
      old = wh[d];
      wh[d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    rank[r] = old + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  // per digit (thread d): offsets of each warp, tile total, publication
  const int d = tid;
  uint32_t total = 0;
  for (int w = 0; w < kOSWarps; ++w) {
    const uint32_t c = s_wh[w * 256 + d];
    s_wh[w * 256 + d] = total;
    total += c;
  }
  uint32_t* status = ws + kOSHeader + ((int64_t)pass * n_tiles) * 256;
  st_relaxed_u32(&status[tile * 256 + d], (tile == 0 ? kOSInc : kOSAgg) | total);
  s_loc[d] = block_excl_scan256(total, s_w);
  // decoupled look-back over earlier tiles (bounded waits), four
  // predecessors' status words loaded at a time
  uint32_t excl = 0;
  if (tile > 0) {
    bool done = false;
    for (int64_t t = tile - 1; t >= 0 && !done; t -= kOSLookBatch) {
      uint32_t v[kOSLookBatch];
#pragma unroll
      for (int i = 0; i < kOSLookBatch; ++i)
        v[i] = (t - i >= 0) ? ld_relaxed_u32(&status[(t - i) * 256 + d]) : 0u;
#pragma unroll
      for (int i = 0; i < kOSLookBatch; ++i) {
        if (done || t - i < 0) break;
        const uint32_t* sp = &status[(t - i) * 256 + d];
        uint32_t sv = v[i];
        uint32_t spins = 0;
        while ((sv & ~kOSValMask) == 0u && ++spins < kOSSpinLimit) {
          if (spins > 32) __nanosleep(64);
          sv = ld_relaxed_u32(sp);
        }
        if ((sv & ~kOSValMask) == 0u) {
          raise_error(err, kErrWaitTimeout);
          done = true;
          break;
        }
        excl += sv & kOSValMask;
        if ((sv & ~kOSValMask) == kOSInc) done = true;
      }
    }
    st_relaxed_u32(&status[tile * 256 + d], kOSInc | ((excl + total) & kOSValMask));
  }
  s_gb[d] = (long long)ws[kOSMaxPasses * 256 + pass * 256 + d] + excl - s_loc[d];
  __syncthreads();
  // local sort by digit in shared memory
#pragma unroll
  for (int r = 0; r < kOSItems; ++r) {
    const int64_t i = wbase + r * 32 + lane;
    if (i < n) {
      const uint32_t dd = digit_of(key[r], shift);
      const uint32_t li = s_loc[dd] + s_wh[warp * 256 + dd] + rank[r];
      s_keys[li] = key[r];
      s_vals[li] = vin[i];
    }
  }
  __syncthreads();
  // digit runs out to their global positions
  const int cnt = (int)imin64(kOSTile, n - tile * kOSTile);
  for (int j = tid; j < cnt; j += kOSThreads) {
    const K k = s_keys[j];
    const long long pos = s_gb[digit_of(k, shift)] + j;
    kout[pos] = k;
    vout[pos] = s_vals[j];
  }
}

template <typename K>
static size_t onesweep_smem() {
  return (size_t)kOSTile * (sizeof(K) + 4) + (size_t)kOSWarps * 256 * 4 + 256 * 4 + 256 * 8;
}

template <typename K>
void radix_sort_pairs(K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                      int begin_bit, int end_bit, uint32_t* hist, uint32_t* scan_ws,
                      cudaStream_t st, bool* result_in_alt, uint32_t* err) {
  *result_in_alt = false;
  if (n <= 1) return;
  if (n >= kOSMaxItems) {
    radix_sort_pairs_3phase(keys, keys_alt, vals, vals_alt, n, begin_bit, end_bit, hist, scan_ws,
                            st, result_in_alt);
    return;
  }
  const int passes = (end_bit - begin_bit + 7) / 8;
  const int64_t n_tiles = ceil_div(n, kOSTile);
  uint32_t* ws = hist;
  NBGB_CUDA(cudaMemsetAsync(ws, 0, ((size_t)kOSHeader + (size_t)passes * n_tiles * 256) * 4, st));
  const unsigned hb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 4096), num_sms() * 4));
  onesweep_hist_kernel<K><<<hb, 256, 0, st>>>(keys, n, begin_bit, passes, ws);
  NBGB_LAUNCH_CHECK();
  const size_t smem = onesweep_smem<K>();
  NBGB_CUDA(cudaFuncSetAttribute(onesweep_pass_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  K* kin = keys;
  K* kout = keys_alt;
  uint32_t* vin = vals;
  uint32_t* vout = vals_alt;
  bool alt = false;
  for (int p = 0; p < passes; ++p) {
    onesweep_pass_kernel<K><<<(unsigned)n_tiles, kOSThreads, smem, st>>>(
        kin, vin, kout, vout, n, begin_bit + 8 * p, p, n_tiles, ws, err);
    NBGB_LAUNCH_CHECK();
    std::swap(kin, kout);
    std::swap(vin, vout);
    alt = !alt;
  }
  *result_in_alt = alt;
}

size_t radix_hist_elems(int64_t n) {
  const int64_t tiles = ceil_div(std::max<int64_t>(n, 1), kSortTile);
  return (size_t)kOSHeader + (size_t)kOSMaxPasses * 256 * tiles;  // covers the 3-phase layout too
}

template void radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, int64_t, int,
                                         int, uint32_t*, uint32_t*, cudaStream_t, bool*,
                                         uint32_t*);
template void radix_sort_pairs<unsigned long long>(unsigned long long*, unsigned long long*,
                                                   uint32_t*, uint32_t*, int64_t, int, int,
                                                   uint32_t*, uint32_t*, cudaStream_t, bool*,
                                                   uint32_t*);

}  // namespace nbgb
