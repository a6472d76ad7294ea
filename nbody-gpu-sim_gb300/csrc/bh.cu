// bh.cu -- Barnes-Hut on the device: path keys, radix sort, octree from
// sorted keys, bottom-up centre of mass, warp-cooperative walk (K2-K6), for
// one system or for many independent systems ("segments") in one pass.
//
// Replaces BarnesHutTree::build/computeForces and BarnesHutCalculator
// (src/cuda/force_barnes_hut.cu:125-583), whose octree is built on the host
// by sequential insertion and copied to the device every step.
//
// Tree.  The reference inserts bodies in Morton order into a point-region
// octree with one body per leaf, splitting leaves by float geometric
// subdivision (child centre = c +- half/2, octant bit0 = x >= c, bit1 = y,
// bit2 = z) down to depth 32, where bodies merge (:391-510).  Without the
// node-budget merge (:449-453, which only fires for N below ~64) that tree
// is canonical: a node exists for every octant-path prefix whose parent holds
// >= 2 bodies, a leaf is the shortest prefix unique to its body, and depth-32
// cells hold all their bodies.  It is built here in parallel:
//   1. per segment, the bounding box and the reference's root cube; every
//      body's path key = its 32 octants, computed with the reference's float
//      operations (levels 1..21 in a high 63-bit key, 22..32 in a low key);
//   2. stable radix sort by the high key, then (several segments) by
//      segment; bodies sharing segment and high key are put in (low key,
//      Morton key, index) order, i.e. the reference's insertion order inside
//      a shared depth-32 cell;
//   3. l_k = common levels of adjacent sorted keys of one segment; body k
//      starts the internal nodes of depths l_{k-1}+1 .. min(l_k, 31) and
//      (unless it shares a depth-32 cell with k-1) one leaf of depth
//      min(32, max(l_{k-1}, l_k) + 1); the first body of a segment also
//      starts the segment's root;
//   4. an exclusive scan of those counts numbers the nodes in depth-first
//      pre-order (children in octant order): every subtree, and every
//      segment's tree, is a contiguous index range, and
//      skip(P) = first node of body end(P)+1;
//   5. centres of mass bottom-up with per-node arrival counters, summing
//      children in octant order with the reference's float operations
//      (:514-538), so masses and centres of mass are bit-identical.
//
// Walk.  One warp walks its segment's pre-order range for 32 consecutive
// targets (path-sorted, so spatially close).  Every lane applies the
// reference's per-target rules (contains_i, leaf self-subtraction, opening
// test 4h^2/(d^2+eps^2) < theta^2, :175-243); the warp descends into a node
// if any active lane opens it, and a lane that accepted a node sleeps until
// the cursor leaves that node's subtree.  Each lane therefore sums exactly
// the reference's interaction set for its target (no stack, no local
// memory, broadcast node loads).  With leaf_capacity > 1 a subtree holding
// at most that many bodies is summed body by body when opened.  The group walk
// (one list per group of nearby bodies) is in bh_group.cu; the node record,
// state and shared parameters in bh_tree.cuh.
#include <algorithm>
#include <atomic>
#include <vector>

#include "bh.cuh"
#include "bh_tree.cuh"
#include "common.cuh"
#include "geom.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "sort.cuh"

namespace nbgb {

void bh_state_delete(BHState* p) { delete p; }

// ----------------------------------------------------------------- keys --
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// computeMortonCode (force_barnes_hut.cu:42-50) on (p - min) * inv.
__device__ __forceinline__ uint32_t morton_of(float4 p, const BBox& b) {
  float nx = __fmul_rn(__fsub_rn(p.x, b.min[0]), b.inv[0]);
  float ny = __fmul_rn(__fsub_rn(p.y, b.min[1]), b.inv[1]);
  float nz = __fmul_rn(__fsub_rn(p.z, b.min[2]), b.inv[2]);
  uint32_t ix = (uint32_t)__fmul_rn(fminf(fmaxf(nx, 0.0f), 1.0f), 1023.0f);
  uint32_t iy = (uint32_t)__fmul_rn(fminf(fmaxf(ny, 0.0f), 1.0f), 1023.0f);
  uint32_t iz = (uint32_t)__fmul_rn(fminf(fmaxf(nz, 0.0f), 1.0f), 1023.0f);
  return (spread3(ix) << 2) | (spread3(iy) << 1) | spread3(iz);
}

// Octant path of a position through the reference's subdivision: the high
// key (levels 1..21, 3 bits each, level 1 most significant) and the low key
// (levels 22..32).
__device__ __forceinline__ void path_key(float4 p, const BBox& b, u64& hi, u64& lo) {
  float cx = b.center[0], cy = b.center[1], cz = b.center[2], h = b.half;
  u64 a = 0, c = 0;
#pragma unroll
  for (int lev = 1; lev <= kMaxDepth; ++lev) {
    const uint32_t o = (p.x >= cx ? 1u : 0u) | (p.y >= cy ? 2u : 0u) | (p.z >= cz ? 4u : 0u);
    const float hs = __fmul_rn(h, 0.5f);
    cx = __fadd_rn(cx, (o & 1u) ? hs : -hs);
    cy = __fadd_rn(cy, (o & 2u) ? hs : -hs);
    cz = __fadd_rn(cz, (o & 4u) ? hs : -hs);
    h = hs;
    if (lev <= kHiLevels)
      a = (a << 3) | o;
    else
      c = (c << 3) | o;
  }
  hi = a;
  lo = c;
}

// ----------------------------------------------------- segment setup --
__global__ void seg_of_kernel(const int64_t* __restrict__ base, int nseg, int64_t n,
                              int32_t* __restrict__ seg_of) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {  // last s with base[s] <= q
      const int mid = (lo + hi + 1) >> 1;
      if (base[mid] <= q)
        lo = mid;
      else
        hi = mid - 1;
    }
    seg_of[q] = lo;
  }
}

// Order-preserving float <-> uint32 (for exact min/max with integer atomics).
__device__ __forceinline__ uint32_t f2ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Per-segment min/max of the bodies.  A block reduces a contiguous chunk;
// when the chunk lies in one segment (the common case) it issues one atomic
// per bound, otherwise each warp (or lane) does.  Min/max are exact, so the
// result equals the reference's computeBoundingBoxKernel (:78-122).
__global__ void seg_bounds_kernel(const float4* __restrict__ pm, SegView sv, int64_t n, int nseg,
                                  uint32_t* __restrict__ mm) {
  __shared__ float s_red[32][6];
  __shared__ int s_same;
  const int64_t c0 = (int64_t)blockIdx.x * blockDim.x * 4;
  const int64_t c1 = imin64(c0 + (int64_t)blockDim.x * 4, n);
  if (c0 >= n) return;
  if (threadIdx.x == 0) s_same = (sv.seg_of[c0] == sv.seg_of[c1 - 1]);
  __syncthreads();
  const bool same = s_same;
  float v[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = 0; r < 4; ++r) {
    const int64_t q = c0 + (int64_t)r * blockDim.x + threadIdx.x;
    if (q < c1) {
      const float4 p = pm[sv.arena((uint32_t)q)];
      if (same) {
        v[0] = fminf(v[0], p.x);
        v[1] = fminf(v[1], p.y);
        v[2] = fminf(v[2], p.z);
        v[3] = fmaxf(v[3], p.x);
        v[4] = fmaxf(v[4], p.y);
        v[5] = fmaxf(v[5], p.z);
      } else {
        const int s = sv.seg_of[q];
        atomicMin(&mm[0 * nseg + s], f2ord(p.x));
        atomicMin(&mm[1 * nseg + s], f2ord(p.y));
        atomicMin(&mm[2 * nseg + s], f2ord(p.z));
        atomicMax(&mm[3 * nseg + s], f2ord(p.x));
        atomicMax(&mm[4 * nseg + s], f2ord(p.y));
        atomicMax(&mm[5 * nseg + s], f2ord(p.z));
      }
    }
  }
  if (!same) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      v[a] = fminf(v[a], __shfl_down_sync(0xffffffffu, v[a], o));
      v[3 + a] = fmaxf(v[3 + a], __shfl_down_sync(0xffffffffu, v[3 + a], o));
    }
  if (lane == 0)
    for (int a = 0; a < 6; ++a) s_red[warp][a] = v[a];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      for (int a = 0; a < 3; ++a) {
        v[a] = fminf(v[a], s_red[w][a]);
        v[3 + a] = fmaxf(v[3 + a], s_red[w][3 + a]);
      }
    const int s = sv.seg_of[c0];
    for (int a = 0; a < 3; ++a) {
      atomicMin(&mm[a * nseg + s], f2ord(v[a]));
      atomicMax(&mm[(3 + a) * nseg + s], f2ord(v[3 + a]));
    }
  }
}

// Per segment: the reference's derived constants with its float operations
//   Morton scale  inv = 1.0f / (max - min + 0.001f)            (:313-320)
//   root centre   (min + max) * 0.5f                           (:418-419)
//   root half     max(ex, ey, ez) * 0.5f + 0.001f, first max   (:420-422)
__global__ void seg_box_kernel(const uint32_t* __restrict__ mm, int nseg, BBox* __restrict__ box,
                               uint32_t* err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) {
    BBox o;
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
      const float mn = ord2f(mm[a * nseg + s]), mx = ord2f(mm[(3 + a) * nseg + s]);
      o.min[a] = mn;
      o.max[a] = mx;
      ok = ok && isfinite(mn) && isfinite(mx);
      o.inv[a] = __fdiv_rn(1.0f, __fadd_rn(__fsub_rn(mx, mn), 0.001f));
      o.center[a] = __fmul_rn(__fadd_rn(mn, mx), 0.5f);
    }
    const float ex = __fsub_rn(o.max[0], o.min[0]), ey = __fsub_rn(o.max[1], o.min[1]),
                ez = __fsub_rn(o.max[2], o.min[2]);
    float ms = ex;
    if (ms < ey) ms = ey;
    if (ms < ez) ms = ez;
    o.half = __fadd_rn(__fmul_rn(ms, 0.5f), 0.001f);
    o.valid = ok ? 1 : 0;
    if (!ok) raise_error(err, kErrBadInput);
    box[s] = o;
  }
}

// High path key of every body in concatenated order (values = indices).
__global__ void path_hi_index_kernel(const float4* __restrict__ pm, SegView sv, int64_t n,
                                     u64* __restrict__ hi, uint32_t* __restrict__ idx) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    u64 h, l;
    path_key(pm[sv.arena((uint32_t)q)], sv.box[sv.seg_of[q]], h, l);
    hi[q] = h;
    idx[q] = (uint32_t)q;
  }
}

__global__ void seg_key_kernel(const uint32_t* __restrict__ idx, const int32_t* __restrict__ seg_of,
                               int64_t n, uint32_t* __restrict__ sk) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    sk[k] = (uint32_t)seg_of[idx[k]];
}

// Final order: segment, both path keys and the body itself per position.
__global__ void path_final_kernel(const float4* __restrict__ pm, SegView sv,
                                  const uint32_t* __restrict__ body, int64_t n,
                                  int32_t* __restrict__ kseg, u64* __restrict__ hi,
                                  u64* __restrict__ lo, float4* __restrict__ spm) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q = body[k];
    const int s = sv.seg_of[q];
    const float4 p = pm[sv.off[s] + ((int64_t)q - sv.base[s])];
    u64 h, l;
    path_key(p, sv.box[s], h, l);
    kseg[k] = s;
    hi[k] = h;
    lo[k] = l;
    spm[k] = p;
  }
}

// Tie key inside a run of equal (segment, high key): low key, then Morton
// key, then index.
__device__ __forceinline__ bool tie_less(const float4& pa, uint32_t a, const float4& pc,
                                         uint32_t c, const BBox& b) {
  u64 ha, la, hc, lc;
  path_key(pa, b, ha, la);
  path_key(pc, b, hc, lc);
  if (la != lc) return la < lc;
  const uint32_t ma = morton_of(pa, b), mc = morton_of(pc, b);
  if (ma != mc) return ma < mc;
  return a < c;
}

// Runs of equal (segment, high key) -- bodies sharing their first 21
// octants, tiny in practice -- are insertion-sorted by one thread per run;
// positions of a run that moved get their body, low key and payload fixed.
// A run already in order (e.g. coincident bodies) costs one comparison per
// body.
__global__ void tie_order_kernel(SegView sv, int64_t n, const int32_t* __restrict__ kseg,
                                 const u64* __restrict__ hi, uint32_t* __restrict__ body,
                                 u64* __restrict__ lo, float4* __restrict__ spm) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k + 1 < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (k > 0 && hi[k - 1] == hi[k] && kseg[k - 1] == kseg[k]) continue;
    if (hi[k + 1] != hi[k] || kseg[k + 1] != kseg[k]) continue;
    int64_t e = k + 1;
    while (e + 1 < n && hi[e + 1] == hi[k] && kseg[e + 1] == kseg[k]) ++e;
    const BBox b = sv.box[kseg[k]];
    bool moved = false;
    for (int64_t i = k + 1; i <= e; ++i) {
      const uint32_t cur = body[i];
      const float4 pc = spm[i];
      int64_t j = i - 1;
      while (j >= k && tie_less(pc, cur, spm[j], body[j], b)) {
        body[j + 1] = body[j];
        spm[j + 1] = spm[j];
        --j;
        moved = true;
      }
      body[j + 1] = cur;
      spm[j + 1] = pc;
    }
    if (moved)
      for (int64_t i = k; i <= e; ++i) {
        u64 h, l;
        path_key(spm[i], b, h, l);
        lo[i] = l;
      }
  }
}

// Morton keys scattered back to index order (for the on-demand key sort of a
// single system).
__global__ void morton_scatter_kernel(const float4* __restrict__ spm,
                                      const uint32_t* __restrict__ body, int64_t n,
                                      const BBox* __restrict__ box, uint32_t* __restrict__ keys,
                                      uint32_t* __restrict__ idx) {
  const BBox b = *box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = body[k];
    keys[i] = morton_of(spm[k], b);
    idx[i] = i;
  }
}

__device__ __forceinline__ int common_levels(u64 h0, u64 l0, u64 h1, u64 l1) {
  if (h0 != h1) return (__clzll(h0 ^ h1) - 1) / 3;  // bit 63 unused
  if (l0 != l1) return kHiLevels + (__clzll(l0 ^ l1) - 31) / 3;  // bits 63..33 unused
  return kMaxDepth;
}

// l_k (0 across a segment boundary) and per-body node counts: internal +
// leaf, + the root at the first body of a segment.
__global__ void lcp_count_kernel(const int32_t* __restrict__ kseg, const u64* __restrict__ hi,
                                 const u64* __restrict__ lo, int64_t n, uint8_t* __restrict__ lcp,
                                 uint32_t* __restrict__ cnt) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const bool first = (k == 0) || kseg[k - 1] != kseg[k];
    const bool last = (k + 1 == n) || kseg[k + 1] != kseg[k];
    const int lk = last ? 0 : common_levels(hi[k], lo[k], hi[k + 1], lo[k + 1]);
    const int lp = first ? 0 : common_levels(hi[k - 1], lo[k - 1], hi[k], lo[k]);
    if (k + 1 < n) lcp[k] = (uint8_t)lk;
    const int fd = first ? 1 : lp + 1;
    const int top = last ? 0 : min(lk, kMaxDepth - 1);
    uint32_t c = (uint32_t)max(0, top - fd + 1);
    const bool leaf_start = first || (lp < kMaxDepth);
    c += leaf_start ? 1u : 0u;
    if (first) c += 1u;  // the segment's root
    cnt[k] = c;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cnt[n] = 0;
}

// Range end of the depth-d node that contains sorted body k: the largest j of
// the same segment with common_levels(key_k, key_j) >= d.  Keys are sorted
// and segments contiguous, so the predicate is monotone in j: gallop, then
// bisect (Karras-style, O(log range)).
__device__ __forceinline__ bool same_prefix(const int32_t* kseg, const u64* hi, const u64* lo,
                                            int32_t s0, u64 h0, u64 l0, int64_t j, int d) {
  return kseg[j] == s0 && common_levels(h0, l0, hi[j], lo[j]) >= d;
}

__device__ __forceinline__ int64_t range_end(const int32_t* __restrict__ kseg,
                                             const u64* __restrict__ hi, const u64* __restrict__ lo,
                                             int64_t n, int64_t k, int d) {
  const u64 h0 = hi[k], l0 = lo[k];
  const int32_t s0 = kseg[k];
  int64_t good = k, step = 1;
  while (k + step < n && same_prefix(kseg, hi, lo, s0, h0, l0, k + step, d)) {
    good = k + step;
    step <<= 1;
  }
  int64_t bad = (k + step < n) ? k + step : n;
  while (bad - good > 1) {
    const int64_t mid = good + ((bad - good) >> 1);
    if (same_prefix(kseg, hi, lo, s0, h0, l0, mid, d))
      good = mid;
    else
      bad = mid;
  }
  return good;
}

struct EmitArgs {
  const int32_t* kseg;
  const uint8_t* lcp;
  const u64* hi;
  const u64* lo;
  const uint32_t* nstart;
  const float4* spm;
  const BBox* box;
  const int64_t* base;  // segment s occupies sorted positions [base[s], base[s+1])
  int64_t n;
  int64_t cap;
  Node* nodes;
  int32_t* parent;
  int32_t* visit;
  int32_t* seg_root;
  int32_t* seg_end;
  int32_t* seg_depth;
  int32_t* leaf_of;  // per sorted body: the leaf node it starts, or -1
  uint32_t* err;
};

__global__ void emit_nodes_kernel(EmitArgs a) {
  const uint32_t total = a.nstart[a.n];
  if ((int64_t)total > a.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(a.err, kErrTreeCapacity);
    return;
  }
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = a.kseg[k];
    const bool first = (k == 0) || a.kseg[k - 1] != s;
    const bool last = (k + 1 == a.n) || a.kseg[k + 1] != s;
    const int lk = last ? 0 : (int)a.lcp[k];
    const int lp = first ? 0 : (int)a.lcp[k - 1];
    const int fd = first ? 1 : lp + 1;
    const int top = last ? 0 : min(lk, kMaxDepth - 1);
    uint32_t idx = a.nstart[k];
    const float4 p = a.spm[k];
    const BBox b = a.box[s];
    if (first) {
      const int64_t send = a.base[s + 1];  // one past the segment's last position
      const uint32_t skip = (send < a.n) ? a.nstart[send] : total;
      a.nodes[idx].geom = make_float4(b.center[0], b.center[1], b.center[2], b.half);
      a.nodes[idx].info = make_int4((int)skip, 0, (int)k, (int)(send - k));
      a.parent[idx] = -1;
      a.visit[idx] = 0;
      a.seg_root[s] = (int32_t)idx;
      a.seg_end[s] = (int32_t)skip;
      ++idx;
    }
    // internal nodes of depth fd..top: slots claimed here (owner = k in
    // parent[]); their cubes are written below on the way down to k's leaf
    // (every owned depth lies above it), the rest by internal_nodes_kernel,
    // one thread per node
    const int n_int = max(0, top - fd + 1);
    const uint32_t int0 = idx;
    for (int j = 0; j < n_int; ++j) a.parent[idx + j] = (int32_t)k;
    idx += n_int;
    const bool leaf_start = first || (lp < kMaxDepth);
    int md = -1;
    if (!leaf_start) a.leaf_of[k] = -1;
    if (leaf_start) {
      const int ld = min(kMaxDepth, max(lp, lk) + 1);
      float cx = b.center[0], cy = b.center[1], cz = b.center[2], h = b.half;
      for (int lev = 1; lev <= ld; ++lev) {
        const uint32_t o = (p.x >= cx ? 1u : 0u) | (p.y >= cy ? 2u : 0u) | (p.z >= cz ? 4u : 0u);
        const float hs = __fmul_rn(h, 0.5f);
        cx = __fadd_rn(cx, (o & 1u) ? hs : -hs);
        cy = __fadd_rn(cy, (o & 2u) ? hs : -hs);
        cz = __fadd_rn(cz, (o & 4u) ? hs : -hs);
        h = hs;
        if (lev >= fd && lev <= top) a.nodes[int0 + (lev - fd)].geom = make_float4(cx, cy, cz, h);
      }
      int64_t e = k;
      while (e + 1 < a.n && a.kseg[e + 1] == s && (int)a.lcp[e] >= kMaxDepth) ++e;
      a.nodes[idx].geom = make_float4(cx, cy, cz, h);
      a.nodes[idx].info = make_int4((int)(idx + 1), (ld << 8) | 1, (int)k, (int)(e - k + 1));
      a.parent[idx] = -1;
      a.visit[idx] = 0;
      a.leaf_of[k] = (int32_t)idx;
      // reference max_depth_: depth of the inserting body's last loop level
      md = (ld == kMaxDepth && e > k) ? kMaxDepth : ld - 1;
    }
    // per-segment maximum: reduced over the lanes of the same segment, one
    // atomic per group and only while it can still raise the stored value
    const unsigned peers = __match_any_sync(__activemask(), s);
    const int gmax = __reduce_max_sync(peers, md);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && gmax > __ldcg(&a.seg_depth[s]))
      atomicMax(&a.seg_depth[s], gmax);
  }
}

// Internal nodes, one thread per node: the owner body k (the first body of
// the node's range) and the depth follow from k's slot numbering, the range
// end from a search over the sorted keys (the cube was written by
// emit_nodes_kernel on k's path).
__global__ void internal_nodes_kernel(EmitArgs a) {
  const uint32_t total = a.nstart[a.n];
  if ((int64_t)total > a.cap) return;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k32 = a.parent[q];
    if (k32 < 0) continue;  // a root or a leaf
    const int64_t k = k32;
    const int32_t s = a.kseg[k];
    const bool first = (k == 0) || a.kseg[k - 1] != s;
    const int fd = first ? 1 : (int)a.lcp[k - 1] + 1;
    const int d = fd + (int)(q - (int64_t)a.nstart[k]) - (first ? 1 : 0);
    const int64_t e = range_end(a.kseg, a.hi, a.lo, a.n, k, d);
    const uint32_t skip = (e + 1 < a.n) ? a.nstart[e + 1] : total;
    a.nodes[q].info = make_int4((int)skip, d << 8, (int)k, (int)(e - k + 1));
    a.visit[q] = 0;
  }
}

// Where link_kernel writes the group walk's groups.
struct GroupSink {
  const uint32_t* body;  // path-sorted position -> concatenated body index
  const int32_t* seg_of;
  int4* groups;          // first body, count, segment: classes 0 and 1
  int4* groups2;         // classes 2 and 3
  GroupCounters* gc;
  int gmax;              // largest group (32 or 64 bodies)
  int64_t gcap;          // groups capacity
  const uint32_t* body_cost;           // last walk's cost per body
  const unsigned long long* cost_acc;  // last walk's total cost, groups
};

// Parent links and child counts (children of P: P+1, skip(P+1), ... < skip(P)).
// With GROUPS it also emits the group walk's groups: roots with at most
// gmax bodies; below larger nodes, runs of consecutive children with at
// most gmax bodies in total (merged only when the parent holds at most
// kGroupMergeMax bodies: sibling cells of a large sparse node can lie far
// apart); depth-32 leaves larger than a group are split.  Every body
// belongs to exactly one group, and a group is one contiguous range of
// path-sorted bodies.  Groups go to four cost classes (GroupCounters) by
// the last walk's cost of their first body's group: classes 0 and 1 to the
// front and back of groups, 2 and 3 to those of groups2; the walk takes
// class 0 first, so the longest groups start early and its last tasks are
// short ones.
template <bool GROUPS>
__global__ void link_kernel(const Node* __restrict__ nodes, const uint32_t* __restrict__ nstart,
                            int64_t n, int64_t cap, int32_t* __restrict__ parent,
                            int32_t* __restrict__ nchild, GroupSink gs) {
  const uint32_t total = nstart[n];
  if ((int64_t)total > cap) return;
  const int gmax = gs.gmax;
  unsigned long long mean = ~0ull;  // no estimates before the first walk
  if (GROUPS && gs.cost_acc[1]) mean = gs.cost_acc[0] / gs.cost_acc[1];
  auto emit = [&](int f, int c) {
    const uint32_t b = gs.body[f];
    const unsigned long long e = gs.body_cost[b];
    const int cls = mean == ~0ull ? 3 : (e > 2 * mean ? 0 : (e > mean ? 1 : (2 * e > mean ? 2 : 3)));
    const uint32_t k = atomicAdd(&gs.gc->nclass[cls], 1u);
    int4* arr = cls < 2 ? gs.groups : gs.groups2;
    const int64_t g = (cls & 1) ? gs.gcap - 1 - (int64_t)k : (int64_t)k;
    arr[g] = make_int4(f, c, gs.seg_of[b], 0);
  };
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < (int64_t)total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 ip = nodes[p].info;  // skip, depth << 8 | leaf, first, count
    if (ip.y & 1) {
      nchild[p] = 0;
      if (GROUPS && ip.w > gmax)
        for (int f = 0; f < ip.w; f += gmax) emit(ip.z + f, min(gmax, ip.w - f));
      continue;
    }
    if (GROUPS && (ip.y >> 8) == 0 && ip.w <= gmax) emit(ip.z, ip.w);  // a small root
    const bool grp = GROUPS && ip.w > gmax, merge = ip.w <= kGroupMergeMax;
    int c = (int)p + 1, nc = 0, gf = 0, gn = 0;
    while (c < ip.x) {
      parent[c] = (int)p;
      ++nc;
      const int4 ci = nodes[c].info;
      if (grp) {
        if (ci.w > gmax) {
          if (gn) emit(gf, gn);
          gn = 0;
        } else if (gn && merge && gn + ci.w <= gmax) {
          gn += ci.w;
        } else {
          if (gn) emit(gf, gn);
          gf = ci.z;
          gn = ci.w;
        }
      }
      c = ci.x;
    }
    if (grp && gn) emit(gf, gn);
    nchild[p] = nc;
  }
}

// Arrival counter increment with acquire-release ordering at GPU scope.
__device__ __forceinline__ int arrive_acq_rel(int32_t* p) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// --------------------------------------------- reference-identical tree --
// NBGB_FLAG_REFERENCE_TREE: the reference's host build
// (BarnesHutTree::buildTreeOnHost, force_barnes_hut.cu:391-543) replayed by
// one device thread -- insertion in Morton order, leaf splitting, the node
// budget of 2N (a leaf is no longer split once node_count + 33 >= 2N, later
// bodies merge into it, :449-453), depth-32 merges (:490-507), the
// bottom-up centre of mass in descending node order (:514-538) -- with the
// reference's float operations, then renumbered depth-first into the walk's
// node records.  The canonical device build equals this tree whenever the
// budget does not fire; for small systems (N below about 100) it can fire.
constexpr int64_t kRefTreeMaxBodies = 65536;

struct RefNode {
  float cx, cy, cz, half;
  float comx, comy, comz, mass;
  int32_t child[8];
  int32_t pidx;   // first inserted body (original index), -1 for internal nodes
  int32_t count;  // bodies
  int32_t leaf;
  int32_t size;   // nodes in the subtree (renumbering)
  int32_t minpos; // smallest sorted position of a body in the subtree
};

__device__ void ref_node_default(RefNode& r) {
  r.cx = r.cy = r.cz = r.half = 0.f;
  r.comx = r.comy = r.comz = r.mass = 0.f;
  for (int c = 0; c < 8; ++c) r.child[c] = -1;
  r.pidx = -1;
  r.count = 0;
  r.leaf = 1;
  r.size = 1;
  r.minpos = 0x7fffffff;
}

__device__ __forceinline__ int ref_octant(float x, float y, float z, const RefNode& r) {
  return (x >= r.cx ? 1 : 0) | (y >= r.cy ? 2 : 0) | (z >= r.cz ? 4 : 0);
}

// mergeParticleIntoLeaf (:355-365)
__device__ void ref_merge(RefNode& r, int32_t q, float4 p) {
  const float t = __fadd_rn(r.mass, p.w);
  r.comx = __fdiv_rn(__fadd_rn(__fmul_rn(r.comx, r.mass), __fmul_rn(p.x, p.w)), t);
  r.comy = __fdiv_rn(__fadd_rn(__fmul_rn(r.comy, r.mass), __fmul_rn(p.y, p.w)), t);
  r.comz = __fdiv_rn(__fadd_rn(__fmul_rn(r.comz, r.mass), __fmul_rn(p.z, p.w)), t);
  r.mass = t;
  r.count += 1;
  if (r.pidx < 0) r.pidx = q;
}

// allocateLeaf (:368-389); false when the node array is full
__device__ bool ref_alloc_leaf(RefNode* rn, int64_t max_nodes, int& count, int parent, int oct,
                               int32_t q, float4 p) {
  if ((int64_t)count >= max_nodes) return false;
  const int ni = count++;
  RefNode& pa = rn[parent];
  pa.child[oct] = ni;
  pa.leaf = 0;
  const float hs = __fmul_rn(pa.half, 0.5f);
  RefNode& c = rn[ni];
  ref_node_default(c);
  c.cx = __fadd_rn(pa.cx, (oct & 1) ? hs : -hs);
  c.cy = __fadd_rn(pa.cy, (oct & 2) ? hs : -hs);
  c.cz = __fadd_rn(pa.cz, (oct & 4) ? hs : -hs);
  c.half = hs;
  c.pidx = q;
  c.count = 1;
  c.mass = p.w;
  c.comx = p.x;
  c.comy = p.y;
  c.comz = p.z;
  return true;
}

struct RefTreeArgs {
  const float4* pm;       // bodies by original index (one segment at offset 0)
  const uint32_t* order;  // original indices in (Morton key, index) order
  const uint32_t* body;   // sorted position -> original index
  const BBox* box;
  int64_t n;
  int64_t cap;            // walk node records available
  RefNode* rn;            // 2n reference nodes
  int32_t* pos_of;        // original index -> sorted position
  Node* nodes;
  int32_t* parent;
  uint32_t* nstart;       // nstart[n] = node count (the walk's capacity check)
  uint32_t* scalars;      // [0] node count
  int32_t* seg_root;
  int32_t* seg_end;
  int32_t* seg_depth;
  uint32_t* err;
};

__global__ void ref_tree_kernel(RefTreeArgs a) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int64_t n = a.n, max_nodes = 2 * n;  // the reference's max_nodes_ (:253)
  const BBox b = *a.box;
  RefNode* rn = a.rn;
  ref_node_default(rn[0]);
  rn[0].cx = b.center[0];
  rn[0].cy = b.center[1];
  rn[0].cz = b.center[2];
  rn[0].half = b.half;
  rn[0].leaf = 0;
  rn[0].count = (int32_t)n;
  int count = 1, max_depth = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t q = (int32_t)a.order[i];
    const float4 p = a.pm[q];
    int cur = 0, depth = 0;
    bool merged = false;
    while (depth < kMaxDepth) {
      RefNode& nd = rn[cur];
      if (nd.leaf) {
        if ((int64_t)count + kMaxDepth + 1 >= max_nodes) {  // the node budget
          ref_merge(nd, q, p);
          merged = true;
          break;
        }
        const int32_t eq = nd.pidx;
        const float4 ep = make_float4(nd.comx, nd.comy, nd.comz, nd.mass);
        nd.leaf = 0;
        nd.pidx = -1;
        nd.count = 0;
        nd.mass = 0.f;
        nd.comx = nd.comy = nd.comz = 0.f;
        const int eo = ref_octant(ep.x, ep.y, ep.z, nd);
        if (nd.child[eo] < 0 && !ref_alloc_leaf(rn, max_nodes, count, cur, eo, eq, ep)) {
          raise_error(a.err, kErrTreeCapacity);
          return;
        }
      }
      const int oct = ref_octant(p.x, p.y, p.z, rn[cur]);
      const int ch = rn[cur].child[oct];
      if (ch < 0) {
        if (!ref_alloc_leaf(rn, max_nodes, count, cur, oct, q, p)) {
          raise_error(a.err, kErrTreeCapacity);
          return;
        }
        break;
      }
      cur = ch;
      ++depth;
    }
    if (!merged && depth >= kMaxDepth) {  // coincident bodies: merge at depth 32
      int leaf = cur;
      while (!rn[leaf].leaf)
        for (int c = 0; c < 8; ++c)
          if (rn[leaf].child[c] >= 0) {
            leaf = rn[leaf].child[c];
            break;
          }
      ref_merge(rn[leaf], q, p);
    }
    max_depth = max(max_depth, depth);
  }
  if ((int64_t)count > a.cap) {
    raise_error(a.err, kErrTreeCapacity);
    return;
  }
  for (int64_t k = 0; k < n; ++k) a.pos_of[a.body[k]] = (int32_t)k;
  // centre of mass bottom-up (children have larger indices than their
  // parent), with subtree sizes and smallest body positions
  for (int i = count - 1; i >= 0; --i) {
    RefNode& nd = rn[i];
    nd.size = 1;
    if (nd.leaf) {
      nd.minpos = a.pos_of[nd.pidx];
      continue;
    }
    float tm = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
    int32_t cnt = 0;
    nd.minpos = 0x7fffffff;
    for (int c = 0; c < 8; ++c) {
      const int ci = nd.child[c];
      if (ci < 0) continue;
      const RefNode& ch = rn[ci];
      tm = __fadd_rn(tm, ch.mass);
      sx = __fadd_rn(sx, __fmul_rn(ch.comx, ch.mass));
      sy = __fadd_rn(sy, __fmul_rn(ch.comy, ch.mass));
      sz = __fadd_rn(sz, __fmul_rn(ch.comz, ch.mass));
      cnt += ch.count;
      nd.size += ch.size;
      nd.minpos = min(nd.minpos, ch.minpos);
    }
    nd.mass = tm;
    nd.count = cnt;
    if (tm > 0.f) {
      nd.comx = __fdiv_rn(sx, tm);
      nd.comy = __fdiv_rn(sy, tm);
      nd.comz = __fdiv_rn(sz, tm);
    }
  }
  // depth-first renumbering (octant order), skip = next node after the
  // subtree, next-sibling flags for the walk records
  struct Item {
    int ref, parent, depth, next;
  };
  Item stack[8 * (kMaxDepth + 2)];
  int sp = 0, id = 0;
  stack[sp++] = Item{0, -1, 0, 0};
  while (sp > 0) {
    const Item it = stack[--sp];
    const RefNode& nd = rn[it.ref];
    const int me = id++;
    const int4 info = make_int4(me + nd.size, (it.depth << 8) | (nd.leaf ? 1 : 0),
                                nd.leaf ? a.pos_of[nd.pidx] : nd.minpos, nd.count);
    Node& o = a.nodes[me];
    o.com = make_float4(nd.comx, nd.comy, nd.comz, nd.mass);
    o.geom = make_float4(nd.cx, nd.cy, nd.cz, nd.half);
    o.info = info;
    o.walk = walk_record(info, nd.half, nd.mass, it.next != 0);
    a.parent[me] = it.parent;
    if (nd.leaf) continue;
    int last = -1;
    for (int c = 7; c >= 0; --c)
      if (nd.child[c] >= 0) {
        stack[sp++] = Item{nd.child[c], me, it.depth + 1, last >= 0 ? 1 : 0};
        last = c;
      }
  }
  a.nstart[n] = (uint32_t)count;
  a.scalars[0] = (uint32_t)count;
  a.seg_root[0] = 0;
  a.seg_end[0] = count;
  a.seg_depth[0] = max_depth;
}

constexpr int kComThreads = 64;

// Leaves: mass/com as the reference's allocateLeaf + mergeParticleIntoLeaf
// (force_barnes_hut.cu:355-389); then the last-arriving child of each node
// computes that node from all its children in octant order (:514-538).
__global__ void com_kernel(Node* __restrict__ nodes, const float4* __restrict__ spm,
                           const uint32_t* __restrict__ nstart, int64_t n, int64_t cap,
                           const int32_t* __restrict__ parent, const int32_t* __restrict__ nchild,
                           int32_t* __restrict__ visit, const int32_t* __restrict__ leaf_of) {
  const uint32_t total = nstart[n];
  if ((int64_t)total > cap) return;
  // one thread per sorted body; the bodies that start a leaf carry it
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = leaf_of[k];
    if (p < 0) continue;
    const int4 ip = nodes[p].info;
    float4 b0 = spm[ip.z];
    float m = b0.w, cx = b0.x, cy = b0.y, cz = b0.z;
    for (int j = 1; j < ip.w; ++j) {
      const float4 q = spm[ip.z + j];
      const float t = __fadd_rn(m, q.w);
      cx = __fdiv_rn(__fadd_rn(__fmul_rn(cx, m), __fmul_rn(q.x, q.w)), t);
      cy = __fdiv_rn(__fadd_rn(__fmul_rn(cy, m), __fmul_rn(q.y, q.w)), t);
      cz = __fdiv_rn(__fadd_rn(__fmul_rn(cz, m), __fmul_rn(q.z, q.w)), t);
      m = t;
    }
    nodes[p].com = make_float4(cx, cy, cz, m);
    int node = parent[p];
    nodes[p].walk = walk_record(ip, nodes[p].geom.w, m, has_next_sibling(nodes, ip.x, node));
    while (node >= 0) {
      // release: this child's centre of mass is visible to the sibling that
      // arrives last; acquire: the last one sees every sibling's
      if (arrive_acq_rel(&visit[node]) != nchild[node] - 1) break;
      const int4 in = nodes[node].info;
      float tm = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
      int c = node + 1;
      while (c < in.x) {
        const float4 q = __ldcg(&nodes[c].com);
        tm = __fadd_rn(tm, q.w);
        sx = __fadd_rn(sx, __fmul_rn(q.x, q.w));
        sy = __fadd_rn(sy, __fmul_rn(q.y, q.w));
        sz = __fadd_rn(sz, __fmul_rn(q.z, q.w));
        c = nodes[c].info.x;
      }
      float4 r = make_float4(0.f, 0.f, 0.f, tm);
      if (tm > 0.0f) {
        r.x = __fdiv_rn(sx, tm);
        r.y = __fdiv_rn(sy, tm);
        r.z = __fdiv_rn(sz, tm);
      }
      __stcg(&nodes[node].com, r);
      const int up = parent[node];
      nodes[node].walk = walk_record(in, nodes[node].geom.w, r.w, has_next_sibling(nodes, in.x, up));
      node = up;
    }
  }
}

// ----------------------------------------------------------------- walk --
struct WalkArgs {
  const Node* nodes;
  const float4* spm;
  const uint32_t* body;
  const uint32_t* nstart;
  SegView sv;
  const WarpTask* tasks;
  int64_t ntasks;
  const int32_t* seg_root;
  const int32_t* seg_end;
  int64_t n;
  int64_t cap;
  float theta2;
  float th_lo;  // theta2 * (1 - 2^-16)
  float th_hi;  // theta2 * (1 + 2^-16)
  float eps2;
  float G;
  int leaf_cap;
  float* ax;
  float* ay;
  float* az;
  int32_t* counts;                  // per-body interaction counts (or null)
  unsigned long long* inter_total;  // sum of interactions (or null)
  uint32_t* task_ctr;               // zeroed before the launch
};

// The reference's opening test `size2 / dist2 < theta2` with the correctly
// rounded quotient (force_barnes_hut.cu:222-224), decided by two FP32
// products against thresholds theta2 (1 -+ 2^-16) whenever size2 is not
// within 2^-16 (relative) of theta2 * dist2 -- almost always -- and by the
// IEEE division otherwise.  With |rounding| <= 2^-24 per product, a product
// test that fires implies the exact quotient is below theta2 (1 - 2^-17),
// resp. above theta2 (1 + 2^-17), so the outcome equals the IEEE comparison.
__device__ __forceinline__ bool opening_accept(float size2, float d2, float th_lo, float th_hi,
                                               float theta2) {
  if (size2 < d2 * th_lo) return true;
  if (size2 > d2 * th_hi) return false;
  return __fdiv_rn(size2, d2) < theta2;
}

__device__ __forceinline__ void bh_add(float px, float py, float pz, float m, float xi, float yi,
                                       float zi, float eps2, float& sx, float& sy, float& sz) {
  const float dx = __fsub_rn(px, xi), dy = __fsub_rn(py, yi), dz = __fsub_rn(pz, zi);
  const float d2 = __fadd_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))), eps2);
  const float r = rsqrt_approx(d2);
  const float f = (m * r) * (r * r);
  sx = fmaf(f, dx, sx);
  sy = fmaf(f, dy, sy);
  sz = fmaf(f, dz, sz);
}

template <bool COUNT, bool BUCKET>
__global__ void __launch_bounds__(256, BUCKET ? 6 : (COUNT ? 7 : 8)) bh_walk_kernel(WalkArgs a) {
  const uint32_t total = a.nstart[a.n];
  const bool tree_ok = (int64_t)total <= a.cap;
  const int lane = threadIdx.x & 31;
  // persistent warps take the next task (32 path-consecutive targets) from a
  // counter: the walk cost per task varies a lot, so this balances the SMs
  while (true) {
    uint32_t t32 = 0;
    if (lane == 0) t32 = atomicAdd(a.task_ctr, 1u);
    const int64_t t = __shfl_sync(0xffffffffu, t32, 0);
    if (t >= a.ntasks) break;
    const WarpTask task = a.tasks[t];
    const int64_t k = task.first + lane;
    const bool valid = k < task.end;
    const float4 pi = valid ? a.spm[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const f2 pi_xy = f2_make(pi.x, pi.y);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    int cnt = 0;
    int resume = valid ? 0 : 0x7fffffff;
    int node = tree_ok ? a.seg_root[task.seg] : 0;
    const int node_end = tree_ok ? a.seg_end[task.seg] : 0;
    while (node < node_end) {
      // one 32-byte load (centre of mass + cube) as four x/y, z/w pairs, one
      // 8-byte load (skip and flags, size2); x and y differences are taken
      // as packed FP32x2 (same IEEE rounding per component)
      f2 cm_xy, cm_zw, g_xy, g_zw;
      ld_node2(&a.nodes[node], cm_xy, cm_zw, g_xy, g_zw);
      float4 cm, g;
      f2_split(cm_xy, cm.x, cm.y);
      f2_split(cm_zw, cm.z, cm.w);
      f2_split(g_xy, g.x, g.y);
      f2_split(g_zw, g.z, g.w);
      float tx, ty;  // target minus cube centre
      f2_split(f2_sub(pi_xy, g_xy), tx, ty);
      // the bucket walk also needs the node's body range (same 16-byte load)
      int4 wr;
      if (BUCKET) {
        wr = __ldg(&a.nodes[node].walk);
      } else {
        const int2 w2 = __ldg(reinterpret_cast<const int2*>(&a.nodes[node].walk));
        wr = make_int4(w2.x, w2.y, 0, 0);
      }
      const int skip = wr.x & (int)(kWalkZero - 1u);
      if ((uint32_t)wr.x >= kWalkZero) {  // a leaf, or zero mass
        if ((uint32_t)wr.x & kWalkZero) {  // force_barnes_hut.cu:172-173
          node = skip;
          continue;
        }
        // leaf (force_barnes_hut.cu:185-203)
        if (node >= resume) {
          float me = cm.w, cx = cm.x, cy = cm.y, cz = cm.z;
          bool use = true;
          if (fabsf(tx) <= g.w && fabsf(ty) <= g.w && fabsf(__fsub_rn(pi.z, g.z)) <= g.w) {
            me = __fsub_rn(cm.w, pi.w);
            use = me > 0.0f;
            if (use) {
              cx = __fdiv_rn(__fsub_rn(__fmul_rn(cm.x, cm.w), __fmul_rn(pi.x, pi.w)), me);
              cy = __fdiv_rn(__fsub_rn(__fmul_rn(cm.y, cm.w), __fmul_rn(pi.y, pi.w)), me);
              cz = __fdiv_rn(__fsub_rn(__fmul_rn(cm.z, cm.w), __fmul_rn(pi.z, pi.w)), me);
            }
          }
          if (use) {
            bh_add(cx, cy, cz, me, pi.x, pi.y, pi.z, a.eps2, sx, sy, sz);
            if (COUNT) ++cnt;
          }
        }
        node = skip;
        continue;
      }
      // internal node (force_barnes_hut.cu:205-243)
      const bool active = node >= resume;
      const bool contains =
          fabsf(tx) <= g.w && fabsf(ty) <= g.w && fabsf(__fsub_rn(pi.z, g.z)) <= g.w;
      float dx, dy;
      f2_split(f2_sub(cm_xy, pi_xy), dx, dy);
      const float dz = __fsub_rn(cm.z, pi.z);
      const float d2 = __fadd_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))), a.eps2);
      const float size2 = __int_as_float(wr.y);
      const bool accept = !contains && opening_accept(size2, d2, a.th_lo, a.th_hi, a.theta2);
      const bool open = active && !accept;
      if (active && accept) {
        const float r = rsqrt_approx(d2);
        const float f = (cm.w * r) * (r * r);
        sx = fmaf(f, dx, sx);
        sy = fmaf(f, dy, sy);
        sz = fmaf(f, dz, sz);
        if (COUNT) ++cnt;
        resume = skip;
      }
      if (BUCKET && (int)((uint32_t)wr.w & ~kWalkNext) <= a.leaf_cap) {
        // a subtree of at most leaf_cap bodies: the lanes that open it sum
        // its bodies directly (all read the same body: one broadcast load)
        if (open) {
          const int64_t self = k - wr.z;
          const int nb = (int)((uint32_t)wr.w & ~kWalkNext);
          for (int j = 0; j < nb; ++j) {
            const float4 q = __ldg(&a.spm[wr.z + j]);
            if (j != self) {
              bh_add(q.x, q.y, q.z, q.w, pi.x, pi.y, pi.z, a.eps2, sx, sy, sz);
              if (COUNT) ++cnt;
            }
          }
        }
        node = skip;
        continue;
      }
      node = __any_sync(0xffffffffu, open) ? node + 1 : skip;
    }
    if (valid) {
      const int64_t i = a.sv.arena(a.body[k]);
      a.ax[i] = a.G * sx;
      a.ay[i] = a.G * sy;
      a.az[i] = a.G * sz;
      if (COUNT && a.counts) a.counts[i] = cnt;
    }
    if (COUNT && a.inter_total) {
      unsigned long long c = valid ? (unsigned long long)cnt : 0ull;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
      if (lane == 0) atomicAdd(a.inter_total, c);
    }
  }
}

static unsigned grid1d(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), threads), (int64_t)num_sms() * 32));
}

// ------------------------------------------------------ host driver --
size_t bh_state_bytes(const BHState* p) {
  if (!p) return 0;
  const BHState& h = *p;
  return h.tables.bytes() + h.seg_of.bytes() + h.seg_minmax.bytes() + h.box.bytes() +
         h.seg_root.bytes() + h.seg_end.bytes() + h.seg_depth.bytes() + h.mkeys.bytes() + h.mkeys_alt.bytes() + h.midx.bytes() +
         h.midx_alt.bytes() + h.klo.bytes() + h.khi.bytes() + h.khi_alt.bytes() +
         h.pidx.bytes() + h.pidx_alt.bytes() + h.sk.bytes() + h.sk_alt.bytes() + h.kseg.bytes() +
         h.hist.bytes() + h.scan_ws.bytes() + h.lcp.bytes() + h.ncnt.bytes() + h.nstart.bytes() +
         h.scalars.bytes() + h.nodes.bytes() +
         h.node_parent.bytes() + h.node_nchild.bytes() + h.node_visit.bytes() +
         h.leaf_of.bytes() + h.ref_nodes.bytes() + h.ref_pos.bytes() + h.spm.bytes() +
         h.walk_ctr.bytes() + h.groups.bytes() + h.groups2.bytes() + h.body_cost.bytes() + h.cost_acc.bytes() +
         h.group_ctr.bytes() + h.group_ovf.bytes();
}

size_t bh_bytes_estimate(int64_t n) { return (size_t)n * 480 + (64u << 10); }

BHState* bh_state_new() { return new BHState(); }

size_t bh_segment_table_bytes(const int64_t* n_per, int nseg) {
  int64_t ntask = 0;
  for (int s = 0; s < nseg; ++s) ntask += ceil_div(n_per[s], 32);
  return ((size_t)nseg * 2 + 1) * sizeof(int64_t) + (size_t)ntask * sizeof(WarpTask);
}

// Segment tables -- arena offsets, first concatenated index (prefix sums of
// the sizes) and warp tasks -- go up in one copy; seg_of is derived on the
// device.
void bh_set_segments(BHState& h, const int64_t* off, const int64_t* n_per, int nseg,
                     cudaStream_t st, char* staging) {
  if (nseg < 1) fail(NBGB_ERR_INVALID_ARG, "Validation Error: no Barnes-Hut segment");
  const size_t bytes = bh_segment_table_bytes(n_per, nseg);
  if (!staging) {
    NBGB_CUDA(cudaStreamSynchronize(st));  // the internal staging buffer is reused below
    staging = h.h_tables.ensure(bytes);
  }
  int64_t* hoff = reinterpret_cast<int64_t*>(staging);
  int64_t* hbase = hoff + nseg;
  WarpTask* ht = reinterpret_cast<WarpTask*>(hbase + nseg + 1);
  int64_t t = 0, n = 0;
  for (int s = 0; s < nseg; ++s) {
    if (n_per[s] < 1) fail(NBGB_ERR_INVALID_ARG, "Validation Error: empty Barnes-Hut segment");
    hoff[s] = off[s];
    hbase[s] = n;
    for (int64_t f = n; f < n + n_per[s]; f += 32) ht[t++] = WarpTask{f, n + n_per[s], s, 0};
    n += n_per[s];
  }
  hbase[nseg] = n;
  char* d = grow(h.tables, bytes);
  NBGB_CUDA(cudaMemcpyAsync(d, staging, bytes, cudaMemcpyHostToDevice, st));
  h.nseg = nseg;
  h.ntasks = t;
  h.n = n;
  if (n > h.reserve) h.reserve = std::max(n, h.reserve + h.reserve / 2);
  h.seg_off_p = reinterpret_cast<int64_t*>(d);
  h.seg_base_p = h.seg_off_p + nseg;
  h.tasks_p = reinterpret_cast<WarpTask*>(h.seg_base_p + nseg + 1);
  int32_t* so = grow(h.seg_of, (size_t)h.reserve);
  seg_of_kernel<<<grid1d(n), 256, 0, st>>>(h.seg_base_p, nseg, n, so);
  NBGB_LAUNCH_CHECK();
}

// Builds the trees of all segments (positions and masses read from `pm` at
// each segment's offset).
void bh_build(BHState& h, const float4* pm, cudaStream_t st, uint32_t* err, bool groups,
              int group_max, bool ref_tree, StageTimer* timer) {
  stage_mark(timer, "barnes_hut.bounds");
  h.built = false;  // until every kernel of this build is enqueued
  h.groups_ready = false;
  h.keys_valid = false;
  const int64_t n = h.n;
  const int nseg = h.nseg;
  const size_t R = (size_t)h.reserve;  // per-body buffers are sized for the reserve
  SegView sv{h.seg_off_p, h.seg_base_p, h.seg_of.ptr, grow(h.box, (size_t)nseg)};
  // 1. per-segment bounds and root cubes
  uint32_t* mm = grow(h.seg_minmax, (size_t)nseg * 6);
  NBGB_CUDA(cudaMemsetAsync(mm, 0xFF, (size_t)nseg * 3 * sizeof(uint32_t), st));
  NBGB_CUDA(cudaMemsetAsync(mm + (size_t)nseg * 3, 0x00, (size_t)nseg * 3 * sizeof(uint32_t), st));
  seg_bounds_kernel<<<(unsigned)ceil_div(n, 1024), 256, 0, st>>>(pm, sv, n, nseg, mm);
  NBGB_LAUNCH_CHECK();
  seg_box_kernel<<<(unsigned)ceil_div(nseg, 128), 128, 0, st>>>(mm, nseg, h.box.ptr, err);
  NBGB_LAUNCH_CHECK();
  // 2. keys and order
  uint32_t* hist = grow(h.hist, radix_hist_elems((int64_t)R));
  uint32_t* sws = grow(h.scan_ws, scan_workspace_elems((int64_t)radix_hist_elems((int64_t)R)) +
                                      scan_workspace_elems((int64_t)R + 1));
  u64* hi = grow(h.khi, R);
  u64* hi2 = grow(h.khi_alt, R);
  u64* lo = grow(h.klo, R);
  uint32_t* pb = grow(h.pidx, R);
  uint32_t* pb2 = grow(h.pidx_alt, R);
  stage_mark(timer, "barnes_hut.keys");
  path_hi_index_kernel<<<grid1d(n), 256, 0, st>>>(pm, sv, n, hi, pb);
  NBGB_LAUNCH_CHECK();
  stage_mark(timer, "barnes_hut.sort");
  bool alt = false;
  radix_sort_pairs<u64>(hi, hi2, pb, pb2, n, 0, 64, hist, sws, st, &alt, err);
  uint32_t* body = alt ? pb2 : pb;
  uint32_t* body_other = alt ? pb : pb2;
  stage_mark(timer, "barnes_hut.order");
  if (nseg > 1) {
    // stable sort by segment: (segment, path) order
    uint32_t* sk = grow(h.sk, R);
    uint32_t* sk2 = grow(h.sk_alt, R);
    seg_key_kernel<<<grid1d(n), 256, 0, st>>>(body, h.seg_of.ptr, n, sk);
    NBGB_LAUNCH_CHECK();
    int bits = 1;
    while (bits < 31 && (1 << bits) < nseg) ++bits;
    bool alt2 = false;
    radix_sort_pairs<uint32_t>(sk, sk2, body, body_other, n, 0, ((bits + 7) / 8) * 8, hist, sws,
                               st, &alt2, err);
    if (alt2) std::swap(body, body_other);
  }
  h.body = body;
  int32_t* kseg = grow(h.kseg, R);
  float4* spm = grow(h.spm, R);
  path_final_kernel<<<grid1d(n), 256, 0, st>>>(pm, sv, body, n, kseg, hi, lo, spm);
  NBGB_LAUNCH_CHECK();
  tie_order_kernel<<<grid1d(n), 256, 0, st>>>(sv, n, kseg, hi, body, lo, spm);
  NBGB_LAUNCH_CHECK();
  h.keys_valid = false;  // Morton (key, index) pairs are produced on demand
  if (ref_tree) {
    if (nseg != 1 || n > kRefTreeMaxBodies)
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: the reference tree takes one system of at most 65536 bodies");
    // insertion order: the reference's Morton keys, stably sorted (:308-328)
    stage_mark(timer, "barnes_hut.reference_tree");
    uint32_t* mk = grow(h.mkeys, R);
    uint32_t* mi = grow(h.midx, R);
    uint32_t* mk2 = grow(h.mkeys_alt, R);
    uint32_t* mi2 = grow(h.midx_alt, R);
    morton_scatter_kernel<<<grid1d(n), 256, 0, st>>>(spm, body, n, h.box.ptr, mk, mi);
    NBGB_LAUNCH_CHECK();
    radix_sort_pairs<uint32_t>(mk, mk2, mi, mi2, n, 0, 32, hist, sws, st, &h.m_alt, err);
    h.keys_valid = true;
    const int64_t cap_min = 2 * n + 64;
    if (h.cap < cap_min) h.cap = cap_min;
    RefTreeArgs ra;
    ra.pm = pm;
    ra.order = h.m_alt ? mi2 : mi;
    ra.body = body;
    ra.box = h.box.ptr;
    ra.n = n;
    ra.cap = h.cap;
    ra.rn = reinterpret_cast<RefNode*>(grow(h.ref_nodes, (size_t)(2 * n + 1) * sizeof(RefNode)));
    ra.pos_of = grow(h.ref_pos, R);
    ra.nodes = grow(h.nodes, (size_t)h.cap);
    ra.parent = grow(h.node_parent, (size_t)h.cap);
    ra.nstart = grow(h.nstart, R + 1);
    ra.scalars = grow(h.scalars, 2);
    ra.seg_root = grow(h.seg_root, 1);
    ra.seg_end = grow(h.seg_end, 1);
    ra.seg_depth = grow(h.seg_depth, 1);
    ra.err = err;
    ref_tree_kernel<<<1, 1, 0, st>>>(ra);
    NBGB_LAUNCH_CHECK();
    h.groups_ready = false;
    h.built = true;
    return;
  }
  // 3.-4. node counts, numbering, emission
  stage_mark(timer, "barnes_hut.nodes");
  uint8_t* lcp = grow(h.lcp, R);
  uint32_t* cnt = grow(h.ncnt, R + 1);
  uint32_t* nst = grow(h.nstart, R + 1);
  uint32_t* sc = grow(h.scalars, 2);
  lcp_count_kernel<<<grid1d(n), 256, 0, st>>>(kseg, hi, lo, n, lcp, cnt);
  NBGB_LAUNCH_CHECK();
  scan_exclusive_u32(cnt, nst, n + 1, sws, sc, st);
  int32_t* sdepth = grow(h.seg_depth, (size_t)nseg);
  NBGB_CUDA(cudaMemsetAsync(sdepth, 0, (size_t)nseg * sizeof(int32_t), st));
  const int64_t min_cap = 2 * n + 64 * (int64_t)nseg;
  if (h.cap < min_cap) h.cap = 3 * n + 64 * (int64_t)nseg;
  if (h.cap >= kMaxWalkNodes)
    fail(NBGB_ERR_OVERFLOW, "Barnes-Hut node capacity above 2^30 nodes: too many bodies in one tree build");
  Node* nodes = grow(h.nodes, (size_t)h.cap);
  int32_t* par = grow(h.node_parent, (size_t)h.cap);
  int32_t* nch = grow(h.node_nchild, (size_t)h.cap);
  int32_t* vis = grow(h.node_visit, (size_t)h.cap);
  int32_t* leaf_of = grow(h.leaf_of, R);
  EmitArgs ea{kseg, lcp, hi, lo, nst, spm, h.box.ptr, h.seg_base_p, n, h.cap, nodes, par,
              vis, grow(h.seg_root, (size_t)nseg), grow(h.seg_end, (size_t)nseg), sdepth,
              leaf_of, err};
  emit_nodes_kernel<<<grid1d(n), 256, 0, st>>>(ea);
  NBGB_LAUNCH_CHECK();
  internal_nodes_kernel<<<grid1d(h.cap), 256, 0, st>>>(ea);
  NBGB_LAUNCH_CHECK();
  if (groups) {
    h.group_max = group_max > 0 ? group_max : bh_group_max(n);
    uint32_t* bc_old = h.body_cost.ptr;
    uint32_t* bc = grow(h.body_cost, R);
    if (bc != bc_old) NBGB_CUDA(cudaMemsetAsync(bc, 0, h.body_cost.cap * sizeof(uint32_t), st));
    unsigned long long* acc_old = h.cost_acc.ptr;
    unsigned long long* acc = grow(h.cost_acc, 2);
    if (acc != acc_old) NBGB_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), st));
    int4* gr = grow(h.groups, R);
    int4* gr2 = h.groups2.ensure(h.groups.cap);
    GroupSink gs{h.body, h.seg_of.ptr, gr, gr2,
                 reinterpret_cast<GroupCounters*>(grow(h.group_ctr, sizeof(GroupCounters))),
                 h.group_max, (int64_t)h.groups.cap, bc, acc};
    NBGB_CUDA(cudaMemsetAsync(gs.gc, 0, sizeof(GroupCounters), st));
    link_kernel<true><<<grid1d(h.cap), 256, 0, st>>>(nodes, nst, n, h.cap, par, nch, gs);
    NBGB_LAUNCH_CHECK();
    // the coming walk adds up its own costs
    NBGB_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), st));
  } else {
    link_kernel<false><<<grid1d(h.cap), 256, 0, st>>>(nodes, nst, n, h.cap, par, nch, GroupSink{});
  }
  NBGB_LAUNCH_CHECK();
  h.groups_ready = groups;
  // one thread per body that starts a leaf (found through leaf_of, so no
  // thread idles on an unused node slot): it carries centres of mass up the
  // tree, so bodies are not chained per thread (one resident wave of threads
  // striding over the node slots was 0.3 ms per serving tick slower); blocks
  // of two warps, so that a block waiting for one long climb holds few slots
  stage_mark(timer, "barnes_hut.com");
  com_kernel<<<(unsigned)ceil_div(std::max<int64_t>(n, 1), kComThreads), kComThreads, 0, st>>>(
      nodes, spm, nst, n, h.cap, par, nch, vis, leaf_of);
  NBGB_LAUNCH_CHECK();
  h.built = true;
}

// Resident 256-thread blocks per SM of one walk instantiation.
template <bool COUNT, bool BUCKET>
static int walk_occupancy() {
  static const int occ = [] {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, bh_walk_kernel<COUNT, BUCKET>, 256, 0);
    return std::max(b, 1);
  }();
  return occ;
}

// Forces for every segment: acc written at each segment's arena offset.
void bh_walk(BHState& h, const BHWalkParams& p, float* ax, float* ay, float* az, int32_t* counts,
             unsigned long long* inter_total, uint32_t* err, cudaStream_t st) {
  if (p.group_walk) {
    bh_group_walk(h, p, ax, ay, az, counts, inter_total, err, st);
    return;
  }
  WalkArgs w;
  w.nodes = h.nodes.ptr;
  w.spm = h.spm.ptr;
  w.body = h.body;
  w.nstart = h.nstart.ptr;
  w.sv = SegView{h.seg_off_p, h.seg_base_p, h.seg_of.ptr, h.box.ptr};
  w.tasks = h.tasks_p;
  w.ntasks = h.ntasks;
  w.seg_root = h.seg_root.ptr;
  w.seg_end = h.seg_end.ptr;
  w.n = h.n;
  w.cap = h.cap;
  w.theta2 = p.theta * p.theta;
  w.th_lo = w.theta2 * (1.0f - 1.52587890625e-05f);
  w.th_hi = w.theta2 * (1.0f + 1.52587890625e-05f);
  w.eps2 = p.softening * p.softening;
  w.G = p.G;
  w.leaf_cap = p.leaf_capacity;
  w.ax = ax;
  w.ay = ay;
  w.az = az;
  w.counts = counts;
  w.inter_total = inter_total;
  w.task_ctr = grow(h.walk_ctr, 1);
  NBGB_CUDA(cudaMemsetAsync(w.task_ctr, 0, sizeof(uint32_t), st));
  const bool count = counts != nullptr || inter_total != nullptr;
  const bool bucket = p.leaf_capacity > 1;
  // one resident wave of persistent warps
  const int64_t need = ceil_div(h.ntasks * 32, 256);
  auto grid = [&](int occ) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)num_sms() * occ));
  };
  if (count) {
    if (bucket)
      bh_walk_kernel<true, true><<<grid(walk_occupancy<true, true>()), 256, 0, st>>>(w);
    else
      bh_walk_kernel<true, false><<<grid(walk_occupancy<true, false>()), 256, 0, st>>>(w);
  } else {
    if (bucket)
      bh_walk_kernel<false, true><<<grid(walk_occupancy<false, true>()), 256, 0, st>>>(w);
    else
      bh_walk_kernel<false, false><<<grid(walk_occupancy<false, false>()), 256, 0, st>>>(w);
  }
  NBGB_LAUNCH_CHECK();
}

// Node capacity that any realistic input fits (the canonical tree has ~1.5N
// nodes; 4N + 64 per segment leaves room for strongly clustered sets).  Used
// when there is no per-call synchronization (no read-back to regrow).
// Every buffer a canonical build (and its walk) of the current segment set
// uses, allocated ahead: bh_build then allocates nothing.  The ensemble calls
// this before it changes any state in a tick, so that running out of device
// memory aborts the tick cleanly instead of half-way through a step.
void bh_reserve_buffers(BHState& h, bool groups) {
  const int64_t n = h.n;
  const int nseg = std::max(h.nseg, 1);
  const size_t R = (size_t)h.reserve;
  const int64_t min_cap = 2 * n + 64 * (int64_t)nseg;
  if (h.cap < min_cap) h.cap = 3 * n + 64 * (int64_t)nseg;
  if (h.cap >= kMaxWalkNodes)
    fail(NBGB_ERR_OVERFLOW, "Barnes-Hut node capacity above 2^30 nodes: too many bodies in one tree build");
  grow(h.box, (size_t)nseg);
  grow(h.seg_minmax, (size_t)nseg * 6);
  grow(h.hist, radix_hist_elems((int64_t)R));
  grow(h.scan_ws, scan_workspace_elems((int64_t)radix_hist_elems((int64_t)R)) +
                      scan_workspace_elems((int64_t)R + 1));
  grow(h.khi, R);
  grow(h.khi_alt, R);
  grow(h.klo, R);
  grow(h.pidx, R);
  grow(h.pidx_alt, R);
  if (nseg > 1) {
    grow(h.sk, R);
    grow(h.sk_alt, R);
  }
  grow(h.kseg, R);
  grow(h.spm, R);
  grow(h.lcp, R);
  grow(h.ncnt, R + 1);
  grow(h.nstart, R + 1);
  grow(h.scalars, 2);
  grow(h.seg_depth, (size_t)nseg);
  grow(h.nodes, (size_t)h.cap);
  grow(h.node_parent, (size_t)h.cap);
  grow(h.node_nchild, (size_t)h.cap);
  grow(h.node_visit, (size_t)h.cap);
  grow(h.leaf_of, R);
  grow(h.seg_root, (size_t)nseg);
  grow(h.seg_end, (size_t)nseg);
  grow(h.walk_ctr, 1);
  if (groups) {
    grow(h.groups, R);
    h.groups2.ensure(h.groups.cap);
    // fresh cost estimates (zero: no order yet), complete before any stream
    // of the caller uses them
    uint32_t* bc_old = h.body_cost.ptr;
    uint32_t* bc = grow(h.body_cost, R);
    unsigned long long* acc_old = h.cost_acc.ptr;
    unsigned long long* acc = grow(h.cost_acc, 2);
    if (bc != bc_old || acc != acc_old) {
      NBGB_CUDA(cudaMemset(bc, 0, h.body_cost.cap * sizeof(uint32_t)));
      NBGB_CUDA(cudaMemset(acc, 0, 2 * sizeof(unsigned long long)));
      NBGB_CUDA(cudaDeviceSynchronize());
    }
    grow(h.group_ctr, sizeof(GroupCounters));
    grow(h.group_ovf, (size_t)kOvfChunks * kOvfChunk);
  }
}

void bh_reserve_async(BHState& h) {
  const int64_t c = 4 * h.reserve + 64 * (int64_t)std::max(h.nseg, 1);
  if (h.cap < c) h.cap = std::max(c, h.cap + h.cap / 2);
}

// The calculator path: one segment at offset 0.
void bh_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay, float* az) {
  if (!c->bh) c->bh.reset(new BHState());
  BHState& h = *c->bh;
  cudaStream_t st = c->stream;
  uint32_t* err = c->err.ensure(1);
  if (h.nseg != 1 || h.n != n) {
    const int64_t off = 0;
    bh_set_segments(h, &off, &n, 1, st, nullptr);
  }
  const bool sync = (c->params.flags & NBGB_FLAG_SYNC) != 0;
  const bool ref_tree = (c->params.flags & NBGB_FLAG_REFERENCE_TREE) != 0;
  const bool groups = (c->params.flags & NBGB_FLAG_GROUP_WALK) != 0;
  StageTimer* timer = stage_timer(c);
  if (!sync) bh_reserve_async(h);
  for (int attempt = 0; attempt < 2; ++attempt) {
    // asynchronously the reference's tree is always replayed; synchronously
    // the canonical tree is built first and replaced only where it can differ
    bh_build(h, pm, st, err, groups, c->params.group_size, ref_tree && !sync, timer);
    if (!sync) break;  // capacity overflow surfaces through the device error word
    // The node count is data dependent: read it back and regrow once if the
    // capacity was too small (the kernels skipped their work in that case).
    uint32_t* hs = h.h_scalars.ensure(2);
    NBGB_CUDA(cudaMemcpyAsync(hs, h.scalars.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    if ((int64_t)hs[0] <= h.cap) {
      // The reference stops splitting once node_count + 33 >= 2N.  Its node
      // count only grows during the insertion and ends at the canonical
      // count when the budget never fires, so a canonical count below
      // 2N - 33 proves that it never fires and the trees are the same.
      if (ref_tree && (int64_t)hs[0] + kMaxDepth + 1 >= 2 * n)
        bh_build(h, pm, st, err, groups, c->params.group_size, true, timer);
      break;
    }
    NBGB_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    h.cap = (int64_t)hs[0] + (int64_t)hs[0] / 8 + 64;
  }
  BHWalkParams wp{c->params.G, c->params.softening, c->params.theta, c->params.leaf_capacity,
                  (c->params.flags & NBGB_FLAG_GROUP_WALK) ? 1 : 0};
  const bool count = (c->params.flags & NBGB_FLAG_COUNT_INTERACTIONS) != 0;
  int32_t* counts = count ? c->counts.ensure((size_t)n) : nullptr;
  stage_mark(timer, "barnes_hut.walk");
  bh_walk(h, wp, ax, ay, az, counts, nullptr, err, st);
}

// ------------------------------------------------------------- export --
__global__ void export_nodes_kernel(const Node* __restrict__ nodes, const uint32_t* __restrict__ body,
                                    int64_t total, nbgb_octree_node* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 in = nodes[p].info;
    const float4 g = nodes[p].geom, cm = nodes[p].com;
    nbgb_octree_node& o = out[p];
    o.center[0] = g.x;
    o.center[1] = g.y;
    o.center[2] = g.z;
    o.half_size = g.w;
    o.center_of_mass[0] = cm.x;
    o.center_of_mass[1] = cm.y;
    o.center_of_mass[2] = cm.z;
    o.total_mass = cm.w;
    o.is_leaf = (uint8_t)(in.y & 1);
    o.pad_[0] = o.pad_[1] = o.pad_[2] = 0;
    o.particle_count = in.w;
    o.particle_index = (in.y & 1) ? (int32_t)body[in.z] : -1;
    for (int j = 0; j < 8; ++j) o.children[j] = -1;
  }
}

__global__ void export_children_kernel(const Node* __restrict__ nodes,
                                       const int32_t* __restrict__ parent,
                                       const u64* __restrict__ hi, const u64* __restrict__ lo,
                                       int64_t total, nbgb_octree_node* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (parent[p] < 0) continue;  // a root
    const int4 in = nodes[p].info;
    const int d = in.y >> 8;
    const int64_t f = in.z;
    const uint32_t oct = (d <= kHiLevels) ? (uint32_t)((hi[f] >> (3 * (kHiLevels - d))) & 7u)
                                          : (uint32_t)((lo[f] >> (3 * (kMaxDepth - d))) & 7u);
    out[parent[p]].children[oct] = (int32_t)p;
  }
}

}  // namespace nbgb

using namespace nbgb;

extern "C" {

nbgb_status nbgb_bh_tree_stats(nbgb_calculator* c, int32_t* node_count, int32_t* max_depth) {
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT || !c->bh->built) return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  uint32_t total = 0;
  int32_t depth = 0;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  if (cudaMemcpy(&total, h.scalars.ptr, sizeof total, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&depth, h.seg_depth.ptr, sizeof depth, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  if (node_count) *node_count = (int32_t)total;
  if (max_depth) *max_depth = depth;
  return NBGB_OK;
}

nbgb_status nbgb_bh_copy_sorted_keys(nbgb_calculator* c, uint32_t* keys, int32_t* indices,
                                     size_t n) {
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT || !c->bh->built) return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  if (n != (size_t)h.n || h.nseg != 1) return NBGB_ERR_INVALID_ARG;
  if (!h.keys_valid) {
    // The reference's Morton keys and their stable sort
    // (force_barnes_hut.cu:308-328), from the bodies of the last build.
    try {
      const int64_t nn = h.n;
      uint32_t* mk = h.mkeys.ensure((size_t)nn);
      uint32_t* mi = h.midx.ensure((size_t)nn);
      uint32_t* mk2 = h.mkeys_alt.ensure((size_t)nn);
      uint32_t* mi2 = h.midx_alt.ensure((size_t)nn);
      morton_scatter_kernel<<<grid1d(nn), 256, 0, c->stream>>>(h.spm.ptr, h.body, nn, h.box.ptr,
                                                              mk, mi);
      NBGB_LAUNCH_CHECK();
      radix_sort_pairs<uint32_t>(mk, mk2, mi, mi2, nn, 0, 32, h.hist.ptr, h.scan_ws.ptr,
                                 c->stream, &h.m_alt);
      h.keys_valid = true;
    } catch (const Error& e) {
      return e.status;
    }
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  const uint32_t* k = h.m_alt ? h.mkeys_alt.ptr : h.mkeys.ptr;
  const uint32_t* v = h.m_alt ? h.midx_alt.ptr : h.midx.ptr;
  if (keys && cudaMemcpy(keys, k, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  if (indices && cudaMemcpy(indices, v, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  return NBGB_OK;
}

nbgb_status nbgb_bh_copy_nodes(nbgb_calculator* c, nbgb_octree_node* nodes, size_t capacity) {
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT || !nodes || !c->bh->built)
    return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  uint32_t total32 = 0;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  if (cudaMemcpy(&total32, h.scalars.ptr, sizeof total32, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  const int64_t total = total32;
  if ((size_t)total > capacity || total > h.cap) return NBGB_ERR_INVALID_ARG;
  nbgb_octree_node* d = nullptr;
  if (cudaMalloc(&d, (size_t)std::max<int64_t>(total, 1) * sizeof(nbgb_octree_node)) != cudaSuccess)
    return NBGB_ERR_OOM;
  unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, 256), 4096));
  export_nodes_kernel<<<blocks, 256, 0, c->stream>>>(h.nodes.ptr, h.body, total, d);
  export_children_kernel<<<blocks, 256, 0, c->stream>>>(h.nodes.ptr, h.node_parent.ptr,
                                                        h.khi.ptr, h.klo.ptr, total, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(nodes, d, (size_t)total * sizeof(nbgb_octree_node), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

nbgb_status nbgb_copy_interaction_counts(nbgb_calculator* c, int32_t* counts, size_t n) {
  if (!c || !counts || c->method == NBGB_DIRECT_N2) return NBGB_ERR_INVALID_ARG;
  if (!(c->params.flags & NBGB_FLAG_COUNT_INTERACTIONS) || !c->counts.ptr ||
      c->counts.cap < n || (int64_t)n != c->last_n)
    return NBGB_ERR_INVALID_ARG;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  return cudaMemcpy(counts, c->counts.ptr, n * 4, cudaMemcpyDeviceToHost) == cudaSuccess
             ? NBGB_OK
             : NBGB_ERR_CUDA;
}

int32_t nbgb_bh_group_size(uint64_t count) {
  return nbgb::bh_group_max(count > (uint64_t)INT64_MAX ? INT64_MAX : (int64_t)count);
}

}  // extern "C"
