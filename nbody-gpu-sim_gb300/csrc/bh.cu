// bh.cu -- Barnes-Hut on the device: Morton keys, radix sort, octree from
// sorted path keys, bottom-up centre of mass, warp-cooperative walk (K2-K6).
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
// cells hold all their bodies.  This file builds exactly that tree in
// parallel:
//   1. path key of every body: its 32 octants, computed with the
//      reference's float operations from the reference's root cube;
//   2. stable radix sort by path key (ties keep Morton order = the
//      reference's insertion order, which fixes merged-leaf sums);
//   3. l_k = common levels of adjacent sorted keys; body k starts the
//      internal nodes of depths l_{k-1}+1 .. min(l_k, 31) and (unless it
//      shares a depth-32 cell with k-1) one leaf of depth
//      min(32, max(l_{k-1}, l_k) + 1);
//   4. an exclusive scan of those counts numbers the nodes in depth-first
//      pre-order (children in octant order), so every subtree is a
//      contiguous index range and skip(P) = first node of body end(P)+1;
//   5. centres of mass bottom-up with per-node arrival counters, summing
//      children in octant order with the reference's float operations
//      (:514-538), so masses and centres of mass are bit-identical.
//
// Walk.  One warp walks the pre-order array for 32 consecutive targets
// (Morton/path-sorted, so spatially close).  Every lane applies the
// reference's per-target rules (contains_i, leaf self-subtraction, opening
// test 4h^2/(d^2+eps^2) < theta^2, :175-243); the warp descends into a node
// if any active lane opens it, and a lane that accepted a node sleeps until
// the cursor leaves that node's subtree.  Each lane therefore sums exactly
// the reference's interaction set for its target (no stack, no local
// memory, broadcast node loads).  With leaf_capacity > 1 a subtree holding
// at most that many bodies is summed body by body when opened.
#include "common.cuh"
#include "geom.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "sort.cuh"

namespace nbgb {

using u64 = unsigned long long;
constexpr int kHiLevels = 21;  // levels 1..21 in the high key (63 bits)
constexpr int kMaxDepth = 32;  // force_barnes_hut.cu:24

struct BHState {
  DevBuf<float> bbox_part;
  DevBuf<BBox> box;
  DevBuf<uint32_t> mkeys, mkeys_alt, midx, midx_alt;  // Morton sort
  DevBuf<u64> klo, klo_alt, khi, khi_alt;             // path keys
  DevBuf<uint32_t> pidx, pidx_alt;
  DevBuf<uint32_t> hist, scan_ws;
  DevBuf<uint8_t> lcp;
  DevBuf<uint32_t> ncnt;    // n + 1
  DevBuf<uint32_t> nstart;  // n + 1
  DevBuf<uint32_t> scalars; // [0] total nodes, [1] max depth
  HostPinned<uint32_t> h_scalars;
  DevBuf<float4> node_com, node_geom;
  DevBuf<int4> node_info;  // skip, first, count, flags (bit0 leaf, bits 8.. depth)
  DevBuf<int32_t> node_parent, node_nchild, node_visit;
  DevBuf<float4> spm;      // bodies in path order
  int64_t n = 0;
  int64_t cap = 0;
  bool m_alt = false;      // Morton result in *_alt
  bool keys_valid = false; // Morton (key, index) pairs computed for the last build
  const uint32_t* body = nullptr;  // path-sorted body indices
  const u64* hi_sorted = nullptr;
};

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

__global__ void morton_kernel(const float4* __restrict__ pm, int64_t n, const BBox* __restrict__ box,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  const BBox b = *box;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = morton_of(pm[i], b);
    idx[i] = (uint32_t)i;
  }
}

// Octant path of a position through the reference's subdivision: returns the
// high key (levels 1..21, 3 bits each, level 1 most significant) and the low
// key (levels 22..32).
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

// Centre and half size of the depth-d cell on a body's path.
__device__ __forceinline__ float4 cell_at_depth(float4 p, const BBox& b, int d) {
  float cx = b.center[0], cy = b.center[1], cz = b.center[2], h = b.half;
  for (int lev = 1; lev <= d; ++lev) {
    const uint32_t o = (p.x >= cx ? 1u : 0u) | (p.y >= cy ? 2u : 0u) | (p.z >= cz ? 4u : 0u);
    const float hs = __fmul_rn(h, 0.5f);
    cx = __fadd_rn(cx, (o & 1u) ? hs : -hs);
    cy = __fadd_rn(cy, (o & 2u) ? hs : -hs);
    cz = __fadd_rn(cz, (o & 4u) ? hs : -hs);
    h = hs;
  }
  return make_float4(cx, cy, cz, h);
}

// After the Morton sort: low path keys in Morton order (values = bodies).
__global__ void path_lo_kernel(const float4* __restrict__ pm, const uint32_t* __restrict__ body,
                               int64_t n, const BBox* __restrict__ box, u64* __restrict__ lo,
                               uint32_t* __restrict__ out_body) {
  const BBox b = *box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = body[k];
    u64 h, l;
    path_key(pm[i], b, h, l);
    lo[k] = l;
    out_body[k] = i;
  }
}

__global__ void path_hi_kernel(const float4* __restrict__ pm, const uint32_t* __restrict__ body,
                               int64_t n, const BBox* __restrict__ box, u64* __restrict__ hi) {
  const BBox b = *box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    u64 h, l;
    path_key(pm[body[k]], b, h, l);
    hi[k] = h;
  }
}

// Final order: low keys recomputed in path order, bodies gathered (x,y,z,m).
__global__ void path_final_kernel(const float4* __restrict__ pm, const uint32_t* __restrict__ body,
                                  int64_t n, const BBox* __restrict__ box, u64* __restrict__ lo,
                                  float4* __restrict__ spm) {
  const BBox b = *box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = pm[body[k]];
    u64 h, l;
    path_key(p, b, h, l);
    lo[k] = l;
    spm[k] = p;
  }
}

// High path key of every body in index order (values = body indices).
__global__ void path_hi_index_kernel(const float4* __restrict__ pm, int64_t n,
                                     const BBox* __restrict__ box, u64* __restrict__ hi,
                                     uint32_t* __restrict__ idx) {
  const BBox b = *box;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    u64 h, l;
    path_key(pm[i], b, h, l);
    hi[i] = h;
    idx[i] = (uint32_t)i;
  }
}

// Tie key of a body: low path key, then Morton key, then index.
__device__ __forceinline__ bool tie_less(const float4* __restrict__ pm, const BBox& b, uint32_t a,
                                         uint32_t c) {
  u64 ha, la, hc, lc;
  const float4 pa = pm[a], pc = pm[c];
  path_key(pa, b, ha, la);
  path_key(pc, b, hc, lc);
  if (la != lc) return la < lc;
  const uint32_t ma = morton_of(pa, b), mc = morton_of(pc, b);
  if (ma != mc) return ma < mc;
  return a < c;
}

// Runs of equal high keys (bodies sharing their first 21 octants; tiny in
// practice) are put in (low key, Morton key, index) order by one thread per
// run with an insertion sort.  A run that is already in order (e.g. many
// coincident bodies) costs one comparison per body.
__global__ void tie_order_kernel(const float4* __restrict__ pm, int64_t n,
                                 const BBox* __restrict__ box, const u64* __restrict__ hi,
                                 uint32_t* __restrict__ body) {
  const BBox b = *box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k + 1 < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (k > 0 && hi[k - 1] == hi[k]) continue;  // not the start of a run
    if (hi[k + 1] != hi[k]) continue;           // run of one
    int64_t e = k + 1;
    while (e + 1 < n && hi[e + 1] == hi[k]) ++e;
    for (int64_t i = k + 1; i <= e; ++i) {
      const uint32_t cur = body[i];
      int64_t j = i - 1;
      while (j >= k && tie_less(pm, b, cur, body[j])) {
        body[j + 1] = body[j];
        --j;
      }
      body[j + 1] = cur;
    }
  }
}

// Morton keys scattered back to index order (for the on-demand key sort).
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

// l_k for k in [0, n-1); per-body node counts (internal + leaf, + root at 0).
__global__ void lcp_count_kernel(const u64* __restrict__ hi, const u64* __restrict__ lo, int64_t n,
                                 uint8_t* __restrict__ lcp, uint32_t* __restrict__ cnt) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int lk = (k + 1 < n) ? common_levels(hi[k], lo[k], hi[k + 1], lo[k + 1]) : 0;
    const int lp = (k > 0) ? common_levels(hi[k - 1], lo[k - 1], hi[k], lo[k]) : 0;
    if (k + 1 < n) lcp[k] = (uint8_t)lk;
    const int fd = (k > 0) ? lp + 1 : 1;
    const int top = (k + 1 < n) ? min(lk, kMaxDepth - 1) : 0;
    uint32_t c = (uint32_t)max(0, top - fd + 1);
    const bool leaf_start = (k == 0) || (lp < kMaxDepth);
    c += leaf_start ? 1u : 0u;
    if (k == 0) c += 1u;  // root
    cnt[k] = c;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cnt[n] = 0;
}

// Range end of the depth-d node that contains sorted body k: the largest j
// with common_levels(key_k, key_j) >= d.  Keys are sorted, so that predicate
// is monotone in j: gallop, then bisect (Karras-style, O(log range)).
__device__ __forceinline__ int64_t range_end(const u64* __restrict__ hi, const u64* __restrict__ lo,
                                             int64_t n, int64_t k, int d) {
  const u64 h0 = hi[k], l0 = lo[k];
  int64_t good = k, step = 1;
  while (k + step < n && common_levels(h0, l0, hi[k + step], lo[k + step]) >= d) {
    good = k + step;
    step <<= 1;
  }
  int64_t bad = (k + step < n) ? k + step : n;
  while (bad - good > 1) {
    const int64_t mid = good + ((bad - good) >> 1);
    if (common_levels(h0, l0, hi[mid], lo[mid]) >= d)
      good = mid;
    else
      bad = mid;
  }
  return good;
}

struct EmitArgs {
  const uint8_t* lcp;
  const u64* hi;
  const u64* lo;
  const uint32_t* nstart;
  const uint32_t* body;
  const float4* spm;
  const BBox* box;
  int64_t n;
  int64_t cap;
  float4* geom;
  int4* info;
  int32_t* visit;
  uint32_t* scalars;
  uint32_t* err;
};

__global__ void emit_nodes_kernel(EmitArgs a) {
  const uint32_t total = a.nstart[a.n];
  if ((int64_t)total > a.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(a.err, kErrTreeCapacity);
    return;
  }
  const BBox b = *a.box;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int lk = (k + 1 < a.n) ? (int)a.lcp[k] : 0;
    const int lp = (k > 0) ? (int)a.lcp[k - 1] : 0;
    const int fd = (k > 0) ? lp + 1 : 1;
    const int top = (k + 1 < a.n) ? min(lk, kMaxDepth - 1) : 0;
    uint32_t idx = a.nstart[k];
    const float4 p = a.spm[k];
    if (k == 0) {
      a.geom[0] = make_float4(b.center[0], b.center[1], b.center[2], b.half);
      a.info[0] = make_int4((int)total, 0, (int)a.n, 0);
      a.visit[0] = 0;
      ++idx;
    }
    // walk the path of body k once, emitting internal nodes of depth fd..top
    float cx = b.center[0], cy = b.center[1], cz = b.center[2], h = b.half;
    const bool leaf_start = (k == 0) || (lp < kMaxDepth);
    const int ld = min(kMaxDepth, max(lp, lk) + 1);
    const int last = leaf_start ? ld : top;
    for (int lev = 1; lev <= last; ++lev) {
      const uint32_t o = (p.x >= cx ? 1u : 0u) | (p.y >= cy ? 2u : 0u) | (p.z >= cz ? 4u : 0u);
      const float hs = __fmul_rn(h, 0.5f);
      cx = __fadd_rn(cx, (o & 1u) ? hs : -hs);
      cy = __fadd_rn(cy, (o & 2u) ? hs : -hs);
      cz = __fadd_rn(cz, (o & 4u) ? hs : -hs);
      h = hs;
      if (lev >= fd && lev <= top) {
        const int64_t e = range_end(a.hi, a.lo, a.n, k, lev);
        const uint32_t skip = (e + 1 < a.n) ? a.nstart[e + 1] : total;
        a.geom[idx] = make_float4(cx, cy, cz, h);
        a.info[idx] = make_int4((int)skip, (int)k, (int)(e - k + 1), lev << 8);
        a.visit[idx] = 0;
        ++idx;
      }
    }
    if (leaf_start) {
      int64_t e = k;
      while (e + 1 < a.n && (int)a.lcp[e] >= kMaxDepth) ++e;  // bodies sharing a depth-32 cell
      a.geom[idx] = make_float4(cx, cy, cz, h);
      a.info[idx] = make_int4((int)(idx + 1), (int)k, (int)(e - k + 1), (ld << 8) | 1);
      a.visit[idx] = 0;
      // reference max_depth_: depth of the inserting body's last loop level
      const int md = (ld == kMaxDepth && e > k) ? kMaxDepth : ld - 1;
      atomicMax(&a.scalars[1], (uint32_t)md);
    }
  }
}

// Parent links and child counts (children of P: P+1, skip(P+1), ... < skip(P)).
__global__ void link_kernel(const int4* __restrict__ info, const uint32_t* __restrict__ nstart,
                            int64_t n, int64_t cap, int32_t* __restrict__ parent,
                            int32_t* __restrict__ nchild) {
  const uint32_t total = nstart[n];
  if ((int64_t)total > cap) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < (int64_t)total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 ip = info[p];
    if (p == 0) parent[0] = -1;
    if (ip.w & 1) {
      nchild[p] = 0;
      continue;
    }
    int c = (int)p + 1, nc = 0;
    while (c < ip.x) {
      parent[c] = (int)p;
      ++nc;
      c = info[c].x;
    }
    nchild[p] = nc;
  }
}

// Leaves: mass/com as the reference's allocateLeaf + mergeParticleIntoLeaf
// (force_barnes_hut.cu:355-389); then the last-arriving child of each node
// computes that node from all its children in octant order (:514-538).
__global__ void com_kernel(const int4* __restrict__ info, const float4* __restrict__ spm,
                           const uint32_t* __restrict__ nstart, int64_t n, int64_t cap,
                           const int32_t* __restrict__ parent, const int32_t* __restrict__ nchild,
                           int32_t* __restrict__ visit, float4* __restrict__ com) {
  const uint32_t total = nstart[n];
  if ((int64_t)total > cap) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < (int64_t)total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 ip = info[p];
    if (!(ip.w & 1)) continue;
    float4 b0 = spm[ip.y];
    float m = b0.w, cx = b0.x, cy = b0.y, cz = b0.z;
    for (int j = 1; j < ip.z; ++j) {
      const float4 q = spm[ip.y + j];
      const float t = __fadd_rn(m, q.w);
      cx = __fdiv_rn(__fadd_rn(__fmul_rn(cx, m), __fmul_rn(q.x, q.w)), t);
      cy = __fdiv_rn(__fadd_rn(__fmul_rn(cy, m), __fmul_rn(q.y, q.w)), t);
      cz = __fdiv_rn(__fadd_rn(__fmul_rn(cz, m), __fmul_rn(q.z, q.w)), t);
      m = t;
    }
    com[p] = make_float4(cx, cy, cz, m);
    int node = parent[p];
    while (node >= 0) {
      __threadfence();
      const int arrived = atomicAdd(&visit[node], 1);
      if (arrived != nchild[node] - 1) break;
      __threadfence();
      const int4 in = info[node];
      float tm = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
      int c = node + 1;
      while (c < in.x) {
        const float4 q = __ldcg(&com[c]);
        tm = __fadd_rn(tm, q.w);
        sx = __fadd_rn(sx, __fmul_rn(q.x, q.w));
        sy = __fadd_rn(sy, __fmul_rn(q.y, q.w));
        sz = __fadd_rn(sz, __fmul_rn(q.z, q.w));
        c = info[c].x;
      }
      float4 r = make_float4(0.f, 0.f, 0.f, tm);
      if (tm > 0.0f) {
        r.x = __fdiv_rn(sx, tm);
        r.y = __fdiv_rn(sy, tm);
        r.z = __fdiv_rn(sz, tm);
      }
      __stcg(&com[node], r);
      node = parent[node];
    }
  }
}

// ----------------------------------------------------------------- walk --
struct WalkArgs {
  const float4* com;
  const float4* geom;
  const int4* info;
  const float4* spm;
  const uint32_t* body;
  const uint32_t* nstart;
  int64_t n;
  int64_t cap;
  float theta2;
  float eps2;
  float G;
  int leaf_cap;
  float* ax;
  float* ay;
  float* az;
  int32_t* counts;
};

// The reference's opening test `size2 / dist2 < theta2` with the correctly
// rounded quotient (force_barnes_hut.cu:222-224), decided from the MUFU
// reciprocal whenever the approximate quotient is far (2^-16 relative) from
// the threshold, which is almost always; only the near-threshold cases pay
// for the IEEE division.  The outcome equals the IEEE comparison.
__device__ __forceinline__ bool opening_accept(float size2, float d2, float theta2) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d2));
  const float q = size2 * r;
  if (q < theta2 * (1.0f - 1.52587890625e-05f)) return true;
  if (q > theta2 * (1.0f + 1.52587890625e-05f)) return false;
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

// One warp, 32 targets, each lane applying the reference's per-target rules
// (union traversal; see the file header).  Adds into sx/sy/sz/cnt.
template <bool COUNT, bool BUCKET>
__device__ __forceinline__ void lane_walk(const WalkArgs& a, int64_t k, bool valid, float4 pi,
                                          uint32_t total, bool tree_ok, float& sx, float& sy,
                                          float& sz, int& cnt) {
    int resume = valid ? 0 : 0x7fffffff;
    int node = tree_ok ? 0 : (int)total;
    while (node < (int)total) {
      const float4 cm = a.com[node];
      const int4 in = a.info[node];
      if (cm.w == 0.0f) {  // force_barnes_hut.cu:172-173
        node = in.x;
        continue;
      }
      const float4 g = a.geom[node];
      const bool active = node >= resume;
      const bool contains = fabsf(__fsub_rn(pi.x, g.x)) <= g.w &&
                            fabsf(__fsub_rn(pi.y, g.y)) <= g.w &&
                            fabsf(__fsub_rn(pi.z, g.z)) <= g.w;
      if (in.w & 1) {  // leaf
        if (active) {
          float me = cm.w, cx = cm.x, cy = cm.y, cz = cm.z;
          bool use = true;
          if (contains) {
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
        node = in.x;
        continue;
      }
      const float dx = __fsub_rn(cm.x, pi.x), dy = __fsub_rn(cm.y, pi.y),
                  dz = __fsub_rn(cm.z, pi.z);
      const float d2 = __fadd_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))), a.eps2);
      const float size2 = __fmul_rn(__fmul_rn(4.0f, g.w), g.w);
      const bool accept = !contains && opening_accept(size2, d2, a.theta2);
      const bool open = active && !accept;
      if (active && accept) {
        const float r = rsqrt_approx(d2);
        const float f = (cm.w * r) * (r * r);
        sx = fmaf(f, dx, sx);
        sy = fmaf(f, dy, sy);
        sz = fmaf(f, dz, sz);
        if (COUNT) ++cnt;
        resume = in.x;
      }
      if (BUCKET && in.z <= a.leaf_cap) {
        if (open) {
          for (int j = 0; j < in.z; ++j) {
            const int64_t s = (int64_t)in.y + j;
            if (s == k) continue;
            const float4 q = a.spm[s];
            bh_add(q.x, q.y, q.z, q.w, pi.x, pi.y, pi.z, a.eps2, sx, sy, sz);
            if (COUNT) ++cnt;
          }
        }
        node = in.x;
        continue;
      }
      node = __any_sync(0xffffffffu, open) ? node + 1 : in.x;
    }
}

template <bool COUNT, bool BUCKET>
__global__ void __launch_bounds__(256) bh_walk_kernel(WalkArgs a) {
  const uint32_t total = a.nstart[a.n];
  const bool tree_ok = (int64_t)total <= a.cap;
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t wbase = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; wbase < a.n;
       wbase += warps * 32) {
    const int64_t k = wbase + lane;
    const bool valid = k < a.n;
    const float4 pi = valid ? a.spm[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    int cnt = 0;
    lane_walk<COUNT, BUCKET>(a, k, valid, pi, total, tree_ok, sx, sy, sz, cnt);
    if (valid) {
      const uint32_t i = a.body[k];
      a.ax[i] = a.G * sx;
      a.ay[i] = a.G * sy;
      a.az[i] = a.G * sz;
      if (COUNT) a.counts[i] = cnt;
    }
  }
}

static unsigned grid1d(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), threads), (int64_t)num_sms() * 32));
}

// Builds the tree for n packed bodies; returns false if the node capacity
// was too small (the needed count is then in h.h_scalars after a sync).
static void bh_build(nbgb_calculator* c, BHState& h, const float4* pm, int64_t n) {
  cudaStream_t st = c->stream;
  uint32_t* err = c->err.ensure(1);
  h.n = n;
  float* part = h.bbox_part.ensure((size_t)bbox_blocks(n) * 6);
  BBox* box = h.box.ensure(1);
  launch_bbox(pm, n, part, box, err, st);
  uint32_t* hist = h.hist.ensure(radix_hist_elems(n));
  uint32_t* sws = h.scan_ws.ensure(scan_workspace_elems((int64_t)radix_hist_elems(n)) +
                                   scan_workspace_elems(n + 1));
  // Path keys in index order, stable radix sort by the high key (levels
  // 1..21, 8 passes), then bodies that share their high key are ordered by
  // (low key, Morton key, index): the full path order with the reference's
  // insertion order (stable Morton order) inside a shared depth-32 cell.
  u64* lo = h.klo.ensure((size_t)n);
  u64* hi = h.khi.ensure((size_t)n);
  u64* hi2 = h.khi_alt.ensure((size_t)n);
  uint32_t* pb = h.pidx.ensure((size_t)n);
  uint32_t* pb2 = h.pidx_alt.ensure((size_t)n);
  path_hi_index_kernel<<<grid1d(n), 256, 0, st>>>(pm, n, box, hi, pb);
  NBGB_LAUNCH_CHECK();
  bool alt = false;
  radix_sort_pairs<u64>(hi, hi2, pb, pb2, n, 0, 64, hist, sws, st, &alt);
  h.body = alt ? pb2 : pb;
  h.hi_sorted = alt ? hi2 : hi;
  tie_order_kernel<<<grid1d(n), 256, 0, st>>>(pm, n, box, h.hi_sorted, const_cast<uint32_t*>(h.body));
  NBGB_LAUNCH_CHECK();
  h.keys_valid = false;  // Morton (key, index) pairs are produced on demand
  float4* spm = h.spm.ensure((size_t)n);
  path_final_kernel<<<grid1d(n), 256, 0, st>>>(pm, h.body, n, box, lo, spm);
  NBGB_LAUNCH_CHECK();
  // node counts, numbering, emission
  uint8_t* lcp = h.lcp.ensure((size_t)n);
  uint32_t* cnt = h.ncnt.ensure((size_t)n + 1);
  uint32_t* nst = h.nstart.ensure((size_t)n + 1);
  uint32_t* sc = h.scalars.ensure(2);
  lcp_count_kernel<<<grid1d(n), 256, 0, st>>>(h.hi_sorted, lo, n, lcp, cnt);
  NBGB_LAUNCH_CHECK();
  scan_exclusive_u32(cnt, nst, n + 1, sws, sc, st);
  NBGB_CUDA(cudaMemsetAsync(sc + 1, 0, sizeof(uint32_t), st));
  if (h.cap < 2 * n + 64) h.cap = 0;
  if (h.cap == 0) h.cap = 3 * n + 64;
  float4* geom = h.node_geom.ensure((size_t)h.cap);
  float4* com = h.node_com.ensure((size_t)h.cap);
  int4* info = h.node_info.ensure((size_t)h.cap);
  int32_t* par = h.node_parent.ensure((size_t)h.cap);
  int32_t* nch = h.node_nchild.ensure((size_t)h.cap);
  int32_t* vis = h.node_visit.ensure((size_t)h.cap);
  EmitArgs ea{lcp, h.hi_sorted, lo, nst, h.body, spm, box, n, h.cap, geom, info, vis, sc, err};
  emit_nodes_kernel<<<grid1d(n), 256, 0, st>>>(ea);
  NBGB_LAUNCH_CHECK();
  link_kernel<<<grid1d(h.cap), 256, 0, st>>>(info, nst, n, h.cap, par, nch);
  NBGB_LAUNCH_CHECK();
  com_kernel<<<grid1d(h.cap), 256, 0, st>>>(info, spm, nst, n, h.cap, par, nch, vis, com);
  NBGB_LAUNCH_CHECK();
}

size_t bh_state_bytes(const BHState* p) {
  if (!p) return 0;
  const BHState& h = *p;
  return h.bbox_part.bytes() + h.box.bytes() + h.mkeys.bytes() + h.mkeys_alt.bytes() +
         h.midx.bytes() + h.midx_alt.bytes() + h.klo.bytes() + h.klo_alt.bytes() +
         h.khi.bytes() + h.khi_alt.bytes() + h.pidx.bytes() + h.pidx_alt.bytes() +
         h.hist.bytes() + h.scan_ws.bytes() + h.lcp.bytes() + h.ncnt.bytes() + h.nstart.bytes() +
         h.scalars.bytes() + h.node_com.bytes() + h.node_geom.bytes() + h.node_info.bytes() +
         h.node_parent.bytes() + h.node_nchild.bytes() + h.node_visit.bytes() + h.spm.bytes();
}

// Node capacity that any realistic input fits (the canonical tree has ~1.5N
// nodes; 4N + 64 leaves room for strongly clustered sets).  Used when the
// calculator runs without per-call synchronization (no read-back to regrow).
static int64_t bh_async_capacity(int64_t n) { return 4 * n + 64; }

void bh_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay, float* az) {
  if (!c->bh) c->bh.reset(new BHState());
  BHState& h = *c->bh;
  cudaStream_t st = c->stream;
  const bool sync = (c->params.flags & NBGB_FLAG_SYNC) != 0;
  if (!sync && h.cap < bh_async_capacity(n)) h.cap = bh_async_capacity(n);
  for (int attempt = 0; attempt < 2; ++attempt) {
    bh_build(c, h, pm, n);
    if (!sync) break;  // capacity overflow surfaces through the device error word
    // The node count is data dependent: read it back and regrow once if the
    // capacity was too small (the kernels skipped their work in that case).
    uint32_t* hs = h.h_scalars.ensure(2);
    NBGB_CUDA(cudaMemcpyAsync(hs, h.scalars.ptr, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    if ((int64_t)hs[0] <= h.cap) break;
    // clear the capacity error raised by the emit kernel and grow
    NBGB_CUDA(cudaMemsetAsync(c->err.ptr, 0, sizeof(uint32_t), st));
    h.cap = (int64_t)hs[0] + (int64_t)hs[0] / 8 + 64;
  }
  WalkArgs w;
  w.com = h.node_com.ptr;
  w.geom = h.node_geom.ptr;
  w.info = h.node_info.ptr;
  w.spm = h.spm.ptr;
  w.body = h.body;
  w.nstart = h.nstart.ptr;
  w.n = n;
  w.cap = h.cap;
  const float th = c->params.theta, eps = c->params.softening;
  w.theta2 = th * th;
  w.eps2 = eps * eps;
  w.G = c->params.G;
  w.leaf_cap = c->params.leaf_capacity;
  w.ax = ax;
  w.ay = ay;
  w.az = az;
  const bool count = (c->params.flags & NBGB_FLAG_COUNT_INTERACTIONS) != 0;
  w.counts = count ? c->counts.ensure((size_t)n) : nullptr;
  const bool bucket = c->params.leaf_capacity > 1;
  const unsigned blocks = grid1d(n);
  if (count) {
    if (bucket) bh_walk_kernel<true, true><<<blocks, 256, 0, st>>>(w);
    else bh_walk_kernel<true, false><<<blocks, 256, 0, st>>>(w);
  } else {
    if (bucket) bh_walk_kernel<false, true><<<blocks, 256, 0, st>>>(w);
    else bh_walk_kernel<false, false><<<blocks, 256, 0, st>>>(w);
  }
  NBGB_LAUNCH_CHECK();
}

// ------------------------------------------------------------- export --
__global__ void export_nodes_kernel(const float4* __restrict__ com, const float4* __restrict__ geom,
                                    const int4* __restrict__ info, const int32_t* __restrict__ parent,
                                    const uint32_t* __restrict__ body, const u64* __restrict__ hi,
                                    const u64* __restrict__ lo, int64_t total,
                                    nbgb_octree_node* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 in = info[p];
    const float4 g = geom[p], cm = com[p];
    nbgb_octree_node& o = out[p];
    o.center[0] = g.x;
    o.center[1] = g.y;
    o.center[2] = g.z;
    o.half_size = g.w;
    o.center_of_mass[0] = cm.x;
    o.center_of_mass[1] = cm.y;
    o.center_of_mass[2] = cm.z;
    o.total_mass = cm.w;
    o.is_leaf = (uint8_t)(in.w & 1);
    o.pad_[0] = o.pad_[1] = o.pad_[2] = 0;
    o.particle_count = in.z;
    o.particle_index = (in.w & 1) ? (int32_t)body[in.y] : -1;
    for (int j = 0; j < 8; ++j) o.children[j] = -1;
  }
}

__global__ void export_children_kernel(const int4* __restrict__ info,
                                       const int32_t* __restrict__ parent,
                                       const u64* __restrict__ hi, const u64* __restrict__ lo,
                                       int64_t total, nbgb_octree_node* __restrict__ out) {
  for (int64_t p = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int4 in = info[p];
    const int d = in.w >> 8;
    const int64_t f = in.y;
    const uint32_t oct = (d <= kHiLevels) ? (uint32_t)((hi[f] >> (3 * (kHiLevels - d))) & 7u)
                                          : (uint32_t)((lo[f] >> (3 * (kMaxDepth - d))) & 7u);
    out[parent[p]].children[oct] = (int32_t)p;
  }
}

}  // namespace nbgb

using namespace nbgb;

extern "C" {

nbgb_status nbgb_bh_tree_stats(nbgb_calculator* c, int32_t* node_count, int32_t* max_depth) {
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT) return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  uint32_t s[2] = {0, 0};
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  if (cudaMemcpy(s, h.scalars.ptr, sizeof s, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  if (node_count) *node_count = (int32_t)s[0];
  if (max_depth) *max_depth = (int32_t)s[1];
  return NBGB_OK;
}

nbgb_status nbgb_bh_copy_sorted_keys(nbgb_calculator* c, uint32_t* keys, int32_t* indices,
                                     size_t n) {
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT) return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  if (n != (size_t)h.n) return NBGB_ERR_INVALID_ARG;
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
  if (!c || !c->bh || c->method != NBGB_BARNES_HUT || !nodes) return NBGB_ERR_INVALID_ARG;
  BHState& h = *c->bh;
  uint32_t s[2] = {0, 0};
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  if (cudaMemcpy(s, h.scalars.ptr, sizeof s, cudaMemcpyDeviceToHost) != cudaSuccess)
    return NBGB_ERR_CUDA;
  const int64_t total = s[0];
  if ((size_t)total > capacity || total > h.cap) return NBGB_ERR_INVALID_ARG;
  nbgb_octree_node* d = nullptr;
  if (cudaMalloc(&d, (size_t)total * sizeof(nbgb_octree_node)) != cudaSuccess) return NBGB_ERR_OOM;
  unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, 256), 4096));
  export_nodes_kernel<<<blocks, 256, 0, c->stream>>>(h.node_com.ptr, h.node_geom.ptr,
                                                     h.node_info.ptr, h.node_parent.ptr, h.body,
                                                     h.hi_sorted, h.klo.ptr, total, d);
  export_children_kernel<<<blocks, 256, 0, c->stream>>>(h.node_info.ptr, h.node_parent.ptr,
                                                        h.hi_sorted, h.klo.ptr, total, d);
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

}  // extern "C"
