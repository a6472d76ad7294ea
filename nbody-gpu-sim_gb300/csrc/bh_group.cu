// bh_group.cu -- the Barnes-Hut group walk (NBGB_FLAG_GROUP_WALK): one
// interaction list per group of at most 32 or 64 nearby bodies, built by one
// warp that tests 32 nodes at a time and evaluated by all its lanes.  Groups
// come from the tree build (link_kernel in bh.cu), filed in cost classes
// learned from the previous walk.
#include <algorithm>
#include <atomic>

#include "bh_tree.cuh"
#include "kernels.cuh"

namespace nbgb {

// ---------------------------------------------------------- group walk --
// Barnes-Hut with a per-group opening test: the bodies of one small subtree
// (or of consecutive small sibling subtrees, at most 64 bodies) share one
// interaction list, built by one warp that tests 32 nodes at a time.  A cell
// is accepted for the whole group when its cube does not touch the group's
// bounding box and size2 < theta2 (d_min^2 + eps^2), d_min being the distance
// from the cell's centre of mass to the box: every accepted cell passes the
// reference's per-target test (force_barnes_hut.cu:218-224) for every body of
// the group, so each target sees an equal or finer cell set than in the
// reference walk.  Leaves contribute their bodies; with leaf_capacity > 1 a
// node of at most that many bodies that is not accepted contributes its
// bodies instead of being opened (buckets).  The list is evaluated by
// all lanes at once, one target per lane (2 or 4 lanes per target in groups
// of at most 16 or 8 bodies, two targets per lane in groups of more than 32),
// in packed FP32x2 arithmetic.
struct GroupWalkArgs {
  const Node* nodes;
  const float4* spm;
  const uint32_t* body;
  const uint32_t* nstart;
  SegView sv;
  const int4* groups;   // cost classes 0 (front) and 1 (back)
  const int4* groups2;  // cost classes 2 (front) and 3 (back)
  const int32_t* seg_root;
  int64_t n;
  int64_t cap;
  float theta2;
  float eps2;
  float G;
  float* ax;
  float* ay;
  float* az;
  int32_t* counts;                  // per-body list lengths without the body itself (or null)
  unsigned long long* inter_total;  // sum of counts (or null)
  GroupCounters* gc;
  int* ovf;                         // kOvfChunks x kOvfChunk stack overflow entries
  uint32_t* err;
  int stack_limit;                  // shared stack entries used (64 .. kGStack)
  int leaf_cap;                     // > 1: an opened node of at most this many bodies adds
                                    // its bodies (buckets) instead of its children
  int64_t gcap;                     // groups capacity: light groups fill it from the back
  uint32_t* body_cost;              // out: per body, its group's cost (for the next build)
  unsigned long long* cost_acc;     // out: total cost, groups
};

// Floats as unsigned integers with the same order (finite values).
__device__ __forceinline__ uint32_t ord_of(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_of(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// One pair of list entries (packed x, y, z, m) added to one target.
template <bool ZERO_EPS>
__device__ __forceinline__ void pair_add(f2 xj, f2 yj, f2 zj, f2 m, f2 px, f2 py, f2 pz, f2 e2,
                                         f2& ax2, f2& ay2, f2& az2) {
  const f2 dx = f2_sub(xj, px);
  const f2 dy = f2_sub(yj, py);
  const f2 dz = f2_sub(zj, pz);
  const f2 d2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, e2)));
  float d2l, d2h;
  f2_split(d2, d2l, d2h);
  float rl = rsqrt_approx(d2l), rh = rsqrt_approx(d2h);
  if (ZERO_EPS) {  // coincident bodies (and the target itself) add nothing
    rl = d2l > 0.0f ? rl : 0.0f;
    rh = d2h > 0.0f ? rh : 0.0f;
  }
  const f2 rr = f2_make(rl, rh);
  const f2 f = f2_mul(f2_mul(m, rr), f2_mul(rr, rr));
  ax2 = f2_fma(f, dx, ax2);
  ay2 = f2_fma(f, dy, ay2);
  az2 = f2_fma(f, dz, az2);
}

__device__ __forceinline__ f2 ring_pair(const float* e, int j) {
  return f2{*reinterpret_cast<const unsigned long long*>(e + j)};
}

// Adds list entries [base, base + cnt) of the ring (cnt a multiple of 4)
// to the lane's target, two entries per packed operation.  With rep > 1
// lanes per body (small groups), replica r takes every rep-th pair.
template <bool ZERO_EPS, bool FULL>
__device__ __forceinline__ void group_eval(const float* ex, const float* ey, const float* ez,
                                           const float* em, int base, int cnt, int r, int rep,
                                           float4 pi, float eps2, f2& ax2, f2& ay2, f2& az2) {
  const f2 px = f2_make(pi.x, pi.x), py = f2_make(pi.y, pi.y), pz = f2_make(pi.z, pi.z);
  const f2 e2 = f2_make(eps2, eps2);
  // FULL: one lane per body and a whole 32-entry chunk (fixed trip count);
  // entries are read as pairs straight into packed registers
  const int j0 = FULL ? 0 : 2 * r, jn = FULL ? 32 : cnt, js = FULL ? 2 : 2 * rep;
#pragma unroll(FULL ? 16 : 1)
  for (int j = j0; j < jn; j += js)
    pair_add<ZERO_EPS>(ring_pair(ex, base + j), ring_pair(ey, base + j), ring_pair(ez, base + j),
                       ring_pair(em, base + j), px, py, pz, e2, ax2, ay2, az2);
}

// Groups of 33..64 bodies: each lane sums body `lane` over the whole list
// and, for the h = count - 32 second bodies, lanes b, b + w, ... (w = 8, 16
// or 32 >= h; REP2 = 32 / w replicas) sum second body b, replica r taking
// pair r of every REP2 consecutive pairs, so no lane idles in the second
// half when h <= 16.  The first body's pairs are read once for the whole
// warp (broadcast); each replica reads its own pair for the second body.
template <bool ZERO_EPS, bool FULL, int REP2>
__device__ __forceinline__ void group_eval2(const float* ex, const float* ey, const float* ez,
                                            const float* em, int base, int cnt, int r2,
                                            float4 pi, float4 pj, float eps2, f2& ax2, f2& ay2,
                                            f2& az2, f2& bx2, f2& by2, f2& bz2) {
  const f2 px = f2_make(pi.x, pi.x), py = f2_make(pi.y, pi.y), pz = f2_make(pi.z, pi.z);
  const f2 qx = f2_make(pj.x, pj.x), qy = f2_make(pj.y, pj.y), qz = f2_make(pj.z, pj.z);
  const f2 e2 = f2_make(eps2, eps2);
  const int jn = FULL ? 32 : cnt;
#pragma unroll(FULL ? 8 / REP2 : 1)
  for (int j = 0; j < jn; j += 2 * REP2) {
    if (REP2 == 1) {
      const f2 xj = ring_pair(ex, base + j), yj = ring_pair(ey, base + j),
               zj = ring_pair(ez, base + j), m = ring_pair(em, base + j);
      pair_add<ZERO_EPS>(xj, yj, zj, m, px, py, pz, e2, ax2, ay2, az2);
      pair_add<ZERO_EPS>(xj, yj, zj, m, qx, qy, qz, e2, bx2, by2, bz2);
    } else {
#pragma unroll
      for (int r = 0; r < REP2; ++r)
        pair_add<ZERO_EPS>(ring_pair(ex, base + j + 2 * r), ring_pair(ey, base + j + 2 * r),
                           ring_pair(ez, base + j + 2 * r), ring_pair(em, base + j + 2 * r), px,
                           py, pz, e2, ax2, ay2, az2);
      const int jb = base + j + 2 * r2;
      pair_add<ZERO_EPS>(ring_pair(ex, jb), ring_pair(ey, jb), ring_pair(ez, jb),
                         ring_pair(em, jb), qx, qy, qz, e2, bx2, by2, bz2);
    }
  }
}

// CNT: 0 no counting; 1 the total only (list lengths minus one per body of
// nonzero mass, whose own leaf is in its list); 2 exact per-body counts (the
// own leaf tracked as it is listed) and their total.
// TWO: groups of up to 64 bodies (two targets per lane above 32; 80
// registers, 3 blocks per SM); otherwise groups of up to 32 (64 registers,
// 4 blocks per SM).
template <int CNT, bool ZERO_EPS, bool TWO>
__global__ void __launch_bounds__(kGWarps * 32, TWO ? 3 : 4) bh_group_walk_kernel(GroupWalkArgs a) {
  constexpr bool COUNT = CNT == 2;
  __shared__ int s_stack[kGWarps][kGStack];
  __shared__ __align__(16) float s_ring[kGWarps][4][kGRing];
  __shared__ __align__(16) float4 s_box[kGWarps][2];  // group box: centre, half sizes
  const uint32_t total = a.nstart[a.n];
  if ((int64_t)total > a.cap) return;  // the tree build failed and said so
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
  int* stk = s_stack[wid];
  float* ex = s_ring[wid][0];
  float* ey = s_ring[wid][1];
  float* ez = s_ring[wid][2];
  float* em = s_ring[wid][3];
  // the cost classes in order: class 0 (longest) first
  const uint32_t c0 = *(volatile uint32_t*)&a.gc->nclass[0];
  const uint32_t c01 = c0 + *(volatile uint32_t*)&a.gc->nclass[1];
  const uint32_t c012 = c01 + *(volatile uint32_t*)&a.gc->nclass[2];
  const uint32_t ngroups = c012 + *(volatile uint32_t*)&a.gc->nclass[3];
  int* ovf = nullptr;  // this warp's overflow chunk, taken on first use
  while (true) {
    uint32_t t32 = 0;
    if (lane == 0) t32 = atomicAdd(&a.gc->task, 1u);
    const uint32_t t = __shfl_sync(full, t32, 0);
    if (t >= ngroups) break;
    const int4 g = t < c0     ? a.groups[t]
                   : t < c01  ? a.groups[a.gcap - 1 - (int64_t)(t - c0)]
                   : t < c012 ? a.groups2[t - c01]
                              : a.groups2[a.gcap - 1 - (int64_t)(t - c012)];
    // a group of at most 8 (16) bodies gives each body 4 (2) lanes, each
    // summing a share of the list: lane = replica * gw + body; in a group of
    // more than 32 bodies every lane sums body `lane`, and its h - 32 second
    // bodies get 32 / gw2 lanes each the same way (lane = replica * gw2 + b)
    const bool two = TWO && g.y > 32;
    const int gw = g.y <= 8 ? 8 : (g.y <= 16 ? 16 : 32);
    const int rep = 32 / gw, tl = lane & (gw - 1), rr = lane / gw;
    const int h2 = two ? g.y - 32 : 0, gw2 = h2 <= 8 ? 8 : (h2 <= 16 ? 16 : 32);
    const int rep2 = 32 / gw2, tl2 = lane & (gw2 - 1), rr2 = lane / gw2;
    const bool valid = tl < g.y, valid2 = two && tl2 < h2;
    const int k = g.x + (valid ? tl : 0), k2 = g.x + (valid2 ? 32 + tl2 : 0);
    const float4 pi = a.spm[k];
    const float4 pj = two ? a.spm[k2] : pi;  // invalid second bodies repeat body 0
    {
      const float lox = float_of(__reduce_min_sync(full, min(ord_of(pi.x), ord_of(pj.x))));
      const float loy = float_of(__reduce_min_sync(full, min(ord_of(pi.y), ord_of(pj.y))));
      const float loz = float_of(__reduce_min_sync(full, min(ord_of(pi.z), ord_of(pj.z))));
      const float hix = float_of(__reduce_max_sync(full, max(ord_of(pi.x), ord_of(pj.x))));
      const float hiy = float_of(__reduce_max_sync(full, max(ord_of(pi.y), ord_of(pj.y))));
      const float hiz = float_of(__reduce_max_sync(full, max(ord_of(pi.z), ord_of(pj.z))));
      if (lane == 0) {  // centre and half sizes, the halves widened past rounding
        const float cx = __fmul_rn(__fadd_rn(lox, hix), 0.5f);
        const float cy = __fmul_rn(__fadd_rn(loy, hiy), 0.5f);
        const float cz = __fmul_rn(__fadd_rn(loz, hiz), 0.5f);
        s_box[wid][0] = make_float4(cx, cy, cz, 0.f);
        s_box[wid][1] = make_float4(
            __fmul_rn(fmaxf(__fsub_rn(hix, cx), __fsub_rn(cx, lox)), kBoxWiden),
            __fmul_rn(fmaxf(__fsub_rn(hiy, cy), __fsub_rn(cy, loy)), kBoxWiden),
            __fmul_rn(fmaxf(__fsub_rn(hiz, cz), __fsub_rn(cz, loz)), kBoxWiden), 0.f);
      }
    }
    f2 ax2 = f2_make(0.f, 0.f), ay2 = ax2, az2 = ax2, bx2 = ax2, by2 = ax2, bz2 = ax2;
    uint32_t wr = 0, rd = 0;  // list entries written / evaluated
    uint64_t selfmask = 0;    // bodies (by index in the group) whose own leaf is in the list
    // evaluates ring entries [base, base + cnt); full: a whole 32-entry chunk
    auto eval = [&](int base, int cnt, bool full_chunk) {
      if (two) {
#define NBGB_EVAL2(F, R)                                                                        \
  group_eval2<ZERO_EPS, F, R>(ex, ey, ez, em, base, F ? 32 : cnt, rr2, pi, pj, a.eps2, ax2, ay2, \
                              az2, bx2, by2, bz2)
        if (rep2 == 1) {
          if (full_chunk) NBGB_EVAL2(true, 1); else NBGB_EVAL2(false, 1);
        } else if (rep2 == 2) {
          if (full_chunk) NBGB_EVAL2(true, 2); else NBGB_EVAL2(false, 2);
        } else {
          if (full_chunk) NBGB_EVAL2(true, 4); else NBGB_EVAL2(false, 4);
        }
#undef NBGB_EVAL2
      } else if (full_chunk && rep == 1) {
        group_eval<ZERO_EPS, true>(ex, ey, ez, em, base, 32, 0, 1, pi, a.eps2, ax2, ay2, az2);
      } else {
        group_eval<ZERO_EPS, false>(ex, ey, ez, em, base, cnt, rr, rep, pi, a.eps2, ax2, ay2,
                                    az2);
      }
    };
    int sp = 1, gsp = 0;
    bool failed = false;
    if (lane == 0) stk[0] = a.seg_root[g.z];
    __syncwarp();
    while (sp > 0 || gsp > 0) {
      if (sp == 0) {  // refill from the overflow chunk
        const int m = min(gsp, a.stack_limit / 2);
        for (int j = lane; j < m; j += 32) stk[j] = ovf[gsp - m + j];
        gsp -= m;
        sp = m;
        __syncwarp();
      }
      if (sp > a.stack_limit - 32) {  // a step adds at most 32: spill the oldest half
        const int half = a.stack_limit / 2;
        if (!ovf) {
          uint32_t c32 = 0;
          if (lane == 0) c32 = atomicAdd(&a.gc->ovf, 1u);
          const uint32_t c = __shfl_sync(full, c32, 0);
          if (c < (uint32_t)kOvfChunks) ovf = a.ovf + (size_t)c * kOvfChunk;
        }
        if (!ovf || gsp + half > kOvfChunk) {
          failed = true;
          break;
        }
        for (int j = lane; j < half; j += 32) ovf[gsp + j] = stk[j];
        __syncwarp();
        for (int j = lane; j < sp - half; j += 32) stk[j] = stk[half + j];
        gsp += half;
        sp -= half;
        __syncwarp();
      }
      const int m = min(sp, 32);
      sp -= m;
      const bool have = lane < m;
      const int node = have ? stk[sp + lane] : 0;
      __syncwarp();
      f2 cm_xy = f2_make(0.f, 0.f), cm_zw = cm_xy, g_xy = cm_xy, g_zw = cm_xy;
      int4 w = make_int4((int)kWalkZero, 0, 0, 0);
      if (have) {
        ld_node2(&a.nodes[node], cm_xy, cm_zw, g_xy, g_zw);
        w = __ldg(&a.nodes[node].walk);
      }
      float4 cm, ge;
      f2_split(cm_xy, cm.x, cm.y);
      f2_split(cm_zw, cm.z, cm.w);
      f2_split(g_xy, ge.x, ge.y);
      f2_split(g_zw, ge.z, ge.w);
      const uint32_t wx = (uint32_t)w.x;
      const bool next = have && ((uint32_t)w.w & kWalkNext);
      const int cnt = (int)((uint32_t)w.w & ~kWalkNext);
      bool entry = false, open = false, multi = false;
      if (!(wx & kWalkZero)) {
        if (wx & kWalkLeaf) {
          entry = cnt == 1;
          multi = cnt > 1;
        } else {
          const float4 bc = s_box[wid][0], bh = s_box[wid][1];
          // cube and box touch / distance of the centre of mass outside the box
          const bool overlap = fabsf(__fsub_rn(ge.x, bc.x)) <= __fadd_rn(ge.w, bh.x) &&
                               fabsf(__fsub_rn(ge.y, bc.y)) <= __fadd_rn(ge.w, bh.y) &&
                               fabsf(__fsub_rn(ge.z, bc.z)) <= __fadd_rn(ge.w, bh.z);
          const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(cm.x, bc.x)), bh.x), 0.0f);
          const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(cm.y, bc.y)), bh.y), 0.0f);
          const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(cm.z, bc.z)), bh.z), 0.0f);
          const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
          entry = !overlap && __int_as_float(w.y) < __fmul_rn(a.theta2, d2);
          // an opened bucket (at most leaf_cap bodies) lists its bodies
          multi = !entry && cnt <= a.leaf_cap;
          open = !entry && !multi;
        }
      }
      // next siblings below first children, so the walk goes depth first
      const unsigned bs = __ballot_sync(full, next), bo = __ballot_sync(full, open);
      if (next) stk[sp + __popc(bs & lt)] = (int)(wx & (kWalkZero - 1u));
      if (open) stk[sp + __popc(bs) + __popc(bo & lt)] = node + 1;
      sp += __popc(bs) + __popc(bo);
      const unsigned be = __ballot_sync(full, entry);
      if (entry) {
        const int slot = (int)((wr + __popc(be & lt)) & (kGRing - 1));
        ex[slot] = cm.x;
        ey[slot] = cm.y;
        ez[slot] = cm.z;
        em[slot] = cm.w;
      }
      wr += __popc(be);
      if (COUNT) {  // lane-local here, combined over the warp at the end
        const uint32_t rel = (uint32_t)(w.z - g.x);
        if (entry && (wx & kWalkLeaf) && rel < (uint32_t)g.y) selfmask |= 1ull << rel;
      }
      __syncwarp();
      if (wr - rd >= 32) {
        eval((int)(rd & (kGRing - 1)), 32, true);
        rd += 32;
        __syncwarp();
      }
      // bodies of small runs (opened buckets, small depth-32 leaves): every
      // such lane appends body j of its run in round j
      const bool small = multi && cnt <= kGSmallRun;
      if (__any_sync(full, small)) {
        const int left = small ? cnt : 0;
        if (COUNT && small) {  // the group's bodies inside this run list themselves
          const int lo = max(w.z, g.x), hi = min(w.z + cnt, g.x + g.y);
          if (lo < hi) selfmask |= ((1ull << (hi - lo)) - 1ull) << (lo - g.x);
        }
        for (int j = 0;; ++j) {
          const bool e = j < left;
          const unsigned bj = __ballot_sync(full, e);
          if (!bj) break;
          if (e) {
            const float4 q = a.spm[w.z + j];
            const int slot = (int)((wr + __popc(bj & lt)) & (kGRing - 1));
            ex[slot] = q.x;
            ey[slot] = q.y;
            ez[slot] = q.z;
            em[slot] = q.w;
          }
          wr += __popc(bj);
          __syncwarp();
          if (wr - rd >= 32) {
            eval((int)(rd & (kGRing - 1)), 32, true);
            rd += 32;
            __syncwarp();
          }
        }
      }
      // larger multi-body (depth-32) leaves: 32 bodies at a time, one leaf
      // after the other
      unsigned bm = __ballot_sync(full, multi && !small);
      while (bm) {
        const int src = __ffs(bm) - 1;
        bm &= bm - 1;
        const int f = __shfl_sync(full, w.z, src), c = __shfl_sync(full, cnt, src);
        if (COUNT) {
          const uint32_t o = (uint32_t)(k - f), o2 = (uint32_t)(k2 - f);
          if (valid && rr == 0 && o < (uint32_t)c) selfmask |= 1ull << tl;
          if (valid2 && o2 < (uint32_t)c) selfmask |= 1ull << (32 + tl2);
        }
        for (int b = 0; b < c; b += 32) {
          const bool e = b + lane < c;
          if (e) {
            const float4 q = a.spm[f + b + lane];
            const int slot = (int)((wr + lane) & (kGRing - 1));
            ex[slot] = q.x;
            ey[slot] = q.y;
            ez[slot] = q.z;
            em[slot] = q.w;
          }
          wr += (uint32_t)min(32, c - b);
          __syncwarp();
          if (wr - rd >= 32) {
            eval((int)(rd & (kGRing - 1)), 32, false);
            rd += 32;
            __syncwarp();
          }
        }
      }
    }
    if (failed) {
      if (lane == 0) raise_error(a.err, kErrWalkStack);
      const float nan = __int_as_float(0x7fc00000);
      ax2 = ay2 = az2 = bx2 = by2 = bz2 = f2_make(nan, nan);
    } else {
      // the rest of the list, padded to a multiple of 8 with massless entries
      // (the evaluation takes up to four pairs at a time)
      const int left = (int)(wr - rd), padded = (left + 7) & ~7;
      if (lane >= left && lane < padded) {
        const int slot = (int)((rd + lane) & (kGRing - 1));
        ex[slot] = 3.0e18f;
        ey[slot] = 0.0f;
        ez[slot] = 0.0f;
        em[slot] = 0.0f;
      }
      __syncwarp();
      if (padded) eval((int)(rd & (kGRing - 1)), padded, false);
      __syncwarp();
    }
    for (int o = gw; o < 32; o <<= 1) {  // add up the replicas of each body
      ax2 = f2_add(ax2, f2_shfl_xor(ax2, o));
      ay2 = f2_add(ay2, f2_shfl_xor(ay2, o));
      az2 = f2_add(az2, f2_shfl_xor(az2, o));
    }
    if (two)
      for (int o = gw2; o < 32; o <<= 1) {  // and the replicas of the second bodies
        bx2 = f2_add(bx2, f2_shfl_xor(bx2, o));
        by2 = f2_add(by2, f2_shfl_xor(by2, o));
        bz2 = f2_add(bz2, f2_shfl_xor(bz2, o));
      }
    if (COUNT)
      selfmask = (uint64_t)__reduce_or_sync(full, (uint32_t)selfmask) |
                 ((uint64_t)__reduce_or_sync(full, (uint32_t)(selfmask >> 32)) << 32);
    const int cnt_lane = (int)wr - (int)((selfmask >> tl) & 1u);
    const int cnt_lane2 = (int)wr - (int)((selfmask >> (32 + tl2)) & 1u);
    const bool owner = valid && rr == 0, owner2 = valid2 && rr2 == 0;
    if (owner) {
      float sx0, sx1, sy0, sy1, sz0, sz1;
      f2_split(ax2, sx0, sx1);
      f2_split(ay2, sy0, sy1);
      f2_split(az2, sz0, sz1);
      const int64_t i = a.sv.arena(a.body[k]);
      a.ax[i] = a.G * (sx0 + sx1);
      a.ay[i] = a.G * (sy0 + sy1);
      a.az[i] = a.G * (sz0 + sz1);
      if (COUNT && a.counts) a.counts[i] = cnt_lane;
    }
    if (owner2) {
      float sx0, sx1, sy0, sy1, sz0, sz1;
      f2_split(bx2, sx0, sx1);
      f2_split(by2, sy0, sy1);
      f2_split(bz2, sz0, sz1);
      const int64_t i = a.sv.arena(a.body[k2]);
      a.ax[i] = a.G * (sx0 + sx1);
      a.ay[i] = a.G * (sy0 + sy1);
      a.az[i] = a.G * (sz0 + sz1);
      if (COUNT && a.counts) a.counts[i] = cnt_lane2;
    }
    {  // this group's cost, for the order of the next build's groups
      const uint32_t cost = wr * (two ? 2u : 1u);
      if (owner) a.body_cost[a.body[k]] = cost;
      if (owner2) a.body_cost[a.body[k2]] = cost;
      if (lane == 0) {
        atomicAdd(&a.cost_acc[0], (unsigned long long)cost);
        atomicAdd(&a.cost_acc[1], 1ull);
      }
    }
    if (CNT > 0 && a.inter_total) {
      const int own = CNT == 2 ? cnt_lane : (int)wr - (pi.w != 0.0f ? 1 : 0);
      const int own2 = CNT == 2 ? cnt_lane2 : (int)wr - (pj.w != 0.0f ? 1 : 0);
      unsigned long long c = (owner ? (unsigned long long)own : 0ull) +
                             (owner2 ? (unsigned long long)own2 : 0ull);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(full, c, o);
      if (lane == 0) atomicAdd(a.inter_total, c);
    }
  }
}

template <int CNT, bool ZERO_EPS, bool TWO>
static int group_walk_occupancy() {
  static const int occ = [] {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, bh_group_walk_kernel<CNT, ZERO_EPS, TWO>,
                                                  kGWarps * 32,
                                                  0);
    return std::max(b, 1);
  }();
  return occ;
}

template <int CNT, bool ZERO_EPS, bool TWO>
static void launch_group_walk_t(const GroupWalkArgs& g, int64_t n, cudaStream_t st) {
  // persistent warps: one resident wave, never more warps than bodies
  const int64_t blocks = std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(n, kGWarps),
                           (int64_t)num_sms() * group_walk_occupancy<CNT, ZERO_EPS, TWO>()));
  bh_group_walk_kernel<CNT, ZERO_EPS, TWO><<<(unsigned)blocks, kGWarps * 32, 0, st>>>(g);
}

template <int CNT, bool ZERO_EPS>
static void launch_group_walk(const GroupWalkArgs& g, int64_t n, bool two, cudaStream_t st) {
  if (two)
    launch_group_walk_t<CNT, ZERO_EPS, true>(g, n, st);
  else
    launch_group_walk_t<CNT, ZERO_EPS, false>(g, n, st);
}

// Shared stack entries the group walk uses before spilling to global memory
// (a test hook: lowering it exercises the spill path on small inputs).
static std::atomic<int> g_group_stack_limit{kGStack};

void bh_set_group_stack_limit(int entries) { g_group_stack_limit.store(entries); }

void bh_group_walk(BHState& h, const BHWalkParams& p, float* ax, float* ay, float* az,
                          int32_t* counts, unsigned long long* inter_total, uint32_t* err,
                          cudaStream_t st) {
  const int64_t n = h.n;
  if (!h.groups_ready)
    fail(NBGB_ERR_INVALID_ARG, "Barnes-Hut group walk without groups from the tree build");
  int4* groups = h.groups.ptr;
  GroupCounters* gc = reinterpret_cast<GroupCounters*>(h.group_ctr.ptr);
  int* ovf = grow(h.group_ovf, (size_t)kOvfChunks * kOvfChunk);
  // the walk's task and overflow counters (the group count stays)
  NBGB_CUDA(cudaMemsetAsync(&gc->task, 0, 2 * sizeof(uint32_t), st));
  GroupWalkArgs g;
  g.nodes = h.nodes.ptr;
  g.spm = h.spm.ptr;
  g.body = h.body;
  g.nstart = h.nstart.ptr;
  g.sv = SegView{h.seg_off_p, h.seg_base_p, h.seg_of.ptr, h.box.ptr};
  g.groups = groups;
  g.groups2 = h.groups2.ptr;
  g.seg_root = h.seg_root.ptr;
  g.n = n;
  g.cap = h.cap;
  g.theta2 = p.theta * p.theta;
  g.eps2 = p.softening * p.softening;
  g.G = p.G;
  g.ax = ax;
  g.ay = ay;
  g.az = az;
  g.counts = counts;
  g.inter_total = inter_total;
  g.gc = gc;
  g.ovf = ovf;
  g.err = err;
  g.stack_limit = g_group_stack_limit.load();
  g.leaf_cap = p.leaf_capacity;
  g.gcap = (int64_t)h.groups.cap;
  g.body_cost = h.body_cost.ptr;
  g.cost_acc = h.cost_acc.ptr;
  const int cnt = counts ? 2 : (inter_total ? 1 : 0);
  const bool zero_eps = g.eps2 == 0.0f;
  const bool two = h.group_max > 32;
  if (cnt == 2) {
    if (zero_eps)
      launch_group_walk<2, true>(g, n, two, st);
    else
      launch_group_walk<2, false>(g, n, two, st);
  } else if (cnt == 1) {
    if (zero_eps)
      launch_group_walk<1, true>(g, n, two, st);
    else
      launch_group_walk<1, false>(g, n, two, st);
  } else {
    if (zero_eps)
      launch_group_walk<0, true>(g, n, two, st);
    else
      launch_group_walk<0, false>(g, n, two, st);
  }
  NBGB_LAUNCH_CHECK();
}

}  // namespace nbgb
