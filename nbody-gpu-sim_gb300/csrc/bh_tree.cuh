// bh_tree.cuh -- Barnes-Hut state shared by the tree build and reference
// walk (bh.cu) and the group walk (bh_group.cu): the 64-byte node record and
// its walk-record flags, the per-state buffers, the segment view, and the
// group walk's parameters.
#pragma once

#include <algorithm>

#include "bh.cuh"
#include "common.cuh"
#include "geom.cuh"
#include "runtime.cuh"

namespace nbgb {

using u64 = unsigned long long;
constexpr int kHiLevels = 21;  // levels 1..21 in the high key (63 bits)
constexpr int kMaxDepth = 32;  // force_barnes_hut.cu:24

// One octree node, 64 bytes (one walk visit touches one 64-byte block).
struct __align__(16) Node {
  float4 com;   // centre of mass, total mass
  float4 geom;  // cube centre, half size
  int4 info;    // skip (next node outside the subtree), depth << 8 | leaf,
                // first body, body count
  int4 walk;    // for the walk: skip | leaf << 31 | zero mass << 30, bits of 4 h^2,
                // first body, body count | has a next sibling << 31
};

constexpr uint32_t kWalkLeaf = 1u << 31;
constexpr uint32_t kWalkZero = 1u << 30;
constexpr uint32_t kWalkNext = 1u << 31;  // in walk.w: the node has a next sibling
constexpr int64_t kMaxWalkNodes = (int64_t)1 << 30;  // skip indices below the flag bits

// The walk record of a node whose centre of mass is final: skip and flags,
// and the opening test's size2 = 4 h^2 (force_barnes_hut.cu:222) rounded as
// the reference rounds it.
__device__ __forceinline__ int4 walk_record(const int4& in, float h, float mass, bool next) {
  uint32_t w = (uint32_t)in.x;
  if (in.y & 1) w |= kWalkLeaf;
  if (mass == 0.0f) w |= kWalkZero;
  return make_int4((int)w, __float_as_int(__fmul_rn(__fmul_rn(4.0f, h), h)), in.z,
                   (int)((uint32_t)in.w | (next ? kWalkNext : 0u)));
}

// A node has a next sibling when its subtree ends before its parent's.
__device__ __forceinline__ bool has_next_sibling(const Node* nodes, int skip, int par) {
  return par >= 0 && skip < nodes[par].info.x;
}

struct BHState {
  // segment tables (device; single-system calls fill one segment)
  DevBuf<char> tables;           // seg_off [nseg], seg_base [nseg + 1], tasks [ntasks]
  int64_t* seg_off_p = nullptr;
  int64_t* seg_base_p = nullptr;
  WarpTask* tasks_p = nullptr;
  DevBuf<int32_t> seg_of;
  DevBuf<uint32_t> seg_minmax;   // [6][nseg] ordered-uint encoded bounds
  DevBuf<BBox> box;              // [nseg]
  DevBuf<int32_t> seg_root, seg_end, seg_depth;  // per segment
  HostPinned<char> h_tables;
  int32_t nseg = 0;
  int64_t ntasks = 0;
  // keys and order
  DevBuf<uint32_t> mkeys, mkeys_alt, midx, midx_alt;  // on-demand Morton sort
  DevBuf<u64> klo, khi, khi_alt;
  DevBuf<uint32_t> pidx, pidx_alt, sk, sk_alt;
  DevBuf<int32_t> kseg;          // segment of sorted position k
  DevBuf<uint32_t> hist, scan_ws;
  DevBuf<uint8_t> lcp;
  DevBuf<uint32_t> ncnt;    // n + 1
  DevBuf<uint32_t> nstart;  // n + 1
  DevBuf<uint32_t> scalars; // [0] total nodes
  HostPinned<uint32_t> h_scalars;
  DevBuf<Node> nodes;
  DevBuf<int32_t> node_parent, node_nchild, node_visit;
  DevBuf<int32_t> leaf_of;  // per sorted body: the leaf it starts, or -1
  DevBuf<char> ref_nodes;   // reference-identical build: the reference's node array
  DevBuf<int32_t> ref_pos;  // reference-identical build: original index -> sorted position
  DevBuf<float4> spm;      // bodies in path order
  DevBuf<uint32_t> walk_ctr;  // next warp task of the walk
  DevBuf<int4> groups;        // group walk: first body, count, segment; cost classes 0 / 1
                              // from the front / back of groups, 2 / 3 of groups2
  DevBuf<int4> groups2;
  DevBuf<uint32_t> body_cost;  // group walk: per concatenated body, the cost of its
                               // group in the last walk (list entries x bodies per lane)
  DevBuf<unsigned long long> cost_acc;  // the last walk's total cost and group count
  bool groups_ready = false;  // the last build emitted groups
  int group_max = 32;           // largest group of the last build (32 or 64 bodies)
  DevBuf<char> group_ctr;     // group walk: GroupCounters
  DevBuf<int> group_ovf;      // group walk: stack overflow chunks
  int64_t n = 0;
  int64_t reserve = 0;  // bodies the per-body buffers are sized for (>= n)
  int64_t cap = 0;      // node capacity
  bool m_alt = false;       // Morton result in *_alt
  bool keys_valid = false;  // Morton (key, index) pairs computed for the last build
  const uint32_t* body = nullptr;  // path-sorted concatenated body indices
  bool built = false;  // the last build finished (the inspection calls read its buffers)
};

struct SegView {
  const int64_t* off;   // arena offset of segment s
  const int64_t* base;  // first concatenated index of segment s (nseg + 1 entries)
  const int32_t* seg_of;
  const BBox* box;
  __device__ __forceinline__ int64_t arena(uint32_t q) const {
    const int s = seg_of[q];
    return off[s] + ((int64_t)q - base[s]);
  }
};

// Barnes-Hut group walk parameters (see the group walk below).
constexpr int kGroupSize = 64;        // largest group (two bodies per lane above 32)
constexpr int kGroupSmall = 32;       // groups of builds below kGroup64MinBodies bodies
constexpr int64_t kGroup64MinBodies = 262144;  // from here on groups of up to 64 bodies
constexpr int kGroupMergeMax = 1024;  // sibling subtrees merge only under parents this small
constexpr int kGWarps = 8;            // warps (groups in flight) per block
constexpr int kGStack = 512;          // per-warp shared stack (nodes to test)
constexpr int kGRing = 64;            // per-warp ring of pending list entries
constexpr int kGSmallRun = 16;        // bucket / leaf bodies listed lane-parallel up to this
constexpr int kOvfChunk = 8704;       // per-warp stack overflow: 32 x 8 siblings x 34 levels
constexpr int kOvfChunks = 256;       // overflow chunks per launch
constexpr float kBoxWiden = 0x1.000004p0f;  // 1 + 2^-22: covers the half sizes' rounding

// Groups by their estimated cost (the last walk's cost of their first
// body's group) against the last walk's mean: class 0 above 2x the mean,
// 1 above the mean, 2 above half of it, 3 the rest (and groups without an
// estimate); the walk takes the classes in that order.
constexpr int kCostClasses = 4;
struct GroupCounters {
  uint32_t nclass[kCostClasses];  // groups emitted per cost class
  uint32_t task;                  // next group of the walk
  uint32_t ovf;                   // overflow chunks handed out
  uint32_t pad[2];
};

// Largest group of a build over n bodies (all segments together): groups of
// up to 64 bodies halve the traversal per body and the list reads per
// interaction, but give half as many warps, which only pays when the walk
// has enough groups to fill the GPU.
inline int bh_group_max(int64_t n) { return n >= kGroup64MinBodies ? kGroupSize : kGroupSmall; }

// Centre of mass and cube of a node in one 256-bit load (read-only path),
// as the register pairs (com x, y), (com z, mass), (centre x, y), (centre z, half).
__device__ __forceinline__ void ld_node2(const Node* p, f2& cm_xy, f2& cm_zw, f2& g_xy, f2& g_zw) {
  asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];"
      : "=l"(cm_xy.v), "=l"(cm_zw.v), "=l"(g_xy.v), "=l"(g_zw.v)
      : "l"(p));
}

// Grows a buffer to hold n elements, with 1.5x headroom when it has to
// reallocate (a reallocation synchronises the device).
template <typename T>
inline T* grow(DevBuf<T>& b, size_t n) {
  if (n <= b.cap && b.ptr) return b.ptr;
  return b.ensure(std::max(n, b.cap + b.cap / 2));
}

// The group walk for every segment (bh_group.cu); needs groups from the
// last build (bh_build with groups).
void bh_group_walk(BHState& h, const BHWalkParams& p, float* ax, float* ay, float* az,
                   int32_t* counts, unsigned long long* inter_total, uint32_t* err,
                   cudaStream_t st);

}  // namespace nbgb
