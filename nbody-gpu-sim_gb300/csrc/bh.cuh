// bh.cuh -- Barnes-Hut build and walk over one or many independent systems
// ("segments") stored in one packed (x, y, z, m) array (bh.cu).
#pragma once

#include "common.cuh"

namespace nbgb {

struct BHState;
struct StageTimer;

// 32 consecutive path-sorted targets of one segment, walked by one warp.
struct WarpTask {
  int64_t first;  // first sorted position
  int64_t end;    // one past the segment's last sorted position
  int32_t seg;
  int32_t pad_;
};

struct BHWalkParams {
  float G;
  float softening;
  float theta;
  int leaf_capacity;  // > 1: subtrees of at most this many bodies are summed body by body
  int group_walk;     // 1: one interaction list per group of <= 64 nearby bodies, cells
                      // accepted by the group's bounding box (opened buckets of at most
                      // leaf_capacity bodies list their bodies)
};

BHState* bh_state_new();
void bh_state_delete(BHState* p);
size_t bh_state_bytes(const BHState* p);
// Device bytes per body a segmented state needs at its asynchronous node
// capacity (upper bound used for admission control).
size_t bh_bytes_estimate(int64_t n);

// Segment s = bodies pm[off[s] .. off[s] + n_per[s]).  Buffers grow
// geometrically, so a slowly growing total does not reallocate every call.
// `staging` is a pinned host buffer of bh_segment_table_bytes() bytes that
// the caller keeps untouched until the copies enqueued on `st` have run;
// null = an internal buffer, with a synchronisation of `st` first.
size_t bh_segment_table_bytes(const int64_t* n_per, int nseg);
void bh_set_segments(BHState& h, const int64_t* off, const int64_t* n_per, int nseg,
                     cudaStream_t st, char* staging);
// Node capacity for use without a read-back (4 nodes per body + 64 per segment).
void bh_reserve_async(BHState& h);
// Allocates every buffer bh_build / bh_walk of the current segments needs.
void bh_reserve_buffers(BHState& h, bool groups);
// Trees of all segments (bit-identical, per segment, to the single-system tree);
// `groups` also emits the group walk's groups.
// groups: emit the group walk's groups, of at most group_max bodies (32 or
// 64; 0 = by the body count, bh_group_max).
// ref_tree: the reference's insertion tree (node budget included) instead of
// the canonical one; one segment of at most 65,536 bodies, no groups.
// timer: stage marks for NBGB_FLAG_STAGE_TIMINGS (or null).
void bh_build(BHState& h, const float4* pm, cudaStream_t st, uint32_t* err, bool groups,
              int group_max = 0, bool ref_tree = false, StageTimer* timer = nullptr);
// Accelerations of all segments, written at each segment's offset into
// ax/ay/az.  counts (per arena index) and inter_total (running sum) are
// optional; err receives device error bits (group walk stack overflow).
void bh_walk(BHState& h, const BHWalkParams& p, float* ax, float* ay, float* az, int32_t* counts,
             unsigned long long* inter_total, uint32_t* err, cudaStream_t st);
// Shared-memory stack entries of the group walk before it spills (64 .. 512).
void bh_set_group_stack_limit(int entries);

}  // namespace nbgb
