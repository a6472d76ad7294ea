// bh.cu -- Barnes-Hut (placeholder until the device octree lands).
#include "common.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {
struct BHState {};
void bh_state_delete(BHState* p) { delete p; }
void bh_forces(nbgb_calculator*, const float4*, int64_t, float*, float*, float*) {
  fail(NBGB_ERR_INVALID_ARG, "Barnes-Hut is not available in this build");
}
}  // namespace nbgb

using namespace nbgb;
extern "C" {
nbgb_status nbgb_bh_tree_stats(nbgb_calculator*, int32_t*, int32_t*) { return NBGB_ERR_INVALID_ARG; }
nbgb_status nbgb_bh_copy_sorted_keys(nbgb_calculator*, uint32_t*, int32_t*, size_t) { return NBGB_ERR_INVALID_ARG; }
nbgb_status nbgb_bh_copy_nodes(nbgb_calculator*, nbgb_octree_node*, size_t) { return NBGB_ERR_INVALID_ARG; }
nbgb_status nbgb_copy_interaction_counts(nbgb_calculator*, int32_t*, size_t) { return NBGB_ERR_INVALID_ARG; }
}
