// hash.cu -- spatial hash (placeholder until the counting-sort grid lands).
#include "common.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {
struct HashState {};
void hash_state_delete(HashState* p) { delete p; }
void hash_forces(nbgb_calculator*, const float4*, int64_t, float*, float*, float*) {
  fail(NBGB_ERR_INVALID_ARG, "spatial hash is not available in this build");
}
}  // namespace nbgb

using namespace nbgb;
extern "C" {
nbgb_status nbgb_hash_grid_info(nbgb_calculator*, int32_t*, float*, float*, int64_t*) { return NBGB_ERR_INVALID_ARG; }
nbgb_status nbgb_hash_copy_cells(nbgb_calculator*, int32_t*, int32_t*, int32_t*, int32_t*) { return NBGB_ERR_INVALID_ARG; }
}
