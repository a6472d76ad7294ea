// geom.cu -- bounding box of the packed positions (K2 first half).
//
// Replaces computeBoundingBoxKernel + atomicMin/MaxFloat and the host wrapper
// that mallocs, copies and frees six scalars every step
// (src/cuda/force_barnes_hut.cu:53-122,266-306).  Min/max are exact, so the
// result equals the reference's whatever the reduction order.  Two kernels,
// no atomics, no host round trip: per-block partials, then one block folds
// them and (optionally) derives the Barnes-Hut root cube and Morton scale.
#include "common.cuh"
#include "geom.cuh"
#include "kernels.cuh"

namespace nbgb {

__global__ void bbox_partial_kernel(const float4* __restrict__ pm, int64_t n,
                                    float* __restrict__ part) {
  float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = pm[i];
    mn[0] = fminf(mn[0], p.x);
    mn[1] = fminf(mn[1], p.y);
    mn[2] = fminf(mn[2], p.z);
    mx[0] = fmaxf(mx[0], p.x);
    mx[1] = fmaxf(mx[1], p.y);
    mx[2] = fmaxf(mx[2], p.z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mn[a] = fminf(mn[a], __shfl_down_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_down_sync(0xffffffffu, mx[a], o));
    }
  }
  __shared__ float s[32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    for (int a = 0; a < 3; ++a) {
      s[warp][a] = mn[a];
      s[warp][3 + a] = mx[a];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; ++w)
      for (int a = 0; a < 3; ++a) {
        s[0][a] = fminf(s[0][a], s[w][a]);
        s[0][3 + a] = fmaxf(s[0][3 + a], s[w][3 + a]);
      }
    for (int k = 0; k < 6; ++k) part[(int64_t)blockIdx.x * 6 + k] = s[0][k];
  }
}

// Folds the partials into `box` and derives the Barnes-Hut constants with the
// reference's float operations:
//   Morton scale  inv = 1.0f / (max - min + 0.001f)            (:313-320)
//   root centre   (min + max) * 0.5f                           (:418-419)
//   root half     max(ex, ey, ez) * 0.5f + 0.001f, first max   (:420-422)
// Rounding is pinned with _rn intrinsics (no contraction).
__global__ void bbox_final_kernel(const float* __restrict__ part, int nblocks, BBox* __restrict__ box,
                                  uint32_t* err) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
  for (int b = 0; b < nblocks; ++b)
    for (int a = 0; a < 3; ++a) {
      mn[a] = fminf(mn[a], part[b * 6 + a]);
      mx[a] = fmaxf(mx[a], part[b * 6 + 3 + a]);
    }
  BBox o;
  bool ok = true;
  for (int a = 0; a < 3; ++a) {
    o.min[a] = mn[a];
    o.max[a] = mx[a];
    ok = ok && isfinite(mn[a]) && isfinite(mx[a]);
    o.inv[a] = __fdiv_rn(1.0f, __fadd_rn(__fsub_rn(mx[a], mn[a]), 0.001f));
    o.center[a] = __fmul_rn(__fadd_rn(mn[a], mx[a]), 0.5f);
  }
  float ex = __fsub_rn(mx[0], mn[0]), ey = __fsub_rn(mx[1], mn[1]), ez = __fsub_rn(mx[2], mn[2]);
  float ms = ex;
  if (ms < ey) ms = ey;
  if (ms < ez) ms = ez;
  o.half = __fadd_rn(__fmul_rn(ms, 0.5f), 0.001f);
  o.valid = ok ? 1 : 0;
  if (!ok) raise_error(err, kErrBadInput);
  *box = o;
}

int bbox_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256 * 4), (int64_t)num_sms() * 2));
}

void launch_bbox(const float4* pm, int64_t n, float* partials, BBox* box, uint32_t* err,
                 cudaStream_t st) {
  const int nb = bbox_blocks(n);
  bbox_partial_kernel<<<nb, 256, 0, st>>>(pm, n, partials);
  NBGB_LAUNCH_CHECK();
  bbox_final_kernel<<<1, 32, 0, st>>>(partials, nb, box, err);
  NBGB_LAUNCH_CHECK();
}

}  // namespace nbgb
