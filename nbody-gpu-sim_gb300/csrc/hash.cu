// hash.cu -- spatial hash: stable counting sort by cell + 27-cell cutoff
// gather (K7).
//
// Replaces SpatialHashGrid::build / computeForces and
// SpatialHashCalculator::computeForces (src/cuda/force_spatial_hash.cu:241-388):
//  * bbox on the device (geom.cu), padded by 0.001f on the host with the
//    reference's float operations, dims = (int)ceilf((max-min)/cell) + 1,
//    1e8-cell cap (:232-260).  One 40-byte device-to-host read per build
//    (the reference does 12 allocations and 12 synchronous copies).
//  * cell id = clamp(floor((p - min) / cell)) with IEEE division, linear
//    x + y*gx + z*gx*gy (:29-50); the effective cell size is
//    max(cell_size, cutoff) (:382).
//  * the reference's atomics-based count/scan/scatter (:53-81,292-308) is a
//    stable radix sort of (cell id, particle index): same cell_start /
//    cell_end, and within a cell ascending particle index (the reference's
//    within-cell order is whatever its atomics produced).
//  * positions+masses are gathered into cell order (float4), so the force
//    kernel streams contiguous memory per neighbour cell.
//  * force: targets in cell order; 27 neighbours dz, dy, dx; skip j == i;
//    accept d^2 < rc^2 on the unsoftened distance, then add
//    m_j d (d^2 + eps^2)^-3/2; scaled by G at the end (:84-158).  d^2 is
//    fma(dz,dz, fma(dy,dy, dx*dx)) with _rn intrinsics, the contraction nvcc
//    gives the reference's source, so neighbour counts match the oracle
//    bit-exactly.
#include <cmath>

#include "common.cuh"
#include "geom.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "sort.cuh"

namespace nbgb {

struct HashState {
  DevBuf<float> bbox_part;
  DevBuf<BBox> box;
  HostPinned<BBox> h_box;
  DevBuf<uint32_t> keys, keys_alt, vals, vals_alt;
  DevBuf<uint32_t> hist, scan_ws;
  DevBuf<int32_t> particle_cell;
  DevBuf<uint32_t> cell_start;  // total_cells + 1
  DevBuf<float4> sorted_pm;
  // last build
  int64_t n = 0;
  int dims[3] = {0, 0, 0};
  float bmin[3] = {0, 0, 0};
  float cell = 0.f;
  int64_t total = 0;
  bool in_alt = false;
  bool built = false;  // the last build finished (the inspection calls read its buffers)
  const uint32_t* sorted_cells() const { return in_alt ? keys_alt.ptr : keys.ptr; }
  const uint32_t* sorted_idx() const { return in_alt ? vals_alt.ptr : vals.ptr; }
};

void hash_state_delete(HashState* p) { delete p; }

struct GridArgs {
  float bmin[3];
  float cell;
  int dims[3];
};

__global__ void hash_assign_kernel(const float4* __restrict__ pm, int64_t n, GridArgs g,
                                   int32_t* __restrict__ particle_cell,
                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = pm[i];
    int cx = (int)floorf(__fdiv_rn(__fsub_rn(p.x, g.bmin[0]), g.cell));
    int cy = (int)floorf(__fdiv_rn(__fsub_rn(p.y, g.bmin[1]), g.cell));
    int cz = (int)floorf(__fdiv_rn(__fsub_rn(p.z, g.bmin[2]), g.cell));
    cx = max(0, min(cx, g.dims[0] - 1));
    cy = max(0, min(cy, g.dims[1] - 1));
    cz = max(0, min(cz, g.dims[2] - 1));
    int32_t id = cx + cy * g.dims[0] + cz * g.dims[0] * g.dims[1];
    particle_cell[i] = id;
    keys[i] = (uint32_t)id;
    vals[i] = (uint32_t)i;
  }
}

// start[c] = number of particles with cell < c (lower bound in the sorted
// cell ids), c in [0, total]; end[c] = start[c + 1].
__global__ void hash_cell_start_kernel(const uint32_t* __restrict__ sorted_cells, int64_t n,
                                       int64_t total, uint32_t* __restrict__ start) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c <= total;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((int64_t)sorted_cells[mid] < c)
        lo = mid + 1;
      else
        hi = mid;
    }
    start[c] = (uint32_t)lo;
  }
}

__global__ void hash_gather_kernel(const float4* __restrict__ pm, const uint32_t* __restrict__ idx,
                                   int64_t n, float4* __restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = pm[idx[k]];
}

template <bool COUNT>
__global__ void __launch_bounds__(256) hash_force_kernel(
    const float4* __restrict__ spm, const uint32_t* __restrict__ sorted_cells,
    const uint32_t* __restrict__ sorted_idx, const uint32_t* __restrict__ start, int64_t n,
    GridArgs g, float cut2, float eps2, float G, float* __restrict__ ax, float* __restrict__ ay,
    float* __restrict__ az, int32_t* __restrict__ counts) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const float4 pi = spm[k];
    const int id = (int)sorted_cells[k];
    const int gxy = g.dims[0] * g.dims[1];
    const int cz = id / gxy;
    const int rem = id - cz * gxy;
    const int cy = rem / g.dims[0];
    const int cx = rem - cy * g.dims[0];
    float sx = 0.f, sy = 0.f, sz = 0.f;
    int cnt = 0;
    for (int oz = -1; oz <= 1; ++oz) {
      const int nz = cz + oz;
      if (nz < 0 || nz >= g.dims[2]) continue;
      for (int oy = -1; oy <= 1; ++oy) {
        const int ny = cy + oy;
        if (ny < 0 || ny >= g.dims[1]) continue;
        {
          // cells cx-1 .. cx+1 of this row are consecutive in the sorted
          // array: one range, in the reference's cell order
          const int row = ny * g.dims[0] + nz * gxy;
          const uint32_t s = start[row + max(cx - 1, 0)];
          const uint32_t e = start[row + min(cx + 1, g.dims[0] - 1) + 1];
          for (uint32_t j = s; j < e; ++j) {
            if ((int64_t)j == k) continue;
            const float4 pj = spm[j];
            const float dx = __fsub_rn(pj.x, pi.x);
            const float dy = __fsub_rn(pj.y, pi.y);
            const float dz = __fsub_rn(pj.z, pi.z);
            float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
            if (d2 < cut2) {
              d2 = __fadd_rn(d2, eps2);
              const float r = rsqrt_approx(d2);
              const float f = (pj.w * r) * (r * r);
              sx = fmaf(f, dx, sx);
              sy = fmaf(f, dy, sy);
              sz = fmaf(f, dz, sz);
              if (COUNT) ++cnt;
            }
          }
        }
      }
    }
    const uint32_t i = sorted_idx[k];
    ax[i] = G * sx;
    ay[i] = G * sy;
    az[i] = G * sz;
    if (COUNT) counts[i] = cnt;
  }
}

static unsigned grid1d(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), threads), (int64_t)num_sms() * 32));
}

void hash_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay,
                 float* az) {
  if (!c->hash) c->hash.reset(new HashState());
  HashState& h = *c->hash;
  h.built = false;
  StageTimer* timer = stage_timer(c);
  stage_mark(timer, "spatial_hash.bounds");
  cudaStream_t st = c->stream;
  uint32_t* err = c->err.ensure(1);
  // 1. bounding box -> host (sizes the grid)
  float* part = h.bbox_part.ensure((size_t)bbox_blocks(n) * 6);
  BBox* box = h.box.ensure(1);
  launch_bbox(pm, n, part, box, err, st);
  BBox* hb = h.h_box.ensure(1);
  NBGB_CUDA(cudaMemcpyAsync(hb, box, sizeof(BBox), cudaMemcpyDeviceToHost, st));
  NBGB_CUDA(cudaStreamSynchronize(st));
  if (!hb->valid) fail(NBGB_ERR_INVALID_ARG, "Validation Error: non-finite particle position");
  const float cell = std::max(c->params.cell_size, c->params.cutoff);
  GridArgs g;
  int64_t total = 1;
  for (int a = 0; a < 3; ++a) {
    volatile float lo = hb->min[a] - 0.001f;  // force float rounding of each step
    volatile float hi = hb->max[a] + 0.001f;
    float ext = hi - lo;
    volatile float q = ext / cell;
    g.bmin[a] = lo;
    g.dims[a] = (int)std::ceil((float)q) + 1;
    total *= (int64_t)g.dims[a];
  }
  g.cell = cell;
  if (total > 100000000)
    fail(NBGB_ERR_OVERFLOW, "Spatial hash grid too large: reduce cell_size or bounding box");
  h.n = n;
  h.total = total;
  h.cell = cell;
  for (int a = 0; a < 3; ++a) {
    h.dims[a] = g.dims[a];
    h.bmin[a] = g.bmin[a];
  }
  // 2. assign cells
  stage_mark(timer, "spatial_hash.assign");
  int32_t* pc = h.particle_cell.ensure((size_t)n);
  uint32_t* keys = h.keys.ensure((size_t)n);
  uint32_t* vals = h.vals.ensure((size_t)n);
  uint32_t* keys_alt = h.keys_alt.ensure((size_t)n);
  uint32_t* vals_alt = h.vals_alt.ensure((size_t)n);
  hash_assign_kernel<<<grid1d(n), 256, 0, st>>>(pm, n, g, pc, keys, vals);
  NBGB_LAUNCH_CHECK();
  // 3. stable sort by cell id
  stage_mark(timer, "spatial_hash.sort");
  int bits = 1;
  while (bits < 32 && ((int64_t)1 << bits) < total) ++bits;
  const int end_bit = ((bits + 7) / 8) * 8;
  uint32_t* hist = h.hist.ensure(radix_hist_elems(n));
  uint32_t* sws = h.scan_ws.ensure(scan_workspace_elems((int64_t)radix_hist_elems(n)) +
                                   scan_workspace_elems(total + 1));
  radix_sort_pairs<uint32_t>(keys, keys_alt, vals, vals_alt, n, 0, end_bit, hist, sws, st,
                             &h.in_alt, c->err.ensure(1));
  // 4. cell starts
  stage_mark(timer, "spatial_hash.cells");
  uint32_t* start = h.cell_start.ensure((size_t)total + 1);
  hash_cell_start_kernel<<<grid1d(total + 1), 256, 0, st>>>(h.sorted_cells(), n, total, start);
  NBGB_LAUNCH_CHECK();
  // 5. payload in cell order
  float4* spm = h.sorted_pm.ensure((size_t)n);
  hash_gather_kernel<<<grid1d(n), 256, 0, st>>>(pm, h.sorted_idx(), n, spm);
  NBGB_LAUNCH_CHECK();
  // 6. cutoff gather
  stage_mark(timer, "spatial_hash.forces");
  const float eps = c->params.softening, rc = c->params.cutoff;
  const bool count = (c->params.flags & NBGB_FLAG_COUNT_INTERACTIONS) != 0;
  int32_t* counts = count ? c->counts.ensure((size_t)n) : nullptr;
  if (count)
    hash_force_kernel<true><<<grid1d(n), 256, 0, st>>>(spm, h.sorted_cells(), h.sorted_idx(),
                                                         start, n, g, rc * rc, eps * eps,
                                                         c->params.G, ax, ay, az, counts);
  else
    hash_force_kernel<false><<<grid1d(n), 256, 0, st>>>(spm, h.sorted_cells(), h.sorted_idx(),
                                                          start, n, g, rc * rc, eps * eps,
                                                          c->params.G, ax, ay, az, counts);
  NBGB_LAUNCH_CHECK();
  h.built = true;
}

}  // namespace nbgb

using namespace nbgb;

extern "C" {

nbgb_status nbgb_hash_grid_info(nbgb_calculator* c, int32_t dims[3], float bbox_min[3],
                                float* cell_size, int64_t* total_cells) {
  if (!c || !c->hash || c->method != NBGB_SPATIAL_HASH || !c->hash->built)
    return NBGB_ERR_INVALID_ARG;
  const HashState& h = *c->hash;
  for (int a = 0; a < 3; ++a) {
    if (dims) dims[a] = h.dims[a];
    if (bbox_min) bbox_min[a] = h.bmin[a];
  }
  if (cell_size) *cell_size = h.cell;
  if (total_cells) *total_cells = h.total;
  return NBGB_OK;
}

nbgb_status nbgb_hash_copy_cells(nbgb_calculator* c, int32_t* cell_start, int32_t* cell_end,
                                 int32_t* particle_cells, int32_t* sorted_indices) {
  if (!c || !c->hash || c->method != NBGB_SPATIAL_HASH || !c->hash->built)
    return NBGB_ERR_INVALID_ARG;
  HashState& h = *c->hash;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return NBGB_ERR_CUDA;
  const size_t tot = (size_t)h.total, n = (size_t)h.n;
  cudaError_t e = cudaSuccess;
  if (cell_start && e == cudaSuccess)
    e = cudaMemcpy(cell_start, h.cell_start.ptr, tot * 4, cudaMemcpyDeviceToHost);
  if (cell_end && e == cudaSuccess)
    e = cudaMemcpy(cell_end, h.cell_start.ptr + 1, tot * 4, cudaMemcpyDeviceToHost);
  if (particle_cells && e == cudaSuccess)
    e = cudaMemcpy(particle_cells, h.particle_cell.ptr, n * 4, cudaMemcpyDeviceToHost);
  if (sorted_indices && e == cudaSuccess)
    e = cudaMemcpy(sorted_indices, h.sorted_idx(), n * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

}  // extern "C"
