// direct.cu -- tiled direct-N^2 gravity (K1), packing, energies.
//
// Replaces computeForcesDirectKernel / launchDirectForceKernel
// (src/cuda/force_direct.cu:10-98).  Law: a_i = G * sum_{j != i} m_j d
// (d^2 + eps^2)^-3/2 with d = x_j - x_i.
//
// Layout: sources are a packed float4 array (x, y, z, m), padded with zero
// mass up to a multiple of the j-tile, so the inner loop has no bounds test
// and no self test: with eps > 0 the j == i term is exactly 0 (d = 0).
// j-tiles of kTile bodies are staged into shared memory by the bulk-copy
// engine (cp.async.bulk + mbarrier, kStages deep) and read as broadcast
// 16-byte shared loads.  Each thread owns I targets in registers.
//
// Accumulation: per target, each j-tile is summed in plain FP32 and folded
// into a running (sum, error) pair with an error-free two-sum (compensated
// per j-tile).  COMP = false gives the plain single-accumulator FP32 sum.
#include "common.cuh"
#include "kernels.cuh"
#include "direct_core.cuh"

namespace nbgb {

// ---------------------------------------------------------------------------
// Packing: SoA (pos_x, pos_y, pos_z, mass) -> float4 (x, y, z, m), zero pad.
// ---------------------------------------------------------------------------
__global__ void pack_soa_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                const float* __restrict__ z, const float* __restrict__ m,
                                int64_t n, int64_t n_pad, float4* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    out[i] = (i < n) ? make_float4(x[i], y[i], z[i], m[i]) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

void launch_pack_soa(const float* x, const float* y, const float* z, const float* m, int64_t n,
                     int64_t n_pad, float4* out, cudaStream_t st) {
  if (n_pad <= 0) return;
  int threads = 256;
  int64_t blocks = std::min<int64_t>(ceil_div(n_pad, threads), (int64_t)num_sms() * 8);
  pack_soa_kernel<<<(unsigned)blocks, threads, 0, st>>>(x, y, z, m, n, n_pad, out);
  NBGB_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// The direct kernel: CTA (blockIdx.x) owns kDirThreads*I targets, split
// (blockIdx.y) owns a contiguous run of j-tiles.
// ---------------------------------------------------------------------------
template <int I, bool PAIRED, bool COMP, bool ZERO_SOFT>
__global__ void __launch_bounds__(kDirThreads) direct_kernel(DirectArgs a) {
  static_assert(!PAIRED || (I % 2 == 0), "paired path needs an even target count");
  __shared__ alignas(128) float4 s_j[kDirStages][kDirTile];
  __shared__ alignas(8) uint64_t s_bar[kDirStages];
  TileRing ring{s_j, s_bar, 0};
  ring_init(ring);

  const int tid = threadIdx.x;
  const int64_t tgt_base = (int64_t)blockIdx.x * (kDirThreads * I);
  const int split = blockIdx.y;
  const int64_t tile0 = (int64_t)split * a.tiles_per_split;
  const int64_t tile1 = imin64(tile0 + a.tiles_per_split, a.n_tiles);
  const int nt = (int)imax64(tile1 - tile0, 0);

  // Targets: thread tid owns tgt_base + tid + q*kDirThreads (coalesced I/O).
  float xi[I], yi[I], zi[I];
#pragma unroll
  for (int q = 0; q < I; ++q) {
    int64_t i = tgt_base + tid + (int64_t)q * kDirThreads;
    float4 p = (i < a.n_tgt) ? a.tgt[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    xi[q] = p.x;
    yi[q] = p.y;
    zi[q] = p.z;
  }
  float sx[I], sy[I], sz[I];
  if (!direct_tiles<kDirThreads, I, PAIRED, COMP, ZERO_SOFT>(ring, a.src + tile0 * kDirTile, nt,
                                                             xi, yi, zi, a.eps2, sx, sy, sz,
                                                             a.err))
    return;
  const float G = a.G;
#pragma unroll
  for (int q = 0; q < I; ++q) {
    int64_t i = tgt_base + tid + (int64_t)q * kDirThreads;
    if (i >= a.n_tgt) continue;
    if (a.partial) {
      a.partial[(int64_t)split * a.n_tgt_pad + i] = make_float4(sx[q], sy[q], sz[q], 0.f);
    } else {
      a.out_x[i] = G * sx[q];
      a.out_y[i] = G * sy[q];
      a.out_z[i] = G * sz[q];
    }
  }
}

// Sum the j-split partials in split order (deterministic), then scale by G.
__global__ void direct_reduce_kernel(const float4* __restrict__ partial, int splits,
                                     int64_t n_tgt, int64_t n_tgt_pad, float G,
                                     float* __restrict__ ox, float* __restrict__ oy,
                                     float* __restrict__ oz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_tgt;
       i += (int64_t)gridDim.x * blockDim.x) {
    float sx = 0.f, sy = 0.f, sz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f, e;
    for (int s = 0; s < splits; ++s) {
      float4 p = partial[(int64_t)s * n_tgt_pad + i];
      sx = two_sum(sx, p.x, e);
      ex += e;
      sy = two_sum(sy, p.y, e);
      ey += e;
      sz = two_sum(sz, p.z, e);
      ez += e;
    }
    ox[i] = G * (sx + ex);
    oy[i] = G * (sy + ey);
    oz[i] = G * (sz + ez);
  }
}

template <int I, bool PAIRED, bool COMP, bool ZS>
static void launch_one(const DirectArgs& a, dim3 grid, cudaStream_t st) {
  direct_kernel<I, PAIRED, COMP, ZS><<<grid, kDirThreads, 0, st>>>(a);
  NBGB_LAUNCH_CHECK();
}

template <int I, bool PAIRED>
static int occupancy_of() {
  int blocks = 0;
  NBGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &blocks, direct_kernel<I, PAIRED, true, false>, kDirThreads, 0));
  return blocks > 0 ? blocks : 1;
}

DirectPlan plan_direct(int64_t n_src, int64_t n_tgt, DirectVariant v) {
  DirectPlan p;
  p.variant = v;
  p.targets_per_cta = kDirThreads * direct_targets_per_thread(v);
  p.n_tiles = ceil_div(std::max<int64_t>(n_src, 1), kDirTile);
  p.n_src_pad = p.n_tiles * kDirTile;
  p.i_blocks = ceil_div(std::max<int64_t>(n_tgt, 1), p.targets_per_cta);
  p.n_tgt_pad = p.i_blocks * p.targets_per_cta;
  int occ = (v == DirectVariant::kPaired8) ? occupancy_of<8, true>() : occupancy_of<4, false>();
  int64_t slots = (int64_t)num_sms() * occ;
  // Choose the j-split so that i_blocks * splits fills whole waves of the
  // resident CTA slots (every CTA does the same work), with >= 4 tiles each.
  int64_t max_split = std::max<int64_t>(1, std::min<int64_t>(p.n_tiles / 4, 128));
  int best = 1;
  double best_eff = -1.0;
  for (int64_t s = 1; s <= max_split; ++s) {
    int64_t items = p.i_blocks * s;
    double waves = (double)items / (double)slots;
    double eff = waves / std::ceil(waves);
    // Prefer fewer splits unless the efficiency gain is material.
    if (eff > best_eff + 0.02) {
      best_eff = eff;
      best = (int)s;
    }
    if (eff >= 0.97) break;
  }
  p.splits = best;
  p.tiles_per_split = ceil_div(p.n_tiles, p.splits);
  p.splits = (int)ceil_div(p.n_tiles, p.tiles_per_split);
  return p;
}

int direct_targets_per_thread(DirectVariant v) {
  return v == DirectVariant::kPaired8 ? 8 : 4;
}

void launch_direct(const DirectPlan& p, const float4* src, const float4* tgt, int64_t n_tgt,
                   float G, float eps2, bool compensated, float4* partial, float* ox, float* oy,
                   float* oz, uint32_t* err, cudaStream_t st) {
  if (n_tgt <= 0) return;
  DirectArgs a;
  a.src = src;
  a.tgt = tgt;
  a.n_tgt = n_tgt;
  a.n_tgt_pad = p.n_tgt_pad;
  a.n_tiles = p.n_tiles;
  a.tiles_per_split = p.tiles_per_split;
  a.eps2 = eps2;
  a.G = G;
  a.partial = (p.splits > 1) ? partial : nullptr;
  a.out_x = ox;
  a.out_y = oy;
  a.out_z = oz;
  a.err = err;
  dim3 grid((unsigned)p.i_blocks, (unsigned)p.splits);
  const bool zs = !(eps2 > 0.f);
  if (p.variant == DirectVariant::kPaired8) {
    if (zs) {
      compensated ? launch_one<8, true, true, true>(a, grid, st)
                  : launch_one<8, true, false, true>(a, grid, st);
    } else {
      compensated ? launch_one<8, true, true, false>(a, grid, st)
                  : launch_one<8, true, false, false>(a, grid, st);
    }
  } else {
    if (zs) {
      compensated ? launch_one<4, false, true, true>(a, grid, st)
                  : launch_one<4, false, false, true>(a, grid, st);
    } else {
      compensated ? launch_one<4, false, true, false>(a, grid, st)
                  : launch_one<4, false, false, false>(a, grid, st);
    }
  }
  if (p.splits > 1) {
    int threads = 256;
    int64_t blocks = std::min<int64_t>(ceil_div(n_tgt, threads), (int64_t)num_sms() * 8);
    direct_reduce_kernel<<<(unsigned)blocks, threads, 0, st>>>(partial, p.splits, n_tgt,
                                                               p.n_tgt_pad, G, ox, oy, oz);
    NBGB_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// Energies (FP64 reductions).
// ---------------------------------------------------------------------------

// Deterministic two-level reduction of per-thread doubles: block sums go to
// `partials`, a single block then adds them in order.
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* partials) {
  __shared__ double s_red[32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) s_red[warp][k] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = (lane < nw) ? s_red[lane][k] : 0.0;
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) partials[(int64_t)blockIdx.x * NV + k] = t;
    }
  }
}

template <int NV>
__global__ void finish_reduce_kernel(const double* __restrict__ partials, int nblocks,
                                     double* __restrict__ out) {
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += partials[(int64_t)b * NV + k];
  __shared__ double s[NV][256];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k][threadIdx.x] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int j = 0; j < (int)blockDim.x; ++j) t += s[k][j];
      out[k] = t;
    }
  }
}

// KE (and optionally momentum) from FP32 SoA velocities.
__global__ void ke_f32_kernel(const float* __restrict__ vx, const float* __restrict__ vy,
                              const float* __restrict__ vz, const float* __restrict__ m,
                              int64_t n, double* partials) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double a = vx[i], b = vy[i], c = vz[i], mm = m[i];
    v[0] += 0.5 * mm * (a * a + b * b + c * c);
    v[1] += mm * a;
    v[2] += mm * b;
    v[3] += mm * c;
  }
  block_reduce_store<4>(v, partials);
}

// KE and momentum from FP64 velocities.
__global__ void ke_f64_kernel(const double* __restrict__ vx, const double* __restrict__ vy,
                              const double* __restrict__ vz, const float4* __restrict__ pm,
                              int64_t n, double* partials) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double a = vx[i], b = vy[i], c = vz[i], mm = pm[i].w;
    v[0] += 0.5 * mm * (a * a + b * b + c * c);
    v[1] += mm * a;
    v[2] += mm * b;
    v[3] += mm * c;
  }
  block_reduce_store<4>(v, partials);
}

// Potential: phi_i = -sum_{j != i} m_j / sqrt(d^2 + eps^2), FP32 pairs with
// one Newton step on the MUFU rsqrt (near-correctly-rounded), compensated
// per 256-body chunk; PE = G/2 sum_i m_i phi_i accumulated in FP64.
__global__ void pe_kernel(const float4* __restrict__ src, int64_t n, float eps2,
                          double* partials) {
  __shared__ float4 s_j[256];
  double acc[1] = {0.0};
  const int64_t n_chunks = ceil_div(n, 256);
  for (int64_t ib = blockIdx.x; ib * 256 < n; ib += gridDim.x) {
    int64_t i = ib * 256 + threadIdx.x;
    float4 pi = (i < n) ? src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float s = 0.f, e = 0.f;
    for (int64_t c = 0; c < n_chunks; ++c) {
      __syncthreads();
      int64_t j = c * 256 + threadIdx.x;
      s_j[threadIdx.x] = (j < n) ? src[j] : make_float4(0.f, 0.f, 0.f, 0.f);
      __syncthreads();
      float t = 0.f;
      const int lim = (int)imin64(256, n - c * 256);
      for (int k = 0; k < lim; ++k) {
        float4 pj = s_j[k];
        float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        float d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        float r = rsqrt_approx(d2);
        r = r * fmaf(-0.5f * d2, r * r, 1.5f);
        bool self = (c * 256 + k) == i;
        t = self ? t : fmaf(-pj.w, r, t);
      }
      float err;
      s = two_sum(s, t, err);
      e += err;
    }
    if (i < n) acc[0] += 0.5 * (double)pi.w * ((double)s + (double)e);
  }
  block_reduce_store<1>(acc, partials);
}

void launch_kinetic_f32(const float* vx, const float* vy, const float* vz, const float* m,
                        int64_t n, double* partials, int nblocks, double* out, cudaStream_t st) {
  ke_f32_kernel<<<nblocks, 256, 0, st>>>(vx, vy, vz, m, n, partials);
  NBGB_LAUNCH_CHECK();
  finish_reduce_kernel<4><<<1, 256, 0, st>>>(partials, nblocks, out);
  NBGB_LAUNCH_CHECK();
}

void launch_kinetic_f64(const double* vx, const double* vy, const double* vz, const float4* pm,
                        int64_t n, double* partials, int nblocks, double* out, cudaStream_t st) {
  ke_f64_kernel<<<nblocks, 256, 0, st>>>(vx, vy, vz, pm, n, partials);
  NBGB_LAUNCH_CHECK();
  finish_reduce_kernel<4><<<1, 256, 0, st>>>(partials, nblocks, out);
  NBGB_LAUNCH_CHECK();
}

void launch_potential(const float4* src, int64_t n, float eps2, double* partials, int nblocks,
                      double* out, cudaStream_t st) {
  pe_kernel<<<nblocks, 256, 0, st>>>(src, n, eps2, partials);
  NBGB_LAUNCH_CHECK();
  finish_reduce_kernel<1><<<1, 256, 0, st>>>(partials, nblocks, out);
  NBGB_LAUNCH_CHECK();
}

// ----------------------------------------------- FP64-state kernels --
// Forces and potential from FP64 positions in FP64 arithmetic: the
// full-FP64 system variant and the energy of every FP64-state system.
// 256-body tiles of (x, y, z, m) in shared memory, one target per thread,
// self excluded by index, rsqrt from the CUDA math library.
__global__ void __launch_bounds__(256) direct_f64_state_kernel(
    const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
    const float4* __restrict__ pm, int64_t n, double G, double eps2, double* __restrict__ ax,
    double* __restrict__ ay, double* __restrict__ az) {
  __shared__ double4 s_j[256];
  for (int64_t base = (int64_t)blockIdx.x * 256; base < n; base += (int64_t)gridDim.x * 256) {
    const int64_t i = base + threadIdx.x;
    const bool valid = i < n;
    const double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0, zi = valid ? z[i] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t c = 0; c < n; c += 256) {
      __syncthreads();
      const int64_t j = c + threadIdx.x;
      s_j[threadIdx.x] = (j < n) ? make_double4(x[j], y[j], z[j], (double)pm[j].w)
                                 : make_double4(0.0, 0.0, 0.0, 0.0);
      __syncthreads();
      const int lim = (int)imin64(256, n - c);
      for (int k = 0; k < lim; ++k) {
        if (c + k == i) continue;
        const double4 q = s_j[k];
        const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
        const double d2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
        const double r = rsqrt(d2);
        const double f = q.w * r * r * r;
        sx = fma(f, dx, sx);
        sy = fma(f, dy, sy);
        sz = fma(f, dz, sz);
      }
    }
    if (valid) {
      ax[i] = G * sx;
      ay[i] = G * sy;
      az[i] = G * sz;
    }
  }
}

__global__ void __launch_bounds__(256) pe_f64_kernel(const double* __restrict__ x,
                                                     const double* __restrict__ y,
                                                     const double* __restrict__ z,
                                                     const float4* __restrict__ pm, int64_t n,
                                                     double eps2, double* partials) {
  __shared__ double4 s_j[256];
  double acc[1] = {0.0};
  for (int64_t base = (int64_t)blockIdx.x * 256; base < n; base += (int64_t)gridDim.x * 256) {
    const int64_t i = base + threadIdx.x;
    const bool valid = i < n;
    const double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0, zi = valid ? z[i] : 0.0;
    double s = 0.0;
    for (int64_t c = 0; c < n; c += 256) {
      __syncthreads();
      const int64_t j = c + threadIdx.x;
      s_j[threadIdx.x] = (j < n) ? make_double4(x[j], y[j], z[j], (double)pm[j].w)
                                 : make_double4(0.0, 0.0, 0.0, 0.0);
      __syncthreads();
      const int lim = (int)imin64(256, n - c);
      for (int k = 0; k < lim; ++k) {
        if (c + k == i) continue;
        const double4 q = s_j[k];
        const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
        s -= q.w * rsqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2))));
      }
    }
    if (valid) acc[0] += 0.5 * (double)pm[i].w * s;
  }
  block_reduce_store<1>(acc, partials);
}

void launch_direct_f64_state(const double* x, const double* y, const double* z, const float4* pm,
                             int64_t n, double G, double eps2, double* ax, double* ay, double* az,
                             cudaStream_t st) {
  if (n <= 0) return;
  const unsigned blocks =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)num_sms() * 8));
  direct_f64_state_kernel<<<blocks, 256, 0, st>>>(x, y, z, pm, n, G, eps2, ax, ay, az);
  NBGB_LAUNCH_CHECK();
}

void launch_potential_f64(const double* x, const double* y, const double* z, const float4* pm,
                          int64_t n, double eps2, double* partials, int nblocks, double* out,
                          cudaStream_t st) {
  pe_f64_kernel<<<nblocks, 256, 0, st>>>(x, y, z, pm, n, eps2, partials);
  NBGB_LAUNCH_CHECK();
  finish_reduce_kernel<1><<<1, 256, 0, st>>>(partials, nblocks, out);
  NBGB_LAUNCH_CHECK();
}

}  // namespace nbgb

// ---------------------------------------------------------------------------
// FP64 direct sum (the full-FP64 variant; accuracy reference on the GPU).
// ---------------------------------------------------------------------------
namespace nbgb {

__global__ void direct_f64_kernel(const float4* __restrict__ src, int64_t n_src,
                                  const int64_t* __restrict__ targets, int64_t n_tgt, double G,
                                  double eps2, double* __restrict__ ax, double* __restrict__ ay,
                                  double* __restrict__ az) {
  __shared__ float4 s_j[256];
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n_tgt;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    const bool valid = t < n_tgt;
    const int64_t i = valid ? (targets ? targets[t] : t) : 0;
    const float4 pi = src[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t c = 0; c < n_src; c += 256) {
      __syncthreads();
      const int64_t j = c + threadIdx.x;
      s_j[threadIdx.x] = (j < n_src) ? src[j] : make_float4(0.f, 0.f, 0.f, 0.f);
      __syncthreads();
      const int lim = (int)imin64(256, n_src - c);
      for (int k = 0; k < lim; ++k) {
        if (c + k == i) continue;
        const float4 pj = s_j[k];
        const double dx = (double)pj.x - (double)pi.x, dy = (double)pj.y - (double)pi.y,
                     dz = (double)pj.z - (double)pi.z;
        const double d2 = dx * dx + dy * dy + dz * dz + eps2;
        const double inv = 1.0 / sqrt(d2);
        const double f = (double)pj.w * inv * inv * inv;
        sx += f * dx;
        sy += f * dy;
        sz += f * dz;
      }
    }
    if (valid) {
      ax[t] = G * sx;
      ay[t] = G * sy;
      az[t] = G * sz;
    }
  }
}

}  // namespace nbgb

extern "C" nbgb_status nbgb_direct_f64(const float* d_src_xyzm, int64_t n_src,
                                       const int64_t* d_targets, int64_t n_targets, double G,
                                       double eps, double* d_ax, double* d_ay, double* d_az,
                                       void* stream) {
  using namespace nbgb;
  try {
    if (!d_src_xyzm || !d_ax || !d_ay || !d_az || n_src < 0 || n_targets < 0)
      return NBGB_ERR_INVALID_ARG;
    if (n_targets == 0) return NBGB_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t blocks = std::min<int64_t>(ceil_div(n_targets, 256), (int64_t)num_sms() * 8);
    direct_f64_kernel<<<(unsigned)blocks, 256, 0, st>>>(
        reinterpret_cast<const float4*>(d_src_xyzm), n_src, d_targets, n_targets, G, eps * eps,
        d_ax, d_ay, d_az);
    NBGB_LAUNCH_CHECK();
    return NBGB_OK;
  } catch (const Error& e) {
    return e.status;
  }
}
