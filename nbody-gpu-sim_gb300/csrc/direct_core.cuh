// direct_core.cuh -- the direct-sum tile engine shared by the one-system
// kernel (direct.cu) and the ensemble work-queue kernel (ensemble.cu).
//
// One CTA of THREADS threads computes THREADS*I targets against a run of
// kDirTile-body j-tiles that the bulk-copy engine streams into a kDirStages
// ring of shared-memory buffers (cp.async.bulk + mbarrier).  The ring state
// (barrier phases) lives across calls, so a persistent CTA can process many
// work items without re-initialising barriers.
#pragma once

#include "common.cuh"
#include "kernels.cuh"

namespace nbgb {

struct TileRing {
  float4 (*buf)[kDirTile];  // [kDirStages][kDirTile] in shared memory
  uint64_t* bar;            // [kDirStages] mbarriers, count 1
  uint32_t consumed;        // tiles consumed so far by this CTA (phase tracking)
};

__device__ __forceinline__ void ring_init(TileRing& r) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kDirStages; ++s) mbar_init(&r.bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  r.consumed = 0;
}

// Sums, for I targets per thread, the contributions of tiles [0, nt) of
// `src` (each kDirTile float4 (x,y,z,m), zero-mass padded).  Returns false
// if a bounded wait ran out (the error word is set; all threads agree).
template <int THREADS, int I, bool PAIRED, bool COMP, bool ZERO_SOFT>
__device__ __forceinline__ bool direct_tiles(TileRing& ring, const float4* __restrict__ src, int nt,
                                             const float (&xi)[I], const float (&yi)[I],
                                             const float (&zi)[I], float eps2, float (&sx)[I],
                                             float (&sy)[I], float (&sz)[I], uint32_t* err) {
  constexpr uint32_t kBytes = kDirTile * sizeof(float4);
  const int tid = threadIdx.x;
  const uint32_t c0 = ring.consumed;
  if (tid == 0) {
    for (int j = 0; j < kDirStages && j < nt; ++j) {
      const int s = (int)((c0 + j) % kDirStages);
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&ring.bar[s], kBytes);
      bulk_g2s(ring.buf[s], src + (int64_t)j * kDirTile, kBytes, &ring.bar[s]);
    }
  }
  float ex[I], ey[I], ez[I];
#pragma unroll
  for (int q = 0; q < I; ++q) {
    sx[q] = sy[q] = sz[q] = 0.f;
    ex[q] = ey[q] = ez[q] = 0.f;
  }
  bool bad = false;
  int t = 0;
  for (; t < nt; ++t) {
    const uint32_t c = c0 + (uint32_t)t;
    const int s = (int)(c % kDirStages);
    const uint32_t parity = (c / kDirStages) & 1u;
    if (!bad && !mbar_wait(&ring.bar[s], parity, err)) bad = true;
    if (!bad) {
      const float4* __restrict__ tile = ring.buf[s];
      float tx[I], ty[I], tz[I];
#pragma unroll
      for (int q = 0; q < I; ++q) tx[q] = ty[q] = tz[q] = 0.f;
      if constexpr (PAIRED) {
        constexpr int P = I / 2;
        f2 xp[P], yp[P], zp[P], ax2[P], ay2[P], az2[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          xp[p] = f2_make(xi[2 * p], xi[2 * p + 1]);
          yp[p] = f2_make(yi[2 * p], yi[2 * p + 1]);
          zp[p] = f2_make(zi[2 * p], zi[2 * p + 1]);
          ax2[p] = ay2[p] = az2[p] = f2_make(0.f, 0.f);
        }
        const f2 e2 = f2_make(eps2, eps2);
#pragma unroll 32
        for (int k = 0; k < kDirTile; ++k) {
          const float4 pj = tile[k];
          const f2 xj = f2_make(pj.x, pj.x), yj = f2_make(pj.y, pj.y), zj = f2_make(pj.z, pj.z);
          const f2 mj = f2_make(pj.w, pj.w);
#pragma unroll
          for (int p = 0; p < P; ++p) {
            f2 dx = f2_sub(xj, xp[p]);
            f2 dy = f2_sub(yj, yp[p]);
            f2 dz = f2_sub(zj, zp[p]);
            f2 d2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, e2)));
            float d2l, d2h;
            f2_split(d2, d2l, d2h);
            float rl = rsqrt_approx(d2l), rh = rsqrt_approx(d2h);
            if constexpr (ZERO_SOFT) {
              rl = (d2l > 0.f) ? rl : 0.f;
              rh = (d2h > 0.f) ? rh : 0.f;
            }
            f2 r = f2_make(rl, rh);
            f2 f = f2_mul(f2_mul(mj, r), f2_mul(r, r));
            ax2[p] = f2_fma(f, dx, ax2[p]);
            ay2[p] = f2_fma(f, dy, ay2[p]);
            az2[p] = f2_fma(f, dz, az2[p]);
          }
        }
#pragma unroll
        for (int p = 0; p < P; ++p) {
          f2_split(ax2[p], tx[2 * p], tx[2 * p + 1]);
          f2_split(ay2[p], ty[2 * p], ty[2 * p + 1]);
          f2_split(az2[p], tz[2 * p], tz[2 * p + 1]);
        }
      } else {
#pragma unroll 4
        for (int k = 0; k < kDirTile; ++k) {
          const float4 pj = tile[k];
#pragma unroll
          for (int q = 0; q < I; ++q) {
            float dx = pj.x - xi[q];
            float dy = pj.y - yi[q];
            float dz = pj.z - zi[q];
            float d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
            float r = rsqrt_approx(d2);
            if constexpr (ZERO_SOFT) r = (d2 > 0.f) ? r : 0.f;
            float f = (pj.w * r) * (r * r);
            tx[q] = fmaf(f, dx, tx[q]);
            ty[q] = fmaf(f, dy, ty[q]);
            tz[q] = fmaf(f, dz, tz[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < I; ++q) {
        if constexpr (COMP) {
          float e;
          sx[q] = two_sum(sx[q], tx[q], e);
          ex[q] += e;
          sy[q] = two_sum(sy[q], ty[q], e);
          ey[q] += e;
          sz[q] = two_sum(sz[q], tz[q], e);
          ez[q] += e;
        } else {
          sx[q] += tx[q];
          sy[q] += ty[q];
          sz[q] += tz[q];
        }
      }
    }
    if (__syncthreads_or(bad)) {
      bad = true;
      break;
    }
    if (tid == 0 && t + kDirStages < nt) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&ring.bar[s], kBytes);
      bulk_g2s(ring.buf[s], src + (int64_t)(t + kDirStages) * kDirTile, kBytes, &ring.bar[s]);
    }
  }
  if (bad) {
    // drain (bounded) the copies still in flight on every stage
    if (tid == 0) {
      for (int j = t; j < nt && j < t + kDirStages; ++j) {
        const uint32_t c = c0 + (uint32_t)j;
        mbar_wait(&ring.bar[c % kDirStages], (c / kDirStages) & 1u, nullptr, 1u << 16);
      }
    }
    return false;
  }
  ring.consumed = c0 + (uint32_t)nt;
  if constexpr (COMP) {
#pragma unroll
    for (int q = 0; q < I; ++q) {
      sx[q] += ex[q];
      sy[q] += ey[q];
      sz[q] += ez[q];
    }
  }
  return true;
}

}  // namespace nbgb
