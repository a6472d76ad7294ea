// kernels.cuh -- launcher declarations shared by the nbgb translation units.
#pragma once

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace nbgb {

// ----------------------------------------------------------------- direct --
constexpr int kDirThreads = 128;  // threads per CTA of the direct kernel
constexpr int kDirTile = 256;     // bodies per shared-memory j-tile (4 KB)
constexpr int kDirStages = 3;     // bulk-copy pipeline depth

enum class DirectVariant : int {
  kScalar4 = 0,  // 4 targets/thread, scalar FP32 (12 FP32 ops + 1 MUFU per pair)
  kPaired8 = 1,  // 8 targets/thread, packed f32x2 arithmetic
};

struct DirectArgs {
  const float4* src;  // padded sources (x, y, z, m)
  const float4* tgt;  // targets (x, y, z, .)
  int64_t n_tgt;
  int64_t n_tgt_pad;
  int64_t n_tiles;
  int64_t tiles_per_split;
  float eps2;
  float G;
  float4* partial;  // [splits][n_tgt_pad] when splits > 1, else null
  float* out_x;
  float* out_y;
  float* out_z;
  uint32_t* err;
};

struct DirectPlan {
  DirectVariant variant = DirectVariant::kScalar4;
  int targets_per_cta = 0;
  int64_t n_tiles = 0;
  int64_t n_src_pad = 0;  // sources must be padded (zero mass) to this length
  int64_t i_blocks = 0;
  int64_t n_tgt_pad = 0;
  int splits = 1;
  int64_t tiles_per_split = 0;
  size_t partial_bytes() const { return splits > 1 ? (size_t)splits * n_tgt_pad * 16 : 0; }
};

int direct_targets_per_thread(DirectVariant v);
DirectPlan plan_direct(int64_t n_src, int64_t n_tgt, DirectVariant v);
void launch_direct(const DirectPlan& p, const float4* src, const float4* tgt, int64_t n_tgt,
                   float G, float eps2, bool compensated, float4* partial, float* ox, float* oy,
                   float* oz, uint32_t* err, cudaStream_t st);
void launch_pack_soa(const float* x, const float* y, const float* z, const float* m, int64_t n,
                     int64_t n_pad, float4* out, cudaStream_t st);

// Energies: `partials` needs nblocks * 4 doubles; out[0..3] = KE, Px, Py, Pz
// (kinetic) or out[0] = sum_i m_i phi_i / 2 without G (potential).
void launch_kinetic_f32(const float* vx, const float* vy, const float* vz, const float* m,
                        int64_t n, double* partials, int nblocks, double* out, cudaStream_t st);
void launch_kinetic_f64(const double* vx, const double* vy, const double* vz, const float4* pm,
                        int64_t n, double* partials, int nblocks, double* out, cudaStream_t st);
void launch_potential(const float4* src, int64_t n, float eps2, double* partials, int nblocks,
                      double* out, cudaStream_t st);

// ------------------------------------------------------------- integrator --
// FP32 SoA Velocity Verlet (reference semantics).
void launch_vv_positions(const nbgb_particle_data& d, float dt, bool store_old, float4* pack,
                         int64_t n_pad, cudaStream_t st);
void launch_vv_velocities(const nbgb_particle_data& d, float dt, cudaStream_t st);
void launch_store_old(const nbgb_particle_data& d, cudaStream_t st);

// FP64-state kick-drift: v += a*kick; x += v*dt; pack (float)x into pm.xyz.
void launch_kick_drift(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                       double* vz, const float* ax, const float* ay, const float* az,
                       double kick, double dt, float4* pm, cudaStream_t st);
// FP64-state kick: v += a*kick.
void launch_kick(int64_t n, double* vx, double* vy, double* vz, const float* ax,
                 const float* ay, const float* az, double kick, cudaStream_t st);
// The same with FP64 accelerations (full-FP64 system).
void launch_kick_drift(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                       double* vz, const double* ax, const double* ay, const double* az,
                       double kick, double dt, float4* pm, cudaStream_t st);
void launch_kick(int64_t n, double* vx, double* vy, double* vz, const double* ax,
                 const double* ay, const double* az, double kick, cudaStream_t st);
// Direct forces and potential energy in FP64 from FP64 positions (masses
// from pm.w).
void launch_direct_f64_state(const double* x, const double* y, const double* z, const float4* pm,
                             int64_t n, double G, double eps2, double* ax, double* ay, double* az,
                             cudaStream_t st);
void launch_potential_f64(const double* x, const double* y, const double* z, const float4* pm,
                          int64_t n, double eps2, double* partials, int nblocks, double* out,
                          cudaStream_t st);

}  // namespace nbgb
