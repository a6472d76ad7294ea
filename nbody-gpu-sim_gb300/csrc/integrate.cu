// integrate.cu -- Velocity Verlet kernels (K8).
//
// Two families:
//  * FP32 SoA kernels with the reference's semantics (src/cuda/integrator.cu:
//    updatePositionsKernel :12-22, updateVelocitiesKernel :25-37,
//    storeAccelerationsKernel :40-49).  storeOld + updatePositions are fused
//    into one pass that can also emit the packed (x, y, z, m) force input.
//  * FP64-state kick-drift-kick for the device-resident system path: x, v in
//    FP64, FP32 accelerations, FP32 packed positions for the force kernels.
//    KDK with a full kick between steps equals the reference's
//    x += v dt + a dt^2/2; v += (a_old + a_new) dt/2 algebraically.
#include "common.cuh"
#include "kernels.cuh"

namespace nbgb {

// The FP32 kernels take the reference's SoA struct, whose arrays the compiler
// must assume may alias: each one issues all of a body's loads before its
// first store, so the loads of the three components are in flight together
// (with a load-store-load order per component the velocity update ran at
// 72 % of the copy bandwidth instead of 96 %).  The arithmetic expressions are
// the reference's.

static inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), threads), (int64_t)num_sms() * 16);
  return (unsigned)std::max<int64_t>(b, 1);
}

__global__ void vv_positions_kernel(nbgb_particle_data d, float dt, bool store_old, float4* pack,
                                    int64_t n_pad) {
  const int64_t n = (int64_t)d.count;
  const float dt2_half = 0.5f * dt * dt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n) {
      const float ax = d.acc_x[i], ay = d.acc_y[i], az = d.acc_z[i];
      const float px = d.pos_x[i], py = d.pos_y[i], pz = d.pos_z[i];
      const float vx = d.vel_x[i], vy = d.vel_y[i], vz = d.vel_z[i];
      const float m = pack ? d.mass[i] : 0.f;
      if (store_old) {
        d.acc_old_x[i] = ax;
        d.acc_old_y[i] = ay;
        d.acc_old_z[i] = az;
      }
      const float x = px + fmaf(vx, dt, ax * dt2_half);
      const float y = py + fmaf(vy, dt, ay * dt2_half);
      const float z = pz + fmaf(vz, dt, az * dt2_half);
      d.pos_x[i] = x;
      d.pos_y[i] = y;
      d.pos_z[i] = z;
      if (pack) pack[i] = make_float4(x, y, z, m);
    } else if (pack) {
      pack[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

__global__ void vv_velocities_kernel(nbgb_particle_data d, float dt) {
  const int64_t n = (int64_t)d.count;
  const float dt_half = 0.5f * dt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float vx = d.vel_x[i], vy = d.vel_y[i], vz = d.vel_z[i];
    const float ox = d.acc_old_x[i], oy = d.acc_old_y[i], oz = d.acc_old_z[i];
    const float ax = d.acc_x[i], ay = d.acc_y[i], az = d.acc_z[i];
    d.vel_x[i] = vx + (ox + ax) * dt_half;
    d.vel_y[i] = vy + (oy + ay) * dt_half;
    d.vel_z[i] = vz + (oz + az) * dt_half;
  }
}

__global__ void store_old_kernel(nbgb_particle_data d) {
  const int64_t n = (int64_t)d.count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ax = d.acc_x[i], ay = d.acc_y[i], az = d.acc_z[i];
    d.acc_old_x[i] = ax;
    d.acc_old_y[i] = ay;
    d.acc_old_z[i] = az;
  }
}

void launch_vv_positions(const nbgb_particle_data& d, float dt, bool store_old, float4* pack,
                         int64_t n_pad, cudaStream_t st) {
  int64_t lim = pack ? std::max<int64_t>(n_pad, (int64_t)d.count) : (int64_t)d.count;
  if (lim <= 0) return;
  vv_positions_kernel<<<grid_for(lim, 256), 256, 0, st>>>(d, dt, store_old, pack, lim);
  NBGB_LAUNCH_CHECK();
}

void launch_vv_velocities(const nbgb_particle_data& d, float dt, cudaStream_t st) {
  if (d.count == 0) return;
  vv_velocities_kernel<<<grid_for((int64_t)d.count, 256), 256, 0, st>>>(d, dt);
  NBGB_LAUNCH_CHECK();
}

void launch_store_old(const nbgb_particle_data& d, cudaStream_t st) {
  if (d.count == 0) return;
  store_old_kernel<<<grid_for((int64_t)d.count, 256), 256, 0, st>>>(d);
  NBGB_LAUNCH_CHECK();
}

template <typename A>
__global__ void kick_drift_kernel(int64_t n, double* __restrict__ x, double* __restrict__ y,
                                  double* __restrict__ z, double* __restrict__ vx,
                                  double* __restrict__ vy, double* __restrict__ vz,
                                  const A* __restrict__ ax, const A* __restrict__ ay,
                                  const A* __restrict__ az, double kick, double dt,
                                  float4* __restrict__ pm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double u = fma((double)ax[i], kick, vx[i]);
    double v = fma((double)ay[i], kick, vy[i]);
    double w = fma((double)az[i], kick, vz[i]);
    double px = fma(u, dt, x[i]);
    double py = fma(v, dt, y[i]);
    double pz = fma(w, dt, z[i]);
    vx[i] = u;
    vy[i] = v;
    vz[i] = w;
    x[i] = px;
    y[i] = py;
    z[i] = pz;
    float4 o = pm[i];
    o.x = (float)px;
    o.y = (float)py;
    o.z = (float)pz;
    pm[i] = o;
  }
}

template <typename A>
__global__ void kick_kernel(int64_t n, double* __restrict__ vx, double* __restrict__ vy,
                            double* __restrict__ vz, const A* __restrict__ ax,
                            const A* __restrict__ ay, const A* __restrict__ az, double kick) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    vx[i] = fma((double)ax[i], kick, vx[i]);
    vy[i] = fma((double)ay[i], kick, vy[i]);
    vz[i] = fma((double)az[i], kick, vz[i]);
  }
}

template <typename A>
static void kick_drift_any(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                           double* vz, const A* ax, const A* ay, const A* az, double kick,
                           double dt, float4* pm, cudaStream_t st) {
  if (n <= 0) return;
  kick_drift_kernel<A><<<grid_for(n, 256), 256, 0, st>>>(n, x, y, z, vx, vy, vz, ax, ay, az, kick,
                                                         dt, pm);
  NBGB_LAUNCH_CHECK();
}

template <typename A>
static void kick_any(int64_t n, double* vx, double* vy, double* vz, const A* ax, const A* ay,
                     const A* az, double kick, cudaStream_t st) {
  if (n <= 0) return;
  kick_kernel<A><<<grid_for(n, 256), 256, 0, st>>>(n, vx, vy, vz, ax, ay, az, kick);
  NBGB_LAUNCH_CHECK();
}

void launch_kick_drift(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                       double* vz, const float* ax, const float* ay, const float* az,
                       double kick, double dt, float4* pm, cudaStream_t st) {
  kick_drift_any(n, x, y, z, vx, vy, vz, ax, ay, az, kick, dt, pm, st);
}
void launch_kick_drift(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                       double* vz, const double* ax, const double* ay, const double* az,
                       double kick, double dt, float4* pm, cudaStream_t st) {
  kick_drift_any(n, x, y, z, vx, vy, vz, ax, ay, az, kick, dt, pm, st);
}
void launch_kick(int64_t n, double* vx, double* vy, double* vz, const float* ax, const float* ay,
                 const float* az, double kick, cudaStream_t st) {
  kick_any(n, vx, vy, vz, ax, ay, az, kick, st);
}
void launch_kick(int64_t n, double* vx, double* vy, double* vz, const double* ax,
                 const double* ay, const double* az, double kick, cudaStream_t st) {
  kick_any(n, vx, vy, vz, ax, ay, az, kick, st);
}

}  // namespace nbgb
