// mirror.cu -- FP64 position/velocity state behind the reference's FP32
// ParticleData, for ParticleSystem::update through the drop-in adapter.
//
// The reference integrates in FP32 (src/cuda/integrator.cu:175-189:
// a_old = a; x += v dt + a dt^2/2; a = F(x); v += (a_old + a) dt/2).  The
// precision rules of this library keep x and v in FP64 across steps and only
// the pairwise force arithmetic in FP32.  A mirror holds x, v in FP64 for one
// ParticleData (keyed by its pos_x device pointer); every step
//   kick-drift:  a_old = a (the reference's storeOldAccelerations);
//                v' = v + a dt/2 and x' = x + v' dt in FP64; pos = (float) x'
//   forces:      the caller's calculator on the FP32 positions
//   kick:        v'' = v' + a_new dt/2 in FP64; vel = (float) v''
// which equals the reference's update algebraically, and the FP32 SoA is
// the rounded FP64 state after every step (what ParticleSystem::getState
// and copyToHost read).  An element whose FP32 value no longer equals its
// rounded FP64 value was changed by the caller (reset, initialisation,
// checkpoint load): the mirror takes the FP32 value again.
#include <memory>
#include <mutex>
#include <unordered_map>

#include "common.cuh"
#include "runtime.cuh"

namespace nbgb {

struct Mirror {
  DevBuf<double> x, y, z, vx, vy, vz;
  int64_t n = 0;
  bool seeded = false;
};

static std::mutex g_mirror_mu;
static std::unordered_map<const float*, std::unique_ptr<Mirror>> g_mirrors;

static Mirror& mirror_of(const nbgb_particle_data& d) {
  std::lock_guard<std::mutex> lk(g_mirror_mu);
  auto& m = g_mirrors[d.pos_x];
  if (!m) m = std::make_unique<Mirror>();
  const int64_t n = (int64_t)d.count;
  if (m->n != n) {
    m->x.ensure((size_t)n);
    m->y.ensure((size_t)n);
    m->z.ensure((size_t)n);
    m->vx.ensure((size_t)n);
    m->vy.ensure((size_t)n);
    m->vz.ensure((size_t)n);
    m->n = n;
    m->seeded = false;
  }
  return *m;
}

// The FP64 value, or the FP32 one where the caller changed it.
__device__ __forceinline__ double synced(double m, float f, bool seeded) {
  return (seeded && (float)m == f) ? m : (double)f;
}

__global__ void mirror_kick_drift_kernel(nbgb_particle_data d, double* __restrict__ x,
                                         double* __restrict__ y, double* __restrict__ z,
                                         double* __restrict__ vx, double* __restrict__ vy,
                                         double* __restrict__ vz, double kick, double dt,
                                         bool seeded) {
  const int64_t n = (int64_t)d.count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float fx = d.pos_x[i], fy = d.pos_y[i], fz = d.pos_z[i];
    const float fvx = d.vel_x[i], fvy = d.vel_y[i], fvz = d.vel_z[i];
    const float ax = d.acc_x[i], ay = d.acc_y[i], az = d.acc_z[i];
    const double X = synced(x[i], fx, seeded), Y = synced(y[i], fy, seeded),
                 Z = synced(z[i], fz, seeded);
    const double U = fma((double)ax, kick, synced(vx[i], fvx, seeded));
    const double V = fma((double)ay, kick, synced(vy[i], fvy, seeded));
    const double W = fma((double)az, kick, synced(vz[i], fvz, seeded));
    const double px = fma(U, dt, X), py = fma(V, dt, Y), pz = fma(W, dt, Z);
    d.acc_old_x[i] = ax;
    d.acc_old_y[i] = ay;
    d.acc_old_z[i] = az;
    x[i] = px;
    y[i] = py;
    z[i] = pz;
    vx[i] = U;
    vy[i] = V;
    vz[i] = W;
    d.pos_x[i] = (float)px;
    d.pos_y[i] = (float)py;
    d.pos_z[i] = (float)pz;
  }
}

__global__ void mirror_kick_kernel(nbgb_particle_data d, double* __restrict__ vx,
                                   double* __restrict__ vy, double* __restrict__ vz,
                                   double kick) {
  const int64_t n = (int64_t)d.count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double U = fma((double)d.acc_x[i], kick, vx[i]);
    const double V = fma((double)d.acc_y[i], kick, vy[i]);
    const double W = fma((double)d.acc_z[i], kick, vz[i]);
    vx[i] = U;
    vy[i] = V;
    vz[i] = W;
    d.vel_x[i] = (float)U;
    d.vel_y[i] = (float)V;
    d.vel_z[i] = (float)W;
  }
}

static unsigned mirror_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), 256), (int64_t)num_sms() * 16));
}

static void check_state(const nbgb_particle_data* d, float dt) {
  if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
  if (!(dt > 0.f) || !std::isfinite(dt))
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Time step must be positive and finite");
  if (d->count == 0) return;
  if (!d->pos_x || !d->pos_y || !d->pos_z || !d->vel_x || !d->vel_y || !d->vel_z ||
      !d->acc_x || !d->acc_y || !d->acc_z || !d->acc_old_x || !d->acc_old_y || !d->acc_old_z)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: null position, velocity or acceleration array");
}

template <typename F>
static nbgb_status mirror_guarded(F&& f) {
  try {
    f();
    return set_error(NBGB_OK, std::string());
  } catch (const Error& e) {
    return set_error(e.status, e.what());
  } catch (const std::bad_alloc&) {
    return set_error(NBGB_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return set_error(NBGB_ERR_CUDA, e.what());
  }
}

}  // namespace nbgb

using namespace nbgb;

extern "C" {

nbgb_status nbgb_state_kick_drift(const nbgb_particle_data* d, float dt, void* stream) {
  return mirror_guarded([&] {
    check_state(d, dt);
    if (d->count == 0) return;
    Mirror& m = mirror_of(*d);
    const double h = 0.5 * (double)dt;
    mirror_kick_drift_kernel<<<mirror_grid(m.n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        *d, m.x.ptr, m.y.ptr, m.z.ptr, m.vx.ptr, m.vy.ptr, m.vz.ptr, h, (double)dt, m.seeded);
    NBGB_LAUNCH_CHECK();
    m.seeded = true;
  });
}

nbgb_status nbgb_state_kick(const nbgb_particle_data* d, float dt, void* stream) {
  return mirror_guarded([&] {
    check_state(d, dt);
    if (d->count == 0) return;
    Mirror& m = mirror_of(*d);
    if (!m.seeded) fail(NBGB_ERR_INVALID_ARG, "Validation Error: kick before kick-drift");
    mirror_kick_kernel<<<mirror_grid(m.n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        *d, m.vx.ptr, m.vy.ptr, m.vz.ptr, 0.5 * (double)dt);
    NBGB_LAUNCH_CHECK();
  });
}

nbgb_status nbgb_state_release(const nbgb_particle_data* d) {
  return mirror_guarded([&] {
    if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
    std::unique_ptr<Mirror> m;
    {
      std::lock_guard<std::mutex> lk(g_mirror_mu);
      auto it = g_mirrors.find(d->pos_x);
      if (it == g_mirrors.end()) return;
      m = std::move(it->second);
      g_mirrors.erase(it);
    }
    // device work on the mirror must finish before its memory is freed
    NBGB_CUDA(cudaDeviceSynchronize());
  });
}

}  // extern "C"
