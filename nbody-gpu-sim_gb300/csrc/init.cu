// init.cu -- initial conditions generated on the device.
//
// The reference generates its initial states on the host with std::mt19937
// (ParticleInitializer::initUniform / initSpherical / initDisk,
// src/cuda/particle_init.cu:167-234) and copies them up.  Here every body is
// drawn independently by one thread from a counter-based generator, so an
// N = 10^8 state is produced in HBM in milliseconds and the same seed gives
// the same state bit for bit on any launch shape.  The distributions follow
// the reference's formulas (uniform box; uniform ball r = cbrt(u) R with
// isotropic directions; disk r = sqrt(u) R, |z| <= thickness/2, v =
// rotation_speed sqrt(r) tangential) plus a Plummer sphere (radius from the
// cumulative mass profile, speeds by von Neumann rejection against the
// distribution function, centred on zero momentum).  The random streams are
// not the reference's: for the reference's exact host states use its own
// initialiser (as nbgb_sim does).
//
// Generator: body i, draw k -> the SplitMix64 output function (Steele, Lea,
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014, with
// Stafford's "Mix13" finaliser constants) applied to seed + golden ratio *
// (16 i + k + 1); top 24 bits -> float in [0, 1), top 53 bits -> double.
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t seed, uint64_t i, uint32_t k) {
  return mix64(seed + 0x9e3779b97f4a7c15ull * (16ull * i + k + 1ull));
}
__device__ __forceinline__ float u01f(uint64_t seed, uint64_t i, uint32_t k) {
  return (float)(draw(seed, i, k) >> 40) * 5.9604644775390625e-08f;  // 2^-24
}
__device__ __forceinline__ double u01d(uint64_t seed, uint64_t i, uint32_t k) {
  return (double)(draw(seed, i, k) >> 11) * 1.1102230246251565e-16;  // 2^-53
}

struct InitArgs {
  nbgb_particle_data d;
  nbgb_init_params p;
  uint64_t seed;
};

__global__ void init_kernel(InitArgs a) {
  const int64_t n = (int64_t)a.d.count;
  const nbgb_init_params& p = a.p;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z, vx = 0.f, vy = 0.f, vz = 0.f, m;
    const float mass_u = u01f(a.seed, i, 15);
    m = p.min_mass + (p.max_mass - p.min_mass) * mass_u;
    if (p.distribution == NBGB_DIST_UNIFORM) {
      x = p.min_bounds[0] + (p.max_bounds[0] - p.min_bounds[0]) * u01f(a.seed, i, 0);
      y = p.min_bounds[1] + (p.max_bounds[1] - p.min_bounds[1]) * u01f(a.seed, i, 1);
      z = p.min_bounds[2] + (p.max_bounds[2] - p.min_bounds[2]) * u01f(a.seed, i, 2);
    } else if (p.distribution == NBGB_DIST_SPHERICAL) {
      const float r = cbrtf(u01f(a.seed, i, 0)) * p.radius;
      const float th = u01f(a.seed, i, 1) * 2.0f * 3.14159265f;
      const float ph = acosf(2.0f * u01f(a.seed, i, 2) - 1.0f);
      x = p.center[0] + r * sinf(ph) * cosf(th);
      y = p.center[1] + r * sinf(ph) * sinf(th);
      z = p.center[2] + r * cosf(ph);
    } else if (p.distribution == NBGB_DIST_DISK) {
      const float r = sqrtf(u01f(a.seed, i, 0)) * p.radius;
      const float th = u01f(a.seed, i, 1) * 2.0f * 3.14159265f;
      x = p.center[0] + r * cosf(th);
      y = p.center[1] + r * sinf(th);
      z = p.center[2] + (u01f(a.seed, i, 2) - 0.5f) * p.thickness;
      const float v = p.rotation_speed * sqrtf(r);
      vx = -v * sinf(th);
      vy = v * cosf(th);
    } else {  // Plummer sphere, FP64 sampling
      const double A = p.plummer_a, M = p.total_mass, G = p.G;
      double u = u01d(a.seed, i, 0);
      if (u <= 0.0) u = 1.1102230246251565e-16;
      const double r = A / sqrt(pow(u, -2.0 / 3.0) - 1.0);
      const double ct = 2.0 * u01d(a.seed, i, 1) - 1.0, st = sqrt(fmax(0.0, 1.0 - ct * ct));
      const double ph = 2.0 * 3.141592653589793 * u01d(a.seed, i, 2);
      x = (float)(r * st * cos(ph));
      y = (float)(r * st * sin(ph));
      z = (float)(r * ct);
      // speed fraction q with density q^2 (1 - q^2)^3.5 (bounded rejection)
      // (acceptance ~0.5 per attempt: 64 attempts fail with probability 1e-19)
      double q = 0.0;
      for (uint32_t t = 0; t < 64; ++t) {
        const uint64_t s2 = a.seed + 0xa0761d6478bd642full * t;  // attempt t's stream
        const double x1 = u01d(s2, i, 6), x2 = 0.1 * u01d(s2, i, 7);
        q = x1;
        if (x2 < x1 * x1 * pow(1.0 - x1 * x1, 3.5)) break;
      }
      const double vesc = sqrt(2.0 * G * M) * pow(r * r + A * A, -0.25);
      const double cv = 2.0 * u01d(a.seed, i, 3) - 1.0, sv = sqrt(fmax(0.0, 1.0 - cv * cv));
      const double pv = 2.0 * 3.141592653589793 * u01d(a.seed, i, 4);
      vx = (float)(q * vesc * sv * cos(pv));
      vy = (float)(q * vesc * sv * sin(pv));
      vz = (float)(q * vesc * cv);
      m = (float)(M / (double)n);
    }
    a.d.pos_x[i] = x;
    a.d.pos_y[i] = y;
    a.d.pos_z[i] = z;
    a.d.vel_x[i] = vx;
    a.d.vel_y[i] = vy;
    a.d.vel_z[i] = vz;
    a.d.mass[i] = m;
    if (a.d.acc_x) a.d.acc_x[i] = 0.f;
    if (a.d.acc_y) a.d.acc_y[i] = 0.f;
    if (a.d.acc_z) a.d.acc_z[i] = 0.f;
    if (a.d.acc_old_x) a.d.acc_old_x[i] = 0.f;
    if (a.d.acc_old_y) a.d.acc_old_y[i] = 0.f;
    if (a.d.acc_old_z) a.d.acc_old_z[i] = 0.f;
  }
}

// Plummer: mass-weighted mean position and velocity, per-block partials in
// FP64 and one fixed-order final sum (deterministic), then the shift.
constexpr int kInitThreads = 256;

__global__ void moment_partial_kernel(nbgb_particle_data d, double* __restrict__ part) {
  const int64_t n = (int64_t)d.count;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double m = d.mass[i];
    v[0] += m * d.pos_x[i];
    v[1] += m * d.pos_y[i];
    v[2] += m * d.pos_z[i];
    v[3] += m * d.vel_x[i];
    v[4] += m * d.vel_y[i];
    v[5] += m * d.vel_z[i];
    v[6] += m;
  }
  __shared__ double s[7][kInitThreads];
  for (int c = 0; c < 7; ++c) s[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int w = kInitThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 7; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 7; ++c) part[blockIdx.x * 7 + c] = s[c][0];
}

// one block: partials summed in a fixed order -> mean position, velocity
__global__ void moment_final_kernel(const double* __restrict__ part, int nblocks,
                                    double* __restrict__ mean) {
  __shared__ double s[7][kInitThreads];
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
    for (int c = 0; c < 7; ++c) v[c] += part[b * 7 + c];
  for (int c = 0; c < 7; ++c) s[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int w = kInitThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 7; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 6; ++c) mean[c] = s[6][0] > 0.0 ? s[c][0] / s[6][0] : 0.0;
}

__global__ void shift_kernel(nbgb_particle_data d, const double* __restrict__ mean) {
  const double m0 = mean[0], m1 = mean[1], m2 = mean[2], m3 = mean[3], m4 = mean[4], m5 = mean[5];
  const int64_t n = (int64_t)d.count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    d.pos_x[i] = (float)((double)d.pos_x[i] - m0);
    d.pos_y[i] = (float)((double)d.pos_y[i] - m1);
    d.pos_z[i] = (float)((double)d.pos_z[i] - m2);
    d.vel_x[i] = (float)((double)d.vel_x[i] - m3);
    d.vel_y[i] = (float)((double)d.vel_y[i] - m4);
    d.vel_z[i] = (float)((double)d.vel_z[i] - m5);
  }
}

__global__ void offset_kernel(nbgb_particle_data d, float cx, float cy, float cz) {
  const int64_t n = (int64_t)d.count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    d.pos_x[i] += cx;
    d.pos_y[i] += cy;
    d.pos_z[i] += cz;
  }
}

}  // namespace nbgb

using namespace nbgb;

extern "C" {

void nbgb_init_params_default(nbgb_init_params* p, int32_t distribution) {
  if (!p) return;
  *p = nbgb_init_params{};
  p->distribution = distribution;
  // ParticleSystem::initialize's parameters (src/core/particle_system.cpp:77-101)
  for (int a = 0; a < 3; ++a) {
    p->center[a] = 0.0f;
    p->min_bounds[a] = -10.0f;
    p->max_bounds[a] = 10.0f;
  }
  p->radius = 10.0f;
  p->min_mass = 1.0f;
  p->max_mass = 1.0f;
  p->thickness = 1.0f;
  p->rotation_speed = 0.5f;
  p->plummer_a = 1.0f;
  p->total_mass = 1.0f;
  p->G = 1.0f;
}

nbgb_status nbgb_init_particles_device(nbgb_particle_data* d, const nbgb_init_params* p,
                                       uint64_t seed, void* stream) {
  try {
    if (!d || !p) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    if (d->count == 0) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count must be greater than 0");
    if (!d->pos_x || !d->pos_y || !d->pos_z || !d->vel_x || !d->vel_y || !d->vel_z || !d->mass)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null device array");
    if (p->distribution < NBGB_DIST_UNIFORM || p->distribution > NBGB_DIST_PLUMMER)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: unknown initial distribution");
    if (p->min_mass > p->max_mass || !(p->min_mass >= 0.0f))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: mass range must satisfy 0 <= min <= max");
    if (p->distribution == NBGB_DIST_PLUMMER &&
        !(p->plummer_a > 0.0f && p->total_mass > 0.0f && p->G > 0.0f))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Plummer scale, mass and G must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(NBGB_ERR_NO_DEVICE, "CUDA Error: no CUDA device available");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = (int64_t)d->count;
    const unsigned blocks = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>(ceil_div(n, kInitThreads), (int64_t)num_sms() * 16));
    InitArgs a{*d, *p, seed};
    init_kernel<<<blocks, kInitThreads, 0, st>>>(a);
    NBGB_LAUNCH_CHECK();
    if (p->distribution == NBGB_DIST_PLUMMER) {
      double* part = nullptr;
      NBGB_CUDA(cudaMallocAsync(&part, ((size_t)blocks * 7 + 8) * sizeof(double), st));
      double* mean = part + (size_t)blocks * 7;
      moment_partial_kernel<<<blocks, kInitThreads, 0, st>>>(*d, part);
      NBGB_LAUNCH_CHECK();
      moment_final_kernel<<<1, kInitThreads, 0, st>>>(part, (int)blocks, mean);
      NBGB_LAUNCH_CHECK();
      shift_kernel<<<blocks, kInitThreads, 0, st>>>(*d, mean);
      NBGB_LAUNCH_CHECK();
      NBGB_CUDA(cudaFreeAsync(part, st));
      if (p->center[0] != 0.0f || p->center[1] != 0.0f || p->center[2] != 0.0f) {
        offset_kernel<<<blocks, kInitThreads, 0, st>>>(*d, p->center[0], p->center[1], p->center[2]);
        NBGB_LAUNCH_CHECK();
      }
    }
    NBGB_CUDA(cudaStreamSynchronize(st));
    return NBGB_OK;
  } catch (const Error& e) {
    return set_error(e.status, e.what());
  }
}

}  // extern "C"
