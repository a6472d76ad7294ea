// api.cu -- the C ABI (include/nbgb.h): calculators, integrator, particle
// memory, device-resident FP64 systems.  No exception crosses extern "C".
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {

static thread_local std::string g_last_error;

nbgb_status set_error(nbgb_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

template <typename F>
static nbgb_status guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return NBGB_OK;
  } catch (const Error& e) {
    return set_error(e.status, e.what());
  } catch (const std::bad_alloc&) {
    return set_error(NBGB_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return set_error(NBGB_ERR_CUDA, e.what());
  }
}

int num_sms() {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  NBGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cache[dev]) {
    int v = 0;
    NBGB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    cache[dev] = v > 0 ? v : 1;
  }
  return cache[dev];
}

// Parameter validation mirrors the reference's checks
// (src/utils/error_handling.cpp:47-138) for the fields a calculator uses.
static void validate_params(nbgb_method m, const nbgb_params& p) {
  auto finite = [](float v) { return std::isfinite(v); };
  if (!(finite(p.G) && p.G > 0.f))
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Gravitational constant must be positive and finite");
  if (!finite(p.softening))
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Softening parameter must be a finite number");
  if (p.softening < 0.f)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Softening parameter must be positive");
  if (m == NBGB_BARNES_HUT) {
    if (!finite(p.theta))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Barnes-Hut theta must be a finite number");
    if (p.theta < 0.f || p.theta > 2.0f)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Barnes-Hut theta must be between 0 and 2");
    if (p.leaf_capacity < 1 || p.leaf_capacity > 16)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: leaf capacity must be between 1 and 16");
    if (p.group_size != 0 && p.group_size != 32 && p.group_size != 64)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: group size must be 0, 32 or 64");
    if ((p.flags & NBGB_FLAG_REFERENCE_TREE) &&
        ((p.flags & NBGB_FLAG_GROUP_WALK) || p.leaf_capacity != 1))
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: the reference tree is walked with the reference walk only "
           "(no group walk, leaf capacity 1)");
  }
  if (m == NBGB_SPATIAL_HASH) {
    if (!(finite(p.cell_size) && p.cell_size > 0.f))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Spatial hash cell size must be positive and finite");
    if (!(finite(p.cutoff) && p.cutoff > 0.f))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Spatial hash cutoff must be positive and finite");
  }
  if (p.block_size <= 0 || p.block_size > 1024)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: CUDA block size must be between 1 and 1024");
}

int64_t direct_pad(int64_t n) { return ceil_div(std::max<int64_t>(n, 1), kDirTile) * kDirTile; }

void check_device_errors(nbgb_calculator* c) {
  uint32_t* h = c->h_err.ensure(1);
  uint32_t* d = c->err.ensure(1);
  NBGB_CUDA(cudaMemcpyAsync(h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  NBGB_CUDA(cudaStreamSynchronize(c->stream));
  uint32_t bits = *h;
  if (bits) {
    NBGB_CUDA(cudaMemsetAsync(d, 0, sizeof(uint32_t), c->stream));
    NBGB_CUDA(cudaStreamSynchronize(c->stream));
    std::string msg = "device error word 0x" + std::to_string(bits) + ":";
    nbgb_status s = NBGB_ERR_CUDA;
    if (bits & kErrWaitTimeout) {
      msg += " bounded wait timed out;";
      s = NBGB_ERR_DEVICE_TIMEOUT;
    }
    if (bits & kErrTreeCapacity) {
      msg += " octree capacity exceeded;";
      s = NBGB_ERR_OVERFLOW;
    }
    if (bits & kErrGridCapacity) {
      msg += " spatial hash grid capacity exceeded;";
      s = NBGB_ERR_OVERFLOW;
    }
    if (bits & kErrQueueOverflow) {
      msg += " work queue overflow;";
      s = NBGB_ERR_OVERFLOW;
    }
    if (bits & kErrBadInput) {
      msg += " non-finite input;";
      s = NBGB_ERR_INVALID_ARG;
    }
    if (bits & kErrWalkStack) {
      msg += " Barnes-Hut group walk stack overflow;";
      s = NBGB_ERR_OVERFLOW;
    }
    fail(s, msg);
  }
}

static void direct_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay,
                          float* az) {
  DirectPlan p = plan_direct(n, n, c->variant);
  float4* part = nullptr;
  if (p.splits > 1) part = c->partial.ensure((size_t)p.splits * p.n_tgt_pad);
  const float eps = c->params.softening;
  launch_direct(p, pm, pm, n, c->params.G, eps * eps,
                (c->params.flags & NBGB_FLAG_COMPENSATED) != 0, part, ax, ay, az,
                c->err.ensure(1), c->stream);
}

void forces_packed(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay,
                   float* az) {
  if (n <= 0) return;
  StageTimer* t = stage_timer(c);
  if (t) t->st = c->stream;
  switch (c->method) {
    case NBGB_DIRECT_N2:
      stage_mark(t, "direct.forces");
      direct_forces(c, pm, n, ax, ay, az);
      break;
    case NBGB_BARNES_HUT:
      bh_forces(c, pm, n, ax, ay, az);
      break;
    case NBGB_SPATIAL_HASH:
      hash_forces(c, pm, n, ax, ay, az);
      break;
  }
  if (t) t->end();
}

// ------------------------------------------------------- stage timings --
StageTimer::~StageTimer() {
  for (auto& m : marks) cudaEventDestroy(m.ev);
  for (auto e : spare) cudaEventDestroy(e);
}

int StageTimer::id_of(const char* name) {
  for (size_t i = 0; i < names.size(); ++i)
    if (names[i] == name) return (int)i;
  names.emplace_back(name);
  total_ms.push_back(0.0);
  samples.push_back(0);
  return (int)names.size() - 1;
}

cudaEvent_t StageTimer::record(int stage) {
  cudaEvent_t ev = nullptr;
  if (!spare.empty()) {
    ev = spare.back();
    spare.pop_back();
  } else {
    NBGB_CUDA(cudaEventCreate(&ev));
  }
  marks.push_back(Mark{stage, ev});
  NBGB_CUDA(cudaEventRecord(ev, st));
  return ev;
}

void StageTimer::mark(const char* stage) {
  if (marks.size() > 4096) harvest();  // bounds the events held between queries
  record(id_of(stage));
}

void StageTimer::end() {
  if (!marks.empty() && marks.back().stage >= 0) record(-1);
}

void StageTimer::harvest() {
  if (marks.empty()) return;
  NBGB_CUDA(cudaEventSynchronize(marks.back().ev));
  const size_t last = marks.size() - 1;
  for (size_t i = 0; i < last; ++i) {
    if (marks[i].stage < 0) continue;
    float ms = 0.f;
    NBGB_CUDA(cudaEventElapsedTime(&ms, marks[i].ev, marks[i + 1].ev));
    total_ms[(size_t)marks[i].stage] += ms;
    samples[(size_t)marks[i].stage] += 1;
  }
  // a stage that began at the last mark is still open: keep that mark
  const bool open = marks[last].stage >= 0;
  for (size_t i = 0; i < (open ? last : last + 1); ++i) spare.push_back(marks[i].ev);
  if (open) {
    const Mark keep = marks[last];
    marks.assign(1, keep);
  } else {
    marks.clear();
  }
}

void StageTimer::reset() {
  std::fill(total_ms.begin(), total_ms.end(), 0.0);
  std::fill(samples.begin(), samples.end(), 0);
}

static DirectVariant default_variant() {
  const char* v = std::getenv("NBGB_DIRECT_VARIANT");
  if (v && std::strcmp(v, "scalar4") == 0) return DirectVariant::kScalar4;
  if (v && std::strcmp(v, "paired8") == 0) return DirectVariant::kPaired8;
  // packed FP32x2 halves the FP32 issue slots: 54.5 vs 48.5 TFLOP/s at N = 1M
  return DirectVariant::kPaired8;
}

static void check_particles(const nbgb_particle_data* d, bool need_vel, bool need_old) {
  if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
  if (d->count == 0) return;
  if (d->count > 100000000ull)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count exceeds maximum supported (100M)");
  if (!d->pos_x || !d->pos_y || !d->pos_z || !d->mass || !d->acc_x || !d->acc_y || !d->acc_z)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: null position, mass or acceleration array");
  if (need_vel && (!d->vel_x || !d->vel_y || !d->vel_z))
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: null velocity array");
  if (need_old && (!d->acc_old_x || !d->acc_old_y || !d->acc_old_z))
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: null acc_old array");
}

static void finish_call(nbgb_calculator* c) {
  if (c->params.flags & NBGB_FLAG_SYNC) check_device_errors(c);
}

}  // namespace nbgb

using namespace nbgb;

// ---------------------------------------------------------------------------
// Device-resident FP64 system.
// ---------------------------------------------------------------------------
constexpr int64_t kPotentialF64MaxN = (int64_t)1 << 18;

void nbgb::system_sync_velocity(nbgb_system* s) {
  if (!s->pending_half) return;
  if (s->fp64)
    launch_kick(s->n, s->vx.ptr, s->vy.ptr, s->vz.ptr, s->ax64.ptr, s->ay64.ptr, s->az64.ptr,
                0.5 * s->last_dt, s->calc->stream);
  else
    launch_kick(s->n, s->vx.ptr, s->vy.ptr, s->vz.ptr, s->ax.ptr, s->ay.ptr, s->az.ptr,
                0.5 * s->last_dt, s->calc->stream);
  s->pending_half = false;
}

// Forces at the current state into the system's acceleration arrays.
static void system_forces(nbgb_system* s) {
  nbgb_calculator* c = s->calc;
  if (s->fp64) {
    const double eps = (double)c->params.softening;
    launch_direct_f64_state(s->x.ptr, s->y.ptr, s->z.ptr, s->pm.ptr, s->n, (double)c->params.G,
                            eps * eps, s->ax64.ptr, s->ay64.ptr, s->az64.ptr, c->stream);
  } else {
    forces_packed(c, s->pm.ptr, s->n, s->ax.ptr, s->ay.ptr, s->az.ptr);
  }
}

extern "C" {

void nbgb_params_default(nbgb_params* p) {
  if (!p) return;
  p->G = 1.0f;             // SimulationConfig::G (types.hpp:136)
  p->softening = 0.1f;     // SimulationConfig::softening (:137)
  p->theta = 0.5f;         // barnes_hut_theta (:138)
  p->cell_size = 2.0f;     // spatial_hash_cell_size (:139)
  p->cutoff = 2.0f;        // spatial_hash_cutoff (:140)
  p->block_size = 256;     // cuda_block_size (:141)
  p->leaf_capacity = 1;    // reference tree: one body per leaf
  p->flags = NBGB_FLAG_SYNC | NBGB_FLAG_COMPENSATED;
  p->group_size = 0;       // group walk: by the body count
}

const char* nbgb_last_error(void) { return g_last_error.c_str(); }
const char* nbgb_version(void) { return "nbgb 0.1.0 (sm_103a)"; }
int32_t nbgb_abi_version(void) { return NBGB_ABI_VERSION; }

nbgb_status nbgb_calculator_create(nbgb_method method, const nbgb_params* params,
                                   nbgb_calculator** out) {
  return guarded([&] {
    if (!out) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null output handle");
    *out = nullptr;
    if (method != NBGB_DIRECT_N2 && method != NBGB_BARNES_HUT && method != NBGB_SPATIAL_HASH)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: unknown force method");
    nbgb_params p;
    nbgb_params_default(&p);
    if (params) p = *params;
    validate_params(method, p);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(NBGB_ERR_NO_DEVICE, "CUDA Error: no CUDA device available");
    }
    auto c = std::make_unique<nbgb_calculator>();
    c->method = method;
    c->params = p;
    if (p.flags & NBGB_FLAG_STAGE_TIMINGS) c->timer = std::make_unique<StageTimer>();
    c->variant = default_variant();
    NBGB_CUDA(cudaGetDevice(&c->device));
    NBGB_CUDA(cudaStreamCreate(&c->stream));
    c->own_stream = true;
    uint32_t* e0 = c->err.ensure(1);
    NBGB_CUDA(cudaMemsetAsync(e0, 0, sizeof(uint32_t), c->stream));
    *out = c.release();
  });
}

nbgb_status nbgb_calculator_destroy(nbgb_calculator* calc) {
  return guarded([&] {
    if (!calc) return;
    if (calc->stream) cudaStreamSynchronize(calc->stream);
    if (calc->own_stream && calc->stream) cudaStreamDestroy(calc->stream);
    delete calc;
  });
}

nbgb_status nbgb_calculator_set_params(nbgb_calculator* calc, const nbgb_params* params) {
  return guarded([&] {
    if (!calc || !params) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    validate_params(calc->method, *params);
    calc->params = *params;
    if ((params->flags & NBGB_FLAG_STAGE_TIMINGS) && !calc->timer)
      calc->timer = std::make_unique<StageTimer>();
  });
}

nbgb_status nbgb_calculator_stage_times(nbgb_calculator* calc, int32_t capacity, char* names,
                                        double* total_ms, int64_t* samples, int32_t* count,
                                        int32_t reset) {
  return guarded([&] {
    if (!calc || capacity < 0 || (capacity > 0 && (!names || !total_ms || !samples)))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    StageTimer* t = calc->timer.get();
    int32_t k = 0;
    if (t) {
      t->harvest();
      k = (int32_t)t->names.size();
      for (int32_t i = 0; i < std::min(k, capacity); ++i) {
        std::snprintf(names + 32 * (size_t)i, 32, "%s", t->names[(size_t)i].c_str());
        total_ms[i] = t->total_ms[(size_t)i];
        samples[i] = t->samples[(size_t)i];
      }
      if (reset) t->reset();
    }
    if (count) *count = k;
  });
}

nbgb_status nbgb_calculator_get_params(const nbgb_calculator* calc, nbgb_params* params) {
  return guarded([&] {
    if (!calc || !params) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    *params = calc->params;
  });
}

nbgb_status nbgb_calculator_get_method(const nbgb_calculator* calc, nbgb_method* method) {
  return guarded([&] {
    if (!calc || !method) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    *method = calc->method;
  });
}

nbgb_status nbgb_calculator_set_stream(nbgb_calculator* calc, void* cuda_stream) {
  return guarded([&] {
    if (!calc) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null calculator");
    NBGB_CUDA(cudaStreamSynchronize(calc->stream));
    if (calc->own_stream) NBGB_CUDA(cudaStreamDestroy(calc->stream));
    calc->own_stream = false;
    calc->stream = static_cast<cudaStream_t>(cuda_stream);
    if (!calc->stream) {
      NBGB_CUDA(cudaStreamCreate(&calc->stream));
      calc->own_stream = true;
    }
  });
}

nbgb_status nbgb_calculator_synchronize(nbgb_calculator* calc) {
  return guarded([&] {
    if (!calc) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null calculator");
    check_device_errors(calc);
  });
}

nbgb_status nbgb_compute_forces(nbgb_calculator* calc, const nbgb_particle_data* d) {
  return guarded([&] {
    if (!calc) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null calculator");
    check_particles(d, false, false);
    const int64_t n = (int64_t)d->count;
    calc->last_n = n;
    if (n == 0) return;
    const int64_t n_pad = direct_pad(n);
    float4* pm = calc->pm.ensure((size_t)n_pad);
    launch_pack_soa(d->pos_x, d->pos_y, d->pos_z, d->mass, n, n_pad, pm, calc->stream);
    forces_packed(calc, pm, n, d->acc_x, d->acc_y, d->acc_z);
    finish_call(calc);
  });
}

nbgb_status nbgb_integrate(nbgb_calculator* calc, const nbgb_particle_data* d, float dt) {
  return guarded([&] {
    if (!calc) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null calculator");
    check_particles(d, true, true);
    const int64_t n = (int64_t)d->count;
    calc->last_n = n;
    if (n == 0) return;
    const int64_t n_pad = direct_pad(n);
    float4* pm = calc->pm.ensure((size_t)n_pad);
    // storeOldAccelerations + updatePositions fused, emitting the packed input.
    launch_vv_positions(*d, dt, true, pm, n_pad, calc->stream);
    forces_packed(calc, pm, n, d->acc_x, d->acc_y, d->acc_z);
    launch_vv_velocities(*d, dt, calc->stream);
    finish_call(calc);
  });
}

nbgb_status nbgb_update_positions(const nbgb_particle_data* d, float dt, void* stream) {
  return guarded([&] {
    check_particles(d, true, false);
    launch_vv_positions(*d, dt, false, nullptr, 0, static_cast<cudaStream_t>(stream));
  });
}

nbgb_status nbgb_update_velocities(const nbgb_particle_data* d, float dt, void* stream) {
  return guarded([&] {
    check_particles(d, true, true);
    launch_vv_velocities(*d, dt, static_cast<cudaStream_t>(stream));
  });
}

nbgb_status nbgb_store_old_accelerations(const nbgb_particle_data* d, void* stream) {
  return guarded([&] {
    check_particles(d, false, true);
    launch_store_old(*d, static_cast<cudaStream_t>(stream));
  });
}

static int reduce_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)num_sms() * 4));
}

nbgb_status nbgb_kinetic_energy(const nbgb_particle_data* d, double* ke, void* stream) {
  return guarded([&] {
    if (!ke) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null output");
    if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
    *ke = 0.0;
    if (d->count == 0) return;
    if (!d->vel_x || !d->vel_y || !d->vel_z || !d->mass)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null velocity or mass array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = (int64_t)d->count;
    int nb = reduce_blocks(n);
    DevBuf<double> part;
    double* p = part.ensure((size_t)nb * 4 + 4);
    launch_kinetic_f32(d->vel_x, d->vel_y, d->vel_z, d->mass, n, p, nb, p + (size_t)nb * 4, st);
    double out[4];
    NBGB_CUDA(cudaMemcpyAsync(out, p + (size_t)nb * 4, sizeof out, cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    *ke = out[0];
  });
}

nbgb_status nbgb_potential_energy(const nbgb_particle_data* d, float G, float eps, double* pe,
                                  void* stream) {
  return guarded([&] {
    if (!pe) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null output");
    if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
    *pe = 0.0;
    if (d->count == 0) return;
    if (!d->pos_x || !d->pos_y || !d->pos_z || !d->mass)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null position or mass array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = (int64_t)d->count;
    DevBuf<float4> pm;
    float4* p4 = pm.ensure((size_t)n);
    launch_pack_soa(d->pos_x, d->pos_y, d->pos_z, d->mass, n, n, p4, st);
    int nb = reduce_blocks(n);
    DevBuf<double> part;
    double* p = part.ensure((size_t)nb + 1);
    launch_potential(p4, n, eps * eps, p, nb, p + nb, st);
    double out = 0.0;
    NBGB_CUDA(cudaMemcpyAsync(&out, p + nb, sizeof out, cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    *pe = (double)G * out;
  });
}

// ---------------------------------------------------------------------------
// ParticleDataManager mirror.
// ---------------------------------------------------------------------------
static float** fields(nbgb_particle_data* d) { return &d->pos_x; }
static float* const* cfields(const nbgb_particle_data* d) { return &d->pos_x; }
static_assert(offsetof(nbgb_particle_data, mass) == 12 * sizeof(float*), "layout");

nbgb_status nbgb_particles_alloc_device(nbgb_particle_data* d, size_t count) {
  return guarded([&] {
    if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
    std::memset(d, 0, sizeof *d);
    d->count = count;
    float** f = fields(d);
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(float);
    for (int k = 0; k < 13; ++k) {
      cudaError_t e = alloc_fault_injected() ? cudaErrorMemoryAllocation : cudaMalloc(&f[k], bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        for (int j = 0; j < k; ++j) cudaFree(f[j]);
        std::memset(d, 0, sizeof *d);
        fail(NBGB_ERR_OOM, "Insufficient GPU memory - allocation of particle arrays failed");
      }
    }
    for (int k = 6; k < 12; ++k) NBGB_CUDA(cudaMemset(f[k], 0, bytes));
  });
}

nbgb_status nbgb_particles_free_device(nbgb_particle_data* d) {
  return guarded([&] {
    if (!d) return;
    float** f = fields(d);
    for (int k = 0; k < 13; ++k)
      if (f[k]) cudaFree(f[k]);
    std::memset(d, 0, sizeof *d);
  });
}

static void copy_fields(nbgb_particle_data* dst, const nbgb_particle_data* src,
                        cudaMemcpyKind kind) {
  if (!dst || !src) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
  const size_t bytes = src->count * sizeof(float);
  if (bytes == 0) return;
  // pos, vel, acc and mass; acc_old is not copied (particle_init.cu:134-160).
  const int idx[] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 12};
  float** fd = fields(dst);
  float* const* fs = cfields(src);
  for (int k : idx) {
    if (!fd[k] || !fs[k]) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle array");
    NBGB_CUDA(cudaMemcpy(fd[k], fs[k], bytes, kind));
  }
}

nbgb_status nbgb_particles_copy_to_device(nbgb_particle_data* d, const nbgb_particle_data* h) {
  return guarded([&] { copy_fields(d, h, cudaMemcpyHostToDevice); });
}

nbgb_status nbgb_particles_copy_to_host(nbgb_particle_data* h, const nbgb_particle_data* d) {
  return guarded([&] { copy_fields(h, d, cudaMemcpyDeviceToHost); });
}

// ---------------------------------------------------------------------------
// System API.
// ---------------------------------------------------------------------------
nbgb_status nbgb_system_create(nbgb_calculator* calc, const nbgb_particle_data* h,
                               nbgb_system** out) {
  return guarded([&] {
    if (!calc || !h || !out) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    *out = nullptr;
    if (h->count == 0) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count must be greater than 0");
    if (h->count > 100000000ull)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count exceeds maximum supported (100M)");
    if (!h->pos_x || !h->pos_y || !h->pos_z || !h->vel_x || !h->vel_y || !h->vel_z || !h->mass)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null host array");
    auto s = std::make_unique<nbgb_system>();
    s->calc = calc;
    s->fp64 = (calc->params.flags & NBGB_FLAG_FP64) != 0;
    if (s->fp64 && calc->method != NBGB_DIRECT_N2)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: FP64 forces require the direct method");
    const int64_t n = (int64_t)h->count;
    s->n = n;
    cudaStream_t st = calc->stream;
    std::vector<double> tmp((size_t)n);
    auto up = [&](DevBuf<double>& b, const float* src) {
      double* d = b.ensure((size_t)n);
      for (int64_t i = 0; i < n; ++i) tmp[(size_t)i] = (double)src[i];
      NBGB_CUDA(cudaMemcpyAsync(d, tmp.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st));
      NBGB_CUDA(cudaStreamSynchronize(st));
    };
    up(s->x, h->pos_x);
    up(s->y, h->pos_y);
    up(s->z, h->pos_z);
    up(s->vx, h->vel_x);
    up(s->vy, h->vel_y);
    up(s->vz, h->vel_z);
    s->ax.ensure((size_t)n);
    s->ay.ensure((size_t)n);
    s->az.ensure((size_t)n);
    if (s->fp64) {
      s->ax64.ensure((size_t)n);
      s->ay64.ensure((size_t)n);
      s->az64.ensure((size_t)n);
    }
    const int64_t n_pad = direct_pad(n);
    float4* pm = s->pm.ensure((size_t)n_pad);
    std::vector<float4> hp((size_t)n_pad, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int64_t i = 0; i < n; ++i)
      hp[(size_t)i] = make_float4(h->pos_x[i], h->pos_y[i], h->pos_z[i], h->mass[i]);
    NBGB_CUDA(cudaMemcpyAsync(pm, hp.data(), (size_t)n_pad * sizeof(float4),
                              cudaMemcpyHostToDevice, st));
    system_forces(s.get());
    check_device_errors(calc);
    *out = s.release();
  });
}

nbgb_status nbgb_system_destroy(nbgb_system* sys) {
  return guarded([&] {
    if (!sys) return;
    cudaStreamSynchronize(sys->calc->stream);
    delete sys;
  });
}

nbgb_status nbgb_system_step(nbgb_system* s, float dt, int32_t steps) {
  return guarded([&] {
    if (!s) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null system");
    if (!(dt > 0.f)) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Time step must be positive");
    if (!std::isfinite(dt)) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Time step must be a finite number");
    if (dt > 1.0f) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Time step is too large (max 1.0)");
    if (steps < 0) fail(NBGB_ERR_INVALID_ARG, "Validation Error: negative step count");
    nbgb_calculator* c = s->calc;
    const double h = (double)dt;
    for (int32_t k = 0; k < steps; ++k) {
      double kick = s->pending_half ? 0.5 * s->last_dt + 0.5 * h : 0.5 * h;
      if (s->fp64)
        launch_kick_drift(s->n, s->x.ptr, s->y.ptr, s->z.ptr, s->vx.ptr, s->vy.ptr, s->vz.ptr,
                          s->ax64.ptr, s->ay64.ptr, s->az64.ptr, kick, h, s->pm.ptr, c->stream);
      else
        launch_kick_drift(s->n, s->x.ptr, s->y.ptr, s->z.ptr, s->vx.ptr, s->vy.ptr, s->vz.ptr,
                          s->ax.ptr, s->ay.ptr, s->az.ptr, kick, h, s->pm.ptr, c->stream);
      system_forces(s);
      s->pending_half = true;
      s->last_dt = h;
    }
    if (c->params.flags & NBGB_FLAG_SYNC) {
      system_sync_velocity(s);
      check_device_errors(c);
    }
  });
}

nbgb_status nbgb_system_read(nbgb_system* s, nbgb_particle_data* h) {
  return guarded([&] {
    if (!s || !h) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    if (h->count != (size_t)s->n) fail(NBGB_ERR_INVALID_ARG, "Validation Error: count mismatch");
    system_sync_velocity(s);
    cudaStream_t st = s->calc->stream;
    const size_t n = (size_t)s->n;
    std::vector<double> tmp(n);
    auto down = [&](const DevBuf<double>& b, float* dst) {
      if (!dst) return;
      NBGB_CUDA(cudaMemcpyAsync(tmp.data(), b.ptr, n * 8, cudaMemcpyDeviceToHost, st));
      NBGB_CUDA(cudaStreamSynchronize(st));
      for (size_t i = 0; i < n; ++i) dst[i] = (float)tmp[i];
    };
    down(s->x, h->pos_x);
    down(s->y, h->pos_y);
    down(s->z, h->pos_z);
    down(s->vx, h->vel_x);
    down(s->vy, h->vel_y);
    down(s->vz, h->vel_z);
    if (s->fp64) {
      down(s->ax64, h->acc_x);
      down(s->ay64, h->acc_y);
      down(s->az64, h->acc_z);
    } else {
      if (h->acc_x) NBGB_CUDA(cudaMemcpyAsync(h->acc_x, s->ax.ptr, n * 4, cudaMemcpyDeviceToHost, st));
      if (h->acc_y) NBGB_CUDA(cudaMemcpyAsync(h->acc_y, s->ay.ptr, n * 4, cudaMemcpyDeviceToHost, st));
      if (h->acc_z) NBGB_CUDA(cudaMemcpyAsync(h->acc_z, s->az.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    }
    if (h->mass) {
      std::vector<float4> hp(n);
      NBGB_CUDA(cudaMemcpyAsync(hp.data(), s->pm.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
      NBGB_CUDA(cudaStreamSynchronize(st));
      for (size_t i = 0; i < n; ++i) h->mass[i] = hp[i].w;
    }
    NBGB_CUDA(cudaStreamSynchronize(st));
    check_device_errors(s->calc);
  });
}

nbgb_status nbgb_system_read_f64(nbgb_system* s, double* x, double* y, double* z, double* vx,
                                 double* vy, double* vz) {
  return guarded([&] {
    if (!s) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null system");
    system_sync_velocity(s);
    cudaStream_t st = s->calc->stream;
    const size_t b = (size_t)s->n * 8;
    double* dst[6] = {x, y, z, vx, vy, vz};
    DevBuf<double>* src[6] = {&s->x, &s->y, &s->z, &s->vx, &s->vy, &s->vz};
    for (int k = 0; k < 6; ++k)
      if (dst[k]) NBGB_CUDA(cudaMemcpyAsync(dst[k], src[k]->ptr, b, cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
  });
}

nbgb_status nbgb_system_energy(nbgb_system* s, double* ke, double* pe, double momentum[3]) {
  return guarded([&] {
    if (!s) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null system");
    system_sync_velocity(s);
    nbgb_calculator* c = s->calc;
    cudaStream_t st = c->stream;
    int nb = reduce_blocks(s->n);
    double* p = s->red.ensure((size_t)nb * 4 + 8);
    double* h = s->h_red.ensure(8);
    launch_kinetic_f64(s->vx.ptr, s->vy.ptr, s->vz.ptr, s->pm.ptr, s->n, p, nb,
                       p + (size_t)nb * 4, st);
    NBGB_CUDA(cudaMemcpyAsync(h, p + (size_t)nb * 4, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    double kin[4] = {h[0], h[1], h[2], h[3]};
    double pot = 0.0;
    if (pe) {
      // FP64 positions and arithmetic (the state the system integrates) up
      // to 2^18 bodies; above, the O(N^2) FP64 sum would take seconds on
      // GB300's FP64 pipe, so the FP32 pair terms (Newton-refined rsqrt,
      // compensated per tile, FP64 totals) are summed instead
      if (s->n <= kPotentialF64MaxN) {
        const double eps = (double)c->params.softening;
        launch_potential_f64(s->x.ptr, s->y.ptr, s->z.ptr, s->pm.ptr, s->n, eps * eps, p, nb,
                             p + (size_t)nb * 4, st);
      } else {
        const float eps = c->params.softening;
        launch_potential(s->pm.ptr, s->n, eps * eps, p, nb, p + (size_t)nb * 4, st);
      }
      NBGB_CUDA(cudaMemcpyAsync(h, p + (size_t)nb * 4, sizeof(double), cudaMemcpyDeviceToHost, st));
      NBGB_CUDA(cudaStreamSynchronize(st));
      pot = (double)c->params.G * h[0];
    }
    if (ke) *ke = kin[0];
    if (pe) *pe = pot;
    if (momentum) {
      momentum[0] = kin[1];
      momentum[1] = kin[2];
      momentum[2] = kin[3];
    }
  });
}

}  // extern "C"
