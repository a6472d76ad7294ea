// checkpoint.cu -- the reference's .nbody v1 checkpoints written from and
// read into device memory, plus an FP64 sidecar for the resident state.
//
// File format (unchanged; include/nbody/serialization.hpp:21-32,
// src/utils/serialization.cpp:25-129): a 56-byte header {u32 magic
// 0x4E424F44, u32 version 1, u64 particle_count, f32 simulation_time, dt, G,
// softening, u32 force_method, 4 x u32 reserved, zero tail padding} followed
// by seven float32 arrays pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, mass.
// The reference goes through host std::vectors (ParticleSystem::getState,
// then one write per array); here the arrays are copied from the device
// straight into one pinned buffer laid out as the file image and written
// with one call (read the same way), and the bytes equal the reference
// writer's for the same state.
//
// FP64 sidecar (<path>.f64, no reference counterpart): a 32-byte header
// {u32 magic 0x4E424638, u32 version 2, u64 particle_count, 2 x u64 zero}
// and six float64 arrays x, y, z, vx, vy, vz.  A v1 reader ignores it; the
// loader restores the FP64 state only when every FP64 value rounds to the v1
// file's float32 value, so a restarted run continues exactly where the
// saved one was.
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "runtime.cuh"

namespace nbgb {

constexpr uint32_t kV1Magic = 0x4E424F44u;
constexpr uint32_t kV1Version = 1;
constexpr uint64_t kMaxParticles = 100000000ull;  // serialization.hpp MAX_PARTICLE_COUNT
constexpr uint32_t kSideMagic = 0x4E424638u;
constexpr uint32_t kSideVersion = 2;

struct V1Header {
  uint32_t magic, version;
  uint64_t particle_count;
  float simulation_time, dt, G, softening;
  uint32_t force_method;
  uint32_t reserved[4];
};
static_assert(sizeof(V1Header) == 56, "the v1 header is 56 bytes");

struct SideHeader {
  uint32_t magic, version;
  uint64_t particle_count;
  uint64_t reserved[2];
};
static_assert(sizeof(SideHeader) == 32, "the sidecar header is 32 bytes");

// One process-wide pinned staging buffer (grown, reused; calls serialised).
static std::mutex g_ckpt_mu;
static HostPinned<char> g_ckpt_buf;

struct File {
  std::FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

static char* staging(size_t bytes) { return g_ckpt_buf.ensure(bytes); }

static void write_all(const std::string& path, const void* data, size_t bytes) {
  File fo;
  fo.f = std::fopen(path.c_str(), "wb");
  if (!fo.f) fail(NBGB_ERR_INVALID_ARG, "IO Error: Failed to open file for writing: " + path);
  if (bytes && std::fwrite(data, 1, bytes, fo.f) != bytes)
    fail(NBGB_ERR_INVALID_ARG, "IO Error: Failed to write file: " + path);
  const int rc = std::fclose(fo.f);
  fo.f = nullptr;
  if (rc != 0) fail(NBGB_ERR_INVALID_ARG, "IO Error: Failed to write file: " + path);
}

// Reads and validates a v1 header like Serializer::load
// (serialization.cpp:39-58,111-129).
static V1Header read_v1_header(std::FILE* f) {
  V1Header h;
  if (std::fread(&h, 1, sizeof h, f) != sizeof h)
    fail(NBGB_ERR_INVALID_ARG,
         "Validation Error: Failed to read file header: file may be truncated or corrupted");
  if (h.magic != kV1Magic)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Invalid file format: wrong magic number");
  if (h.version != kV1Version) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Unsupported file version");
  if (h.particle_count > kMaxParticles)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count (" +
                                   std::to_string(h.particle_count) +
                                   ") exceeds maximum allowed (" + std::to_string(kMaxParticles) +
                                   ")");
  if (h.force_method > 2u)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: Invalid force method in file header: " +
                                   std::to_string(h.force_method));
  return h;
}

static V1Header pack_header(const nbgb_checkpoint_header& in, uint64_t n) {
  V1Header h;
  std::memset(&h, 0, sizeof h);
  h.magic = kV1Magic;
  h.version = kV1Version;
  h.particle_count = n;
  h.simulation_time = in.simulation_time;
  h.dt = in.dt;
  h.G = in.G;
  h.softening = in.softening;
  h.force_method = in.force_method;
  return h;
}

static nbgb_checkpoint_header unpack_header(const V1Header& h) {
  nbgb_checkpoint_header o;
  std::memset(&o, 0, sizeof o);
  o.particle_count = h.particle_count;
  o.simulation_time = h.simulation_time;
  o.dt = h.dt;
  o.G = h.G;
  o.softening = h.softening;
  o.force_method = h.force_method;
  return o;
}

// Reads the v1 file image (header and arrays); the arrays land in the
// staging buffer.
static V1Header read_v1(const std::string& path, const float** arrays) {
  File fi;
  fi.f = std::fopen(path.c_str(), "rb");
  if (!fi.f) fail(NBGB_ERR_INVALID_ARG, "IO Error: Failed to open file for reading: " + path);
  const V1Header h = read_v1_header(fi.f);
  const size_t bytes = (size_t)h.particle_count * 7 * sizeof(float);
  char* buf = staging(std::max<size_t>(bytes, 1));
  if (bytes && std::fread(buf, 1, bytes, fi.f) != bytes)
    fail(NBGB_ERR_INVALID_ARG,
         "Validation Error: Failed to read particle data: file may be truncated or corrupted");
  *arrays = reinterpret_cast<const float*>(buf);
  return h;
}

__global__ void f64_to_f32_kernel(const double* __restrict__ src, int64_t n, float* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

__global__ void mass_of_kernel(const float4* __restrict__ pm, int64_t n, float* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = pm[i].w;
}

static unsigned ckpt_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), 256), (int64_t)num_sms() * 8));
}

template <typename F>
static nbgb_status ckpt_guarded(F&& f) {
  try {
    std::lock_guard<std::mutex> lk(g_ckpt_mu);
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

nbgb_status nbgb_checkpoint_save_device(const char* path, const nbgb_particle_data* d,
                                        const nbgb_checkpoint_header* hdr, void* stream) {
  return ckpt_guarded([&] {
    if (!path || !d || !hdr) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    const size_t n = d->count;
    const float* src[7] = {d->pos_x, d->pos_y, d->pos_z, d->vel_x, d->vel_y, d->vel_z, d->mass};
    for (const float* p : src)
      if (n && !p) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null device array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* buf = staging(sizeof(V1Header) + n * 7 * sizeof(float));
    const V1Header h = pack_header(*hdr, n);
    std::memcpy(buf, &h, sizeof h);
    float* arr = reinterpret_cast<float*>(buf + sizeof h);
    for (int k = 0; k < 7 && n; ++k)
      NBGB_CUDA(cudaMemcpyAsync(arr + (size_t)k * n, src[k], n * sizeof(float),
                                cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    write_all(path, buf, sizeof h + n * 7 * sizeof(float));
  });
}

nbgb_status nbgb_checkpoint_load_device(const char* path, nbgb_particle_data* d,
                                        nbgb_checkpoint_header* hdr, void* stream) {
  return ckpt_guarded([&] {
    if (!path) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null path");
    if (!d) {  // header only
      File fi;
      fi.f = std::fopen(path, "rb");
      if (!fi.f)
        fail(NBGB_ERR_INVALID_ARG, std::string("IO Error: Failed to open file for reading: ") + path);
      const V1Header h = read_v1_header(fi.f);
      if (hdr) *hdr = unpack_header(h);
      return;
    }
    const float* arr = nullptr;
    const V1Header h = read_v1(path, &arr);
    const size_t n = h.particle_count;
    if (d->count != n)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: particle data holds " +
                                     std::to_string(d->count) + " particles, the file " +
                                     std::to_string(n));
    float* dst[7] = {d->pos_x, d->pos_y, d->pos_z, d->vel_x, d->vel_y, d->vel_z, d->mass};
    for (float* p : dst)
      if (n && !p) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null device array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int k = 0; k < 7 && n; ++k)
      NBGB_CUDA(cudaMemcpyAsync(dst[k], arr + (size_t)k * n, n * sizeof(float),
                                cudaMemcpyHostToDevice, st));
    NBGB_CUDA(cudaStreamSynchronize(st));  // the staging buffer is reused by the next call
    if (hdr) *hdr = unpack_header(h);
  });
}

nbgb_status nbgb_system_save(nbgb_system* s, const char* path, const nbgb_checkpoint_header* hdr,
                             int32_t with_f64) {
  return ckpt_guarded([&] {
    if (!s || !path || !hdr) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    system_sync_velocity(s);
    cudaStream_t st = s->calc->stream;
    const size_t n = (size_t)s->n;
    // v1: the FP64 state rounded to float32 on the device, then one copy of
    // the seven arrays into the file image
    DevBuf<float> tmp;
    float* t = tmp.ensure(n * 7);
    const DevBuf<double>* f64[6] = {&s->x, &s->y, &s->z, &s->vx, &s->vy, &s->vz};
    for (int k = 0; k < 6; ++k)
      f64_to_f32_kernel<<<ckpt_grid((int64_t)n), 256, 0, st>>>(f64[k]->ptr, (int64_t)n, t + k * n);
    mass_of_kernel<<<ckpt_grid((int64_t)n), 256, 0, st>>>(s->pm.ptr, (int64_t)n, t + 6 * n);
    NBGB_LAUNCH_CHECK();
    const size_t v1 = sizeof(V1Header) + n * 7 * sizeof(float);
    const size_t side = with_f64 ? sizeof(SideHeader) + n * 6 * sizeof(double) : 0;
    char* buf = staging(std::max(v1, side));
    const V1Header h = pack_header(*hdr, n);
    std::memcpy(buf, &h, sizeof h);
    NBGB_CUDA(cudaMemcpyAsync(buf + sizeof h, t, n * 7 * sizeof(float), cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    write_all(path, buf, v1);
    if (!with_f64) return;
    SideHeader sh;
    std::memset(&sh, 0, sizeof sh);
    sh.magic = kSideMagic;
    sh.version = kSideVersion;
    sh.particle_count = n;
    std::memcpy(buf, &sh, sizeof sh);
    double* arr = reinterpret_cast<double*>(buf + sizeof sh);
    for (int k = 0; k < 6; ++k)
      NBGB_CUDA(cudaMemcpyAsync(arr + k * n, f64[k]->ptr, n * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    write_all(std::string(path) + ".f64", buf, side);
  });
}

nbgb_status nbgb_system_load(nbgb_calculator* calc, const char* path, nbgb_system** out,
                             nbgb_checkpoint_header* hdr, int32_t* restored_f64) {
  nbgb_system* sys = nullptr;
  const nbgb_status st0 = ckpt_guarded([&] {
    if (!calc || !path || !out) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    *out = nullptr;
    if (restored_f64) *restored_f64 = 0;
    const float* arr = nullptr;
    const V1Header h = read_v1(path, &arr);
    const size_t n = h.particle_count;
    if (n == 0) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count must be greater than 0");
    // the v1 arrays leave the staging buffer before the sidecar uses it
    std::vector<float> v1(arr, arr + n * 7);
    nbgb_particle_data hp;
    std::memset(&hp, 0, sizeof hp);
    hp.count = n;
    hp.pos_x = v1.data();
    hp.pos_y = v1.data() + n;
    hp.pos_z = v1.data() + 2 * n;
    hp.vel_x = v1.data() + 3 * n;
    hp.vel_y = v1.data() + 4 * n;
    hp.vel_z = v1.data() + 5 * n;
    hp.mass = v1.data() + 6 * n;
    const nbgb_status cs = nbgb_system_create(calc, &hp, &sys);
    if (cs != NBGB_OK) fail(cs, nbgb_last_error());
    if (hdr) *hdr = unpack_header(h);
    // the FP64 sidecar, where it exists and agrees with the v1 arrays
    File fi;
    fi.f = std::fopen((std::string(path) + ".f64").c_str(), "rb");
    if (!fi.f) return;
    SideHeader sh;
    if (std::fread(&sh, 1, sizeof sh, fi.f) != sizeof sh || sh.magic != kSideMagic ||
        sh.version != kSideVersion || sh.particle_count != n)
      return;
    const size_t bytes = n * 6 * sizeof(double);
    double* d64 = reinterpret_cast<double*>(staging(bytes));
    if (std::fread(d64, 1, bytes, fi.f) != bytes) return;
    for (size_t i = 0; i < n * 6; ++i)
      if ((float)d64[i] != v1[i]) return;
    DevBuf<double>* dst[6] = {&sys->x, &sys->y, &sys->z, &sys->vx, &sys->vy, &sys->vz};
    cudaStream_t st = calc->stream;
    for (int k = 0; k < 6; ++k)
      NBGB_CUDA(cudaMemcpyAsync(dst[k]->ptr, d64 + k * n, n * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    NBGB_CUDA(cudaStreamSynchronize(st));
    if (restored_f64) *restored_f64 = 1;
  });
  if (st0 != NBGB_OK) {
    const std::string msg = nbgb_last_error();
    if (sys) nbgb_system_destroy(sys);
    return set_error(st0, msg);
  }
  *out = sys;
  return NBGB_OK;
}

}  // extern "C"
