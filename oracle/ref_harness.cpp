// ref_harness.cpp -- runs the reference's own host-side code on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Linked by oracle/build.py with objects compiled
// in place from the reference sources (nothing of the reference is copied
// into this repository) into oracle/_ref/libnbody_ref.so.  It is used in this
// container to pin the C restatement in oracle/nbody_oracle.c and to generate
// the golden fixtures under tests/golden/.  It cannot run on a machine
// without the reference sources, and nothing on the product path loads it.
//
// The reference's BarnesHutTree keeps its tree on the device and builds it
// on the host from device copies (src/cuda/force_barnes_hut.cu:391-543).  To
// run that host build without a GPU, this file supplies host-memory versions
// of the four CUDA runtime memory calls the build uses (cudaMalloc, cudaFree,
// cudaMemcpy, cudaMemset), and intercepts kernel launches (see below).  The
// shared object is linked with -Bsymbolic, so the reference objects bind to
// these definitions and no device is touched.  No kernel of the reference
// runs through this harness.

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <sstream>
#include <stdexcept>
#include <fstream>
#include <chrono>
#include <algorithm>
#include <cuda_runtime.h>
#include <cuda_runtime_api.h>

// Private members of BarnesHutTree (bbox_min_, buildTreeOnHost, ...) are
// reached by widening access in this translation unit only; access
// specifiers do not change the ABI of the members.
#define private public
#include "nbody/barnes_hut_tree.hpp"
#include "nbody/error_handling.hpp"
#include "nbody/force_calculator.hpp"
#include "nbody/particle_data.hpp"
#include "nbody/serialization.hpp"
#include "nbody/spatial_hash_grid.hpp"
#include "nbody/simulation_state.hpp"
#undef private

// ---- host-memory stand-ins for the CUDA runtime memory calls -------------
extern "C" {
cudaError_t cudaMalloc(void** ptr, size_t size) {
  *ptr = std::malloc(size ? size : 1);
  return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* ptr) {
  std::free(ptr);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind) {
  if (count) std::memcpy(dst, src, count);
  return cudaSuccess;
}
cudaError_t cudaMemset(void* dst, int value, size_t count) {
  if (count) std::memset(dst, value, count);
  return cudaSuccess;
}
}

// ---- kernel launches ------------------------------------------------------
// SpatialHashGrid::build (src/cuda/force_spatial_hash.cu:241-261) computes
// its padded bounding box and grid dimensions on the host, between kernel
// launches.  To run exactly that host code here, launches are intercepted:
// the reference's bounding-box kernel (force_barnes_hut.cu:78-122, an exact
// per-axis min/max) is replaced by the same min/max over the host arrays, and
// every other launch is refused, so build() stops with its own CudaException
// right after the dimensions are set (at the cell-assignment launch).
namespace nbody {
// host-side launch stub of the reference kernel (same symbol nvcc emits)
void computeBoundingBoxKernel(const float* pos_x, const float* pos_y, const float* pos_z,
                              float* min_x, float* min_y, float* min_z, float* max_x,
                              float* max_y, float* max_z, int N);
}  // namespace nbody

static thread_local cudaError_t g_launch_error = cudaSuccess;

extern "C" {
// The launch sequence nvcc emits for `kernel<<<...>>>(args)`: push the
// configuration, look the kernel handle up once, pop the configuration,
// launch.  The handle is the host stub's address here.
unsigned __cudaPushCallConfiguration(dim3, dim3, size_t, struct CUstream_st*) { return 0; }
cudaError_t __cudaPopCallConfiguration(dim3* grid, dim3* block, size_t* shmem, void* stream) {
  *grid = dim3(1, 1, 1);
  *block = dim3(1, 1, 1);
  *shmem = 0;
  *static_cast<cudaStream_t*>(stream) = nullptr;
  return cudaSuccess;
}
cudaError_t __cudaGetKernel(cudaKernel_t* kernel, const void* func) {
  *kernel = reinterpret_cast<cudaKernel_t>(const_cast<void*>(func));
  return cudaSuccess;
}
cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3, dim3, void** args, size_t,
                               cudaStream_t) {
  if (reinterpret_cast<const void*>(kernel) ==
      reinterpret_cast<const void*>(&nbody::computeBoundingBoxKernel)) {
    const float* p[3];
    float* lo[3];
    float* hi[3];
    for (int a = 0; a < 3; ++a) {
      p[a] = *static_cast<const float**>(args[a]);
      lo[a] = *static_cast<float**>(args[3 + a]);
      hi[a] = *static_cast<float**>(args[6 + a]);
    }
    const int n = *static_cast<int*>(args[9]);
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a) {
        *lo[a] = std::min(*lo[a], p[a][i]);
        *hi[a] = std::max(*hi[a], p[a][i]);
      }
    return cudaSuccess;
  }
  g_launch_error = cudaErrorNotSupported;
  return g_launch_error;
}
cudaError_t cudaGetLastError(void) {
  const cudaError_t e = g_launch_error;
  g_launch_error = cudaSuccess;
  return e;
}
cudaError_t cudaPeekAtLastError(void) { return g_launch_error; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
}

static_assert(sizeof(nbody::OctreeNode) == 76, "OctreeNode layout");

extern "C" {

// nbody::computeGravitationalAccelerationCPU (src/cuda/force_direct.cu:109-117)
void ref_pair_accel(const float p1[3], const float p2[3], float m2, float G, float eps,
                    float out[3]) {
  nbody::Vec3 a = nbody::computeGravitationalAccelerationCPU(
      nbody::Vec3(p1[0], p1[1], p1[2]), nbody::Vec3(p2[0], p2[1], p2[2]), m2, G, eps);
  out[0] = a.x;
  out[1] = a.y;
  out[2] = a.z;
}

// nbody::computeMortonCode (src/cuda/force_barnes_hut.cu:42-50)
uint32_t ref_morton_code(float nx, float ny, float nz) {
  return nbody::computeMortonCode(nx, ny, nz);
}

// nbody::SpatialHashGrid::getCellIndex (src/cuda/force_spatial_hash.cu:15-18)
void ref_cell_index(float x, float y, float z, float cell, int out[3]) {
  int3 c = nbody::SpatialHashGrid::getCellIndex(x, y, z, cell);
  out[0] = c.x;
  out[1] = c.y;
  out[2] = c.z;
}

static void copy_out(const nbody::ParticleData& h, float* x, float* y, float* z, float* vx,
                     float* vy, float* vz, float* m) {
  size_t b = h.count * sizeof(float);
  std::memcpy(x, h.pos_x, b);
  std::memcpy(y, h.pos_y, b);
  std::memcpy(z, h.pos_z, b);
  std::memcpy(vx, h.vel_x, b);
  std::memcpy(vy, h.vel_y, b);
  std::memcpy(vz, h.vel_z, b);
  std::memcpy(m, h.mass, b);
}

// nbody::ParticleInitializer::initSpherical (src/cuda/particle_init.cu:187-208)
void ref_init_spherical(int64_t n, float cx, float cy, float cz, float radius, float min_mass,
                        float max_mass, unsigned seed, float* x, float* y, float* z, float* vx,
                        float* vy, float* vz, float* m) {
  nbody::ParticleData h;
  nbody::ParticleDataManager::allocateHost(h, (size_t)n);
  nbody::SphericalDistParams p;
  p.center = nbody::Vec3(cx, cy, cz);
  p.radius = radius;
  p.min_mass = min_mass;
  p.max_mass = max_mass;
  nbody::ParticleInitializer::initSpherical(h, p, seed);
  copy_out(h, x, y, z, vx, vy, vz, m);
  nbody::ParticleDataManager::freeHost(h);
}

// nbody::ParticleInitializer::initUniform (src/cuda/particle_init.cu:167-185)
void ref_init_uniform(int64_t n, const float bmin[3], const float bmax[3], float min_mass,
                      float max_mass, unsigned seed, float* x, float* y, float* z, float* vx,
                      float* vy, float* vz, float* m) {
  nbody::ParticleData h;
  nbody::ParticleDataManager::allocateHost(h, (size_t)n);
  nbody::UniformDistParams p;
  p.min_bounds = nbody::Vec3(bmin[0], bmin[1], bmin[2]);
  p.max_bounds = nbody::Vec3(bmax[0], bmax[1], bmax[2]);
  p.min_mass = min_mass;
  p.max_mass = max_mass;
  nbody::ParticleInitializer::initUniform(h, p, seed);
  copy_out(h, x, y, z, vx, vy, vz, m);
  nbody::ParticleDataManager::freeHost(h);
}

// BarnesHutTree::buildTreeOnHost (src/cuda/force_barnes_hut.cu:391-543) on
// caller-supplied bbox and Morton-sorted indices.  The tree is sized for
// max_particles = n, i.e. 2n nodes, exactly as BarnesHutCalculator sizes it
// on its first call (:577-580).  nodes_out receives node_count 76-byte
// OctreeNode records.  Returns 0, or 1 when nodes_cap is too small.
int ref_build_tree(int64_t n, const float* x, const float* y, const float* z, const float* m,
                   const int32_t* sorted_idx, const float bmin[3], const float bmax[3],
                   void* nodes_out, int64_t nodes_cap, int* node_count, int* max_depth) {
  nbody::BarnesHutTree tree((size_t)n);
  tree.bbox_min_ = nbody::Vec3(bmin[0], bmin[1], bmin[2]);
  tree.bbox_max_ = nbody::Vec3(bmax[0], bmax[1], bmax[2]);
  std::memcpy(tree.d_sorted_indices_, sorted_idx, (size_t)n * sizeof(int32_t));
  nbody::ParticleData pd;
  pd.pos_x = const_cast<float*>(x);
  pd.pos_y = const_cast<float*>(y);
  pd.pos_z = const_cast<float*>(z);
  pd.mass = const_cast<float*>(m);
  pd.count = (size_t)n;
  tree.buildTreeOnHost(&pd);
  *node_count = tree.getNodeCount();
  *max_depth = tree.getMaxDepth();
  if ((int64_t)*node_count > nodes_cap) return 1;
  std::memcpy(nodes_out, tree.getNodes(), (size_t)*node_count * sizeof(nbody::OctreeNode));
  return 0;
}

// nbody::SpatialHashGrid::build up to its first cell kernel
// (src/cuda/force_spatial_hash.cu:190-261): the reference's padded bounding
// box (computeBoundingBox, :190-239) and grid dimensions (:249-252) for the
// given positions and cell size.  Returns 0 with bmin/bmax/dims/total_cells
// filled, 2 when the reference rejects the grid as too large (:257-260),
// 1 on any other outcome.
int ref_hash_grid_setup(int64_t n, const float* x, const float* y, const float* z, float cell,
                        float bmin[3], float bmax[3], int dims[3], int64_t* total_cells) {
  nbody::SpatialHashGrid grid((size_t)n, cell);
  nbody::ParticleData pd;
  pd.pos_x = const_cast<float*>(x);
  pd.pos_y = const_cast<float*>(y);
  pd.pos_z = const_cast<float*>(z);
  pd.count = (size_t)n;
  try {
    grid.build(&pd);
    return 1;  // cannot complete without a device: a launch must have been refused
  } catch (const nbody::CudaException&) {
    // stopped at the cell-assignment launch, after the dimensions were set
  } catch (const std::runtime_error& e) {
    if (std::string(e.what()).find("too large") != std::string::npos) return 2;
    return 1;
  }
  bmin[0] = grid.bbox_min_.x;
  bmin[1] = grid.bbox_min_.y;
  bmin[2] = grid.bbox_min_.z;
  bmax[0] = grid.bbox_max_.x;
  bmax[1] = grid.bbox_max_.y;
  bmax[2] = grid.bbox_max_.z;
  dims[0] = grid.grid_dims_.x;
  dims[1] = grid.grid_dims_.y;
  dims[2] = grid.grid_dims_.z;
  *total_cells = (int64_t)grid.total_cells_;
  return 0;
}

// nbody::Serializer::save (src/utils/serialization.cpp:25-37)
int ref_save_checkpoint(const char* path, int64_t n, float sim_time, float dt, float G,
                        float softening, uint32_t method, const float* x, const float* y,
                        const float* z, const float* vx, const float* vy, const float* vz,
                        const float* m) {
  try {
    nbody::SimulationState s;
    s.particle_count = (size_t)n;
    s.simulation_time = sim_time;
    s.dt = dt;
    s.G = G;
    s.softening = softening;
    s.force_method = static_cast<nbody::ForceMethod>(method);
    s.pos_x.assign(x, x + n);
    s.pos_y.assign(y, y + n);
    s.pos_z.assign(z, z + n);
    s.vel_x.assign(vx, vx + n);
    s.vel_y.assign(vy, vy + n);
    s.vel_z.assign(vz, vz + n);
    s.mass.assign(m, m + n);
    nbody::Serializer::save(std::string(path), s);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// nbody::Serializer::load (src/utils/serialization.cpp:39-75).  Returns 0
// and fills the header fields (arrays when non-null); on a rejected file
// returns 1 and copies the exception text into err.
int ref_load_checkpoint(const char* path, int64_t* n, float* sim_time, float* dt, float* G,
                        float* softening, uint32_t* method, float* x, float* y, float* z,
                        float* vx, float* vy, float* vz, float* m, char* err, int err_cap) {
  try {
    nbody::SimulationState s = nbody::Serializer::load(std::string(path));
    *n = (int64_t)s.particle_count;
    *sim_time = s.simulation_time;
    *dt = s.dt;
    *G = s.G;
    *softening = s.softening;
    *method = (uint32_t)s.force_method;
    if (x) {
      std::memcpy(x, s.pos_x.data(), s.particle_count * 4);
      std::memcpy(y, s.pos_y.data(), s.particle_count * 4);
      std::memcpy(z, s.pos_z.data(), s.particle_count * 4);
      std::memcpy(vx, s.vel_x.data(), s.particle_count * 4);
      std::memcpy(vy, s.vel_y.data(), s.particle_count * 4);
      std::memcpy(vz, s.vel_z.data(), s.particle_count * 4);
      std::memcpy(m, s.mass.data(), s.particle_count * 4);
    }
    return 0;
  } catch (const std::exception& e) {
    if (err && err_cap > 0) {
      std::strncpy(err, e.what(), (size_t)err_cap - 1);
      err[err_cap - 1] = 0;
    }
    return 1;
  }
}

}  // extern "C"
