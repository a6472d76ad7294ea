// nbody_adapter.cpp -- the reference-side binding: definitions of the
// reference's hot-path classes over the nbgb C ABI.
//
// A maintainer of the reference app builds this file (against the
// reference's include/ and this repository's include/nbgb.h) in place of
// src/cuda/force_direct.cu, force_barnes_hut.cu (calculator part),
// force_spatial_hash.cu (calculator part) and integrator.cu, and links
// libnbgb.so.  Everything above these classes (ParticleSystem, the app, the
// benchmarks, the examples) is unchanged.
//
// Mapping (reference declaration -> C ABI):
//   ForceCalculator::computeForces      (force_calculator.hpp:12)  -> nbgb_compute_forces
//   createForceCalculator               (force_calculator.hpp:76)  -> one adapter object per method
//   computeGravitationalAccelerationCPU (force_calculator.hpp:79)  -> kept on the host
//   Integrator::integrate                (integrator.hpp:19)        -> nbgb_state_kick_drift,
//                                                                     computeForces, nbgb_state_kick
//   Integrator::* (the other members)    (integrator.hpp:15-33)     -> nbgb_update_* / nbgb_*_energy
// Status codes are rethrown as the reference's exception types
// (include/nbody/error_handling.hpp).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include <vector>

#include "nbgb.h"
#include "nbody/barnes_hut_tree.hpp"
#include "nbody/error_handling.hpp"
#include "nbody/force_calculator.hpp"
#include "nbody/integrator.hpp"
#include "nbody/performance_observability.hpp"
#include "nbody/spatial_hash_grid.hpp"
#include "nbody/types.hpp"

static_assert(sizeof(nbody::ParticleData) == sizeof(nbgb_particle_data),
              "nbgb_particle_data mirrors nbody::ParticleData");
static_assert(static_cast<int>(nbody::ForceMethod::BARNES_HUT) == NBGB_BARNES_HUT,
              "method numbering");

namespace nbody {
namespace {

[[noreturn]] void rethrow(nbgb_status s) {
  std::string msg = nbgb_last_error();
  const std::string prefix = "Validation Error: ";
  switch (s) {
    case NBGB_ERR_INVALID_ARG:
      if (msg.compare(0, prefix.size(), prefix) == 0) msg = msg.substr(prefix.size());
      throw ValidationException(msg);
    case NBGB_ERR_OOM:
      throw ResourceException(msg.c_str(), 0, 0);
    case NBGB_ERR_OVERFLOW:
      throw std::runtime_error(msg);
    default:
      throw CudaException(nbgb_last_error(), __FILE__, __LINE__);
  }
}

void check(nbgb_status s) {
  if (s != NBGB_OK) rethrow(s);
}

nbgb_particle_data* view(ParticleData* d) { return reinterpret_cast<nbgb_particle_data*>(d); }

// One library calculator per adapter object (keyed by address; released by
// the destructors the reference declares).  Direct calculators declare no
// destructor, so they share one handle whose parameters are set per call
// (the reference is single-threaded: particle_system.hpp:13).
std::mutex g_mu;
std::unordered_map<const void*, nbgb_calculator*> g_handles;

nbgb_calculator* handle(const void* key, nbgb_method m, const nbgb_params& p) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_handles.find(key);
  if (it == g_handles.end()) {
    nbgb_calculator* c = nullptr;
    check(nbgb_calculator_create(m, &p, &c));
    it = g_handles.emplace(key, c).first;
  } else {
    check(nbgb_calculator_set_params(it->second, &p));
  }
  return it->second;
}

void release(const void* key) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_handles.find(key);
  if (it != g_handles.end()) {
    nbgb_calculator_destroy(it->second);
    g_handles.erase(it);
  }
}

nbgb_params params_of(float G, float eps) {
  nbgb_params p;
  nbgb_params_default(&p);
  p.G = G;
  p.softening = eps;
  return p;
}

const int kDirectKey = 0;

}  // namespace

// ------------------------------------------------------------- direct --
DirectForceCalculator::DirectForceCalculator(int block_size) : block_size_(block_size) {}

void DirectForceCalculator::computeForces(ParticleData* d_particles) {
  NBODY_PROFILE_SCOPE("force.direct_n2");
  nbgb_params p = params_of(G_, softening_eps_);
  p.block_size = block_size_ > 0 && block_size_ <= 1024 ? block_size_ : 256;
  check(nbgb_compute_forces(handle(&kDirectKey, NBGB_DIRECT_N2, p), view(d_particles)));
}

// --------------------------------------------------------- Barnes-Hut --
BarnesHutCalculator::BarnesHutCalculator(float theta) : theta_(theta) {}

BarnesHutCalculator::~BarnesHutCalculator() { release(this); }

void BarnesHutCalculator::computeForces(ParticleData* d_particles) {
  NBODY_PROFILE_SCOPE("barnes_hut.build");
  nbgb_params p = params_of(G_, softening_eps_);
  p.theta = theta_;
  // the reference's own tree wherever it differs from the canonical one
  // (synchronous calls check the node count; only small systems pay)
  if (d_particles->count <= 65536) p.flags |= NBGB_FLAG_REFERENCE_TREE;
  check(nbgb_compute_forces(handle(this, NBGB_BARNES_HUT, p), view(d_particles)));
}

// ------------------------------------------------------- spatial hash --
SpatialHashCalculator::SpatialHashCalculator(float cell_size, float cutoff_radius)
    : cell_size_(cell_size), cutoff_radius_(cutoff_radius) {}

SpatialHashCalculator::~SpatialHashCalculator() { release(this); }

void SpatialHashCalculator::computeForces(ParticleData* d_particles) {
  NBODY_PROFILE_SCOPE("force.spatial_hash");
  nbgb_params p = params_of(G_, softening_eps_);
  p.cell_size = cell_size_;
  p.cutoff = cutoff_radius_;
  check(nbgb_compute_forces(handle(this, NBGB_SPATIAL_HASH, p), view(d_particles)));
}

std::unique_ptr<ForceCalculator> createForceCalculator(ForceMethod method,
                                                       const SimulationConfig& config) {
  switch (method) {
    case ForceMethod::BARNES_HUT:
      return std::make_unique<BarnesHutCalculator>(config.barnes_hut_theta);
    case ForceMethod::SPATIAL_HASH:
      return std::make_unique<SpatialHashCalculator>(config.spatial_hash_cell_size,
                                                     config.spatial_hash_cutoff);
    case ForceMethod::DIRECT_N2:
    default:
      return std::make_unique<DirectForceCalculator>(config.cuda_block_size);
  }
}

// Host pair function: unchanged semantics (force_direct.cu:109-117).
Vec3 computeGravitationalAccelerationCPU(const Vec3& p1, const Vec3& p2, float m2, float G,
                                         float eps) {
  Vec3 r = p2 - p1;
  float dist2 = r.length2() + eps * eps;
  float inv = 1.0f / std::sqrt(dist2);
  return r * (G * m2 * (inv * inv * inv));
}

// ------------------------------------------- inspection classes (tests) --
// BarnesHutTree / SpatialHashGrid (barnes_hut_tree.hpp, spatial_hash_grid.hpp)
// are what the reference's tests inspect.  Here they wrap a library
// calculator of their own; the tree and grid are the library's (nodes in the
// reference layout, numbered depth-first instead of in insertion order).
namespace {
// Builds a structure without touching the caller's accelerations: the
// library computes forces as part of a build, into scratch arrays.
void build_into_scratch(nbgb_calculator* c, const ParticleData* d) {
  nbgb_particle_data v = *reinterpret_cast<const nbgb_particle_data*>(d);
  float* acc = nullptr;
  const size_t bytes = std::max<size_t>(d->count, 1) * sizeof(float) * 3;
  CUDA_CHECK(cudaMalloc(&acc, bytes));
  v.acc_x = acc;
  v.acc_y = acc + d->count;
  v.acc_z = acc + 2 * d->count;
  nbgb_status s = nbgb_compute_forces(c, &v);
  cudaFree(acc);
  check(s);
}
}  // namespace

BarnesHutTree::BarnesHutTree(size_t max_particles)
    : d_nodes_(nullptr),
      d_sorted_indices_(nullptr),
      d_morton_codes_(nullptr),
      max_particles_(max_particles),
      max_nodes_(max_particles * 2),
      node_count_(0),
      max_depth_(0) {}

BarnesHutTree::~BarnesHutTree() { release(this); }

namespace {
// The tree the reference's tests inspect: its own insertion tree (2N node
// budget included) up to the reference-tree limit, the canonical device
// tree above it (the two agree whenever the budget does not fire).
nbgb_params tree_params(size_t count, float G = 1.0f, float eps = 0.1f) {
  nbgb_params p = params_of(G, eps);
  if (count <= 65536) p.flags |= NBGB_FLAG_REFERENCE_TREE;
  return p;
}
}  // namespace

void BarnesHutTree::build(const ParticleData* d_particles) {
  NBODY_PROFILE_SCOPE("barnes_hut.build");
  nbgb_calculator* c = handle(this, NBGB_BARNES_HUT, tree_params(d_particles->count));
  build_into_scratch(c, d_particles);
  int32_t nc = 0, md = 0;
  check(nbgb_bh_tree_stats(c, &nc, &md));
  node_count_ = nc;
  max_depth_ = md;
}

void BarnesHutTree::computeForces(ParticleData* d_particles, float theta, float G, float eps) {
  nbgb_params p = tree_params(d_particles->count, G, eps);
  p.theta = theta;
  check(nbgb_compute_forces(handle(this, NBGB_BARNES_HUT, p), view(d_particles)));
}

void BarnesHutTree::copyNodesToHost() {
  nbgb_calculator* c = handle(this, NBGB_BARNES_HUT, tree_params(max_particles_));
  h_nodes_.resize((size_t)std::max(node_count_, 1));
  check(nbgb_bh_copy_nodes(c, reinterpret_cast<nbgb_octree_node*>(h_nodes_.data()),
                           h_nodes_.size()));
}

bool BarnesHutTree::verifyMassConservation(const ParticleData* h_particles) const {
  float total = 0.0f;
  for (size_t i = 0; i < h_particles->count; i++) total += h_particles->mass[i];
  return !h_nodes_.empty() && std::abs(total - h_nodes_[0].total_mass) < 0.001f * total;
}

SpatialHashGrid::SpatialHashGrid(size_t max_particles, float cell_size)
    : d_cell_start_(nullptr),
      d_cell_end_(nullptr),
      d_particle_cell_(nullptr),
      d_sorted_indices_(nullptr),
      d_cell_counts_(nullptr),
      max_particles_(max_particles),
      cell_size_(cell_size),
      total_cells_(0) {
  grid_dims_ = make_int3(0, 0, 0);
}

SpatialHashGrid::~SpatialHashGrid() { release(this); }

int3 SpatialHashGrid::getCellIndex(float x, float y, float z, float cell_size) {
  return make_int3(static_cast<int>(std::floor(x / cell_size)),
                   static_cast<int>(std::floor(y / cell_size)),
                   static_cast<int>(std::floor(z / cell_size)));
}

void SpatialHashGrid::build(const ParticleData* d_particles) {
  nbgb_params p = params_of(1.0f, 0.1f);
  p.cell_size = cell_size_;
  p.cutoff = cell_size_;
  nbgb_calculator* c = handle(this, NBGB_SPATIAL_HASH, p);
  build_into_scratch(c, d_particles);
  int32_t dims[3];
  float bmin[3], cell = 0.f;
  int64_t total = 0;
  check(nbgb_hash_grid_info(c, dims, bmin, &cell, &total));
  grid_dims_ = make_int3(dims[0], dims[1], dims[2]);
  total_cells_ = static_cast<int>(total);
  bbox_min_ = Vec3(bmin[0], bmin[1], bmin[2]);
}

void SpatialHashGrid::computeForces(ParticleData* d_particles, float cutoff, float G, float eps) {
  nbgb_params p = params_of(G, eps);
  p.cell_size = cell_size_;
  p.cutoff = cutoff;
  check(nbgb_compute_forces(handle(this, NBGB_SPATIAL_HASH, p), view(d_particles)));
}

void SpatialHashGrid::copyCellDataToHost(std::vector<int>& cell_start, std::vector<int>& cell_end,
                                         std::vector<int>& particle_cells,
                                         std::vector<int>& sorted_indices) {
  nbgb_calculator* c = handle(this, NBGB_SPATIAL_HASH, params_of(1.0f, 0.1f));
  cell_start.resize((size_t)total_cells_);
  cell_end.resize((size_t)total_cells_);
  particle_cells.resize(max_particles_);
  sorted_indices.resize(max_particles_);
  check(nbgb_hash_copy_cells(c, cell_start.data(), cell_end.data(), particle_cells.data(),
                             sorted_indices.data()));
}

bool SpatialHashGrid::verifyCellAssignment(const ParticleData* h) const {
  for (size_t i = 0; i < h->count; i++) {
    int3 c = getCellIndex(h->pos_x[i] - bbox_min_.x, h->pos_y[i] - bbox_min_.y,
                          h->pos_z[i] - bbox_min_.z, cell_size_);
    c.x = std::max(0, std::min(c.x, grid_dims_.x - 1));
    c.y = std::max(0, std::min(c.y, grid_dims_.y - 1));
    c.z = std::max(0, std::min(c.z, grid_dims_.z - 1));
    const float x0 = bbox_min_.x + c.x * cell_size_, y0 = bbox_min_.y + c.y * cell_size_,
                z0 = bbox_min_.z + c.z * cell_size_;
    if (h->pos_x[i] < x0 || h->pos_x[i] > x0 + cell_size_ || h->pos_y[i] < y0 ||
        h->pos_y[i] > y0 + cell_size_ || h->pos_z[i] < z0 || h->pos_z[i] > z0 + cell_size_)
      return false;
  }
  return true;
}

// --------------------------------------------------------- integrator --
void launchUpdatePositionsKernel(ParticleData* d, float dt, int) {
  check(nbgb_update_positions(view(d), dt, nullptr));
}
void launchUpdateVelocitiesKernel(ParticleData* d, float dt, int) {
  check(nbgb_update_velocities(view(d), dt, nullptr));
}
void launchStoreAccelerationsKernel(ParticleData* d, int) {
  check(nbgb_store_old_accelerations(view(d), nullptr));
}

namespace {
// ParticleData whose FP64 state an integrator keeps (released with it).
std::unordered_map<const Integrator*, std::vector<ParticleData*>> g_integrated;

// NBGB_FP32_VERLET=1: the reference's FP32 update kernels instead of the
// FP64 state.
bool fp32_verlet() {
  const char* v = std::getenv("NBGB_FP32_VERLET");
  return v && v[0] == '1';
}
}  // namespace

Integrator::Integrator(int block_size) : block_size_(block_size) {}
Integrator::~Integrator() {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_integrated.find(this);
  if (it == g_integrated.end()) return;
  for (ParticleData* d : it->second) nbgb_state_release(view(d));
  g_integrated.erase(it);
}
void Integrator::ensureScratchBuffer(size_t) {}  // reductions need no caller-visible scratch

// Velocity Verlet (integrator.cu:175-189) with x and v kept in FP64 between
// steps; the FP32 ParticleData is the rounded state after every step.
void Integrator::integrate(ParticleData* d, ForceCalculator* force_calc, float dt) {
  NBODY_PROFILE_SCOPE("integrator.velocity_verlet");
  if (fp32_verlet()) {
    storeOldAccelerations(d);
    updatePositions(d, dt);
    force_calc->computeForces(d);
    updateVelocities(d, dt);
    return;
  }
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto& v = g_integrated[this];
    if (std::find(v.begin(), v.end(), d) == v.end()) v.push_back(d);
  }
  check(nbgb_state_kick_drift(view(d), dt, nullptr));
  force_calc->computeForces(d);
  check(nbgb_state_kick(view(d), dt, nullptr));
}
void Integrator::updatePositions(ParticleData* d, float dt) {
  launchUpdatePositionsKernel(d, dt, block_size_);
}
void Integrator::updateVelocities(ParticleData* d, float dt) {
  launchUpdateVelocitiesKernel(d, dt, block_size_);
}
void Integrator::storeOldAccelerations(ParticleData* d) {
  launchStoreAccelerationsKernel(d, block_size_);
}
float Integrator::computeKineticEnergy(const ParticleData* d) {
  double ke = 0.0;
  check(nbgb_kinetic_energy(reinterpret_cast<const nbgb_particle_data*>(d), &ke, nullptr));
  return static_cast<float>(ke);
}
float Integrator::computePotentialEnergy(const ParticleData* d, float G, float eps) {
  double pe = 0.0;
  check(nbgb_potential_energy(reinterpret_cast<const nbgb_particle_data*>(d), G, eps, &pe,
                              nullptr));
  return static_cast<float>(pe);
}
float Integrator::computeTotalEnergy(const ParticleData* d, float G, float eps) {
  return computeKineticEnergy(d) + computePotentialEnergy(d, G, eps);
}

}  // namespace nbody
