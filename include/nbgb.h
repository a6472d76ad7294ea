/*
 * nbgb.h -- C ABI of the GB300 (sm_103a) force-and-integrate library.
 *
 * This is the drop-in boundary for the reference's `include/nbody` hot path.
 * Every entry point cites the reference interface it replaces (paths are
 * relative to the reference project root).  Plain C types only: device
 * pointers are `float*` in the caller's address space, streams are
 * `cudaStream_t` passed as `void*` (NULL = the library's own stream), and no
 * C++ exception crosses this boundary -- every call returns an nbgb_status
 * and leaves a message in nbgb_last_error().  The C++ adapter in
 * nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp defines the reference's
 * classes over this ABI and rethrows the reference's exception types.
 *
 * Threading: a calculator, system or ensemble handle must be used by one
 * host thread at a time (the reference's ParticleSystem is documented "Not
 * thread-safe", include/nbody/particle_system.hpp:13).  Distinct handles may
 * be used concurrently from different threads.
 */
#ifndef NBGB_H
#define NBGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBGB_ABI_VERSION 2

/* Status codes.  The C++ adapter maps them to the reference's exceptions
 * (include/nbody/error_handling.hpp): INVALID_ARG -> ValidationException
 * (:98-102), OOM -> ResourceException (:76-95), CUDA -> CudaException
 * (:29-51), OVERFLOW -> std::runtime_error as thrown for an oversize grid
 * (src/cuda/force_spatial_hash.cu:258-260). */
typedef enum nbgb_status {
  NBGB_OK = 0,
  NBGB_ERR_INVALID_ARG = 1,
  NBGB_ERR_OOM = 2,
  NBGB_ERR_CUDA = 3,
  NBGB_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up */
  NBGB_ERR_OVERFLOW = 5,       /* grid above 1e8 cells, or a capacity the device exceeded */
  NBGB_ERR_NOT_READY = 6,      /* asynchronous result not available yet */
  NBGB_ERR_NO_DEVICE = 7
} nbgb_status;

/* == nbody::ForceMethod (include/nbody/types.hpp:35), same numeric values,
 * which are also the values stored in the checkpoint header. */
typedef enum nbgb_method {
  NBGB_DIRECT_N2 = 0,
  NBGB_BARNES_HUT = 1,
  NBGB_SPATIAL_HASH = 2
} nbgb_method;

/* == nbody::ParticleData (include/nbody/types.hpp:96-131): 13 separate FP32
 * arrays and a count, same member order, so a `nbody::ParticleData*` can be
 * passed where a `nbgb_particle_data*` is expected. */
typedef struct nbgb_particle_data {
  float* pos_x;
  float* pos_y;
  float* pos_z;
  float* vel_x;
  float* vel_y;
  float* vel_z;
  float* acc_x;
  float* acc_y;
  float* acc_z;
  float* acc_old_x;
  float* acc_old_y;
  float* acc_old_z;
  float* mass;
  size_t count;
} nbgb_particle_data;

/* Parameters of a force calculator.  Defaults (nbgb_params_default) are the
 * reference's SimulationConfig defaults (include/nbody/types.hpp:133-144)
 * and ForceCalculator members (include/nbody/force_calculator.hpp:22-25). */
typedef struct nbgb_params {
  float G;                /* ForceCalculator::setGravitationalConstant (force_calculator.hpp:19) */
  float softening;        /* ForceCalculator::setSofteningParameter (:15-18); eps^2 derived */
  float theta;            /* BarnesHutCalculator(theta), setTheta (:43,47) */
  float cell_size;        /* SpatialHashCalculator(cell_size, cutoff), setCellSize (:60,64) */
  float cutoff;           /* setCutoffRadius (:65) */
  int32_t block_size;     /* DirectForceCalculator(block_size) (:31); accepted, the
                             library chooses its own tiling */
  int32_t leaf_capacity;  /* Barnes-Hut bucket size: 1 = the reference tree and walk
                             (one body per leaf); 2..16 = subtrees with at most this
                             many bodies are summed body by body when opened (both
                             walks) */
  uint32_t flags;         /* NBGB_FLAG_* */
  int32_t group_size;     /* group walk: largest group, 32 or 64 bodies; 0 (default) =
                             by the body count (nbgb_bh_group_size) */
} nbgb_params;

/* Synchronize the calculator's stream at the end of each call and report any
 * device-side error word (reference semantics: callers read results right
 * after computeForces).  Clear it to enqueue asynchronously and check with
 * nbgb_calculator_synchronize(). */
#define NBGB_FLAG_SYNC 0x1u
/* Per-target compensated (two-sum) accumulation across j-tiles.  Clear it
 * for the plain FP32 sum (one running FP32 accumulator, as the reference). */
#define NBGB_FLAG_COMPENSATED 0x2u
/* Record per-target accepted-interaction counts (Barnes-Hut) or neighbour
 * counts (spatial hash) for nbgb_copy_interaction_counts(). */
#define NBGB_FLAG_COUNT_INTERACTIONS 0x4u
/* nbgb_system over a direct calculator: forces in FP64 from the FP64 state,
 * accelerations kept in FP64 (the full-FP64 reference variant; FP64
 * arithmetic runs at a small fraction of the FP32 rate on GB300). */
#define NBGB_FLAG_FP64 0x8u
/* Barnes-Hut group walk: the bodies of each small subtree (at most 32 or 64,
 * nbgb_params.group_size; consecutive small sibling subtrees merged) share
 * one interaction list; a
 * cell is accepted for the group when its cube does not touch the group's
 * bounding box and 4h^2 < theta^2 (d^2 + eps^2), d the distance from the
 * cell's centre of mass to the box.  Every accepted cell passes the
 * reference's per-target test for every body of the group, so the force
 * error is at most that of the reference walk at the same theta; the
 * interaction sets differ from the reference's.  With leaf_capacity > 1 a
 * node of at most that many bodies that is not accepted adds its bodies to
 * the list instead of being opened (buckets). */
#define NBGB_FLAG_GROUP_WALK 0x10u
/* Barnes-Hut: build the tree exactly as the reference's host build does,
 * including its node budget of 2N (BarnesHutTree::buildTreeOnHost,
 * force_barnes_hut.cu:391-543): once a split could overrun it, later bodies
 * merge into existing leaves.  The default device build makes the canonical
 * octree, which equals the reference's whenever the budget does not fire
 * (in practice from about 100 bodies on).  With this flag the reference's
 * insertion is replayed by one device thread where the trees can differ --
 * with NBGB_FLAG_SYNC only when the canonical tree has at least 2N - 33
 * nodes (otherwise it is the reference's tree), without it always -- for
 * systems of at most 65,536 bodies, with the reference walk (no group walk,
 * leaf_capacity 1).  The drop-in adapter sets it. */
#define NBGB_FLAG_REFERENCE_TREE 0x20u
/* Record the device time of each stage of every force evaluation (CUDA
 * events on the calculator's stream) for nbgb_calculator_stage_times.
 * Stages: direct.forces; barnes_hut.bounds, .keys, .sort, .order, .nodes,
 * .com, .walk (.reference_tree with NBGB_FLAG_REFERENCE_TREE);
 * spatial_hash.bounds, .assign, .sort, .cells, .forces.  The SURVEY-style
 * counterpart of the reference's NBODY_PROFILE_SCOPE phases
 * (performance_observability.hpp:70-78), measured on the device. */
#define NBGB_FLAG_STAGE_TIMINGS 0x40u

/* The largest group of the group walk that a calculator with group_size 0
 * uses for `count` bodies: 32, or 64 from 262,144 bodies on (each lane of a
 * group's warp then sums two bodies; below that, half as many groups would
 * leave SMs idle).  The ensemble always uses 64, so that a system's result
 * does not depend on what else is resident.  Host-only; no reference
 * counterpart. */
int32_t nbgb_bh_group_size(uint64_t count);

void nbgb_params_default(nbgb_params* p);

/* ---------------------------------------------------------------------------
 * Force calculators: nbody::ForceCalculator and its three subclasses
 * (include/nbody/force_calculator.hpp:8-74) and the factory
 * createForceCalculator (:76-77, body src/cuda/force_spatial_hash.cu:391-404).
 * ------------------------------------------------------------------------- */
typedef struct nbgb_calculator nbgb_calculator;

nbgb_status nbgb_calculator_create(nbgb_method method, const nbgb_params* params,
                                   nbgb_calculator** out);
nbgb_status nbgb_calculator_destroy(nbgb_calculator* calc);
nbgb_status nbgb_calculator_set_params(nbgb_calculator* calc, const nbgb_params* params);
nbgb_status nbgb_calculator_get_params(const nbgb_calculator* calc, nbgb_params* params);
/* Device time per stage of the force evaluations made with
 * NBGB_FLAG_STAGE_TIMINGS since it was set or since the last reset: waits for
 * the calculator's stream, then fills up to `capacity` entries -- stage name
 * (NUL-terminated, in names + 32 * i), total milliseconds, number of times
 * the stage ran -- and sets *count to the number of stages (which may exceed
 * capacity).  reset != 0 clears the totals afterwards.  No reference
 * counterpart (its phase timer measures host enqueue time). */
nbgb_status nbgb_calculator_stage_times(nbgb_calculator* calc, int32_t capacity, char* names,
                                        double* total_ms, int64_t* samples, int32_t* count,
                                        int32_t reset);
/* ForceCalculator::getMethod (force_calculator.hpp:13) */
nbgb_status nbgb_calculator_get_method(const nbgb_calculator* calc, nbgb_method* method);
/* All work of the calculator is enqueued on this stream (NULL: a stream the
 * library creates for the calculator). */
nbgb_status nbgb_calculator_set_stream(nbgb_calculator* calc, void* cuda_stream);
/* Waits for the calculator's stream and reports device-side error words. */
nbgb_status nbgb_calculator_synchronize(nbgb_calculator* calc);

/* ForceCalculator::computeForces (force_calculator.hpp:12; direct
 * src/cuda/force_direct.cu:103-106, Barnes-Hut force_barnes_hut.cu:577-583,
 * spatial hash force_spatial_hash.cu:376-388).  Reads pos_x/y/z and mass,
 * OVERWRITES acc_x/y/z, touches nothing else.  Device pointers. */
nbgb_status nbgb_compute_forces(nbgb_calculator* calc, const nbgb_particle_data* d_particles);

/* Direct-sum forces that allocate no device memory (no counterpart in the
 * reference).  For callers that may not call cudaMalloc/cudaFree -- e.g. a
 * host application that owns all device memory through its own pool, or a
 * latency-critical loop that cannot afford cudaMalloc's implicit device
 * synchronisation.  Same contract as nbgb_compute_forces with a direct
 * calculator of the given G and softening: reads pos_x/y/z and mass, writes
 * acc_x/y/z (device pointers), compensated FP32 sums.  Limit: count <=
 * 65536 (larger counts return NBGB_ERR_INVALID_ARG).  Scratch is ~9 MiB of
 * static device memory per device, held until exit.  With lazy module
 * loading (the default of recent CUDA releases) the first call on a device
 * reserves it and resolves its address, so that call may synchronise the
 * device or fail with NBGB_ERR_OOM; a warm-up call with count 0 does exactly
 * that and nothing else.  cudaDeviceReset after the first call on a device
 * is not supported.  The call cannot run while `stream` is being captured
 * (it returns NBGB_ERR_INVALID_ARG): it reads a device error word back and
 * waits for the stream.  All calls share the scratch: calls that overlap on
 * the GPU race and must be serialised by the caller.  Work is enqueued on
 * `stream` (NULL = legacy default stream) and the call waits for it. */
nbgb_status nbgb_compute_forces_direct_noalloc(const nbgb_particle_data* d_particles, float G,
                                               float softening, void* stream);

/* ---------------------------------------------------------------------------
 * Integrator (include/nbody/integrator.hpp:15-33, src/cuda/integrator.cu).
 * FP32 SoA semantics of the reference; device pointers.
 * ------------------------------------------------------------------------- */
/* Integrator::integrate (integrator.cu:175-189): a_old = a; x += v dt +
 * a dt^2/2; a = F(x) via calc; v += (a_old + a) dt/2.  Runs on calc's stream. */
nbgb_status nbgb_integrate(nbgb_calculator* calc, const nbgb_particle_data* d_particles, float dt);
/* Integrator::updatePositions / updateVelocities / storeOldAccelerations
 * (integrator.cu:191-201). */
nbgb_status nbgb_update_positions(const nbgb_particle_data* d_particles, float dt, void* stream);
nbgb_status nbgb_update_velocities(const nbgb_particle_data* d_particles, float dt, void* stream);
nbgb_status nbgb_store_old_accelerations(const nbgb_particle_data* d_particles, void* stream);
/* Integrator::computeKineticEnergy / computePotentialEnergy
 * (integrator.cu:203-240), reduced in FP64 and returned as double (the
 * reference returns the FP32 sum of per-block FP32 partials).  Synchronous. */
nbgb_status nbgb_kinetic_energy(const nbgb_particle_data* d_particles, double* ke, void* stream);
nbgb_status nbgb_potential_energy(const nbgb_particle_data* d_particles, float G, float eps,
                                  double* pe, void* stream);

/* FP64-state Velocity Verlet behind the reference's FP32 ParticleData, for
 * ParticleSystem::update (src/core/particle_system.cpp:122-136) through
 * Integrator::integrate (integrator.cu:175-189).  The library keeps x and v
 * of each ParticleData (keyed by its pos_x device pointer) in FP64 across
 * steps; one step is
 *   nbgb_state_kick_drift:  acc_old = acc; v += acc dt/2 and x += v dt in
 *                           FP64; pos = (float) x
 *   (the caller's forces on pos -> acc)
 *   nbgb_state_kick:        v += acc dt/2 in FP64; vel = (float) v
 * -- the reference's update algebraically, with FP64 state.  After every
 * step pos and vel are the rounded FP64 state.  An element whose FP32 value
 * differs from its rounded FP64 value was changed by the caller and is taken
 * over as the new state.  Enqueued on `stream` (NULL = legacy stream).
 * nbgb_state_release frees a ParticleData's FP64 state (synchronises). */
nbgb_status nbgb_state_kick_drift(const nbgb_particle_data* d_particles, float dt, void* stream);
nbgb_status nbgb_state_kick(const nbgb_particle_data* d_particles, float dt, void* stream);
nbgb_status nbgb_state_release(const nbgb_particle_data* d_particles);

/* ---------------------------------------------------------------------------
 * ParticleDataManager (include/nbody/particle_data.hpp:9-28,
 * src/cuda/particle_init.cu:11-160): 13 separate device arrays, acc and
 * acc_old zeroed; copies move pos, vel, acc and mass (not acc_old), as the
 * reference does (particle_init.cu:134-160).
 * ------------------------------------------------------------------------- */
nbgb_status nbgb_particles_alloc_device(nbgb_particle_data* d, size_t count);
nbgb_status nbgb_particles_free_device(nbgb_particle_data* d);
nbgb_status nbgb_particles_copy_to_device(nbgb_particle_data* d, const nbgb_particle_data* h);
nbgb_status nbgb_particles_copy_to_host(nbgb_particle_data* h, const nbgb_particle_data* d);

/* ---------------------------------------------------------------------------
 * Initial conditions generated on the device (ParticleInitializer::initUniform
 * / initSpherical / initDisk, src/cuda/particle_init.cu:167-234, generate on
 * the host; these write straight into device arrays).  Same formulas as the
 * reference plus a Plummer sphere; the random stream is a counter-based
 * generator (deterministic per seed, independent of the launch shape), not
 * the reference's std::mt19937 sequence.  acc and acc_old are zeroed.
 * Synchronous on `stream`.
 * ------------------------------------------------------------------------- */
typedef enum nbgb_distribution {
  NBGB_DIST_UNIFORM = 0,
  NBGB_DIST_SPHERICAL = 1,
  NBGB_DIST_DISK = 2,
  NBGB_DIST_PLUMMER = 3
} nbgb_distribution;

typedef struct nbgb_init_params {
  int32_t distribution;   /* nbgb_distribution */
  float center[3];        /* spherical, disk, Plummer */
  float radius;           /* spherical, disk */
  float min_bounds[3];    /* uniform */
  float max_bounds[3];
  float min_mass;         /* uniform, spherical, disk: mass uniform in [min, max] */
  float max_mass;
  float thickness;        /* disk */
  float rotation_speed;   /* disk: v = rotation_speed * sqrt(r) */
  float plummer_a;        /* Plummer scale radius, total mass, G (equal masses M/N) */
  float total_mass;
  float G;
} nbgb_init_params;

/* Parameters ParticleSystem::initialize uses (particle_system.cpp:77-101):
 * box [-10, 10]^3, ball / disk radius 10, thickness 1, rotation 0.5, mass 1;
 * Plummer a = 1, M = 1, G = 1. */
void nbgb_init_params_default(nbgb_init_params* p, int32_t distribution);
nbgb_status nbgb_init_particles_device(nbgb_particle_data* d_particles, const nbgb_init_params* p,
                                       uint64_t seed, void* stream);

/* ---------------------------------------------------------------------------
 * Inspection for parity tests: what the reference exposes through
 * BarnesHutTree (include/nbody/barnes_hut_tree.hpp:38-91) and SpatialHashGrid
 * (include/nbody/spatial_hash_grid.hpp:9-62).  Host output buffers; each call
 * synchronizes.  Valid after the calculator's last nbgb_compute_forces.
 * ------------------------------------------------------------------------- */

/* == nbody::OctreeNode (include/nbody/barnes_hut_tree.hpp:9-30), 76 bytes. */
typedef struct nbgb_octree_node {
  float center[3];
  float half_size;
  float center_of_mass[3];
  float total_mass;
  int32_t children[8];
  int32_t particle_index;
  uint8_t is_leaf;
  uint8_t pad_[3];
  int32_t particle_count;
} nbgb_octree_node;

/* BarnesHutTree::getNodeCount / getMaxDepth (barnes_hut_tree.hpp:57-58). */
nbgb_status nbgb_bh_tree_stats(nbgb_calculator* calc, int32_t* node_count, int32_t* max_depth);
/* The (Morton key, particle index) pairs after the stable sort
 * (force_barnes_hut.cu:308-328); n = particle count. */
nbgb_status nbgb_bh_copy_sorted_keys(nbgb_calculator* calc, uint32_t* keys, int32_t* indices,
                                     size_t n);
/* The tree in the reference node layout (BarnesHutTree::copyNodesToHost,
 * force_barnes_hut.cu:557-560).  Node 0 is the root; nodes are numbered in
 * depth-first pre-order (the reference numbers in insertion order), children
 * hold node indices, -1 for empty octants. */
nbgb_status nbgb_bh_copy_nodes(nbgb_calculator* calc, nbgb_octree_node* nodes, size_t capacity);
/* SpatialHashGrid::getGridDims / getCellSize / getTotalCells
 * (spatial_hash_grid.hpp:25-27) plus the padded bbox minimum. */
nbgb_status nbgb_hash_grid_info(nbgb_calculator* calc, int32_t dims[3], float bbox_min[3],
                                float* cell_size, int64_t* total_cells);
/* SpatialHashGrid::copyCellDataToHost (force_spatial_hash.cu:324-340).
 * Within a cell, particles are in ascending index order. */
nbgb_status nbgb_hash_copy_cells(nbgb_calculator* calc, int32_t* cell_start, int32_t* cell_end,
                                 int32_t* particle_cells, int32_t* sorted_indices);
/* Per-target accepted interactions (Barnes-Hut) or neighbours within the
 * cutoff (spatial hash), recorded under NBGB_FLAG_COUNT_INTERACTIONS. */
nbgb_status nbgb_copy_interaction_counts(nbgb_calculator* calc, int32_t* counts, size_t n);

/* ---------------------------------------------------------------------------
 * Device-resident simulation with FP64 position/velocity state: the fast
 * path under ParticleSystem::update (src/core/particle_system.cpp:122-136).
 * Kick-drift-kick (algebraically the reference's Velocity Verlet,
 * src/cuda/integrator.cu:175-189) with x, v in FP64 and FP32 forces (FP64
 * forces from the FP64 state when the calculator has NBGB_FLAG_FP64).
 * ------------------------------------------------------------------------- */
typedef struct nbgb_system nbgb_system;

/* Copies the initial state from HOST arrays (pos, vel, mass of h) and
 * computes a(0) with calc (ParticleSystem::finishInitialization,
 * particle_system.cpp:45-61).  The system keeps a reference to calc. */
nbgb_status nbgb_system_create(nbgb_calculator* calc, const nbgb_particle_data* h_init,
                               nbgb_system** out);
nbgb_status nbgb_system_destroy(nbgb_system* sys);
/* `steps` Velocity-Verlet steps of size dt (ParticleSystem::update x steps). */
nbgb_status nbgb_system_step(nbgb_system* sys, float dt, int32_t steps);
/* FP32 view into HOST arrays (pos, vel, acc, mass; acc_old untouched):
 * ParticleSystem::copyToHost / getState (particle_system.cpp:228-253). */
nbgb_status nbgb_system_read(nbgb_system* sys, nbgb_particle_data* h_out);
/* FP64 state into host arrays (any pointer may be NULL). */
nbgb_status nbgb_system_read_f64(nbgb_system* sys, double* x, double* y, double* z, double* vx,
                                 double* vy, double* vz);
/* FP64 energy and momentum from the FP64 state: KE = sum m v^2/2, PE =
 * -sum_{i<j} G m_i m_j / sqrt(r^2 + eps^2) (integrator.cu:52-120; O(N^2), in
 * FP64 arithmetic up to 2^18 bodies, above that FP32 pair terms with FP64
 * accumulation), P = sum m v. */
nbgb_status nbgb_system_energy(nbgb_system* sys, double* ke, double* pe, double momentum[3]);

/* ---------------------------------------------------------------------------
 * Checkpoints (Serializer::save / load, src/utils/serialization.cpp:25-75):
 * the reference's .nbody v1 file, byte-identical to its writer's, written
 * from and read into device memory through one pinned file image (one write
 * or read per file).  nbgb_system_save can add an FP64 sidecar <path>.f64
 * (32-byte header: magic 0x4E424638, version 2, u64 count, 16 zero bytes;
 * then float64 x, y, z, vx, vy, vz); nbgb_system_load restores the FP64
 * state from it when every value rounds to the v1 file's float32 value
 * (*restored_f64 = 1), so a restarted run continues bitwise where the saved
 * one stood.  Load errors carry the reference's messages.
 * ------------------------------------------------------------------------- */
typedef struct nbgb_checkpoint_header {
  uint64_t particle_count;   /* set by the loaders; ignored on save (the data's count) */
  float simulation_time;
  float dt;
  float G;
  float softening;
  uint32_t force_method;     /* nbgb_method */
} nbgb_checkpoint_header;

/* d_particles: device arrays pos, vel, mass. */
nbgb_status nbgb_checkpoint_save_device(const char* path, const nbgb_particle_data* d_particles,
                                        const nbgb_checkpoint_header* hdr, void* stream);
/* d_particles->count must equal the file's count; d_particles == NULL reads
 * the header only. */
nbgb_status nbgb_checkpoint_load_device(const char* path, nbgb_particle_data* d_particles,
                                        nbgb_checkpoint_header* hdr, void* stream);
/* Saves the system's state (velocities synchronised to its positions). */
nbgb_status nbgb_system_save(nbgb_system* sys, const char* path,
                             const nbgb_checkpoint_header* hdr, int32_t with_f64);
/* A new system on calc from a checkpoint (a(0) computed as in
 * nbgb_system_create). */
nbgb_status nbgb_system_load(nbgb_calculator* calc, const char* path, nbgb_system** out,
                             nbgb_checkpoint_header* hdr, int32_t* restored_f64);

/* ---------------------------------------------------------------------------
 * Ensemble serving (no reference counterpart; the reference runs one
 * ParticleSystem at a time).  Many independent simulations share the GPU:
 * requests are admitted while the HBM budget and the resident cap allow,
 * every resident system advances one Velocity-Verlet step per tick (FP64
 * x/v state, FP32 forces: direct sum for N <= direct_max_n through one
 * persistent work-queue kernel spanning all direct systems; Barnes-Hut for
 * all resident systems as one segmented tree build, captured as a CUDA graph
 * once the resident set is stable, and one batched walk on a side stream),
 * and finished systems retire and free their memory.  The result of a system does not depend on what else
 * is resident (per-system work decomposition), except through the direct
 * kernel configuration the autotuner picks (rounding-level differences).
 * ------------------------------------------------------------------------- */
typedef struct nbgb_ensemble nbgb_ensemble;

typedef struct nbgb_ensemble_config {
  uint64_t hbm_budget_bytes; /* admission budget for system state and trees */
  int32_t max_resident;      /* cap on simultaneously resident systems */
  int32_t direct_max_n;      /* N <= direct_max_n: direct sum, else Barnes-Hut */
  float G;
  float softening;           /* must be > 0 */
  float theta;               /* Barnes-Hut opening angle */
  int32_t leaf_capacity;     /* Barnes-Hut bucket size (1 = reference tree walk) */
  int32_t direct_config;     /* direct kernel configuration; -1 = autotune */
  int32_t use_graphs;        /* run the batched Barnes-Hut pass as a CUDA graph while the
                                set of resident Barnes-Hut systems is unchanged */
  int32_t group_walk;        /* 1 (default) = Barnes-Hut group walk (NBGB_FLAG_GROUP_WALK);
                                0 = the reference's per-target walk */
} nbgb_ensemble_config;

/* One finished request. */
typedef struct nbgb_ensemble_result {
  uint64_t request_id;
  int64_t count;
  int32_t steps;
  int32_t method;        /* nbgb_method used */
  double gpu_ms;         /* tick time from admission to retirement */
} nbgb_ensemble_result;

typedef struct nbgb_ensemble_stats {
  int64_t ticks;
  int64_t particle_steps;       /* sum over ticks of resident bodies */
  double direct_interactions;   /* sum of N (N - 1) over direct system-steps */
  double bh_interactions;       /* interactions summed by the Barnes-Hut walks (device
                                   count; group walk: list lengths minus one per body of
                                   nonzero mass) */
  int64_t admitted;
  int64_t retired;
  int32_t resident;
  int32_t queued;
  uint64_t bytes_reserved;      /* against hbm_budget_bytes */
  int32_t direct_config;        /* configuration in use */
  int32_t tuning;               /* 1 while the autotuner is measuring */
  double direct_kernel_ms;      /* summed device time of the direct work-queue kernel */
  double direct_kernel_interactions; /* interactions those launches computed */
  int64_t kernel_launches;      /* kernels launched by ticks (graph kernel nodes counted) */
  double bh_walk_ms;            /* summed device time of the batched Barnes-Hut walk */
  int64_t bh_bodies;            /* bodies in the current Barnes-Hut segments */
} nbgb_ensemble_stats;

void nbgb_ensemble_config_default(nbgb_ensemble_config* cfg);
nbgb_status nbgb_ensemble_create(const nbgb_ensemble_config* cfg, nbgb_ensemble** out);
nbgb_status nbgb_ensemble_destroy(nbgb_ensemble* ens);
/* Queue a simulation: HOST pos/vel/mass arrays of h_init, `steps` steps of
 * size dt.  The arrays are copied; the call does not touch the GPU. */
nbgb_status nbgb_ensemble_submit(nbgb_ensemble* ens, const nbgb_particle_data* h_init,
                                 int32_t steps, float dt, uint64_t* request_id);
/* Admit what fits, advance every resident system one step, retire the
 * finished ones (their results become pollable when their copies land). */
nbgb_status nbgb_ensemble_tick(nbgb_ensemble* ens, int32_t* resident, int32_t* queued);
/* Pop one finished request.  Returns NBGB_ERR_NOT_READY when none is
 * available.  If h_out is non-NULL and h_out->count (the capacity of its
 * host arrays) is at least result->count, its non-NULL pos/vel/acc/mass
 * arrays receive the final FP32 state (acc = the acceleration at the final
 * positions); state_f64 (6*count doubles x, y, z, vx, vy, vz, or NULL) the
 * FP64 state.  The engine reads results back into pinned host buffers that
 * it recycles after the poll (at most 256 MiB kept idle, all freed by
 * nbgb_ensemble_destroy); the caller's arrays may be pageable. */
nbgb_status nbgb_ensemble_poll(nbgb_ensemble* ens, nbgb_ensemble_result* result,
                               nbgb_particle_data* h_out, double* state_f64);
/* Wait for all retirements in flight. */
nbgb_status nbgb_ensemble_synchronize(nbgb_ensemble* ens);
nbgb_status nbgb_ensemble_get_stats(nbgb_ensemble* ens, nbgb_ensemble_stats* stats);
/* The stream every tick's work joins into (for CUDA-event timing). */
nbgb_status nbgb_ensemble_get_stream(nbgb_ensemble* ens, void** cuda_stream);

/* ---------------------------------------------------------------------------
 * FP64 direct sum on the GPU (the full-FP64 variant of the precision study;
 * no reference counterpart).  Sources: n_src device float4 (x, y, z, m);
 * targets: device indices into the sources (or NULL for all); device double
 * outputs.  Same law as nbgb_compute_forces, self term excluded.
 * ------------------------------------------------------------------------- */
nbgb_status nbgb_direct_f64(const float* d_src_xyzm, int64_t n_src, const int64_t* d_targets,
                            int64_t n_targets, double G, double eps, double* d_ax, double* d_ay,
                            double* d_az, void* stream);

/* ---------------------------------------------------------------------------
 * Diagnostics (no reference counterpart): measured FP32 pipe rates of the
 * current device -- FFMA and packed FFMA2 in TFLOP/s (2 flops per lane-FMA)
 * and MUFU rsqrt in Gop/s -- used as roofline denominators for the force
 * kernels.  Synchronous; any pointer may be NULL.
 * ------------------------------------------------------------------------- */
nbgb_status nbgb_measure_fp32_peak(double* ffma_tflops, double* ffma2_tflops, double* mufu_gops);

/* Failure-detection self-test (no reference counterpart): one thread waits,
 * through the kernels' own bounded mbarrier wait, on a barrier nothing
 * arrives at, giving up after max_iters tries (1 .. 2^20).  Returns
 * NBGB_ERR_DEVICE_TIMEOUT with the device error bits in *error_bits; the
 * context stays usable.  Nothing faults, traps or hangs. */
nbgb_status nbgb_selftest_wait_timeout(uint32_t max_iters, uint32_t* error_bits);

/* Failure injection on the host (no reference counterpart): the nth device
 * allocation the library makes from now on (nth >= 1; 0 switches it off)
 * fails as if the device were out of memory -- the call that needed it
 * returns NBGB_ERR_OOM with its message and nothing is left half-built that
 * a later call would trip over.  Process-wide; nothing reaches the GPU. */
nbgb_status nbgb_selftest_fail_allocation(int32_t nth);

/* Test hook for the Barnes-Hut group walk: the number of shared-memory stack
 * entries (64 .. 512, default 512) a warp uses before it spills the older
 * half of its traversal stack to a global overflow chunk.  Lowering it
 * exercises the spill path on small inputs; when more warps spill in one
 * walk than there are overflow chunks (256), or one warp outgrows its chunk,
 * the walk reports NBGB_ERR_OVERFLOW ("group walk stack overflow") at the
 * next synchronization instead of returning forces.  Process-wide. */
nbgb_status nbgb_selftest_group_walk_stack(int32_t entries);

/* Test hook for nbgb_compute_forces_direct_noalloc: the j-split count the
 * regular direct planner picks for `count` bodies on the current device
 * (*planned_splits) and the count the allocation-free entry point uses after
 * capping it to its static partial-sum scratch (*used_splits, <= 8). */
nbgb_status nbgb_selftest_noalloc_plan(int64_t count, int32_t* planned_splits,
                                       int32_t* used_splits);

/* ---------------------------------------------------------------------------
 * Library information.
 * ------------------------------------------------------------------------- */
/* Message of the last failing call on this thread ("" if none). */
const char* nbgb_last_error(void);
const char* nbgb_version(void);
int32_t nbgb_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NBGB_H */
