// ensemble.cu -- continuous-batching ensemble of independent simulations (K10).
//
// No reference counterpart: the reference runs one ParticleSystem at a time
// (src/core/particle_system.cpp:122-136).  This engine keeps many systems of
// uneven N device-resident and advances all of them per tick:
//
//   arena     one set of SoA arrays (FP64 x, v; FP32 a; FP32 (x,y,z,m)) for
//             all resident systems, carved in 256-body chunks (zero-mass
//             padding to the chunk boundary, so the direct tiles need no
//             bounds test); admission is first-fit within the HBM budget.
//   tick      1. one kick-drift kernel over every resident body (per-system
//                kick: half on the first step, full afterwards);
//             2. Barnes-Hut systems: ONE build + walk over all of them (each
//                system a segment of one key sort; trees and interaction
//                sets per system identical to the single-system path), on
//                a side stream that overlaps the direct kernel; captured as
//                a CUDA graph while the Barnes-Hut resident set is stable;
//             3. direct systems: one persistent kernel whose CTAs pull work
//                items (system, 32..1024-target tile) from a queue spanning
//                all direct systems, largest first;
//             4. retirement: final half kick and an async copy of the state
//                of systems that finished, then their memory is reused.
//   admission a newly admitted system joins the next tick with a zero kick
//             and drift: that tick only computes its a(0) inside the batched
//             passes, so admission launches nothing per system.
//   autotune  the direct kernel's configuration (threads per CTA = warps per
//             tile, targets per thread, scalar or packed FP32x2) is picked
//             by timing every candidate on the current mix; re-tuned when
//             the direct load changes by more than 2x.
#include <algorithm>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "bh.cuh"
#include "common.cuh"
#include "direct_core.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {

constexpr int64_t kChunk = 256;  // arena granularity (== kDirTile)
constexpr int kTimingRing = 8;   // direct-kernel event pairs in flight
// The group walk's largest group in the batched build: fixed, so that a
// system's lists (and results) do not depend on what else is resident; 64
// pays off once the resident Barnes-Hut systems give the walk enough groups.
constexpr int kEnsembleGroupMax = 64;

struct DirectItem {
  int64_t off;  // arena offset of the system
  int32_t n;    // bodies in the system
  int32_t first;  // first target (local index)
};

struct KDBlock {
  int64_t off;  // arena offset of this block's first body
  int32_t count;
  int32_t slot;
};

struct SlotParams {
  double kick;
  double dt;
};

// ----------------------------------------------------------- kernels --
__global__ void ens_kick_drift_kernel(const KDBlock* __restrict__ blocks, int n_blocks,
                                      const SlotParams* __restrict__ sp, double* __restrict__ x,
                                      double* __restrict__ y, double* __restrict__ z,
                                      double* __restrict__ vx, double* __restrict__ vy,
                                      double* __restrict__ vz, const float* __restrict__ ax,
                                      const float* __restrict__ ay, const float* __restrict__ az,
                                      float4* __restrict__ pm) {
  for (int b = blockIdx.x; b < n_blocks; b += gridDim.x) {
    const KDBlock blk = blocks[b];
    if ((int)threadIdx.x >= blk.count) continue;
    const int64_t i = blk.off + threadIdx.x;
    const SlotParams p = sp[blk.slot];
    const double u = fma((double)ax[i], p.kick, vx[i]);
    const double v = fma((double)ay[i], p.kick, vy[i]);
    const double w = fma((double)az[i], p.kick, vz[i]);
    const double px = fma(u, p.dt, x[i]);
    const double py = fma(v, p.dt, y[i]);
    const double pz = fma(w, p.dt, z[i]);
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

// Admission: FP32 host state (staged on the device) -> arena.
__global__ void ens_admit_kernel(const float* __restrict__ stage, int64_t n, int64_t n_pad,
                                 int64_t off, double* __restrict__ x, double* __restrict__ y,
                                 double* __restrict__ z, double* __restrict__ vx,
                                 double* __restrict__ vy, double* __restrict__ vz,
                                 float* __restrict__ ax, float* __restrict__ ay,
                                 float* __restrict__ az, float4* __restrict__ pm) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_pad;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = off + k;
    if (k < n) {
      const float px = stage[k], py = stage[n + k], pz = stage[2 * n + k];
      x[i] = px;
      y[i] = py;
      z[i] = pz;
      vx[i] = stage[3 * n + k];
      vy[i] = stage[4 * n + k];
      vz[i] = stage[5 * n + k];
      pm[i] = make_float4(px, py, pz, stage[6 * n + k]);
    } else {
      x[i] = y[i] = z[i] = vx[i] = vy[i] = vz[i] = 0.0;
      pm[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ax[i] = ay[i] = az[i] = 0.f;
  }
}

template <int THREADS, int I, bool PAIRED>
__global__ void __launch_bounds__(THREADS) ens_direct_kernel(const DirectItem* __restrict__ items,
                                                             int n_items,
                                                             uint32_t* __restrict__ counter,
                                                             const float4* __restrict__ pm,
                                                             float* __restrict__ ax,
                                                             float* __restrict__ ay,
                                                             float* __restrict__ az, float eps2,
                                                             float G, uint32_t* err) {
  __shared__ alignas(128) float4 s_j[kDirStages][kDirTile];
  __shared__ alignas(8) uint64_t s_bar[kDirStages];
  __shared__ int s_item;
  TileRing ring{s_j, s_bar, 0};
  ring_init(ring);
  const int tid = threadIdx.x;
  while (true) {
    if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const DirectItem w = items[it];
    float xi[I], yi[I], zi[I];
#pragma unroll
    for (int q = 0; q < I; ++q) {
      const int li = w.first + tid + q * THREADS;
      const float4 p = (li < w.n) ? pm[w.off + li] : make_float4(0.f, 0.f, 0.f, 0.f);
      xi[q] = p.x;
      yi[q] = p.y;
      zi[q] = p.z;
    }
    float sx[I], sy[I], sz[I];
    const int nt = (int)ceil_div(w.n, kDirTile);
    if (!direct_tiles<THREADS, I, PAIRED, true, false>(ring, pm + w.off, nt, xi, yi, zi, eps2, sx,
                                                       sy, sz, err))
      return;
#pragma unroll
    for (int q = 0; q < I; ++q) {
      const int li = w.first + tid + q * THREADS;
      if (li < w.n) {
        ax[w.off + li] = G * sx[q];
        ay[w.off + li] = G * sy[q];
        az[w.off + li] = G * sz[q];
      }
    }
  }
}

// ----------------------------------------------------- direct configs --
struct DirectConfig {
  int threads;
  int per_thread;
  bool paired;
  const char* name;
};
static const DirectConfig kConfigs[] = {
    {128, 4, false, "t128x4"}, {128, 2, false, "t128x2"}, {64, 4, false, "t64x4"},
    {128, 8, true, "t128x8p"}, {64, 8, true, "t64x8p"},   {256, 2, false, "t256x2"},
};
constexpr int kNumConfigs = sizeof(kConfigs) / sizeof(kConfigs[0]);

template <int T, int I, bool P>
static int occ_of() {
  int b = 0;
  NBGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ens_direct_kernel<T, I, P>, T, 0));
  return std::max(b, 1);
}

static int config_occupancy(int c) {
  switch (c) {
    case 0: return occ_of<128, 4, false>();
    case 1: return occ_of<128, 2, false>();
    case 2: return occ_of<64, 4, false>();
    case 3: return occ_of<128, 8, true>();
    case 4: return occ_of<64, 8, true>();
    default: return occ_of<256, 2, false>();
  }
}

static void launch_config(int c, int grid, const DirectItem* items, int n_items, uint32_t* counter,
                          const float4* pm, float* ax, float* ay, float* az, float eps2, float G,
                          uint32_t* err, cudaStream_t st) {
#define NBGB_ENS_LAUNCH(T, I, P)                                                             \
  ens_direct_kernel<T, I, P><<<grid, T, 0, st>>>(items, n_items, counter, pm, ax, ay, az, eps2, \
                                                 G, err)
  switch (c) {
    case 0: NBGB_ENS_LAUNCH(128, 4, false); break;
    case 1: NBGB_ENS_LAUNCH(128, 2, false); break;
    case 2: NBGB_ENS_LAUNCH(64, 4, false); break;
    case 3: NBGB_ENS_LAUNCH(128, 8, true); break;
    case 4: NBGB_ENS_LAUNCH(64, 8, true); break;
    default: NBGB_ENS_LAUNCH(256, 2, false); break;
  }
#undef NBGB_ENS_LAUNCH
  NBGB_LAUNCH_CHECK();
}

// ------------------------------------------------------------ engine --
struct Request {
  uint64_t id;
  int64_t n;
  int32_t steps;
  float dt;
  std::vector<float> state;  // x, y, z, vx, vy, vz, m (7n)
};

struct ResidentSystem {
  uint64_t id;
  int64_t n;
  int64_t off;
  int64_t n_pad;
  int32_t steps;
  int32_t done = 0;
  float dt;
  int slot;
  nbgb_method method;
  bool fresh = true;          // admitted, a(0) not computed yet
  bool pending_half = false;  // the previous step's closing half kick is still due
  size_t bytes = 0;
  int64_t tick_admitted = 0;
};

// Host-to-device table uploads: the host runs ahead of the device, so a
// pinned source buffer may only be rewritten after the copy that read it
// has executed.  Each upload takes the next of kRing buffers and first waits
// for the event recorded after that buffer's previous copy.
struct UploadRing {
  static constexpr int kRing = 8;
  HostPinned<char> buf[kRing];
  cudaEvent_t ev[kRing] = {};
  bool used[kRing] = {};
  int next = 0;
  int cur = -1;
  void* acquire(size_t bytes) {
    cur = next++ % kRing;
    if (used[cur]) NBGB_CUDA(cudaEventSynchronize(ev[cur]));
    if (!ev[cur]) NBGB_CUDA(cudaEventCreateWithFlags(&ev[cur], cudaEventDisableTiming));
    return buf[cur].ensure(std::max<size_t>(bytes, 1));
  }
  void upload(void* dst, size_t bytes, cudaStream_t st) {
    if (bytes) NBGB_CUDA(cudaMemcpyAsync(dst, buf[cur].ptr, bytes, cudaMemcpyHostToDevice, st));
    mark(st);
  }
  // The current buffer's reader(s) were enqueued on `st` by the caller.
  void mark(cudaStream_t st) {
    NBGB_CUDA(cudaEventRecord(ev[cur], st));
    used[cur] = true;
  }
  ~UploadRing() {
    for (int k = 0; k < kRing; ++k)
      if (ev[k]) cudaEventDestroy(ev[k]);
  }
};

struct Retiring {
  nbgb_ensemble_result res;
  std::unique_ptr<ResidentSystem> sys;
  double* h_state = nullptr;  // pinned: 6n doubles + 3n floats (acc) + n floats (mass)
  size_t h_bytes = 0;         // its capacity (a size class of the pinned pool)
  cudaEvent_t evt = nullptr;
};

// Pinned result buffers are recycled by size class (powers of two from
// 64 KiB): page-locking host memory for every finished request costs about a
// millisecond per megabyte, and cudaFreeHost waits for the device, which
// would drain the tick pipeline at every retirement.
constexpr size_t kPinnedMinBytes = size_t(64) << 10;
constexpr size_t kPinnedPoolMaxBytes = size_t(256) << 20;  // idle buffers kept

struct PinnedPool {
  std::multimap<size_t, void*> idle;  // capacity -> buffer
  size_t idle_bytes = 0;
  void* take(size_t bytes, size_t* cap) {
    size_t c = kPinnedMinBytes;
    while (c < bytes) c <<= 1;
    *cap = c;
    auto it = idle.find(c);
    if (it != idle.end()) {
      void* p = it->second;
      idle.erase(it);
      idle_bytes -= c;
      return p;
    }
    void* p = nullptr;
    NBGB_CUDA(cudaMallocHost(&p, c));
    return p;
  }
  void give(void* p, size_t cap) {
    if (!p) return;
    if (idle_bytes + cap > kPinnedPoolMaxBytes) {
      cudaFreeHost(p);
      return;
    }
    idle.emplace(cap, p);
    idle_bytes += cap;
  }
  ~PinnedPool() {
    for (auto& kv : idle) cudaFreeHost(kv.second);
  }
};

}  // namespace nbgb

using namespace nbgb;

struct nbgb_ensemble {
  nbgb_ensemble_config cfg{};
  int device = 0;
  cudaStream_t main = nullptr;
  // batched Barnes-Hut pass
  cudaStream_t bh_stream = nullptr;
  std::unique_ptr<BHState, BHDeleter> bh;
  DevBuf<unsigned long long> d_bh_inter;  // interactions summed by the walks
  UploadRing up_bh;
  bool bh_dirty = true;   // Barnes-Hut resident set changed
  int64_t bh_n = 0;       // bodies in the Barnes-Hut segments
  int bh_stable = 0;      // ticks since the set last changed
  cudaGraph_t bh_graph = nullptr;  // the tree build
  cudaGraphExec_t bh_exec = nullptr;
  int64_t bh_graph_kernels = 0;
  cudaEvent_t ev_bh = nullptr;
  // walk timing ring (events around each tick's walk on bh_stream)
  cudaEvent_t wev0[kTimingRing] = {}, wev1[kTimingRing] = {};
  bool wev_used[kTimingRing] = {};
  int wev_next = 0;
  double walk_ms = 0.0;
  // arena
  int64_t cap = 0;  // bodies
  DevBuf<double> x, y, z, vx, vy, vz;
  DevBuf<float> ax, ay, az;
  DevBuf<float4> pm;
  std::map<int64_t, int64_t> free_chunks;  // start chunk -> length (chunks)
  uint64_t bytes_reserved = 0;
  // staging for admissions
  DevBuf<float> stage;
  HostPinned<float> h_stage;
  PinnedPool results;  // retirement read-back buffers
  // tables
  DevBuf<KDBlock> d_kd;
  DevBuf<SlotParams> d_slot;
  DevBuf<DirectItem> d_items;
  DevBuf<uint32_t> d_counter;
  DevBuf<uint32_t> d_err;
  DevBuf<float4> part;  // a(0) of direct systems: j-split partials
  UploadRing up_kd, up_slot, up_items;
  int n_kd = 0, n_items = 0;
  bool tables_dirty = true;
  int items_config = -1;
  std::vector<int> free_slots;
  int n_slots = 0;
  // systems
  uint64_t next_id = 1;
  std::deque<Request> queue;
  std::vector<std::unique_ptr<ResidentSystem>> resident;
  std::deque<Retiring> retiring;
  // autotune
  int config = 0;
  bool tuning = false;
  int tune_tick = 0;
  double tune_sum[kNumConfigs] = {};
  int tune_cnt[kNumConfigs] = {};
  double tuned_load = 0.0;
  cudaEvent_t ev_kd = nullptr;
  // direct-kernel timing ring
  cudaEvent_t tev0[kTimingRing] = {}, tev1[kTimingRing] = {};
  bool tev_used[kTimingRing] = {};
  double tev_load[kTimingRing] = {}, tev_inter[kTimingRing] = {};
  int tev_cfg[kTimingRing] = {};
  int tev_next = 0;
  double dk_ms = 0.0, dk_inter = 0.0;
  // stats
  nbgb_ensemble_stats st{};
  double direct_load = 0.0;  // sum N^2 over resident direct systems
  cudaEvent_t stage_evt = nullptr;  // last staging upload (pinned buffer reuse)
};

namespace nbgb {

static int64_t pad_n(int64_t n) { return ceil_div(n, kChunk) * kChunk; }

static bool arena_alloc(nbgb_ensemble* e, int64_t n_pad, int64_t* off) {
  const int64_t need = n_pad / kChunk;
  for (auto it = e->free_chunks.begin(); it != e->free_chunks.end(); ++it) {
    if (it->second >= need) {
      const int64_t start = it->first, len = it->second;
      e->free_chunks.erase(it);
      if (len > need) e->free_chunks[start + need] = len - need;
      *off = start * kChunk;
      return true;
    }
  }
  return false;
}

static void arena_free(nbgb_ensemble* e, int64_t off, int64_t n_pad) {
  int64_t start = off / kChunk, len = n_pad / kChunk;
  auto next = e->free_chunks.lower_bound(start);
  if (next != e->free_chunks.end() && next->first == start + len) {
    len += next->second;
    next = e->free_chunks.erase(next);
  }
  if (next != e->free_chunks.begin()) {
    auto prev = std::prev(next);
    if (prev->first + prev->second == start) {
      prev->second += len;
      return;
    }
  }
  e->free_chunks[start] = len;
}

static size_t arena_bytes_per_body() { return 6 * sizeof(double) + 3 * sizeof(float) + sizeof(float4); }

// Share of the batched tree workspace reserved per Barnes-Hut system
// (buffers at the asynchronous node capacity, with growth headroom).
static size_t bh_estimate_bytes(int64_t n) { return bh_bytes_estimate(n); }

static nbgb_method method_for(const nbgb_ensemble* e, int64_t n) {
  return n <= e->cfg.direct_max_n ? NBGB_DIRECT_N2 : NBGB_BARNES_HUT;
}

static void rebuild_tables(nbgb_ensemble* e) {
  // KD blocks (one per 256 bodies of every resident system)
  int64_t nb = 0;
  for (auto& s : e->resident) nb += s->n_pad / kChunk;
  KDBlock* kd = static_cast<KDBlock*>(e->up_kd.acquire((size_t)std::max<int64_t>(nb, 1) * sizeof(KDBlock)));
  int64_t b = 0;
  for (auto& s : e->resident) {
    for (int64_t c = 0; c < s->n_pad / kChunk; ++c) {
      const int64_t first = c * kChunk;
      kd[b++] = KDBlock{s->off + first, (int32_t)std::max<int64_t>(0, std::min<int64_t>(kChunk, s->n - first)), s->slot};
    }
  }
  e->n_kd = (int)nb;
  KDBlock* dkd = e->d_kd.ensure((size_t)std::max<int64_t>(nb, 1));
  e->up_kd.upload(dkd, (size_t)nb * sizeof(KDBlock), e->main);
  // direct work items, largest systems first (longest-processing-time order)
  const DirectConfig& dc = kConfigs[e->config];
  const int ti = dc.threads * dc.per_thread;
  std::vector<ResidentSystem*> ds;
  for (auto& s : e->resident)
    if (s->method == NBGB_DIRECT_N2) ds.push_back(s.get());
  std::stable_sort(ds.begin(), ds.end(), [](auto* a, auto* b2) { return a->n > b2->n; });
  int64_t ni = 0;
  for (auto* s : ds) ni += ceil_div(s->n, ti);
  DirectItem* it = static_cast<DirectItem*>(e->up_items.acquire((size_t)std::max<int64_t>(ni, 1) * sizeof(DirectItem)));
  int64_t k = 0;
  for (auto* s : ds)
    for (int64_t f = 0; f < s->n; f += ti) it[k++] = DirectItem{s->off, (int32_t)s->n, (int32_t)f};
  e->n_items = (int)ni;
  DirectItem* dit = e->d_items.ensure((size_t)std::max<int64_t>(ni, 1));
  e->up_items.upload(dit, (size_t)ni * sizeof(DirectItem), e->main);
  e->items_config = e->config;
  e->tables_dirty = false;
}

// Segment tables of the batched Barnes-Hut pass (all resident Barnes-Hut
// systems, in resident order), uploaded through the staging ring.
static void bh_tables(nbgb_ensemble* e) {
  std::vector<int64_t> off, cnt;
  for (auto& s : e->resident)
    if (s->method == NBGB_BARNES_HUT) {
      off.push_back(s->off);
      cnt.push_back(s->n);
    }
  e->bh_n = 0;
  for (int64_t c : cnt) e->bh_n += c;
  e->bh_stable = 0;
  if (e->bh_exec) {
    cudaGraphExecDestroy(e->bh_exec);
    e->bh_exec = nullptr;
  }
  if (e->bh_graph) {
    cudaGraphDestroy(e->bh_graph);
    e->bh_graph = nullptr;
  }
  if (off.empty()) return;
  if (!e->bh) e->bh.reset(bh_state_new());
  const int nseg = (int)off.size();
  char* stg = static_cast<char*>(e->up_bh.acquire(bh_segment_table_bytes(cnt.data(), nseg)));
  bh_set_segments(*e->bh, off.data(), cnt.data(), nseg, e->bh_stream, stg);
  e->up_bh.mark(e->bh_stream);
  bh_reserve_async(*e->bh);
  e->bh_dirty = false;  // only once the new tables are in place
}

static void harvest_walk(nbgb_ensemble* e, int k) {
  if (!e->wev_used[k]) return;
  NBGB_CUDA(cudaEventSynchronize(e->wev1[k]));
  float ms = 0.f;
  NBGB_CUDA(cudaEventElapsedTime(&ms, e->wev0[k], e->wev1[k]));
  e->wev_used[k] = false;
  e->walk_ms += ms;
}

// Tree build of every resident Barnes-Hut system, enqueued on bh_stream:
// eagerly right after the set changed, then (with graphs enabled) as a
// graph captured on the first stable tick, when every buffer of the build
// has been allocated.  Then the walk, between timing events.  Returns the
// kernels a graph launched.
static int64_t run_bh_pass(nbgb_ensemble* e) {
  int64_t graph_kernels = 0;
  if (e->bh_exec) {
    NBGB_CUDA(cudaGraphLaunch(e->bh_exec, e->bh_stream));
    graph_kernels = e->bh_graph_kernels;
  } else if (!e->cfg.use_graphs || e->bh_stable < 1) {
    bh_build(*e->bh, e->pm.ptr, e->bh_stream, e->d_err.ptr, e->cfg.group_walk != 0,
             kEnsembleGroupMax);
  } else {
    const int64_t l0 = t_launches;
    NBGB_CUDA(cudaStreamBeginCapture(e->bh_stream, cudaStreamCaptureModeThreadLocal));
    try {
      bh_build(*e->bh, e->pm.ptr, e->bh_stream, e->d_err.ptr, e->cfg.group_walk != 0,
             kEnsembleGroupMax);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(e->bh_stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    NBGB_CUDA(cudaStreamEndCapture(e->bh_stream, &e->bh_graph));
    NBGB_CUDA(cudaGraphInstantiate(&e->bh_exec, e->bh_graph, 0));
    e->bh_graph_kernels = t_launches - l0;
    t_launches = l0;  // captured, not launched: the graph launch counts them
    NBGB_CUDA(cudaGraphLaunch(e->bh_exec, e->bh_stream));
    graph_kernels = e->bh_graph_kernels;
  }
  const int k = e->wev_next % kTimingRing;
  harvest_walk(e, k);
  NBGB_CUDA(cudaEventRecord(e->wev0[k], e->bh_stream));
  const BHWalkParams wp{e->cfg.G, e->cfg.softening, e->cfg.theta, e->cfg.leaf_capacity,
                        e->cfg.group_walk};
  bh_walk(*e->bh, wp, e->ax.ptr, e->ay.ptr, e->az.ptr, nullptr, e->d_bh_inter.ptr, e->d_err.ptr,
          e->bh_stream);
  NBGB_CUDA(cudaEventRecord(e->wev1[k], e->bh_stream));
  e->wev_used[k] = true;
  e->wev_next++;
  return graph_kernels;
}

// Admits, in FIFO order, every queued request that fits the resident cap,
// the HBM budget and the arena.  All admitted states go up in one staging
// copy; a(0) is computed by the next tick's batched passes.
static void admit_batch(nbgb_ensemble* e) {
  struct Pending {
    std::unique_ptr<ResidentSystem> s;
    Request r;
    size_t stage_off;
  };
  std::vector<Pending> batch;
  size_t stage_total = 0;
  while (!e->queue.empty() && (int)(e->resident.size() + batch.size()) < e->cfg.max_resident) {
    Request& r = e->queue.front();
    const nbgb_method m = method_for(e, r.n);
    const int64_t n_pad = pad_n(r.n);
    const size_t est = (size_t)n_pad * arena_bytes_per_body() +
                       (m == NBGB_BARNES_HUT ? bh_estimate_bytes(r.n) : 0);
    if (e->bytes_reserved + est > e->cfg.hbm_budget_bytes) break;
    int64_t off = 0;
    if (!arena_alloc(e, n_pad, &off)) break;
    auto s = std::make_unique<ResidentSystem>();
    s->id = r.id;
    s->n = r.n;
    s->n_pad = n_pad;
    s->off = off;
    s->steps = r.steps;
    s->dt = r.dt;
    s->method = m;
    s->tick_admitted = e->st.ticks;
    s->bytes = est;
    if (e->free_slots.empty()) {
      s->slot = e->n_slots++;
    } else {
      s->slot = e->free_slots.back();
      e->free_slots.pop_back();
    }
    e->bytes_reserved += est;
    const size_t so = stage_total;
    stage_total += (size_t)7 * r.n;
    batch.push_back(Pending{std::move(s), std::move(r), so});
    e->queue.pop_front();
  }
  if (batch.empty()) return;
  // one staging upload; the pinned buffer is reused only after the previous
  // upload has landed.  If the staging memory cannot be had, the requests go
  // back to the front of the queue and their arena space and slots are
  // returned, as if this tick had not admitted them.
  float* hs = nullptr;
  float* ds = nullptr;
  try {
    if (e->stage_evt) NBGB_CUDA(cudaEventSynchronize(e->stage_evt));
    hs = e->h_stage.ensure(stage_total);
    ds = e->stage.ensure(stage_total);
  } catch (...) {
    for (auto it = batch.rbegin(); it != batch.rend(); ++it) {
      arena_free(e, it->s->off, it->s->n_pad);
      e->bytes_reserved -= it->s->bytes;
      e->free_slots.push_back(it->s->slot);
      e->queue.push_front(std::move(it->r));
    }
    throw;
  }
  for (auto& p : batch) std::copy(p.r.state.begin(), p.r.state.end(), hs + p.stage_off);
  NBGB_CUDA(cudaMemcpyAsync(ds, hs, stage_total * sizeof(float), cudaMemcpyHostToDevice, e->main));
  if (!e->stage_evt) NBGB_CUDA(cudaEventCreateWithFlags(&e->stage_evt, cudaEventDisableTiming));
  NBGB_CUDA(cudaEventRecord(e->stage_evt, e->main));
  for (auto& p : batch) {
    ResidentSystem& s = *p.s;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(s.n_pad, 256), 1024));
    ens_admit_kernel<<<blocks, 256, 0, e->main>>>(ds + p.stage_off, s.n, s.n_pad, s.off, e->x.ptr,
                                                   e->y.ptr, e->z.ptr, e->vx.ptr, e->vy.ptr,
                                                   e->vz.ptr, e->ax.ptr, e->ay.ptr, e->az.ptr,
                                                   e->pm.ptr);
    NBGB_LAUNCH_CHECK();
  }
  for (auto& p : batch) {
    ResidentSystem& s = *p.s;
    if (s.method == NBGB_DIRECT_N2)
      e->direct_load += (double)s.n * (double)s.n;
    else
      e->bh_dirty = true;
    e->resident.push_back(std::move(p.s));
    e->st.admitted++;
  }
  e->tables_dirty = true;
}

static void retire(nbgb_ensemble* e, std::unique_ptr<ResidentSystem> s) {
  // final half kick, then copy the state out
  launch_kick(s->n, e->vx.ptr + s->off, e->vy.ptr + s->off, e->vz.ptr + s->off, e->ax.ptr + s->off,
              e->ay.ptr + s->off, e->az.ptr + s->off, 0.5 * (double)s->dt, e->main);
  Retiring r;
  r.res.request_id = s->id;
  r.res.count = s->n;
  r.res.steps = s->steps;
  r.res.method = s->method;
  r.res.gpu_ms = 0.0;
  const size_t n = (size_t)s->n;
  r.h_state = static_cast<double*>(
      e->results.take(n * (6 * sizeof(double) + 4 * sizeof(float)) + 8, &r.h_bytes));
  double* hd = r.h_state;
  DevBuf<double>* src[6] = {&e->x, &e->y, &e->z, &e->vx, &e->vy, &e->vz};
  for (int k = 0; k < 6; ++k)
    NBGB_CUDA(cudaMemcpyAsync(hd + k * n, src[k]->ptr + s->off, n * 8, cudaMemcpyDeviceToHost, e->main));
  float* hf = reinterpret_cast<float*>(hd + 6 * n);
  NBGB_CUDA(cudaMemcpyAsync(hf, e->ax.ptr + s->off, n * 4, cudaMemcpyDeviceToHost, e->main));
  NBGB_CUDA(cudaMemcpyAsync(hf + n, e->ay.ptr + s->off, n * 4, cudaMemcpyDeviceToHost, e->main));
  NBGB_CUDA(cudaMemcpyAsync(hf + 2 * n, e->az.ptr + s->off, n * 4, cudaMemcpyDeviceToHost, e->main));
  NBGB_CUDA(cudaMemcpy2DAsync(hf + 3 * n, sizeof(float), reinterpret_cast<const char*>(e->pm.ptr + s->off) + 12,
                              sizeof(float4), sizeof(float), n, cudaMemcpyDeviceToHost, e->main));
  // device error word (bounded waits, tree capacity, non-finite bounds)
  uint32_t* herr = reinterpret_cast<uint32_t*>(hf + 4 * n);
  NBGB_CUDA(cudaMemcpyAsync(herr, e->d_err.ptr, 4, cudaMemcpyDeviceToHost, e->main));
  herr[1] = 0;
  NBGB_CUDA(cudaEventCreateWithFlags(&r.evt, cudaEventDisableTiming));
  NBGB_CUDA(cudaEventRecord(r.evt, e->main));
  // device work that reuses this memory is ordered after the copies on main
  arena_free(e, s->off, s->n_pad);
  e->bytes_reserved -= s->bytes;
  e->free_slots.push_back(s->slot);
  if (s->method == NBGB_DIRECT_N2)
    e->direct_load -= (double)s->n * (double)s->n;
  else
    e->bh_dirty = true;
  e->st.retired++;
  r.sys = std::move(s);
  e->retiring.push_back(std::move(r));
  e->tables_dirty = true;
}

// Direct-kernel timing ring: every tick's direct kernel is bracketed by a
// pair of events; a pair is harvested (synchronised, elapsed time added to
// the statistics and, while tuning, to its configuration's score) when it is
// reused kTimingRing ticks later or when statistics are read.  This also
// bounds how far the host runs ahead of the device.
static void harvest(nbgb_ensemble* e, int k) {
  if (!e->tev_used[k]) return;
  NBGB_CUDA(cudaEventSynchronize(e->tev1[k]));
  float ms = 0.f;
  NBGB_CUDA(cudaEventElapsedTime(&ms, e->tev0[k], e->tev1[k]));
  e->tev_used[k] = false;
  e->dk_ms += ms;
  e->dk_inter += e->tev_inter[k];
  if (e->tuning) {
    const int c = e->tev_cfg[k];
    e->tune_sum[c] += (double)ms / std::max(e->tev_load[k], 1.0);  // time per unit of load
    e->tune_cnt[c] += 1;
  }
}

static void harvest_all(nbgb_ensemble* e) {
  for (int k = 0; k < kTimingRing; ++k) {
    harvest(e, k);
    harvest_walk(e, k);
  }
}

// Tuning schedule: every configuration runs two ticks; once all are
// measured the fastest per unit of direct load is kept.
static void tune_select(nbgb_ensemble* e) {
  if (!e->tuning) return;
  const int want = std::min(e->tune_tick / 2, kNumConfigs - 1);
  if (e->tune_tick >= 2 * kNumConfigs) harvest_all(e);
  bool all = true;
  for (int c = 0; c < kNumConfigs; ++c) all = all && e->tune_cnt[c] >= 2;
  if (all) {
    int best = 0;
    for (int c = 1; c < kNumConfigs; ++c)
      if (e->tune_sum[c] / e->tune_cnt[c] < e->tune_sum[best] / e->tune_cnt[best]) best = c;
    e->tuning = false;
    e->config = best;
    e->tuned_load = e->direct_load;
    e->tables_dirty = true;
    return;
  }
  if (want != e->config) {
    e->config = want;
    e->tables_dirty = true;
  }
}

static void maybe_start_tuning(nbgb_ensemble* e) {
  if (e->cfg.direct_config >= 0 || e->tuning || e->direct_load <= 0.0) return;
  const double ratio = e->tuned_load > 0 ? e->direct_load / e->tuned_load : 1e9;
  if (ratio > 2.0 || ratio < 0.5) {
    e->tuning = true;
    e->tune_tick = 0;
    for (int c = 0; c < kNumConfigs; ++c) {
      e->tune_sum[c] = 0.0;
      e->tune_cnt[c] = 0;
    }
    e->config = 0;
    e->tables_dirty = true;
  }
}

static void run_tick(nbgb_ensemble* e) {
  const int64_t l0 = t_launches;
  int64_t graph_kernels = 0;
  admit_batch(e);
  maybe_start_tuning(e);
  tune_select(e);
  if (e->resident.empty()) {
    e->st.kernel_launches += t_launches - l0;
    return;
  }
  if (e->tables_dirty || e->items_config != e->config) rebuild_tables(e);
  if (e->bh_dirty) bh_tables(e);
  // per-slot kick factors: a fresh system neither kicks nor drifts (its
  // a(0) is computed below); afterwards the closing half kick of the last
  // step and the opening half kick of this one are merged
  SlotParams* sp = static_cast<SlotParams*>(e->up_slot.acquire((size_t)std::max(e->n_slots, 1) * sizeof(SlotParams)));
  for (auto& s : e->resident)
    sp[s->slot] = s->fresh ? SlotParams{0.0, 0.0}
                           : SlotParams{s->pending_half ? (double)s->dt : 0.5 * (double)s->dt,
                                        (double)s->dt};
  SlotParams* dsp = e->d_slot.ensure((size_t)std::max(e->n_slots, 1));
  e->up_slot.upload(dsp, (size_t)e->n_slots * sizeof(SlotParams), e->main);
  // every device buffer the rest of the tick needs is allocated before the
  // first kernel that changes a system's state: running out of memory ends
  // the tick here, and the next tick repeats it from the same state
  if (e->bh_n > 0 && !e->bh_exec) bh_reserve_buffers(*e->bh, e->cfg.group_walk != 0);
  // 1. kick-drift for everything resident
  if (e->n_kd) {
    const unsigned blocks = (unsigned)std::min(e->n_kd, num_sms() * 16);
    ens_kick_drift_kernel<<<blocks, (int)kChunk, 0, e->main>>>(
        e->d_kd.ptr, e->n_kd, dsp, e->x.ptr, e->y.ptr, e->z.ptr, e->vx.ptr, e->vy.ptr, e->vz.ptr,
        e->ax.ptr, e->ay.ptr, e->az.ptr, e->pm.ptr);
    NBGB_LAUNCH_CHECK();
  }
  NBGB_CUDA(cudaEventRecord(e->ev_kd, e->main));
  // 2. all Barnes-Hut systems: one batched pass on the side stream
  const bool bh_work = e->bh_n > 0;
  if (bh_work) {
    NBGB_CUDA(cudaStreamWaitEvent(e->bh_stream, e->ev_kd, 0));
    graph_kernels = run_bh_pass(e);
    NBGB_CUDA(cudaEventRecord(e->ev_bh, e->bh_stream));
    e->bh_stable++;
  }
  // 3. direct systems: persistent work-queue kernel (always timed)
  if (e->n_items) {
    const int k = e->tev_next % kTimingRing;
    harvest(e, k);
    double inter = 0.0;
    for (auto& s : e->resident)
      if (s->method == NBGB_DIRECT_N2) inter += (double)s->n * (double)(s->n - 1);
    e->tev_load[k] = e->direct_load;
    e->tev_inter[k] = inter;
    e->tev_cfg[k] = e->config;
    NBGB_CUDA(cudaMemsetAsync(e->d_counter.ptr, 0, sizeof(uint32_t), e->main));
    NBGB_CUDA(cudaEventRecord(e->tev0[k], e->main));
    // Beside a Barnes-Hut pass, one CTA per SM: the kernel then runs next to
    // the tree build (a chain of latency-bound kernels that needs resident
    // warps, not issue slots) without crowding it out, and still finishes
    // before the walk (serving bench: 5.79 ms per tick vs 5.98 at full
    // occupancy; 2 per SM 5.86, one per two SMs 5.83).  Alone, full occupancy.
    const int grid = bh_work ? num_sms() : num_sms() * config_occupancy(e->config);
    launch_config(e->config, grid, e->d_items.ptr, e->n_items, e->d_counter.ptr, e->pm.ptr,
                  e->ax.ptr, e->ay.ptr, e->az.ptr, e->cfg.softening * e->cfg.softening, e->cfg.G,
                  e->d_err.ptr, e->main);
    NBGB_CUDA(cudaEventRecord(e->tev1[k], e->main));
    e->tev_used[k] = true;
    e->tev_next++;
    if (e->tuning) e->tune_tick++;
    e->st.direct_interactions += inter;
  }
  if (bh_work) NBGB_CUDA(cudaStreamWaitEvent(e->main, e->ev_bh, 0));
  // 4. bookkeeping and retirement
  e->st.ticks++;
  std::vector<std::unique_ptr<ResidentSystem>> keep;
  for (auto& s : e->resident) {
    if (s->fresh) {
      s->fresh = false;
      continue;
    }
    s->done++;
    s->pending_half = true;
    e->st.particle_steps += s->n;
  }
  for (auto& s : e->resident) {
    if (s->done >= s->steps)
      retire(e, std::move(s));
    else
      keep.push_back(std::move(s));
  }
  e->resident.swap(keep);
  e->st.kernel_launches += t_launches - l0 + graph_kernels;
}

}  // namespace nbgb


template <typename F>
static nbgb_status ens_guard(F&& f) {
  try {
    f();
    return NBGB_OK;
  } catch (const Error& err) {
    set_error(err.status, err.what());
    return err.status;
  } catch (const std::bad_alloc&) {
    return NBGB_ERR_OOM;
  } catch (const std::exception&) {
    return NBGB_ERR_CUDA;
  }
}

extern "C" {

void nbgb_ensemble_config_default(nbgb_ensemble_config* c) {
  if (!c) return;
  c->hbm_budget_bytes = 64ull << 30;
  c->max_resident = 4096;
  c->direct_max_n = 8192;
  c->G = 1.0f;
  c->softening = 0.01f;
  c->theta = 0.5f;
  c->leaf_capacity = 1;  // the reference's tree walk (8 = bodies of small subtrees summed directly)
  c->direct_config = -1;
  c->use_graphs = 1;
  c->group_walk = 1;  // lower force error than the reference walk at the same theta, ~2x faster
}

nbgb_status nbgb_ensemble_create(const nbgb_ensemble_config* cfg, nbgb_ensemble** out) {
  return ens_guard([&] {
    if (!out) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null output handle");
    *out = nullptr;
    nbgb_ensemble_config c;
    nbgb_ensemble_config_default(&c);
    if (cfg) c = *cfg;
    if (!(c.softening > 0.f) || !std::isfinite(c.softening))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Softening parameter must be positive");
    if (!(c.G > 0.f)) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Gravitational constant must be positive and finite");
    if (c.theta < 0.f || c.theta > 2.f) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Barnes-Hut theta must be between 0 and 2");
    if (c.direct_config >= kNumConfigs) fail(NBGB_ERR_INVALID_ARG, "Validation Error: unknown direct configuration");
    if (c.leaf_capacity < 1 || c.leaf_capacity > 16)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: leaf capacity must be between 1 and 16");
    if (c.max_resident < 1 || c.hbm_budget_bytes < (1u << 20))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: budget or resident cap too small");
    auto e = std::make_unique<nbgb_ensemble>();
    e->cfg = c;
    NBGB_CUDA(cudaGetDevice(&e->device));
    NBGB_CUDA(cudaStreamCreateWithFlags(&e->main, cudaStreamNonBlocking));
    // the Barnes-Hut chain (build, then walk) is the tick's critical path:
    // its blocks are scheduled ahead of the direct work queue's
    int prio_lo = 0, prio_hi = 0;
    NBGB_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    NBGB_CUDA(cudaStreamCreateWithPriority(&e->bh_stream, cudaStreamNonBlocking, prio_hi));
    // arena: a quarter of the budget holds body state; the rest is for trees
    e->cap = std::max<int64_t>(kChunk, (int64_t)(c.hbm_budget_bytes / 4 / arena_bytes_per_body()) / kChunk * kChunk);
    e->x.ensure((size_t)e->cap);
    e->y.ensure((size_t)e->cap);
    e->z.ensure((size_t)e->cap);
    e->vx.ensure((size_t)e->cap);
    e->vy.ensure((size_t)e->cap);
    e->vz.ensure((size_t)e->cap);
    e->ax.ensure((size_t)e->cap);
    e->ay.ensure((size_t)e->cap);
    e->az.ensure((size_t)e->cap);
    e->pm.ensure((size_t)e->cap);
    e->free_chunks[0] = e->cap / kChunk;
    e->d_counter.ensure(1);
    e->d_err.ensure(1);
    NBGB_CUDA(cudaMemset(e->d_err.ptr, 0, 4));
    for (int k = 0; k < kTimingRing; ++k) {
      NBGB_CUDA(cudaEventCreate(&e->tev0[k]));
      NBGB_CUDA(cudaEventCreate(&e->tev1[k]));
      NBGB_CUDA(cudaEventCreate(&e->wev0[k]));
      NBGB_CUDA(cudaEventCreate(&e->wev1[k]));
    }
    NBGB_CUDA(cudaEventCreateWithFlags(&e->ev_kd, cudaEventDisableTiming));
    NBGB_CUDA(cudaEventCreateWithFlags(&e->ev_bh, cudaEventDisableTiming));
    e->d_bh_inter.ensure(1);
    NBGB_CUDA(cudaMemset(e->d_bh_inter.ptr, 0, sizeof(unsigned long long)));
    e->config = c.direct_config >= 0 ? c.direct_config : 0;
    *out = e.release();
  });
}

nbgb_status nbgb_ensemble_destroy(nbgb_ensemble* e) {
  return ens_guard([&] {
    if (!e) return;
    cudaDeviceSynchronize();
    for (auto& r : e->retiring) {
      if (r.h_state) cudaFreeHost(r.h_state);
      if (r.evt) cudaEventDestroy(r.evt);
    }
    if (e->bh_exec) cudaGraphExecDestroy(e->bh_exec);
    if (e->bh_graph) cudaGraphDestroy(e->bh_graph);
    e->bh.reset();
    cudaStreamDestroy(e->bh_stream);
    cudaEventDestroy(e->ev_bh);
    for (int k = 0; k < kTimingRing; ++k) {
      cudaEventDestroy(e->tev0[k]);
      cudaEventDestroy(e->tev1[k]);
      cudaEventDestroy(e->wev0[k]);
      cudaEventDestroy(e->wev1[k]);
    }
    cudaEventDestroy(e->ev_kd);
    if (e->stage_evt) cudaEventDestroy(e->stage_evt);
    cudaStreamDestroy(e->main);
    delete e;
  });
}

nbgb_status nbgb_ensemble_submit(nbgb_ensemble* e, const nbgb_particle_data* h, int32_t steps,
                                 float dt, uint64_t* request_id) {
  return ens_guard([&] {
    if (!e || !h) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null argument");
    if (h->count == 0) fail(NBGB_ERR_INVALID_ARG, "Validation Error: Particle count must be greater than 0");
    if (steps < 1) fail(NBGB_ERR_INVALID_ARG, "Validation Error: step count must be positive");
    if (!(dt > 0.f) || dt > 1.f || !std::isfinite(dt))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: Time step must be in (0, 1]");
    if (!h->pos_x || !h->pos_y || !h->pos_z || !h->vel_x || !h->vel_y || !h->vel_z || !h->mass)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null host array");
    Request r;
    r.id = e->next_id++;
    r.n = (int64_t)h->count;
    r.steps = steps;
    r.dt = dt;
    const size_t n = h->count;
    r.state.resize(7 * n);
    const float* src[7] = {h->pos_x, h->pos_y, h->pos_z, h->vel_x, h->vel_y, h->vel_z, h->mass};
    for (int k = 0; k < 7; ++k) std::copy(src[k], src[k] + n, r.state.begin() + k * n);
    const size_t need = (size_t)pad_n(r.n) * arena_bytes_per_body() +
                        (method_for(e, r.n) == NBGB_BARNES_HUT ? bh_estimate_bytes(r.n) : 0);
    if (need > e->cfg.hbm_budget_bytes || pad_n(r.n) > e->cap)
      fail(NBGB_ERR_OOM, "Insufficient GPU memory - request larger than the ensemble budget");
    if (request_id) *request_id = r.id;
    e->queue.push_back(std::move(r));
    e->st.queued = (int32_t)e->queue.size();
  });
}

nbgb_status nbgb_ensemble_tick(nbgb_ensemble* e, int32_t* resident, int32_t* queued) {
  return ens_guard([&] {
    if (!e) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null ensemble");
    run_tick(e);
    if (resident) *resident = (int32_t)e->resident.size();
    if (queued) *queued = (int32_t)e->queue.size();
  });
}

nbgb_status nbgb_ensemble_poll(nbgb_ensemble* e, nbgb_ensemble_result* result,
                               nbgb_particle_data* h_out, double* state_f64) {
  if (!e || !result) return NBGB_ERR_INVALID_ARG;
  if (e->retiring.empty()) return NBGB_ERR_NOT_READY;
  Retiring& r = e->retiring.front();
  cudaError_t q = cudaEventQuery(r.evt);
  if (q == cudaErrorNotReady) return NBGB_ERR_NOT_READY;
  if (q != cudaSuccess) return NBGB_ERR_CUDA;
  *result = r.res;
  const size_t n = (size_t)r.res.count;
  // device error words copied at retirement (bounded waits, tree capacity)
  const uint32_t* herr =
      reinterpret_cast<const uint32_t*>(reinterpret_cast<const float*>(r.h_state + 6 * n) + 4 * n);
  const uint32_t bits = herr[0] | herr[1];
  if (h_out && h_out->count >= n) {
    const double* d = r.h_state;
    float* dst[6] = {h_out->pos_x, h_out->pos_y, h_out->pos_z, h_out->vel_x, h_out->vel_y, h_out->vel_z};
    for (int k = 0; k < 6; ++k)
      if (dst[k])
        for (size_t i = 0; i < n; ++i) dst[k][i] = (float)d[k * n + i];
    const float* f = reinterpret_cast<const float*>(d + 6 * n);
    if (h_out->acc_x) std::copy(f, f + n, h_out->acc_x);
    if (h_out->acc_y) std::copy(f + n, f + 2 * n, h_out->acc_y);
    if (h_out->acc_z) std::copy(f + 2 * n, f + 3 * n, h_out->acc_z);
    if (h_out->mass) std::copy(f + 3 * n, f + 4 * n, h_out->mass);
  }
  if (state_f64) std::copy(r.h_state, r.h_state + 6 * n, state_f64);
  e->results.give(r.h_state, r.h_bytes);
  cudaEventDestroy(r.evt);
  e->retiring.pop_front();
  if (bits) {
    set_error(NBGB_ERR_OVERFLOW, "device error word set during the ensemble run");
    return bits & kErrWaitTimeout ? NBGB_ERR_DEVICE_TIMEOUT : NBGB_ERR_OVERFLOW;
  }
  return NBGB_OK;
}

nbgb_status nbgb_ensemble_synchronize(nbgb_ensemble* e) {
  return ens_guard([&] {
    if (!e) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null ensemble");
    NBGB_CUDA(cudaStreamSynchronize(e->main));
  });
}

nbgb_status nbgb_ensemble_get_stream(nbgb_ensemble* e, void** cuda_stream) {
  if (!e || !cuda_stream) return NBGB_ERR_INVALID_ARG;
  *cuda_stream = static_cast<void*>(e->main);
  return NBGB_OK;
}

nbgb_status nbgb_ensemble_get_stats(nbgb_ensemble* e, nbgb_ensemble_stats* s) {
  if (!e || !s) return NBGB_ERR_INVALID_ARG;
  unsigned long long bh_inter = 0;
  try {
    harvest_all(e);
    NBGB_CUDA(cudaMemcpyAsync(&bh_inter, e->d_bh_inter.ptr, sizeof bh_inter,
                              cudaMemcpyDeviceToHost, e->main));
    NBGB_CUDA(cudaStreamSynchronize(e->main));
  } catch (const Error& err) {
    return err.status;
  }
  *s = e->st;
  s->bh_interactions = (double)bh_inter;
  s->bh_walk_ms = e->walk_ms;
  s->bh_bodies = e->bh_n;
  s->direct_kernel_ms = e->dk_ms;
  s->direct_kernel_interactions = e->dk_inter;
  s->resident = (int32_t)e->resident.size();
  s->queued = (int32_t)e->queue.size();
  s->bytes_reserved = e->bytes_reserved;
  s->direct_config = e->config;
  s->tuning = e->tuning ? 1 : 0;
  return NBGB_OK;
}

}  // extern "C"
