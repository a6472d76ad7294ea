// runtime.cuh -- device buffers and the internal state behind the C handles.
#pragma once

#include <atomic>
#include <memory>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace nbgb {

// Allocation-failure injection (nbgb_selftest_fail_allocation): the
// countdown-th device allocation from now fails as if the device were out of
// memory, without calling the allocator.  0 = off.
extern std::atomic<int64_t> g_alloc_fault_countdown;

inline bool alloc_fault_injected() {
  int64_t c = g_alloc_fault_countdown.load(std::memory_order_relaxed);
  while (c > 0) {
    if (g_alloc_fault_countdown.compare_exchange_weak(c, c - 1)) return c == 1;
  }
  return false;
}

// Growable device allocation (contents are not preserved on growth).
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;  // elements
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  T* ensure(size_t n) {
    if (n <= cap && ptr) return ptr;
    release();
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    cudaError_t e = alloc_fault_injected() ? cudaErrorMemoryAllocation : cudaMalloc(&ptr, bytes);
    if (e != cudaSuccess) {
      ptr = nullptr;
      cudaGetLastError();
      char buf[160];
      std::snprintf(buf, sizeof buf, "device allocation of %zu bytes failed: %s", bytes,
                    cudaGetErrorString(e));
      fail(e == cudaErrorMemoryAllocation ? NBGB_ERR_OOM : NBGB_ERR_CUDA, buf);
    }
    cap = std::max<size_t>(n, 1);
    return ptr;
  }
  size_t bytes() const { return cap * sizeof(T); }
};

// Pinned host scalars used to read small device results.
template <typename T>
struct HostPinned {
  T* ptr = nullptr;
  size_t n = 0;
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() {
    if (ptr) cudaFreeHost(ptr);
  }
  T* ensure(size_t k) {
    if (k <= n && ptr) return ptr;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    NBGB_CUDA(cudaMallocHost(&ptr, std::max<size_t>(k, 1) * sizeof(T)));
    n = std::max<size_t>(k, 1);
    return ptr;
  }
};

// Per-stage device times of a calculator (NBGB_FLAG_STAGE_TIMINGS): an event
// is recorded on the calculator's stream where each stage of a force
// evaluation begins and where the evaluation ends; harvest() waits for the
// last one and adds the time between consecutive events to the stage that
// began at the first.  Events are recycled.
struct StageTimer {
  cudaStream_t st = nullptr;
  std::vector<std::string> names;
  std::vector<double> total_ms;
  std::vector<int64_t> samples;
  struct Mark {
    int stage;  // -1: the end of an evaluation
    cudaEvent_t ev;
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> spare;
  StageTimer() = default;
  StageTimer(const StageTimer&) = delete;
  StageTimer& operator=(const StageTimer&) = delete;
  ~StageTimer();
  void mark(const char* stage);  // begins `stage`, ending the one before
  void end();                    // ends the evaluation's last stage
  void harvest();
  void reset();

 private:
  cudaEvent_t record(int stage);
  int id_of(const char* name);
};

// Marks a stage on an optional timer.
inline void stage_mark(StageTimer* t, const char* stage) {
  if (t) t->mark(stage);
}

struct BHState;    // bh.cu
struct HashState;  // hash.cu
void bh_state_delete(BHState*);
void hash_state_delete(HashState*);

struct BHDeleter {
  void operator()(BHState* p) const { bh_state_delete(p); }
};
struct HashDeleter {
  void operator()(HashState* p) const { hash_state_delete(p); }
};

}  // namespace nbgb

struct nbgb_calculator {
  nbgb_method method = NBGB_DIRECT_N2;
  nbgb_params params{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0;
  nbgb::DirectVariant variant = nbgb::DirectVariant::kScalar4;

  nbgb::DevBuf<float4> pm;        // packed (x, y, z, m) input of the last drop-in call
  nbgb::DevBuf<float4> partial;   // direct j-split partials
  nbgb::DevBuf<uint32_t> err;     // device error word
  nbgb::DevBuf<int32_t> counts;   // per-target interaction / neighbour counts
  nbgb::DevBuf<double> red;       // reduction partials
  nbgb::HostPinned<uint32_t> h_err;
  nbgb::HostPinned<double> h_red;
  int64_t last_n = 0;

  std::unique_ptr<nbgb::BHState, nbgb::BHDeleter> bh;
  std::unique_ptr<nbgb::HashState, nbgb::HashDeleter> hash;
  std::unique_ptr<nbgb::StageTimer> timer;  // NBGB_FLAG_STAGE_TIMINGS
};

// A device-resident system (nbgb_system_*): FP64 x, v; FP32 (or FP64) a;
// packed FP32 (x, y, z, m) for the force kernels.
struct nbgb_system {
  nbgb_calculator* calc = nullptr;
  int64_t n = 0;
  nbgb::DevBuf<double> x, y, z, vx, vy, vz;
  nbgb::DevBuf<float> ax, ay, az;
  nbgb::DevBuf<double> ax64, ay64, az64;  // NBGB_FLAG_FP64: accelerations in FP64
  nbgb::DevBuf<float4> pm;
  nbgb::DevBuf<double> red;
  nbgb::HostPinned<double> h_red;
  bool fp64 = false;
  bool pending_half = false;  // v lags x by half a kick of size last_dt/2
  double last_dt = 0.0;
};

namespace nbgb {

// Applies a system's pending half kick (v then matches x in time).
void system_sync_velocity(nbgb_system* s);

// The calculator's stage timer while NBGB_FLAG_STAGE_TIMINGS is set.
inline StageTimer* stage_timer(nbgb_calculator* c) {
  return (c->params.flags & NBGB_FLAG_STAGE_TIMINGS) ? c->timer.get() : nullptr;
}

// Forces on n bodies given as packed float4 `pm` (padded by the callee's own
// requirements where needed); writes ax/ay/az (length n).  Enqueued on
// calc->stream.  Defined in api.cu; the method backends live in bh.cu and
// hash.cu.
void forces_packed(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay,
                   float* az);
void bh_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay, float* az);
void hash_forces(nbgb_calculator* c, const float4* pm, int64_t n, float* ax, float* ay,
                 float* az);
// Sources padded for the direct kernel: returns the padded length.
int64_t direct_pad(int64_t n);
// Wait for the calculator's stream and turn device error bits into an Error.
void check_device_errors(nbgb_calculator* c);
// Record msg as this thread's nbgb_last_error() text; returns s.
nbgb_status set_error(nbgb_status s, const std::string& msg);

}  // namespace nbgb
