// noalloc.cu -- direct-sum forces that allocate no device memory.
//
// Who needs this: callers that are not allowed to call cudaMalloc (or
// cudaFree) -- for example a simulation step embedded in a host application
// that owns all device memory through its own pool and forbids driver
// allocations, or a latency-critical loop where cudaMalloc's implicit device
// synchronisation and its failure modes under memory pressure are
// unacceptable.  The regular calculator (nbgb_compute_forces) keeps growable
// per-calculator buffers and allocates them on first use; this entry point
// instead uses scratch that lives in file-scope device arrays (about 9 MiB
// per device), held until the process exits.
//
// When the memory is reserved: the arrays belong to this library's device
// module.  With eager module loading that happens when the library's module
// is loaded on the device; with lazy loading (CUDA_MODULE_LOADING=LAZY, the
// default of recent CUDA releases) it happens at the first call on that
// device, which resolves the arrays' device addresses.  That first call can
// therefore fail with NBGB_ERR_OOM under memory pressure or synchronise the
// device; a warm-up call with count 0 does the reservation and nothing else.
//
// Limits: at most kNoAllocMaxBodies bodies per call, direct sum only; not
// callable while its stream is being captured into a CUDA graph (it reads the
// device error word back and waits for the stream); cudaDeviceReset after
// the first call on a device is not supported (the resolved addresses are
// kept per device).  All calls share the same scratch arrays: calls whose
// work overlaps on the GPU (different streams, or different host threads,
// without ordering between them) race on that scratch and must be
// serialised by the caller.
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace nbgb {

constexpr int64_t kNoAllocMaxBodies = 65536;  // multiple of the j-tile (256)
constexpr int kNoAllocMaxSplits = 8;           // j-splits of the partial sums

// Scratch (global memory beyond the caller's inputs and outputs):
//   packed (x, y, z, m) bodies, zero-mass padded      1 MiB
//   per-split partial accelerations                   8 MiB
//   device error word (bounded-wait timeouts)         4 B
static __device__ __align__(256) float4 g_noalloc_bodies[kNoAllocMaxBodies];
static __device__ __align__(256) float4 g_noalloc_partial[kNoAllocMaxSplits * kNoAllocMaxBodies];
static __device__ __align__(256) uint32_t g_noalloc_err[64];

struct NoAllocScratch {
  float4* bodies = nullptr;
  float4* partial = nullptr;
  uint32_t* err = nullptr;
  bool ready = false;
};

// Device addresses of the scratch arrays, resolved once per device with that
// device current.  In host code the array names are host-side stand-ins, not
// device addresses, so kernels only ever receive these resolved pointers.
static std::mutex g_noalloc_mu;
static NoAllocScratch g_noalloc[64];

static NoAllocScratch noalloc_scratch(int dev) {
  if (dev < 0 || dev >= 64)
    fail(NBGB_ERR_INVALID_ARG, "Validation Error: device ordinal beyond the no-allocation table");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocScratch& s = g_noalloc[dev];
  if (!s.ready) {
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&s.bodies), g_noalloc_bodies);
    if (e == cudaSuccess)
      e = cudaGetSymbolAddress(reinterpret_cast<void**>(&s.partial), g_noalloc_partial);
    if (e == cudaSuccess)
      e = cudaGetSymbolAddress(reinterpret_cast<void**>(&s.err), g_noalloc_err);
    if (e != cudaSuccess) {
      cudaGetLastError();
      s = NoAllocScratch{};
      fail(e == cudaErrorMemoryAllocation ? NBGB_ERR_OOM : NBGB_ERR_CUDA,
           std::string("CUDA Error: reserving the static no-allocation scratch: ") +
               cudaGetErrorString(e));
    }
    s.ready = true;
  }
  return s;
}

// The direct plan with its j-splits capped to the static partial-sum array.
// `planned` receives the split count the regular planner chose.
static DirectPlan noalloc_plan(int64_t n, int* planned) {
  DirectPlan p = plan_direct(n, n, DirectVariant::kPaired8);
  if (planned) *planned = p.splits;
  if (p.splits > kNoAllocMaxSplits) {
    p.tiles_per_split = ceil_div(p.n_tiles, kNoAllocMaxSplits);
    p.splits = (int)ceil_div(p.n_tiles, p.tiles_per_split);
  }
  return p;
}

template <typename F>
static nbgb_status noalloc_guarded(F&& f) {
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

extern "C" nbgb_status nbgb_compute_forces_direct_noalloc(const nbgb_particle_data* d, float G,
                                                          float softening, void* stream) {
  return noalloc_guarded([&] {
    if (!d) fail(NBGB_ERR_INVALID_ARG, "Validation Error: null particle data");
    if (!(std::isfinite(G) && G > 0.f))
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: Gravitational constant must be positive and finite");
    if (!std::isfinite(softening) || softening < 0.f)
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: Softening parameter must be a finite, non-negative number");
    const int64_t n = (int64_t)d->count;
    if (n > kNoAllocMaxBodies)
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: the allocation-free direct sum takes at most 65536 bodies per call");
    if (n > 0 &&
        (!d->pos_x || !d->pos_y || !d->pos_z || !d->mass || !d->acc_x || !d->acc_y || !d->acc_z))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: null position, mass or acceleration array");
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    NBGB_CUDA(cudaStreamIsCapturing(cs, &cap));
    if (cap != cudaStreamCaptureStatusNone)
      fail(NBGB_ERR_INVALID_ARG,
           "Validation Error: the allocation-free direct sum cannot run while its stream is "
           "being captured");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
      cudaGetLastError();
      fail(NBGB_ERR_NO_DEVICE, "CUDA Error: no CUDA device");
    }
    // the first call on a device resolves (and, with lazy module loading,
    // reserves) the scratch; a count of 0 stops right after that
    const NoAllocScratch s = noalloc_scratch(dev);
    if (n == 0) return;
    // The error word keeps the previous call's value: clear it first.
    NBGB_CUDA(cudaMemsetAsync(s.err, 0, sizeof(uint32_t), cs));
    const DirectPlan p = noalloc_plan(n, nullptr);
    // Every padded body slot and every partial read below is rewritten by
    // this call, so nothing else of the previous call's contents is used.
    launch_pack_soa(d->pos_x, d->pos_y, d->pos_z, d->mass, n, p.n_src_pad, s.bodies, cs);
    launch_direct(p, s.bodies, s.bodies, n, G, softening * softening, true, s.partial, d->acc_x,
                  d->acc_y, d->acc_z, s.err, cs);
    uint32_t bits = 0;
    NBGB_CUDA(cudaMemcpyAsync(&bits, s.err, sizeof bits, cudaMemcpyDeviceToHost, cs));
    NBGB_CUDA(cudaStreamSynchronize(cs));
    if (bits)
      fail(NBGB_ERR_DEVICE_TIMEOUT,
           "CUDA Error: a bounded device wait of the direct kernel ran out of iterations");
  });
}

extern "C" nbgb_status nbgb_selftest_noalloc_plan(int64_t count, int32_t* planned_splits,
                                                  int32_t* used_splits) {
  return noalloc_guarded([&] {
    if (count < 1 || count > kNoAllocMaxBodies)
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: count must be in [1, 65536]");
    int planned = 0;
    const DirectPlan p = noalloc_plan(count, &planned);
    if ((int64_t)p.splits * p.n_tgt_pad > kNoAllocMaxSplits * kNoAllocMaxBodies ||
        p.n_src_pad > kNoAllocMaxBodies)
      fail(NBGB_ERR_OVERFLOW, "the capped plan does not fit the static scratch");
    if (planned_splits) *planned_splits = planned;
    if (used_splits) *used_splits = p.splits;
  });
}
