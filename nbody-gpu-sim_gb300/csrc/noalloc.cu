// noalloc.cu -- direct-sum forces that allocate no device memory.
//
// Who needs this: callers that are not allowed to call cudaMalloc (or
// cudaFree) -- for example a simulation step embedded in a host application
// that owns all device memory through its own pool and forbids driver
// allocations, or a latency-critical loop where cudaMalloc's implicit device
// synchronisation and its failure modes under memory pressure are
// unacceptable.  The regular calculator (nbgb_compute_forces) keeps growable
// per-calculator buffers and allocates them on first use; this entry point
// instead uses scratch that lives in file-scope device arrays, reserved
// once when the library is loaded on a device and held until the process
// exits (about 9 MiB per device).
//
// Limits: at most kNoAllocMaxBodies bodies per call, direct sum only.
// All calls share the same scratch arrays: calls whose work overlaps on the
// GPU (different streams, or different host threads, without ordering
// between them) race on that scratch and must be serialised by the caller.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

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

static nbgb_status noalloc_scratch(int dev, NoAllocScratch* out) {
  if (dev < 0 || dev >= 64) return NBGB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocScratch& s = g_noalloc[dev];
  if (!s.ready) {
    if (cudaGetSymbolAddress(reinterpret_cast<void**>(&s.bodies), g_noalloc_bodies) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void**>(&s.partial), g_noalloc_partial) != cudaSuccess ||
        cudaGetSymbolAddress(reinterpret_cast<void**>(&s.err), g_noalloc_err) != cudaSuccess) {
      cudaGetLastError();
      s = NoAllocScratch{};
      return NBGB_ERR_CUDA;
    }
    s.ready = true;
  }
  *out = s;
  return NBGB_OK;
}

}  // namespace nbgb

using namespace nbgb;

extern "C" nbgb_status nbgb_compute_forces_direct_noalloc(const nbgb_particle_data* d, float G,
                                                          float softening, void* stream) {
  try {
    if (!d) return NBGB_ERR_INVALID_ARG;
    if (!(std::isfinite(G) && G > 0.f) || !std::isfinite(softening) || softening < 0.f)
      return NBGB_ERR_INVALID_ARG;
    const int64_t n = (int64_t)d->count;
    if (n > kNoAllocMaxBodies) return NBGB_ERR_INVALID_ARG;  // beyond the static scratch
    if (n == 0) return NBGB_OK;
    if (!d->pos_x || !d->pos_y || !d->pos_z || !d->mass || !d->acc_x || !d->acc_y || !d->acc_z)
      return NBGB_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NBGB_ERR_NO_DEVICE;
    NoAllocScratch s;
    nbgb_status st = noalloc_scratch(dev, &s);  // first call on a device resolves the scratch
    if (st != NBGB_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // The error word keeps the previous call's value: clear it first.
    if (cudaMemsetAsync(s.err, 0, sizeof(uint32_t), cs) != cudaSuccess) return NBGB_ERR_CUDA;
    DirectPlan p = plan_direct(n, n, DirectVariant::kPaired8);
    if (p.splits > kNoAllocMaxSplits) {
      p.tiles_per_split = ceil_div(p.n_tiles, kNoAllocMaxSplits);
      p.splits = (int)ceil_div(p.n_tiles, p.tiles_per_split);
    }
    // Every padded body slot and every partial read below is rewritten by
    // this call, so nothing else of the previous call's contents is used.
    launch_pack_soa(d->pos_x, d->pos_y, d->pos_z, d->mass, n, p.n_src_pad, s.bodies, cs);
    launch_direct(p, s.bodies, s.bodies, n, G, softening * softening, true, s.partial, d->acc_x,
                  d->acc_y, d->acc_z, s.err, cs);
    uint32_t bits = 0;
    if (cudaMemcpyAsync(&bits, s.err, sizeof bits, cudaMemcpyDeviceToHost, cs) != cudaSuccess)
      return NBGB_ERR_CUDA;
    if (cudaStreamSynchronize(cs) != cudaSuccess) return NBGB_ERR_CUDA;
    return bits ? NBGB_ERR_DEVICE_TIMEOUT : NBGB_OK;
  } catch (const Error& e) {
    return e.status;
  }
}
