// common.cuh -- shared helpers for the nbgb CUDA kernels (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "nbgb.h"

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "nbgb kernels are written for sm_103a (Blackwell) only"
#endif

namespace nbgb {

// ---------------------------------------------------------------------------
// Host-side error plumbing.  Internals throw nbgb::Error; the C ABI layer
// converts it to an nbgb_status plus a thread-local message.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  nbgb_status status;
  Error(nbgb_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

[[noreturn]] inline void fail(nbgb_status s, const std::string& msg) { throw Error(s, msg); }

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    nbgb_status s = (e == cudaErrorMemoryAllocation) ? NBGB_ERR_OOM
                    : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                        ? NBGB_ERR_NO_DEVICE
                        : NBGB_ERR_CUDA;
    char buf[512];
    std::snprintf(buf, sizeof buf, "CUDA Error: %s (%s) at %s:%d", cudaGetErrorString(e), what,
                  file, line);
    throw Error(s, buf);
  }
}

#define NBGB_CUDA(call) ::nbgb::cuda_check((call), #call, __FILE__, __LINE__)
// Kernel launches issued by this thread (every launch site is followed by
// NBGB_LAUNCH_CHECK); engines report per-call deltas of it.
inline thread_local int64_t t_launches = 0;
#define NBGB_LAUNCH_CHECK()                                                              \
  do {                                                                                   \
    ++::nbgb::t_launches;                                                                \
    ::nbgb::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__);         \
  } while (0)

// ---------------------------------------------------------------------------
// Device error word.  Kernels never trap: a bounded wait that runs out, or a
// capacity that is exceeded, ORs a bit into this word and the kernel returns.
// The host reads it at synchronization points.
// ---------------------------------------------------------------------------
enum DeviceErrorBits : uint32_t {
  kErrWaitTimeout = 1u << 0,    // an mbarrier / flag wait exceeded its iteration limit
  kErrTreeCapacity = 1u << 1,   // octree node count exceeded the allocation
  kErrGridCapacity = 1u << 2,   // spatial hash grid larger than its allocation
  kErrQueueOverflow = 1u << 3,  // ensemble work queue overflow
  kErrBadInput = 1u << 4,       // non-finite bounding box or similar
  kErrWalkStack = 1u << 5,      // Barnes-Hut group walk: traversal stack overflow
};

__device__ __forceinline__ void raise_error(uint32_t* word, uint32_t bits) {
  if (word) atomicOr(word, bits);
}

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t imax64(int64_t a, int64_t b) { return a > b ? a : b; }

// ---------------------------------------------------------------------------
// Arithmetic helpers.
// ---------------------------------------------------------------------------

// MUFU reciprocal square root (max relative error ~2^-22.9), the same
// instruction rsqrtf() lowers to; denormal inputs flush to zero (inputs here
// are r^2 + eps^2 > 0).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Error-free transformation of a + b (Knuth two-sum); returns s, sets e with
// s + e == a + b exactly.  Written with _rn intrinsics so nothing contracts.
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  float s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
  return s;
}

// ---------------------------------------------------------------------------
// Packed FP32x2 (Blackwell `*.f32x2` PTX): two independent FP32 lanes per
// 64-bit register pair, one instruction.
// ---------------------------------------------------------------------------
struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 f2_make(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_split(f2 a, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
__device__ __forceinline__ f2 f2_shfl_xor(f2 a, int lane_mask) {
  f2 r;
  r.v = __shfl_xor_sync(0xffffffffu, a.v, lane_mask);
  return r;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk copy (TMA, non-tensor form) helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arrive on `bar` and announce `bytes` of incoming bulk-copy traffic.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Bulk copy global -> shared, completion signalled on `bar` (complete_tx).
// dst, src 16-byte aligned and bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait for phase `parity` of `bar`.  Returns false (and records a
// timeout in *err) if the phase did not complete within `max_iters` probes.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err,
                                          uint32_t max_iters = (1u << 22)) {
  uint32_t addr = smem_addr(bar);
  for (uint32_t it = 0; it < max_iters; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  raise_error(err, kErrWaitTimeout);
  return false;
}

// ---------------------------------------------------------------------------
// Misc host helpers.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) {
  return (a + b - 1) / b;
}

int num_sms();  // cached SM count of the current device

}  // namespace nbgb
