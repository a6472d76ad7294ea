// probe.cu -- measured FP32 pipe peaks used as roofline denominators.
//
// The direct and Barnes-Hut force stages are bound by the FP32 FMA pipe (no
// stage is a dense contraction, so tensor cores do not apply).  These kernels
// time long independent chains of FFMA, packed FFMA2 (fma.rn.f32x2) and MUFU
// rsqrt on every SM to give the measured rates of this device.
#include "common.cuh"
#include "kernels.cuh"

namespace nbgb {

constexpr int kProbeChains = 16;

__global__ void __launch_bounds__(256) probe_ffma(float* out, int iters, float b, float c) {
  float a[kProbeChains];
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) s += a[k];
  if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(256) probe_ffma2(float* out, int iters, float b, float c) {
  f2 a[kProbeChains / 2];
#pragma unroll
  for (int k = 0; k < kProbeChains / 2; ++k)
    a[k] = f2_make(threadIdx.x * 1e-3f + k, threadIdx.x * 2e-3f + k);
  const f2 bb = f2_make(b, b), cc = f2_make(c, c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kProbeChains / 2; ++k) a[k] = f2_fma(a[k], bb, cc);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kProbeChains / 2; ++k) {
    float lo, hi;
    f2_split(a[k], lo, hi);
    s += lo + hi;
  }
  if (s == 1234.5f) out[0] = s;
}

__global__ void __launch_bounds__(256) probe_mufu(float* out, int iters) {
  float a[kProbeChains];
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) a[k] = 1.0f + threadIdx.x * 1e-3f + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = rsqrt_approx(a[k]);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) s += a[k];
  if (s == 1234.5f) out[0] = s;
}

}  // namespace nbgb

using namespace nbgb;

extern "C" nbgb_status nbgb_measure_fp32_peak(double* ffma_tflops, double* ffma2_tflops,
                                              double* mufu_gops) {
  try {
    const int sms = num_sms();
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float* d_out = nullptr;
    NBGB_CUDA(cudaMalloc(&d_out, sizeof(float)));
    cudaEvent_t e0, e1;
    NBGB_CUDA(cudaEventCreate(&e0));
    NBGB_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](auto launch) {
      float best = 1e30f;
      for (int r = 0; r < 6; ++r) {
        NBGB_CUDA(cudaEventRecord(e0));
        launch();
        NBGB_CUDA(cudaEventRecord(e1));
        NBGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        NBGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (r > 0) best = std::min(best, ms);
      }
      return (double)best;
    };
    const double ops = (double)blocks * threads * iters * kProbeChains;
    double t1 = time_it([&] { probe_ffma<<<blocks, threads>>>(d_out, iters, 0.999f, 1e-3f); });
    double t2 = time_it([&] { probe_ffma2<<<blocks, threads>>>(d_out, iters, 0.999f, 1e-3f); });
    double t3 = time_it([&] { probe_mufu<<<blocks, threads>>>(d_out, iters); });
    NBGB_LAUNCH_CHECK();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_out);
    if (ffma_tflops) *ffma_tflops = 2.0 * ops / (t1 * 1e-3) / 1e12;
    if (ffma2_tflops) *ffma2_tflops = 2.0 * ops / (t2 * 1e-3) / 1e12;
    if (mufu_gops) *mufu_gops = ops / (t3 * 1e-3) / 1e9;
    return NBGB_OK;
  } catch (const Error& e) {
    return e.status;
  }
}
