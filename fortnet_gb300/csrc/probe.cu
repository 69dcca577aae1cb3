// Issue-rate probes of the pipes the featurisation, force and optimiser kernels run on: FP32
// fused multiply-adds, the special-function unit's base-2 exponential (ex2.approx, the MUFU op
// the Gaussians of the ACSF and force kernels use) and FP64 fused multiply-adds (the L-BFGS
// history products).  Each probe keeps every SM busy with
// independent dependency chains, is timed with CUDA events on the context's stream, and gives
// the device's sustained rate: the denominators of the compute rooflines of those kernels.
#include "internal.cuh"

namespace fnetg {

namespace {

constexpr int kProbeThreads = 256;
constexpr int kChains = 8;  // independent chains per thread (covers the pipes' latency)

__global__ void __launch_bounds__(kProbeThreads) fma_probe_kernel(int iters, float seed,
                                                                  float *sink) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = seed + (float)(threadIdx.x + c);
  const float m = 0.999999f, b = 1e-7f;
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int c = 0; c < kChains; c++) x[c] = fmaf(x[c], m, b);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 1234.5f) sink[0] = s;  // keeps the chains alive (a store within the buffer)
}

__global__ void __launch_bounds__(kProbeThreads) fma64_probe_kernel(int iters, double seed,
                                                                    double *sink) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = seed + (double)(threadIdx.x + c);
  const double m = 0.999999, b = 1e-7;
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int c = 0; c < kChains; c++) x[c] = fma(x[c], m, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 1234.5) sink[0] = s;
}

__global__ void __launch_bounds__(kProbeThreads) ex2_probe_kernel(int iters, float seed,
                                                                  float *sink) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = -1e-3f * (seed + (float)(threadIdx.x + c));
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int c = 0; c < kChains; c++) {
        float y;
        asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
        x[c] = -y;  // stays in (-1, 0): the next exponential is in (0.5, 1)
      }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 1234.5f) sink[0] = s;
}

}  // namespace

}  // namespace fnetg

using namespace fnetg;

extern "C" int fnetg_probe_peaks(fnetg_ctx *ctx, double *fp32_tflops, double *ex2_tops,
                                 double *fp64_tflops) {
  if (!ctx) return FNETG_E_INVALID;
  const int sms = num_sms();
  const int grid = sms * 8;  // eight 256-thread CTAs per SM
  // about a quarter of a second per launch or less at the nominal rates (128 FP32 FMA, 16 ex2
  // and 2 FP64 FMA per clock and SM)
  const int iters_of[3] = {256, 32, 4};
  // the loops' sink: a slot of the context's scalars that no result lives in
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  double *sink64 = ctx->d_scalars.as<double>() + 12;
  float *sink = reinterpret_cast<float *>(sink64);
  double best[3] = {0.0, 0.0, 0.0};
  for (int kind = 0; kind < 3; kind++) {
    const int iters = iters_of[kind];
    // threads x iterations x unrolled steps x chains
    const double ops = (double)grid * kProbeThreads * iters * 16.0 * kChains;
    for (int rep = 0; rep < 4; rep++) {  // the first repetition warms up
      FNETG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
      if (kind == 0)
        fma_probe_kernel<<<grid, kProbeThreads, 0, ctx->stream>>>(iters, 1.f, sink);
      else if (kind == 1)
        ex2_probe_kernel<<<grid, kProbeThreads, 0, ctx->stream>>>(iters, 1.f, sink);
      else
        fma64_probe_kernel<<<grid, kProbeThreads, 0, ctx->stream>>>(iters, 1.0, sink64);
      FNETG_CUDA(cudaGetLastError());
      FNETG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
      FNETG_CUDA(cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      FNETG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      if (rep > 0 && ms > 0.f) {
        // an FMA is two FLOPs; an ex2 one operation
        const double rate = ops * (kind == 1 ? 1.0 : 2.0) / (ms * 1e-3) / 1e12;
        best[kind] = std::max(best[kind], rate);
      }
    }
  }
  if (fp32_tflops) *fp32_tflops = best[0];
  if (ex2_tops) *ex2_tops = best[1];
  if (fp64_tflops) *fp64_tflops = best[2];
  return FNETG_OK;
}
