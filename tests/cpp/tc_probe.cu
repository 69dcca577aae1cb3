// Probe of the tensor-core primitives of fortnet_gb300/csrc/tc.cuh: one 128 x 64 x 32 BF16
// product D = A B^T (D[m][n] = sum_k A[m][k] B[n][k]) through tcgen05.mma with FP32
// accumulation in tensor memory, for every combination of K-major and MN-major operands in the
// library's core-matrix layout, compared with an FP64 product of the same BF16 values.
// Prints one line per combination: "a_mn b_mn max_abs_error max_abs_value".
//
// Every shared-memory buffer is followed by 64 KB of padding, so any reading of the descriptor
// strides stays inside the CTA's shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../fortnet_gb300/csrc/tc.cuh"

using namespace fnetg;

constexpr int M = 128, N = 64, K = 32;
constexpr int kPad = 64 * 1024;

__global__ void probe_kernel(const __nv_bfloat16 *a_img, const __nv_bfloat16 *b_img, int a_mn,
                             int b_mn, float *d_out, int *status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  unsigned char *As = sm;                       // M*K bf16 = 8 KB
  unsigned char *Bs = sm + M * K * 2 + kPad;    // N*K bf16 = 4 KB
  // operand images are already in the core-matrix layout: copy them in
  for (int q = threadIdx.x; q < M * K / 8; q += blockDim.x)
    reinterpret_cast<uint4 *>(As)[q] = reinterpret_cast<const uint4 *>(a_img)[q];
  for (int q = threadIdx.x; q < N * K / 8; q += blockDim.x)
    reinterpret_cast<uint4 *>(Bs)[q] = reinterpret_cast<const uint4 *>(b_img)[q];
  if (threadIdx.x == 0) {
    tc::mbar_init(&mbar, 1);
    tc::mbar_fence_init();
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&tmem_base, 64);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base;
  if (threadIdx.x == 0) {
    // A is M x K: K-major stored as (rows m, cols k); MN-major stored as (rows k, cols m)
    const uint32_t a_lbo = a_mn ? 128u : 16u * M, a_sbo = a_mn ? 16u * K : 128u;
    const uint32_t a_kstep = a_mn ? 2u * 128u : 2u * 16u * M;
    const uint32_t b_lbo = b_mn ? 128u : 16u * N, b_sbo = b_mn ? 16u * K : 128u;
    const uint32_t b_kstep = b_mn ? 2u * 128u : 2u * 16u * N;
    const uint32_t idesc = tc::idesc_bf16(M, N, a_mn, b_mn);
    for (int ks = 0; ks < K / 16; ks++) {
      const uint64_t ad = tc::smem_desc(tc::smem_u32(As) + ks * a_kstep, a_lbo, a_sbo);
      const uint64_t bd = tc::smem_desc(tc::smem_u32(Bs) + ks * b_kstep, b_lbo, b_sbo);
      tc::mma_bf16(tbase, ad, bd, idesc, ks > 0);
    }
    tc::mma_commit(&mbar);
  }
  const bool ok = tc::mbar_wait(&mbar, 0);
  if (!ok) atomicExch(status, 1);
  tc::fence_after_sync();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + c0, v);
      tc::tmem_wait_ld();
      const int m = warp * 32 + lane;
      for (int k = 0; k < 16; k++) d_out[m * N + c0 + k] = v[k];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tbase, 64);
}

static float bf16_round(float x) { return __bfloat162float(__float2bfloat16(x)); }

int main() {
  srand(12345);
  std::vector<float> A(M * K), B(N * K);
  for (auto &x : A) x = bf16_round((float)rand() / RAND_MAX * 2.f - 1.f);
  for (auto &x : B) x = bf16_round((float)rand() / RAND_MAX * 2.f - 1.f);
  std::vector<double> D(M * N, 0.0);
  double dmax = 0.0;
  for (int m = 0; m < M; m++)
    for (int n = 0; n < N; n++) {
      double s = 0.0;
      for (int k = 0; k < K; k++) s += (double)A[m * K + k] * (double)B[n * K + k];
      D[m * N + n] = s;
      dmax = std::fmax(dmax, std::fabs(s));
    }
  __nv_bfloat16 *da, *db;
  float *dd;
  int *dst;
  cudaMalloc(&da, M * K * 2);
  cudaMalloc(&db, N * K * 2);
  cudaMalloc(&dd, M * N * 4);
  cudaMalloc(&dst, 4);
  const int smem = M * K * 2 + kPad + N * K * 2 + kPad;
  cudaFuncSetAttribute(probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int failed = 0;
  for (int a_mn = 0; a_mn < 2; a_mn++)
    for (int b_mn = 0; b_mn < 2; b_mn++) {
      std::vector<__nv_bfloat16> ai(M * K), bi(N * K);
      // byte offsets / 2 = element offsets in the core-matrix layout
      for (int m = 0; m < M; m++)
        for (int k = 0; k < K; k++) {
          const uint32_t off = a_mn ? tc::core_off(k, m, K) : tc::core_off(m, k, M);
          ai[off / 2] = __float2bfloat16(A[m * K + k]);
        }
      for (int n = 0; n < N; n++)
        for (int k = 0; k < K; k++) {
          const uint32_t off = b_mn ? tc::core_off(k, n, K) : tc::core_off(n, k, N);
          bi[off / 2] = __float2bfloat16(B[n * K + k]);
        }
      cudaMemcpy(da, ai.data(), M * K * 2, cudaMemcpyHostToDevice);
      cudaMemcpy(db, bi.data(), N * K * 2, cudaMemcpyHostToDevice);
      cudaMemset(dd, 0, M * N * 4);
      cudaMemset(dst, 0, 4);
      probe_kernel<<<1, 128, smem>>>(da, db, a_mn, b_mn, dd, dst);
      cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        printf("cuda error %s\n", cudaGetErrorString(e));
        return 2;
      }
      std::vector<float> got(M * N);
      int st = 0;
      cudaMemcpy(got.data(), dd, M * N * 4, cudaMemcpyDeviceToHost);
      cudaMemcpy(&st, dst, 4, cudaMemcpyDeviceToHost);
      double err = 0.0;
      for (int q = 0; q < M * N; q++) err = std::fmax(err, std::fabs(got[q] - D[q]));
      printf("%d %d %.3e %.3e %d\n", a_mn, b_mn, err, dmax, st);
      if (st || !(err <= 1e-5 * dmax)) failed = 1;
    }
  return failed;
}
