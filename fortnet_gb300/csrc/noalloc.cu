// Allocation-free z-score statistics (fnetg_acsf_zscore_stats_noalloc).
//
// The same reduction as the z-score statistics of fnetg_acsf_zscore(..., compute = 1)
// (acsf.F90:445-511: weighted mean and population standard deviation per ACSF column), with
// three differences that let it run where the caller cannot let the library allocate:
//   * the per-chunk partial sums live in one file-scope device array of kScratchDoubles
//     doubles (1 MiB) instead of a context buffer that grows on demand;
//   * the integer structure weights are read from device memory and the weight total is
//     reduced on the device, so no host-to-device staging buffer is needed;
//   * the statistics are written to a caller-provided device array; the features are left
//     unstandardised.
// Every partial the reduction reads is written earlier in the same call, so nothing in the
// scratch array has to start at zero.  The array is shared by every call on a device:
// overlapping calls (other streams, other contexts on the same device) race on it.
#include <algorithm>
#include <atomic>

#include "internal.cuh"

namespace fnetg {

namespace {

constexpr int64_t kScratchDoubles = 131072;  // 1 MiB
constexpr int kMaxCols = 4095;               // nG + 1 partials per chunk, >= 32 chunks

static __device__ __align__(256) double g_zscore_scratch[kScratchDoubles];

// Chunk b of the atoms (in atom order): partial sums per column f < ng, and in column ng the
// weight total of the chunk.  mean == nullptr: sums of w x; else sums of w (x - mean)^2.
template <typename T>
__global__ void zsum_na_kernel(const T *feat, int nf, int ng, const int32_t *bpos,
                               const int32_t *astruct, const int32_t *w, int64_t N,
                               const double *mean, double *part, int64_t chunk) {
  const int64_t a0 = (int64_t)blockIdx.x * chunk;
  const int64_t a1 = min(N, a0 + chunk);
  for (int f = threadIdx.x; f <= ng; f += blockDim.x) {
    double acc = 0.0;
    for (int64_t a = a0; a < a1; a++) {
      const double wt = w ? (double)w[astruct[a]] : 1.0;
      if (f == ng) {
        acc += wt;
        continue;
      }
      const double x = (double)feat[(int64_t)bpos[a] * nf + f];
      if (mean) {
        const double d = x - mean[f];
        acc += wt * (d * d);
      } else {
        acc += wt * x;
      }
    }
    part[(int64_t)blockIdx.x * (ng + 1) + f] = acc;
  }
}

// out[f] = (sum over chunks of column f) / (sum over chunks of the weight column), then the
// square root for the deviation pass.
__global__ void zfinish_na_kernel(const double *part, int nparts, int ng, double *out,
                                  int is_std) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= ng) return;
  double acc = 0.0, den = 0.0;
  for (int p = 0; p < nparts; p++) {
    acc += part[(int64_t)p * (ng + 1) + f];
    den += part[(int64_t)p * (ng + 1) + ng];
  }
  out[f] = is_std ? sqrt(acc / den) : acc / den;
}

// Scratch address per device, looked up once with that device current.  Host threads making
// their first call on a device at the same time may both look it up; they store the same
// value, and the atomic entries make that well defined.
constexpr int kMaxDevices = 64;
std::atomic<double *> g_scratch_addr[kMaxDevices] = {};

template <typename T>
int run_stats(fnetg_ctx *ctx, const int32_t *d_weights, double *d_zprec, double *scratch) {
  const int ng = (int)ctx->gf.size();
  const int64_t N = ctx->N;
  const int64_t max_parts = kScratchDoubles / (ng + 1);
  const int64_t chunk = std::max<int64_t>(256, (N + max_parts - 1) / max_parts);
  const int nparts = (int)((N + chunk - 1) / chunk);
  const int thr = std::min(256, std::max(32, (ng + 1 + 31) / 32 * 32));
  const T *feat = ctx->d_feat.as<T>();
  const int32_t *bpos = ctx->d_bpos.as<int32_t>();
  const int32_t *astruct = ctx->d_atom_struct.as<int32_t>();
  zsum_na_kernel<T><<<nparts, thr, 0, ctx->stream>>>(feat, ctx->nf, ng, bpos, astruct,
                                                      d_weights, N, nullptr, scratch, chunk);
  zfinish_na_kernel<<<ceil_div(ng, 128), 128, 0, ctx->stream>>>(scratch, nparts, ng, d_zprec, 0);
  zsum_na_kernel<T><<<nparts, thr, 0, ctx->stream>>>(feat, ctx->nf, ng, bpos, astruct,
                                                      d_weights, N, d_zprec, scratch, chunk);
  zfinish_na_kernel<<<ceil_div(ng, 128), 128, 0, ctx->stream>>>(scratch, nparts, ng,
                                                                 d_zprec + ng, 1);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FNETG_OK : fail(ctx, FNETG_E_CUDA, cudaGetErrorString(e));
}

}  // namespace

}  // namespace fnetg

using namespace fnetg;

extern "C" int fnetg_acsf_zscore_stats_noalloc(fnetg_ctx *ctx, const int32_t *d_weights,
                                               double *d_zprec) {
  if (!ctx || !d_zprec) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "zscore_stats_noalloc: no features computed");
  FNETG_CHECK(!ctx->zprec_valid, FNETG_E_INVALID,
              "zscore_stats_noalloc: the features are already standardised (fnetg_acsf_zscore)");
  const int ng = (int)ctx->gf.size();
  FNETG_CHECK(ng >= 1 && ng <= kMaxCols, FNETG_E_UNSUPPORTED,
              "zscore_stats_noalloc: the number of ACSF columns must lie in [1, 4095]");
  FNETG_CHECK(ctx->N > 0, FNETG_E_INVALID, "zscore_stats_noalloc: empty dataset");
  FNETG_CHECK(ctx->device >= 0 && ctx->device < kMaxDevices, FNETG_E_UNSUPPORTED,
              "zscore_stats_noalloc: device ordinal beyond 63");
  // the context's device is made current for the call and the caller's device restored after
  int prev = -1;
  FNETG_CUDA(cudaGetDevice(&prev));
  struct Restore {
    int dev;
    ~Restore() { cudaSetDevice(dev); }
  } restore{prev};
  FNETG_CUDA(cudaSetDevice(ctx->device));
  double *scratch = g_scratch_addr[ctx->device].load(std::memory_order_relaxed);
  if (!scratch) {
    // first call on this device: resolve the scratch array's address
    FNETG_CUDA(cudaGetSymbolAddress((void **)&scratch, g_zscore_scratch));
    g_scratch_addr[ctx->device].store(scratch, std::memory_order_relaxed);
  }
  return ctx->prec == FNETG_FP64 ? run_stats<double>(ctx, d_weights, d_zprec, scratch)
                                 : run_stats<float>(ctx, d_weights, d_zprec, scratch);
}
