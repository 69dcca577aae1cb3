// K6/K7/K8: per-species network forward (TNetwork_fprop / iPredict, lib_nn/network.F90:146-180,
// 314-347), backward with weight/bias gradient accumulation (TNetwork_bprop 248-296 driven by
// TBpnn_sysTrain, lib_nn/bpnn.F90:610-704) and input Jacobians (TNetwork_fdevi 183-244,
// computed here in reverse mode).
//
// Feature rows are stored species-bucketed, so every CTA works on a tile of rows of ONE
// sub-network and reads one weight set.  One thread per row; hidden activations live in
// shared memory (one padded row per thread, bank-conflict free), weights are read from a
// kernel-friendly copy (row-major [d_in][d_out] per layer) through warp-uniform vector
// loads, eight (FP32) or four (FP64) output neurons per pass.  Per-tile weight-gradient
// partials are reduced across tiles in FP64.
#include <algorithm>

#include "internal.cuh"

namespace fnetg {

namespace {

struct NetDesc {
  int nlayer;
  int dims[kMaxLayers];
  int64_t cw[kMaxLayers];  // compute-layout weight offset of layer l (d_l x d_{l+1}, row-major)
  int64_t cb[kMaxLayers];  // compute-layout bias offset of layer l+1
  int64_t stride;          // compute-layout parameters per species
  int act;
  int hidden_w;            // sum of hidden widths (z storage per row)
  int zoff[kMaxLayers];    // offset of layer l's z in a row's scratch (l = 1..L-2)
  int maxw;
};

template <typename T> __device__ __forceinline__ T act_f(int t, T x) {
  switch (t) {
    case FNETG_ACT_TANH: return tanh(x);
    case FNETG_ACT_SIGMOID: return (T)1 / ((T)1 + exp(-x));
    case FNETG_ACT_RELU: return x > (T)0 ? x : (T)0;
    case FNETG_ACT_LRELU: return ((T)0.01 * x > x) ? (T)0.01 * x : x;
    case FNETG_ACT_SOFTPLUS: return log((T)1 + exp(x));
    case FNETG_ACT_BENT: return (sqrt(x * x + (T)1) - (T)1) / (T)2 + x;
    case FNETG_ACT_ATAN: return atan(x);
    case FNETG_ACT_GAUSSIAN: return exp(-(x * x));
    case FNETG_ACT_HEAVISIDE: return x > (T)0 ? (T)1 : (T)0;
    default: return x;
  }
}

template <typename T> __device__ __forceinline__ T act_d(int t, T x) {
  switch (t) {
    case FNETG_ACT_TANH: { T th = tanh(x); return (T)1 - th * th; }
    case FNETG_ACT_SIGMOID: { T sg = (T)1 / ((T)1 + exp(-x)); return sg * ((T)1 - sg); }
    case FNETG_ACT_RELU: return x >= (T)0 ? (T)1 : (T)0;
    case FNETG_ACT_LRELU: return x >= (T)0 ? (T)1 : (T)0.01;
    case FNETG_ACT_SOFTPLUS: return (T)1 / ((T)1 + exp(-x));
    case FNETG_ACT_BENT: return x / ((T)2 * sqrt(x * x + (T)1)) + (T)1;
    case FNETG_ACT_ATAN: return (T)1 / (x * x + (T)1);
    case FNETG_ACT_GAUSSIAN: return (T)-2 * x * exp(-(x * x));
    case FNETG_ACT_HEAVISIDE: return (T)0;
    default: return (T)1;
  }
}

template <> __device__ __forceinline__ float act_f<float>(int t, float x) {
  switch (t) {
    case FNETG_ACT_TANH: return tanhf(x);
    case FNETG_ACT_SIGMOID: return 1.f / (1.f + expf(-x));
    case FNETG_ACT_RELU: return x > 0.f ? x : 0.f;
    case FNETG_ACT_LRELU: return (0.01f * x > x) ? 0.01f * x : x;
    case FNETG_ACT_SOFTPLUS: return logf(1.f + expf(x));
    case FNETG_ACT_BENT: return (sqrtf(x * x + 1.f) - 1.f) / 2.f + x;
    case FNETG_ACT_ATAN: return atanf(x);
    case FNETG_ACT_GAUSSIAN: return expf(-(x * x));
    case FNETG_ACT_HEAVISIDE: return x > 0.f ? 1.f : 0.f;
    default: return x;
  }
}

template <> __device__ __forceinline__ float act_d<float>(int t, float x) {
  switch (t) {
    case FNETG_ACT_TANH: { float th = tanhf(x); return 1.f - th * th; }
    case FNETG_ACT_SIGMOID: { float sg = 1.f / (1.f + expf(-x)); return sg * (1.f - sg); }
    case FNETG_ACT_RELU: return x >= 0.f ? 1.f : 0.f;
    case FNETG_ACT_LRELU: return x >= 0.f ? 1.f : 0.01f;
    case FNETG_ACT_SOFTPLUS: return 1.f / (1.f + expf(-x));
    case FNETG_ACT_BENT: return x / (2.f * sqrtf(x * x + 1.f)) + 1.f;
    case FNETG_ACT_ATAN: return 1.f / (x * x + 1.f);
    case FNETG_ACT_GAUSSIAN: return -2.f * x * expf(-(x * x));
    case FNETG_ACT_HEAVISIDE: return 0.f;
    default: return 1.f;
  }
}

// One dense layer for one row: out[o] = b[o] + sum_k in[k] * W[k][o] for o in [0, dout).
// `in` is a row of stride 1 (shared or global), `W` row-major [din][dout].
template <typename T, int OB>
__device__ __forceinline__ void dense_row(const T *__restrict__ W, const T *__restrict__ b,
                                          const T *in, int din, int dout, T *z_out) {
  for (int o0 = 0; o0 < dout; o0 += OB) {
    T acc[OB];
#pragma unroll
    for (int u = 0; u < OB; u++) acc[u] = (o0 + u < dout) ? b[o0 + u] : (T)0;
    if (o0 + OB <= dout) {
      for (int k = 0; k < din; k++) {
        const T x = in[k];
        const T *w = W + (int64_t)k * dout + o0;
#pragma unroll
        for (int u = 0; u < OB; u++) acc[u] += x * __ldg(w + u);
      }
    } else {
      for (int k = 0; k < din; k++) {
        const T x = in[k];
        const T *w = W + (int64_t)k * dout + o0;
#pragma unroll
        for (int u = 0; u < OB; u++)
          if (o0 + u < dout) acc[u] += x * __ldg(w + u);
      }
    }
#pragma unroll
    for (int u = 0; u < OB; u++)
      if (o0 + u < dout) z_out[o0 + u] = acc[u];
  }
}

template <typename T> struct MlpArgs {
  NetDesc net;
  const T *params;        // compute layout
  const T *feat;          // bucketed rows [N][nf]
  int nf;
  const int4 *tiles;      // (species, row0, nrows, 0)
  const int32_t *bperm;   // row -> atom
  double *out;            // [N][nout] atom order (forward)
  // backward
  const double *delta_out;  // [N][nout] atom order: scaled loss gradient of the outputs
  T *gpart;               // [ntiles][stride] per-tile gradient partials (compute layout)
  // jacobian
  int jac_out;            // output index
  const double *zsd;      // z-score standard deviations (or null), length ng
  int ng;                 // number of ACSF columns (z-score applies to these)
  double *jac64;          // [N][nf] atom order (API)
  T *jacT;                // [N][nf] atom order scaled by 1/sd (forces)
};

// smem row stride (odd in 4-byte words for conflict-free per-thread rows)
__host__ __device__ inline int row_stride(int w, int elem) {
  int s = w;
  if (elem == 4) s |= 1;
  else s = (s % 2 == 0) ? s + 1 : s;
  return s;
}

template <typename T, int OB>
__global__ void mlp_forward_kernel(MlpArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);
  const int4 tl = a.tiles[blockIdx.x];
  const int t = threadIdx.x;
  if (t >= tl.z) return;
  const int64_t row = tl.y + t;
  const NetDesc &n = a.net;
  const T *P = a.params + (int64_t)tl.x * n.stride;
  const int rs = row_stride(2 * n.maxw, sizeof(T));
  T *buf = sm + (int64_t)t * rs;
  T *A = buf, *B = buf + n.maxw;
  const T *in = a.feat + row * a.nf;
  const int L = n.nlayer;
  for (int l = 0; l < L - 1; l++) {
    const int din = n.dims[l], dout = n.dims[l + 1];
    T *dst = (l % 2 == 0) ? A : B;
    dense_row<T, OB>(P + n.cw[l], P + n.cb[l], in, din, dout, dst);
    if (l < L - 2)
      for (int o = 0; o < dout; o++) dst[o] = act_f<T>(n.act, dst[o]);
    in = dst;
  }
  const int nout = n.dims[L - 1];
  const int64_t atom = a.bperm[row];
  for (int o = 0; o < nout; o++) a.out[atom * nout + o] = (double)in[o];
}

// Reverse-mode Jacobian of output jac_out with respect to the row's inputs.
template <typename T, int OB>
__global__ void mlp_jacobian_kernel(MlpArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);
  const int4 tl = a.tiles[blockIdx.x];
  const int t = threadIdx.x;
  if (t >= tl.z) return;
  const int64_t row = tl.y + t;
  const NetDesc &n = a.net;
  const T *P = a.params + (int64_t)tl.x * n.stride;
  const int L = n.nlayer;
  const int rs = row_stride(n.hidden_w + 2 * n.maxw, sizeof(T));
  T *Z = sm + (int64_t)t * rs;        // z of hidden layers
  T *D0 = Z + n.hidden_w;             // delta ping
  T *D1 = D0 + n.maxw;                // delta pong
  // forward, keeping z of the hidden layers
  const T *in = a.feat + row * a.nf;
  for (int l = 0; l < L - 2; l++) {
    const int din = n.dims[l], dout = n.dims[l + 1];
    T *z = Z + n.zoff[l + 1];
    dense_row<T, OB>(P + n.cw[l], P + n.cb[l], in, din, dout, z);
    // activations of layer l+1 are needed as the next input: keep them in D0 temporarily
    T *act = (l % 2 == 0) ? D0 : D1;
    for (int o = 0; o < dout; o++) act[o] = act_f<T>(n.act, z[o]);
    in = act;
  }
  // delta of the output layer (linear): unit vector e_o
  const int nout = n.dims[L - 1];
  T *dcur = D0;
  for (int o = 0; o < nout; o++) dcur[o] = (o == a.jac_out) ? (T)1 : (T)0;
  T *dnext = D1;
  for (int l = L - 2; l >= 0; l--) {
    const int din = n.dims[l], dout = n.dims[l + 1];
    const T *W = P + n.cw[l];
    for (int k = 0; k < din; k++) {
      const T *w = W + (int64_t)k * dout;
      T s = 0;
      for (int o = 0; o < dout; o++) s += __ldg(w + o) * dcur[o];
      if (l >= 1) s *= act_d<T>(n.act, Z[n.zoff[l] + k]);
      dnext[k] = s;
    }
    T *tmp = dcur;
    dcur = dnext;
    dnext = tmp;
  }
  const int64_t atom = a.bperm[row];
  for (int k = 0; k < a.nf; k++) {
    const T v = dcur[k];
    if (a.jac64) a.jac64[atom * a.nf + k] = (double)v;
    if (a.jacT) {
      T s = v;
      if (a.zsd && k < a.ng) {
        const double sd = a.zsd[k];
        if (sd >= 1e-08) s = (T)((double)v / sd);
      }
      a.jacT[atom * a.nf + k] = s;
    }
  }
}

// Forward + backward of a tile; per-tile gradient partials in the compute layout.
template <typename T, int OB>
__global__ void mlp_backward_kernel(MlpArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);
  const int4 tl = a.tiles[blockIdx.x];
  const int t = threadIdx.x;
  const int R = blockDim.x;
  const NetDesc &n = a.net;
  const int L = n.nlayer;
  const T *P = a.params + (int64_t)tl.x * n.stride;
  // per-row scratch: z (hidden), then delta of every layer >= 1 (sum of widths 1..L-1)
  int dw_total = 0;
  for (int l = 1; l < L; l++) dw_total += n.dims[l];
  const int rs = row_stride(n.hidden_w + dw_total, sizeof(T));
  T *row_base = sm + (int64_t)t * rs;
  T *Z = row_base;
  T *Dl = Z + n.hidden_w;             // deltas, layer l at doff(l)
  auto doff = [&](int l) {
    int o = 0;
    for (int m = 1; m < l; m++) o += n.dims[m];
    return o;
  };
  const bool active = t < tl.z;
  const int64_t row = tl.y + (active ? t : 0);
  if (active) {
    const T *in = a.feat + row * a.nf;
    for (int l = 0; l < L - 2; l++) {
      const int din = n.dims[l], dout = n.dims[l + 1];
      T *z = Z + n.zoff[l + 1];
      dense_row<T, OB>(P + n.cw[l], P + n.cb[l], in, din, dout, z);
      // next input: activations, kept in the delta area of layer l+1 until the backward
      T *actbuf = Dl + doff(l + 1);
      for (int o = 0; o < dout; o++) actbuf[o] = act_f<T>(n.act, z[o]);
      in = actbuf;
    }
    // output deltas (linear output layer): scaled loss gradients
    const int nout = n.dims[L - 1];
    const int64_t atom = a.bperm[row];
    T *dL = Dl + doff(L - 1);
    for (int o = 0; o < nout; o++) dL[o] = (T)a.delta_out[atom * nout + o];
    // back-propagate: delta_l = (W_l delta_{l+1}) * f'(z_l) for hidden layers l
    for (int l = L - 2; l >= 1; l--) {
      const int din = n.dims[l], dout = n.dims[l + 1];
      const T *W = P + n.cw[l];
      const T *dn = Dl + doff(l + 1);
      T *dc = Dl + doff(l);
      for (int k = 0; k < din; k++) {
        const T *w = W + (int64_t)k * dout;
        T s = 0;
        for (int o = 0; o < dout; o++) s += __ldg(w + o) * dn[o];
        dc[k] = s * act_d<T>(n.act, Z[n.zoff[l] + k]);
      }
    }
  } else {
    // inactive rows contribute zero deltas
    for (int q = 0; q < dw_total; q++) Dl[q] = (T)0;
    for (int q = 0; q < n.hidden_w; q++) Z[q] = (T)0;
  }
  __syncthreads();
  // weight gradients: dW_l[k][o] = sum_rows a_l[row][k] * delta_{l+1}[row][o];
  // bias gradients db_{l+1}[o] = sum_rows delta_{l+1}[row][o]
  T *G = a.gpart + (int64_t)blockIdx.x * n.stride;
  const int nrows = tl.z;
  for (int l = 0; l < L - 1; l++) {
    const int din = n.dims[l], dout = n.dims[l + 1];
    const int dof = doff(l + 1);
    const int64_t nw = (int64_t)din * dout;
    for (int64_t e = t; e < nw + dout; e += R) {
      T acc = 0;
      if (e < nw) {
        const int k = (int)(e / dout), o = (int)(e % dout);
        for (int r = 0; r < nrows; r++) {
          const T *rb = sm + (int64_t)r * rs;
          T ak;
          if (l == 0) ak = a.feat[(tl.y + r) * (int64_t)a.nf + k];
          else ak = act_f<T>(n.act, rb[n.zoff[l] + k]);
          acc += ak * rb[n.hidden_w + dof + o];
        }
        G[n.cw[l] + e] = acc;
      } else {
        const int o = (int)(e - nw);
        for (int r = 0; r < nrows; r++) acc += sm[(int64_t)r * rs + n.hidden_w + dof + o];
        G[n.cb[l] + o] = acc;
      }
    }
  }
}

// FP64 sum of the per-tile partials of every species, written in the reference layout.
template <typename T>
__global__ void grad_reduce_kernel(const T *gpart, const int4 *tiles, const int64_t *sp_tile0,
                                   NetDesc net, const int64_t *ref_of_compute, int64_t nparams,
                                   double *grad64) {
  const int s = blockIdx.y;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= net.stride) return;
  const int64_t t0 = sp_tile0[s], t1 = sp_tile0[s + 1];
  double acc = 0.0;
  for (int64_t t = t0; t < t1; t++) acc += (double)gpart[t * net.stride + q];
  grad64[(int64_t)s * nparams + ref_of_compute[q]] = acc;
}

// reference layout (FP64 master) -> compute layout (T)
template <typename T>
__global__ void params_convert_kernel(const double *p64, T *pc, NetDesc net,
                                      const int64_t *ref_of_compute, int64_t nparams, int nsp) {
  const int s = blockIdx.y;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= net.stride || s >= nsp) return;
  pc[(int64_t)s * net.stride + q] = (T)p64[(int64_t)s * nparams + ref_of_compute[q]];
}

struct Layouts {
  NetDesc net;
  std::vector<int64_t> ref_of_compute;
};

Layouts make_layouts(fnetg_ctx *ctx) {
  Layouts Lo{};
  NetDesc &n = Lo.net;
  n.nlayer = ctx->nlayer;
  n.act = ctx->act;
  n.maxw = 1;
  for (int l = 0; l < ctx->nlayer; l++) {
    n.dims[l] = ctx->dims[l];
    n.maxw = std::max(n.maxw, ctx->dims[l]);
  }
  int64_t ind = 0;
  n.hidden_w = 0;
  for (int l = 0; l < ctx->nlayer - 1; l++) {
    n.cw[l] = ind;
    ind += (int64_t)ctx->dims[l] * ctx->dims[l + 1];
    n.cb[l] = ind;
    ind += ctx->dims[l + 1];
  }
  n.stride = ind;
  for (int l = 1; l < ctx->nlayer - 1; l++) {
    n.zoff[l] = n.hidden_w;
    n.hidden_w += ctx->dims[l];
  }
  Lo.ref_of_compute.assign(n.stride, 0);
  for (int l = 0; l < ctx->nlayer - 1; l++) {
    const int din = ctx->dims[l], dout = ctx->dims[l + 1];
    for (int k = 0; k < din; k++)
      for (int o = 0; o < dout; o++)
        Lo.ref_of_compute[n.cw[l] + (int64_t)k * dout + o] = ctx->woff[l] + k + (int64_t)din * o;
    for (int o = 0; o < dout; o++) Lo.ref_of_compute[n.cb[l] + o] = ctx->boff[l + 1] + o;
  }
  return Lo;
}


template <typename T> constexpr int out_block() { return sizeof(T) == 4 ? 8 : 4; }

template <typename T> size_t fwd_smem(const NetDesc &n, int R) {
  return sizeof(T) * (size_t)R * row_stride(2 * n.maxw, sizeof(T));
}
template <typename T> size_t jac_smem(const NetDesc &n, int R) {
  return sizeof(T) * (size_t)R * row_stride(n.hidden_w + 2 * n.maxw, sizeof(T));
}
template <typename T> size_t bwd_smem(const NetDesc &n, int R) {
  int dw_total = 0;
  for (int l = 1; l < n.nlayer; l++) dw_total += n.dims[l];
  return sizeof(T) * (size_t)R * row_stride(n.hidden_w + dw_total, sizeof(T));
}

template <typename T> int prepare(fnetg_ctx *ctx, Layouts &Lo, MlpArgs<T> &a) {
  Lo = make_layouts(ctx);
  a = MlpArgs<T>{};
  a.net = Lo.net;
  a.params = ctx->d_params.as<T>();
  a.feat = ctx->d_feat.as<T>();
  a.nf = ctx->nf;
  a.tiles = ctx->d_tiles.as<int4>();
  a.bperm = ctx->d_bperm.as<int32_t>();
  return FNETG_OK;
}

template <typename K> int set_smem(fnetg_ctx *ctx, K kernel, size_t bytes) {
  FNETG_CHECK(bytes <= 227 * 1024, FNETG_E_UNSUPPORTED, "network too wide for shared memory");
  FNETG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return FNETG_OK;
}

template <typename T> int do_params(fnetg_ctx *ctx) {
  Layouts Lo;
  MlpArgs<T> a;
  int rc = prepare<T>(ctx, Lo, a);
  if (rc) return rc;
  FNETG_CUDA(ctx->d_ref_of_compute.ensure(sizeof(int64_t) * std::max<int64_t>(Lo.net.stride, 1)));
  FNETG_CUDA(cudaMemcpy(ctx->d_ref_of_compute.p, Lo.ref_of_compute.data(),
                        sizeof(int64_t) * Lo.net.stride, cudaMemcpyHostToDevice));
  FNETG_CUDA(ctx->d_params.ensure(sizeof(T) * ctx->nsp * Lo.net.stride));
  dim3 grid(ceil_div(Lo.net.stride, 256), ctx->nsp);
  LaunchScope ls(ctx, "params");
  params_convert_kernel<T><<<grid, 256, 0, ctx->stream>>>(
      ctx->d_params64.as<double>(), ctx->d_params.as<T>(), Lo.net,
      ctx->d_ref_of_compute.as<int64_t>(), ctx->nparams, ctx->nsp);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

template <typename T> int do_predict(fnetg_ctx *ctx) {
  Layouts Lo;
  MlpArgs<T> a;
  int rc = prepare<T>(ctx, Lo, a);
  if (rc) return rc;
  const int nout = ctx->dims.back();
  FNETG_CUDA(ctx->d_out.ensure(sizeof(double) * std::max<int64_t>(ctx->N, 1) * nout));
  a.out = ctx->d_out.as<double>();
  if (ctx->ntiles == 0) return FNETG_OK;
  const int R = ctx->tile_rows;
  const size_t sm = fwd_smem<T>(Lo.net, R);
  rc = set_smem(ctx, mlp_forward_kernel<T, out_block<T>()>, sm);
  if (rc) return rc;
  LaunchScope ls(ctx, "mlp_forward");
  mlp_forward_kernel<T, out_block<T>()><<<(unsigned)ctx->ntiles, R, sm, ctx->stream>>>(a);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

template <typename T> int do_jacobian(fnetg_ctx *ctx, int o, void *dstT) {
  Layouts Lo;
  MlpArgs<T> a;
  int rc = prepare<T>(ctx, Lo, a);
  if (rc) return rc;
  const int nf = ctx->nf;
  a.jac_out = o;
  a.ng = (int)ctx->gf.size();
  if (dstT) {
    a.jacT = static_cast<T *>(dstT);
    a.zsd = ctx->zprec_valid ? ctx->d_zprec.as<double>() + ctx->gf.size() : nullptr;
  } else {
    FNETG_CUDA(ctx->d_jac.ensure(sizeof(double) * std::max<int64_t>(ctx->N, 1) * nf));
    a.jac64 = ctx->d_jac.as<double>();
  }
  if (ctx->ntiles == 0) return FNETG_OK;
  const int R = ctx->tile_rows;
  const size_t sm = jac_smem<T>(Lo.net, R);
  rc = set_smem(ctx, mlp_jacobian_kernel<T, out_block<T>()>, sm);
  if (rc) return rc;
  LaunchScope ls(ctx, "mlp_jacobian");
  mlp_jacobian_kernel<T, out_block<T>()><<<(unsigned)ctx->ntiles, R, sm, ctx->stream>>>(a);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

template <typename T> int do_backward(fnetg_ctx *ctx) {
  Layouts Lo;
  MlpArgs<T> a;
  int rc = prepare<T>(ctx, Lo, a);
  if (rc) return rc;
  a.delta_out = ctx->d_lossgrad.as<double>();
  FNETG_CUDA(ctx->d_gpart.ensure(sizeof(T) * std::max<int64_t>(ctx->ntiles, 1) * Lo.net.stride));
  a.gpart = ctx->d_gpart.as<T>();
  FNETG_CUDA(ctx->d_grad64.ensure(sizeof(double) * ctx->nsp * ctx->nparams));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_grad64.p, 0, sizeof(double) * ctx->nsp * ctx->nparams,
                             ctx->stream));
  if (ctx->ntiles > 0) {
    const int R = ctx->tile_rows;
    const size_t sm = bwd_smem<T>(Lo.net, R);
    rc = set_smem(ctx, mlp_backward_kernel<T, out_block<T>()>, sm);
    if (rc) return rc;
    LaunchScope ls(ctx, "mlp_backward");
    mlp_backward_kernel<T, out_block<T>()><<<(unsigned)ctx->ntiles, R, sm, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  {
    dim3 grid(ceil_div(Lo.net.stride, 256), ctx->nsp);
    LaunchScope ls(ctx, "reduce");
    grad_reduce_kernel<T><<<grid, 256, 0, ctx->stream>>>(
        ctx->d_gpart.as<T>(), ctx->d_tiles.as<int4>(), ctx->d_sp_tile0.as<int64_t>(), Lo.net,
        ctx->d_ref_of_compute.as<int64_t>(), ctx->nparams, ctx->d_grad64.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

}  // namespace

int run_params_to_compute(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? do_params<double>(ctx) : do_params<float>(ctx);
}
int run_predict(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? do_predict<double>(ctx) : do_predict<float>(ctx);
}
int run_jacobian(fnetg_ctx *ctx, int o, void *dst) {
  return ctx->prec == FNETG_FP64 ? do_jacobian<double>(ctx, o, dst) : do_jacobian<float>(ctx, o, dst);
}
int run_mlp_backward(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? do_backward<double>(ctx) : do_backward<float>(ctx);
}

}  // namespace fnetg
