// Training with a force term in the loss: L = L_E + c / (3 N) sum_a |F_a - F*_a|^2, with L_E the
// reference's energy loss (lib_common/loss.F90:512-721) and F = -dE/dR the analytical forces
// (forceAnalysis_analytical, lib_analysis/forces.F90:317-425).  The reference trains on
// energies only; this is the force-loss training of the precision form.
//
// The gradient of the force term with respect to the network parameters theta is a mixed
// second derivative.  With x_i the standardised inputs of atom i, J_i = d out_i / d x_i and
// F_k = -sum_i J_i . dx_i/dR_k:
//     dL_F/dtheta = -sum_i d/dtheta (J_i . u_i),   u_i = sum_k dx_i/dR_k . w_k,
//     w_k = dL_F/dF_k = 2 c / (3 N) (F_k - F*_k),
// u is the forward-mode derivative of the features along w (jvp.cu), and J_i . u_i is the
// tangent of the atom's output along u_i, so its parameter gradient is one reverse pass of
// the network carrying activations and tangents together (per layer: z, zdot = W^T t,
// a = tanh z, t = tanh'(z) zdot; reverse: zbar = tanh' abar + tanh'' zdot tbar, zdotbar =
// tanh' tbar, dW += a zbar^T + t zdotbar^T).  The same reverse pass carries the energy
// loss's output gradients, so one kernel yields the whole gradient.
//
// Gradient convention: the energy part is the reference's raw accumulated gradient (not yet
// divided by the summed datapoint weights, bpnn.F90:394-481); the force part is scaled by the
// summed weights, so that after TBpnn_update's normalisation (bpnn.F90:751-766) it is exactly
// dL_F/dtheta.
#include <algorithm>

#include "internal.cuh"

namespace fnetg {

int launch_loss_range(fnetg_ctx *ctx, int s0, int count, int loss);
int launch_loss_reduce(fnetg_ctx *ctx);
int run_features_jvp(fnetg_ctx *ctx, const void *d_w, void *d_u);

namespace {

constexpr int kFlRows = 16;    // atoms per chunk
constexpr int kFlThreads = 128;

struct FlNet {
  int nlayer;
  int dims[kMaxLayers];
  int64_t woff[kMaxLayers], boff[kMaxLayers];
  int64_t nparams;
  // shared-memory plan (elements): per layer input l = 0..L-1: A, T; hidden l = 1..L-2: P, Zd;
  // four adjoint buffers of maxd rows
  int64_t sA[kMaxLayers], sT[kMaxLayers], sP[kMaxLayers], sZ[kMaxLayers], sB[4], total;
};

FlNet make_flnet(fnetg_ctx *ctx) {
  FlNet n{};
  n.nlayer = ctx->nlayer;
  int maxd = 1;
  for (int l = 0; l < ctx->nlayer; l++) {
    n.dims[l] = ctx->dims[l];
    n.woff[l] = ctx->woff[l];
    n.boff[l] = ctx->boff[l];
    if (l >= 1) maxd = std::max(maxd, ctx->dims[l]);
  }
  n.nparams = ctx->nparams;
  int64_t o = 0;
  for (int l = 0; l < n.nlayer; l++) {
    n.sA[l] = o;
    o += (int64_t)n.dims[l] * kFlRows;
    n.sT[l] = o;
    o += (int64_t)n.dims[l] * kFlRows;
    if (l >= 1 && l <= n.nlayer - 2) {
      n.sP[l] = o;
      o += (int64_t)n.dims[l] * kFlRows;
      n.sZ[l] = o;
      o += (int64_t)n.dims[l] * kFlRows;
    }
  }
  for (int b = 0; b < 4; b++) {
    n.sB[b] = o;
    o += (int64_t)maxd * kFlRows;
  }
  n.total = o;
  return n;
}

template <typename T> struct FlArgs {
  FlNet net;
  const double *p64;        // FP64 master parameters [nsp][nparams]
  const T *feat;            // bucketed rows [N][nf]
  const T *u;               // feature tangents [N][nf], atom order
  const int4 *tiles;        // (species, row0, nrows, 0)
  int64_t ntiles;
  const int32_t *bperm;
  const double *delta;      // [N][nout] energy-loss output gradients (nout == 1)
  T *gpart;                 // [ntiles][nparams]
};

template <typename T> __device__ __forceinline__ T tanh_t(T x) { return tanh(x); }
template <> __device__ __forceinline__ float tanh_t<float>(float x) { return tanhf(x); }

// One CTA per tile: chunks of kFlRows atoms through the forward (values + tangents) and the
// reverse pass; per-tile parameter gradients in the reference order.
template <typename T>
__global__ void __launch_bounds__(kFlThreads) fl_backward_kernel(FlArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);
  const FlNet &n = a.net;
  const int L = n.nlayer, nf = n.dims[0];
  const int64_t t = blockIdx.x;
  if (t >= a.ntiles) return;
  const int4 tl = a.tiles[t];
  const double *P = a.p64 + (int64_t)tl.x * n.nparams;
  T *gp = a.gpart + t * n.nparams;
  const int R = kFlRows;
  for (int c0 = 0; c0 < tl.z; c0 += R) {
    const int nr = min(R, tl.z - c0);
    const int64_t row0 = tl.y + c0;
    for (int q = threadIdx.x; q < nf * R; q += blockDim.x) {
      const int k = q / R, r = q % R;
      T x = (T)0, ud = (T)0;
      if (r < nr) {
        x = a.feat[(row0 + r) * nf + k];
        ud = a.u[(int64_t)a.bperm[row0 + r] * nf + k];
      }
      sm[n.sA[0] + q] = x;
      sm[n.sT[0] + q] = ud;
    }
    __syncthreads();
    // forward through the hidden layers: values and tangents
    for (int l = 0; l + 1 <= L - 2; l++) {
      const int din = n.dims[l], dout = n.dims[l + 1];
      for (int q = threadIdx.x; q < dout * R; q += blockDim.x) {
        const int o = q / R, r = q % R;
        T z = (T)P[n.boff[l + 1] + o], zd = (T)0;
        for (int k = 0; k < din; k++) {
          const T w = (T)P[n.woff[l] + k + (int64_t)din * o];
          z += w * sm[n.sA[l] + k * R + r];
          zd += w * sm[n.sT[l] + k * R + r];
        }
        const T av = tanh_t<T>(z);
        const T pv = (T)1 - av * av;
        sm[n.sA[l + 1] + q] = av;
        sm[n.sP[l + 1] + q] = pv;
        sm[n.sZ[l + 1] + q] = zd;
        sm[n.sT[l + 1] + q] = pv * zd;
      }
      __syncthreads();
    }
    // adjoints of the output layer's pre-activations (linear): energy gradient, tangent -1
    T *ZB = sm + n.sB[0], *ZD = sm + n.sB[1], *NB = sm + n.sB[2], *ND = sm + n.sB[3];
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      const bool live = r < nr;
      ZB[r] = live ? (T)a.delta[a.bperm[row0 + r]] : (T)0;
      ZD[r] = live ? (T)-1 : (T)0;
    }
    __syncthreads();
    for (int l = L - 2; l >= 0; l--) {
      const int din = n.dims[l], dout = n.dims[l + 1];
      // dW_l = A_l ZB^T + T_l ZD^T, db_{l+1} = sum ZB
      for (int q = threadIdx.x; q < din * dout + dout; q += blockDim.x) {
        T acc = (T)0;
        int64_t dst;
        if (q < din * dout) {
          const int k = q % din, o = q / din;
          for (int r = 0; r < R; r++)
            acc += sm[n.sA[l] + k * R + r] * ZB[o * R + r] + sm[n.sT[l] + k * R + r] * ZD[o * R + r];
          dst = n.woff[l] + k + (int64_t)din * o;
        } else {
          const int o = q - din * dout;
          for (int r = 0; r < R; r++) acc += ZB[o * R + r];
          dst = n.boff[l + 1] + o;
        }
        gp[dst] = c0 == 0 ? acc : gp[dst] + acc;
      }
      if (l >= 1) {
        // adjoints of layer l's pre-activations
        for (int q = threadIdx.x; q < din * R; q += blockDim.x) {
          const int k = q / R, r = q % R;
          T ab = (T)0, tb = (T)0;
          for (int o = 0; o < dout; o++) {
            const T w = (T)P[n.woff[l] + k + (int64_t)din * o];
            ab += w * ZB[o * R + r];
            tb += w * ZD[o * R + r];
          }
          const T pv = sm[n.sP[l] + q], av = sm[n.sA[l] + q], zd = sm[n.sZ[l] + q];
          ND[q] = pv * tb;
          NB[q] = pv * ab - (T)2 * av * pv * zd * tb;
        }
      }
      __syncthreads();
      T *x = ZB;
      ZB = NB;
      NB = x;
      x = ZD;
      ZD = ND;
      ND = x;
    }
    __syncthreads();
  }
  // parameters this kernel does not produce: the unused output-layer ww(d_L, 1) and the
  // input-layer biases
  for (int64_t q = n.woff[L - 1] + threadIdx.x; q < n.boff[1]; q += blockDim.x) gp[q] = (T)0;
}

template <typename T>
__global__ void fl_reduce_kernel(const T *gpart, const int64_t *sp_tile0, int64_t nparams,
                                 double *grad64) {
  const int s = blockIdx.y;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nparams) return;
  double acc = 0.0;
  for (int64_t t = sp_tile0[s]; t < sp_tile0[s + 1]; t++) acc += (double)gpart[t * nparams + q];
  grad64[(int64_t)s * nparams + q] = acc;
}

// w = scale (F - F*) in the context's arithmetic; per-block sums of |F - F*|^2
template <typename T>
__global__ void fl_prep_kernel(const double *F, const double *Ft, int64_t n, double scale, T *w,
                               double *part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n;
       a += (int64_t)gridDim.x * blockDim.x) {
    for (int c = 0; c < 3; c++) {
      const double v = F[3 * a + c] - Ft[3 * a + c];
      w[3 * a + c] = (T)(scale * v);
      acc += v * v;
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// scalars[2] = c / (3 N) sum |F - F*|^2; scalars[0] += scalars[2] (total loss); scalars[3] = L_E
__global__ void fl_finish_kernel(const double *part, int nb, double coef, double *scalars) {
  double acc = 0.0;
  for (int b = 0; b < nb; b++) acc += part[b];
  scalars[3] = scalars[0];
  scalars[2] = coef * acc;
  scalars[0] = scalars[0] + scalars[2];
}

constexpr int kPrepBlocks = 256;

// The force term of the loss at the current forces: L_F into scalars[2] (and added to the
// total in scalars[0]), the loss's force gradient w scaled by the summed weights, and the
// input tangents u = (dx/dR) w (jvp.cu) into d_fl_u.
template <typename T> int force_loss_terms(fnetg_ctx *ctx) {
  const int64_t N = ctx->N;
  FNETG_CUDA(ctx->d_fl_w.ensure(sizeof(T) * std::max<int64_t>(3 * N, 1)));
  FNETG_CUDA(ctx->d_fl_u.ensure(sizeof(T) * std::max<int64_t>(N, 1) * ctx->nf));
  FNETG_CUDA(ctx->d_fl_part.ensure(sizeof(double) * kPrepBlocks));
  const double c = ctx->fl_weight, n3 = 3.0 * (double)std::max<int64_t>(N, 1);
  {
    LaunchScope ls(ctx, "force_loss");
    fl_prep_kernel<T><<<kPrepBlocks, 256, 0, ctx->stream>>>(
        ctx->d_forces.as<double>(), ctx->d_fl_target.as<double>(), N,
        ctx->sum_weights * 2.0 * c / n3, ctx->d_fl_w.as<T>(), ctx->d_fl_part.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  {
    LaunchScope ls(ctx, "force_loss");
    fl_finish_kernel<<<1, 1, 0, ctx->stream>>>(ctx->d_fl_part.as<double>(), kPrepBlocks, c / n3,
                                               ctx->d_scalars.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  return run_features_jvp(ctx, ctx->d_fl_w.p, ctx->d_fl_u.p);
}

template <typename T> int do_force_gradients(fnetg_ctx *ctx, int loss) {
  FNETG_CHECK(ctx->act == FNETG_ACT_TANH && ctx->dims.back() == 1 && ctx->ngt == 1 &&
                  ctx->nat == 0,
              FNETG_E_UNSUPPORTED,
              "force loss: tanh networks with one output and one global target (energy)");
  FNETG_CHECK(ctx->nb_valid && ctx->zprec_valid, FNETG_E_INVALID,
              "force loss: neighbour list and z-scored features are needed");
  int rc = run_predict(ctx);
  if (rc) return rc;
  rc = launch_loss_range(ctx, 0, ctx->S, loss);
  if (rc) return rc;
  rc = launch_loss_reduce(ctx);
  if (rc) return rc;
  rc = run_forces(ctx);
  if (rc) return rc;
  rc = force_loss_terms<T>(ctx);
  if (rc) return rc;
  FlArgs<T> a{};
  a.net = make_flnet(ctx);
  a.p64 = ctx->d_params64.as<double>();
  a.feat = ctx->d_feat.as<T>();
  a.u = ctx->d_fl_u.as<T>();
  a.tiles = ctx->d_tiles.as<int4>();
  a.ntiles = ctx->ntiles;
  a.bperm = ctx->d_bperm.as<int32_t>();
  a.delta = ctx->d_lossgrad.as<double>();
  FNETG_CUDA(ctx->d_fl_gpart.ensure(sizeof(T) * std::max<int64_t>(ctx->ntiles, 1) * ctx->nparams));
  a.gpart = ctx->d_fl_gpart.as<T>();
  const size_t smem = sizeof(T) * (size_t)a.net.total;
  FNETG_CHECK(smem <= 227 * 1024, FNETG_E_UNSUPPORTED, "force loss: network too wide");
  FNETG_CUDA(raise_smem_limit((const void *)fl_backward_kernel<T>, smem));
  if (ctx->ntiles > 0) {
    LaunchScope ls(ctx, "force_loss_backward");
    fl_backward_kernel<T><<<(unsigned)ctx->ntiles, kFlThreads, smem, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  FNETG_CUDA(ctx->d_grad64.ensure(sizeof(double) * ctx->nsp * ctx->nparams));
  {
    dim3 grid(ceil_div(ctx->nparams, 256), ctx->nsp);
    LaunchScope ls(ctx, "reduce");
    fl_reduce_kernel<T><<<grid, 256, 0, ctx->stream>>>(a.gpart, ctx->d_sp_tile0.as<int64_t>(),
                                                       ctx->nparams, ctx->d_grad64.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

}  // namespace

int run_force_loss_terms(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? force_loss_terms<double>(ctx) : force_loss_terms<float>(ctx);
}

int run_force_gradients(fnetg_ctx *ctx, int loss) {
  return ctx->prec == FNETG_FP64 ? do_force_gradients<double>(ctx, loss)
                                 : do_force_gradients<float>(ctx, loss);
}

}  // namespace fnetg

using namespace fnetg;

extern "C" {

int fnetg_set_force_targets(fnetg_ctx *ctx, double weight, const double *forces) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(weight >= 0.0 && std::isfinite(weight), FNETG_E_INVALID,
              "set_force_targets: weight must be finite and >= 0");
  if (weight == 0.0) {
    ctx->fl_weight = 0.0;
    return FNETG_OK;
  }
  FNETG_CHECK(forces != nullptr, FNETG_E_INVALID, "set_force_targets: no forces");
  const int64_t N = ctx->N;
  for (int64_t q = 0; q < 3 * N; q++)
    FNETG_CHECK(std::isfinite(forces[q]), FNETG_E_INVALID, "set_force_targets: non-finite force");
  FNETG_CUDA(ctx->d_fl_target.ensure(sizeof(double) * std::max<int64_t>(3 * N, 1)));
  if (N > 0)
    FNETG_CUDA(copy_sync(ctx, ctx->d_fl_target.p, forces, sizeof(double) * 3 * N,
                          cudaMemcpyHostToDevice));
  ctx->fl_weight = weight;
  return FNETG_OK;
}

int fnetg_last_losses(fnetg_ctx *ctx, double *loss_energy, double *loss_forces) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->d_scalars.p != nullptr, FNETG_E_INVALID, "last_losses: no loss computed");
  double s[4] = {0, 0, 0, 0};
  FNETG_CUDA(copy_sync(ctx, s, ctx->d_scalars.p, sizeof(double) * 4, cudaMemcpyDeviceToHost));
  if (loss_energy) *loss_energy = ctx->fl_weight > 0.0 ? s[3] : s[0];
  if (loss_forces) *loss_forces = ctx->fl_weight > 0.0 ? s[2] : 0.0;
  return FNETG_OK;
}

}  // extern "C"
