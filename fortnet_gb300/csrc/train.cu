// Training on the device: per-structure output sums, losses and loss gradients
// (lib_common/loss.F90:217-721, TBpnn_sysTrain bpnn.F90:654-701), the gradient
// preparation of TBpnn_update (bpnn.F90:751-766, elastic net nestedtypes.F90:336-370) and
// the optimisers — steepest descent (lib_dftbp/steepdesc.F90:126-204) and L-BFGS with its
// line minimiser (lib_dftbp/lbfgs.F90:283-488, linemin.F90:141-391) — with one CTA per
// sub-network holding the optimiser state in FP64 device memory.
#include <algorithm>

#include "internal.cuh"

namespace fnetg {

int run_mlp_backward(fnetg_ctx *ctx);

namespace {

constexpr double kEps = 2.220446049250313e-16;        // epsilon(1.0_dp)
constexpr double kGoldenMeanP1 = 1.6180339887498949;  // lib_dftbp/constants.F90:131
constexpr int kOptThreads = 512;

struct LossArgs {
  int S;
  const int64_t *off;
  const double *out;      // [N][nout]
  int nout, ngt, nat;
  const double *gt, *at, *aw, *saw;
  const int32_t *w;
  int loss;
  double *delta;          // [N][nout] scaled output gradients
  double *part;           // [S][2] loss numerator / denominator per structure
};

// one CTA of kLossThreads per structure: the structure's atoms strided over the threads, sums
// by warp shuffles and a shared-memory combine (large structures no longer serialise a warp)
constexpr int kLossThreads = 128;

__device__ __forceinline__ double cta_sum(double v, double *sh) {
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) v += __shfl_xor_sync(0xffffffffu, v, k);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kLossThreads / 32; w++) t += sh[w];
  return t;
}

__global__ void __launch_bounds__(kLossThreads) loss_cta_kernel(LossArgs a) {
  __shared__ double sh[kLossThreads / 32];
  const int s = blockIdx.x;
  if (s >= a.S) return;
  const int64_t a0 = a.off[s], a1 = a.off[s + 1];
  const int n = (int)(a1 - a0);
  const double ws = a.w ? (double)a.w[s] : 1.0;
  double num = 0.0, den = 0.0;
  if (a.ngt > 0) {
    double lsum = 0.0;
    for (int o = 0; o < a.ngt; o++) {
      // four outputs requested together per thread (large structures: 2,048 atoms are 16 per
      // thread), partial sums combined in a fixed order
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int64_t at = a0 + threadIdx.x;
      for (; at + 3 * kLossThreads < a1; at += 4 * kLossThreads) {
        s0 += a.out[at * a.nout + o];
        s1 += a.out[(at + kLossThreads) * a.nout + o];
        s2 += a.out[(at + 2 * kLossThreads) * a.nout + o];
        s3 += a.out[(at + 3 * kLossThreads) * a.nout + o];
      }
      for (; at < a1; at += kLossThreads) s0 += a.out[at * a.nout + o];
      double sum = cta_sum((s0 + s1) + (s2 + s3), sh);
      const double t = a.gt[(int64_t)s * a.ngt + o];
      const double lg = lossgrad(a.loss, sum, t);
      lsum += loss_term(a.loss, sum, t);
      // the structure's factor of every atom's output gradient, lg / n * ws (lg w / n ws for
      // atomic weight w; equal to it for w = 1): one FP64 division per structure, not per atom
      const double g = lg / (double)n * ws;
      // atomic weights of four atoms loaded before their four stores (the stores could alias
      // the loads as far as the compiler knows)
      at = a0 + threadIdx.x;
      for (; at + 3 * kLossThreads < a1; at += 4 * kLossThreads) {
        const double w0 = a.aw[at], w1 = a.aw[at + kLossThreads],
                     w2 = a.aw[at + 2 * kLossThreads], w3 = a.aw[at + 3 * kLossThreads];
        a.delta[at * a.nout + o] = g * w0;
        a.delta[(at + kLossThreads) * a.nout + o] = g * w1;
        a.delta[(at + 2 * kLossThreads) * a.nout + o] = g * w2;
        a.delta[(at + 3 * kLossThreads) * a.nout + o] = g * w3;
      }
      for (; at < a1; at += kLossThreads) a.delta[at * a.nout + o] = g * a.aw[at];
    }
    num += ws * a.saw[s] * loss_finish(a.loss, lsum, a.ngt);
    den += ws * a.saw[s];
  }
  if (a.nat > 0) {
    double ln = 0.0, ld = 0.0;
    for (int64_t at = a0 + threadIdx.x; at < a1; at += kLossThreads) {
      double lsum = 0.0;
      for (int t = 0; t < a.nat; t++) {
        const double p = a.out[at * a.nout + a.ngt + t];
        const double tg = a.at[at * a.nat + t];
        lsum += loss_term(a.loss, p, tg);
        a.delta[at * a.nout + a.ngt + t] = lossgrad(a.loss, p, tg) * a.aw[at] / (double)n * ws;
      }
      ln += ws * a.aw[at] * loss_finish(a.loss, lsum, a.nat);
      ld += ws * a.aw[at];
    }
    num += cta_sum(ln, sh);
    den += cta_sum(ld, sh);
  }
  if (threadIdx.x == 0) {
    a.part[2 * s] = num;
    a.part[2 * s + 1] = den;
  }
}

template <int NT> __device__ double block_sum(double v, double *sh) {
  const int t = threadIdx.x;
  __syncthreads();
  sh[t] = v;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (t < o) sh[t] += sh[t + o];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

template <int NT> __device__ double block_max(double v, double *sh) {
  const int t = threadIdx.x;
  __syncthreads();
  sh[t] = v;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (t < o) sh[t] = fmax(sh[t], sh[t + o]);
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void loss_reduce_kernel(const double *part, int S, double *scalars) {
  __shared__ double sh[1024];
  double num = 0.0, den = 0.0;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    num += part[2 * s];
    den += part[2 * s + 1];
  }
  num = block_sum<1024>(num, sh);
  den = block_sum<1024>(den, sh);
  if (threadIdx.x == 0) scalars[0] = num / den;
}

// elastic net (nestedtypes.F90:336-370), 1/sum(w), per-species sum of squares
__global__ void update_prepare_kernel(const double *params, double *grad, int64_t np, int64_t nw,
                                      double lam, double alpha, double sumw, double *sq) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  const double *p = params + s * np;
  double *g = grad + s * np;
  double acc = 0.0;
  for (int64_t q = threadIdx.x; q < np; q += blockDim.x) {
    double v = g[q];
    if (q < nw) {
      const double ww = p[q];
      const double sgn = ww == 0.0 ? 0.0 : (ww > 0.0 ? 1.0 : -1.0);
      v = v + lam / (double)nw * ((1.0 - alpha) * ww + alpha * sgn);
    }
    v = v / sumw;
    g[q] = v;
    acc += v * v;
  }
  acc = block_sum<kOptThreads>(acc, sh);
  if (threadIdx.x == 0) sq[s] = acc;
}

__global__ void norm_finish_kernel(const double *sq, int nsp, double *scalars) {
  double acc = 0.0;
  for (int s = 0; s < nsp; s++) acc += sq[s];
  scalars[1] = sqrt(acc);
}

// ---------------------------------------------------------------- steepest descent
struct SdState {
  double tol, maxdisp, lr;
};

__global__ void sd_kernel(double *params, const double *grad, int64_t np, SdState st,
                          int *conv_flags) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  double *x = params + s * np;
  const double *g = grad + s * np;
  if (conv_flags[s]) return;  // sticky convergence: xNew = xOld
  double gmax = 0.0;
  for (int64_t q = threadIdx.x; q < np; q += blockDim.x) gmax = fmax(gmax, fabs(g[q]));
  gmax = block_max<kOptThreads>(gmax, sh);
  if (gmax < st.tol) {
    if (threadIdx.x == 0) conv_flags[s] = 1;
    return;
  }
  double mx = 0.0;
  for (int64_t q = threadIdx.x; q < np; q += blockDim.x) mx = fmax(mx, fabs(-1.0 * st.lr * g[q]));
  mx = block_max<kOptThreads>(mx, sh);
  for (int64_t q = threadIdx.x; q < np; q += blockDim.x) {
    const double d = -1.0 * st.lr * g[q];
    x[q] = mx <= st.maxdisp ? x[q] + d : x[q] + (st.maxdisp / mx) * d;
  }
}

// ---------------------------------------------------------------- L-BFGS + line minimiser
// state layout per species (doubles): vectors xx, xold, gg, dir, x0, d0, dxt, qq (n each),
// ss, yy (mem*n each), rho, alph (mem each), scalars (32)
// ss, yy (mem*n each), rho, alph (mem each), scalars (32); then the compact form of the
// L-BFGS direction: rinv[a][b] = (R^-1)_ab and rinvt[b][a] = (R^-1)_ab for the upper-triangular
// R_ab = s_a.y_b (a older than b), R_aa = max(|s_a.y_a|, eps); syt[b][a] = s_a.y_b (the column
// of the newest pair), yg[a][b] = y_a.y_b (mem*mem each); ps[a] = s_a.g, py[a] = y_a.g, the
// direction's coefficients cs, cy and the intermediate v3 (mem each), and kLbSplit partial sums
// of the direction (n each).  alph holds v1 = R^-1 S^T g.
enum {
  SC_ITER = 0, SC_STATE, SC_IITER, SC_CONV, SC_XX0, SC_XX1, SC_DX0, SC_DX1, SC_XCUR, SC_MAXX,
  SC_FIRST, SC_CONVERGED, SC_PHASE, SC_NE, SC_USED, SC_GAMMA, SC_NS = 32
};
constexpr int kLbSplit = 8;         // slot groups of the direction's combination
constexpr int kLbMaxMem = 8192;     // history slots (the combination stages a slot group)

struct LbView {
  double *xx, *xold, *gg, *dir, *x0, *d0, *dxt, *qq, *ss, *yy, *rho, *alph, *sc;
  double *rinv, *syt, *yg, *rinvt, *ps, *py, *cs, *cy, *v3, *part;
};

__host__ __device__ inline size_t lb_stride(int64_t n, int mem) {
  return (size_t)8 * n + (size_t)2 * mem * n + (size_t)2 * mem + SC_NS +
         (size_t)4 * mem * mem + (size_t)5 * mem + (size_t)kLbSplit * n;
}

__device__ LbView lb_view(double *base, int64_t n, int mem) {
  LbView v;
  double *p = base;
  v.xx = p; p += n;
  v.xold = p; p += n;
  v.gg = p; p += n;
  v.dir = p; p += n;
  v.x0 = p; p += n;
  v.d0 = p; p += n;
  v.dxt = p; p += n;
  v.qq = p; p += n;
  v.ss = p; p += (size_t)mem * n;
  v.yy = p; p += (size_t)mem * n;
  v.rho = p; p += mem;
  v.alph = p; p += mem;
  v.sc = p; p += SC_NS;
  v.rinv = p; p += (size_t)mem * mem;
  v.syt = p; p += (size_t)mem * mem;
  v.yg = p; p += (size_t)mem * mem;
  v.rinvt = p; p += (size_t)mem * mem;
  v.ps = p; p += mem;
  v.py = p; p += mem;
  v.cs = p; p += mem;
  v.cy = p; p += mem;
  v.v3 = p; p += mem;
  v.part = p;
  return v;
}

struct LbParams {
  int64_t n;
  int mem;
  double tol, maxdisp;
  int linesearch;
  double qn_maxdisp;
  double lm_tol;  // line-minimiser tolerance (L-BFGS: tol; CG: 1e4, conjgrad.F90:120)
};

__device__ double bdot(const double *a, const double *b, int64_t n, double *sh) {
  double acc = 0.0;
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) acc += a[q] * b[q];
  return block_sum<kOptThreads>(acc, sh);
}

__device__ double bmaxabs(const double *a, int64_t n, double *sh) {
  double acc = 0.0;
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) acc = fmax(acc, fabs(a[q]));
  return block_max<kOptThreads>(acc, sh);
}

__device__ void bcopy(double *dst, const double *src, int64_t n) {
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
  __syncthreads();
}

// TLbfgs_calcDirection (lbfgs.F90:387-488) in the compact form of the L-BFGS inverse Hessian
// (Byrd, Nocedal and Schnabel, Math. Program. 63 (1994), eq. 3.7): with the stored pairs as the
// columns of S and Y (oldest first), R the upper triangle of S^T Y with the diagonal
// 1 / rho_a = max(|s_a.y_a|, eps) of the reference's rho, D = diag(1 / rho) and gamma the
// initial diagonal, the two-loop recursion's direction is
//   dir = -H g = -gamma g - S p + gamma Y v1,
//   v1 = R^-1 S^T g,   p = R^-T ((D + gamma Y^T Y) v1 - gamma Y^T g).
// Same arithmetic in exact terms (the recursion is this product written as loops); rounding
// differs by the order of the sums.  The serial chains of the recursion (2 x memory dependent
// dot products over all parameters) become matrix-vector products over memory x memory
// matrices that spread over the whole GPU.  R^-1 is kept from one direction to the next: when
// the oldest pair leaves the ring buffer, the inverse of the remaining trailing block of R is
// the trailing block of R^-1; a new pair adds the column -R^-1 c rho_new (c_a = s_a.y_new) and
// the diagonal rho_new.  Slots never written are skipped (the reference's rho = 0 for them
// changes nothing).
//
// Stage 1 (lbfgs_pre_kernel, one CTA per species): convergence, the line minimiser, and the
// history update s_ne = x - x_old, y_ne = g - g_old.  SC_PHASE tells the later stages what
// to do: 0 nothing (converged or inside a line search), 1 a compact-form direction, 2 the
// first direction -g.
__device__ void lb_history(LbView &v, const LbParams &P, const double *xx, const double *g) {
  const int64_t n = P.n;
  const int mem = P.mem;
  const int iter = (int)v.sc[SC_ITER];
  if (iter == 0) {
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
      v.gg[q] = g[q];
      v.dir[q] = -g[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      v.sc[SC_ITER] = 1;
      v.sc[SC_PHASE] = 2;
    }
    __syncthreads();
    return;
  }
  const int ne = (iter - 1) % mem;
  double *s = v.ss + (size_t)ne * n, *y = v.yy + (size_t)ne * n;
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
    s[q] = xx[q] - v.xold[q];
    y[q] = g[q] - v.gg[q];
    v.xold[q] = xx[q];
    v.gg[q] = g[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    v.sc[SC_NE] = ne;
    v.sc[SC_USED] = iter < mem ? iter : mem;
    v.sc[SC_PHASE] = 1;
  }
  __syncthreads();
}

// Stage 2 (lbfgs_gram_kernel): the inner products that involve the newest pair or the new
// gradient, for every written slot a: s_a.y_ne, y_a.y_ne, s_a.g, y_a.g.  kGramSlots slots per
// CTA share the loads of y_ne and g.
constexpr int kGramSlots = 4;
constexpr int kGramThreads = 256;

// Stages 3-6 (lbfgs_rinv_kernel, lbfgs_v1_kernel, lbfgs_v2_kernel, lbfgs_p_kernel): the new
// column of R^-1 and gamma, v1, v3 = (D + gamma Y^T Y) v1 - gamma Y^T g, p = R^-T v3 and the
// coefficients; a warp per row of the memory x memory matrices, rows in age order
// (k = 0 oldest .. used - 1 newest, slot ne - (used - 1 - k)).
constexpr int kGemvWarps = 8;

// Stage 7 (lbfgs_combine_kernel): kLbSplit partial sums of sum_a cs_a s_a + cy_a y_a over
// slot groups; stage 8 (lbfgs_post_kernel) adds them in a fixed order to -gamma g and runs the
// line minimiser's reset / first step, or the plain step.
constexpr int kCombThreads = 128;

// TLineMin reset (linemin.F90:141-176)
__device__ void lm_reset(LbView &v, const LbParams &P, const double *x0, const double *d0,
                         double first, double *sh) {
  const int64_t n = P.n;
  const double tmp = sqrt(bdot(d0, d0, n, sh));
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
    v.x0[q] = x0[q];
    v.d0[q] = d0[q] / tmp;
  }
  __syncthreads();
  const double dmax = bmaxabs(v.d0, n, sh);
  if (threadIdx.x == 0) {
    v.sc[SC_STATE] = 1;
    v.sc[SC_IITER] = 0;
    v.sc[SC_XX0] = v.sc[SC_XX1] = 0.0;
    v.sc[SC_DX0] = v.sc[SC_DX1] = 0.0;
    v.sc[SC_XCUR] = 0.0;
    v.sc[SC_FIRST] = first;
    v.sc[SC_MAXX] = P.maxdisp / dmax;
    v.sc[SC_CONV] = 0;
  }
  __syncthreads();
}

// next / next_local (linemin.F90:179-391); uu receives the next point, returns convergence
__device__ bool lm_next(LbView &v, const LbParams &P, double fu, const double *du, double *uu,
                        double *sh) {
  const int64_t n = P.n;
  __shared__ int s_ret, s_flip;
  if (v.sc[SC_CONV] != 0.0) {
    bcopy(uu, v.x0, n);
    return true;
  }
  const double dcur0 = bdot(du, v.d0, n, sh);
  if (threadIdx.x == 0) {
    double *sc = v.sc;
    sc[SC_IITER] += 1;
    double dcur = dcur0;
    s_ret = 0;
    s_flip = 0;
    const int iiter = (int)sc[SC_IITER];
    if ((fabs(dcur) < P.lm_tol && (int)sc[SC_STATE] == 3) || iiter > 10) {
      s_ret = 1;
    } else {
      int state = (int)sc[SC_STATE];
      int next_state = state;
      double xnew = 0.0, tmp, qq, aa, bb, cc;
      double xcur = sc[SC_XCUR];
      if (state == 1) {
        if (dcur > 0.0) {
          s_flip = 1;
          dcur = -dcur;
        }
        sc[SC_XX0] = xcur;
        sc[SC_DX0] = dcur;
        xnew = sc[SC_FIRST];
        next_state = 2;
      }
      if (state == 2) {
        if (dcur < 0.0) {
          xnew = xcur + kGoldenMeanP1 * (xcur - sc[SC_XX0]);
          sc[SC_XX0] = xcur;
          sc[SC_DX0] = dcur;
          next_state = 2;
        } else {
          state = 3;
          sc[SC_STATE] = 3;
        }
      }
      if (state == 3) {
        bool done = false;
        next_state = 3;
        double xx0 = sc[SC_XX0], xx1 = sc[SC_XX1], dx0 = sc[SC_DX0], dx1 = sc[SC_DX1];
        if (iiter > 2 && fabs(xx0 - xx1) > kEps) {
          qq = (xcur - xx0) / (xx0 - xx1);
          tmp = dcur - dx0;
          cc = qq * qq * (dx1 - dx0);
          aa = qq * tmp + cc;
          bb = 2.0 * qq * tmp + cc + tmp;
          cc = (qq + 1.0) * dcur;
          tmp = bb * bb - 4 * aa * cc;
          if (tmp >= 0.0) {
            tmp = sqrt(tmp);
            aa = bb > 0.0 ? bb + tmp : bb - tmp;
            if (fabs(aa) > kEps) {
              xnew = xcur - (xcur - xx0) * 2.0 * cc / aa;
              if (((xx0 < xnew) == (xnew < xx1)) && ((dcur < 0.0) == (xnew > xcur))) {
                if (xnew > xcur) {
                  xx0 = xcur;
                  dx0 = dcur;
                } else {
                  xx1 = xcur;
                  dx1 = dcur;
                }
                done = true;
              }
            }
          }
        }
        if (!done) {
          if (dcur < 0.0) {
            xx0 = xcur;
            dx0 = dcur;
          } else {
            xx1 = xcur;
            dx1 = dcur;
          }
          tmp = dx0 - dx1;
          if (fabs(tmp) > kEps) {
            xnew = (xx1 * dx0 - xx0 * dx1) / tmp;
            if ((xx0 < xnew) == (xnew < xx1)) done = true;
          }
        }
        if (!done) xnew = 0.5 * (xx0 + xx1);
        sc[SC_XX0] = xx0;
        sc[SC_XX1] = xx1;
        sc[SC_DX0] = dx0;
        sc[SC_DX1] = dx1;
      }
      tmp = xnew - xcur;
      if (fabs(tmp) <= sc[SC_MAXX]) xcur = xnew;
      else xcur = xcur + copysign(sc[SC_MAXX], tmp);
      sc[SC_XCUR] = xcur;
      sc[SC_STATE] = next_state;
    }
  }
  __syncthreads();
  if (s_ret) {
    const double xcur = v.sc[SC_XCUR];
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
      v.x0[q] = v.x0[q] + xcur * v.d0[q];
      v.d0[q] = du[q];
      uu[q] = v.x0[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      v.sc[SC_XX0] = fu;
      v.sc[SC_XX1] = xcur;
      v.sc[SC_CONV] = 1;
    }
    __syncthreads();
    return true;
  }
  if (s_flip)
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) v.d0[q] = -v.d0[q];
  __syncthreads();
  const double xcur = v.sc[SC_XCUR];
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) uu[q] = v.x0[q] + xcur * v.d0[q];
  __syncthreads();
  return false;
}

// TLbfgs_next (lbfgs.F90:283-359) in five launches (stages above); params holds xNew once
// stage 5 ran.
__global__ void lbfgs_pre_kernel(double *state, size_t stride, double *params, const double *grad,
                                 LbParams P, int *conv_flags) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  LbView v = lb_view(state + (size_t)s * stride, P.n, P.mem);
  const double *dx = grad + (size_t)s * P.n;
  double *xnew = params + (size_t)s * P.n;
  const int64_t n = P.n;
  const double fx = 0.0;  // the reference passes a loss value that the line minimiser only stores
  if (threadIdx.x == 0) v.sc[SC_PHASE] = 0;
  const double gmax = bmaxabs(dx, n, sh);
  if (gmax < P.tol) {
    if (threadIdx.x == 0) conv_flags[s] = 1;
    bcopy(xnew, v.xx, n);
    return;
  }
  if (threadIdx.x == 0) conv_flags[s] = 0;
  bcopy(v.dxt, dx, n);
  if (P.linesearch && (int)v.sc[SC_ITER] > 0) {
    const bool lconv = lm_next(v, P, fx, dx, v.xx, sh);
    if (lconv) {
      bcopy(v.dxt, v.d0, n);
    } else {
      bcopy(xnew, v.xx, n);
      return;
    }
  }
  lb_history(v, P, v.xx, v.dxt);
}

__global__ void __launch_bounds__(kGramThreads) lbfgs_gram_kernel(double *state, size_t stride,
                                                                  LbParams P) {
  __shared__ double red[kGramThreads / 32][4 * kGramSlots];
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int64_t n = P.n;
  const int mem = P.mem;
  const int ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int k0 = blockIdx.x * kGramSlots;
  if (k0 >= used) return;
  const int nk = min(kGramSlots, used - k0);
  int slot[kGramSlots];
#pragma unroll
  for (int i = 0; i < kGramSlots; i++) slot[i] = ((ne - (k0 + min(i, nk - 1))) % mem + mem) % mem;
  const double *yn = v.yy + (size_t)ne * n, *g = v.dxt;
  double acc[4 * kGramSlots];
#pragma unroll
  for (int i = 0; i < 4 * kGramSlots; i++) acc[i] = 0.0;
  for (int64_t q = threadIdx.x; q < n; q += kGramThreads) {
    const double a = yn[q], b = g[q];
#pragma unroll
    for (int i = 0; i < kGramSlots; i++) {
      const double sv = v.ss[(size_t)slot[i] * n + q], yv = v.yy[(size_t)slot[i] * n + q];
      acc[4 * i + 0] = fma(sv, a, acc[4 * i + 0]);
      acc[4 * i + 1] = fma(yv, a, acc[4 * i + 1]);
      acc[4 * i + 2] = fma(sv, b, acc[4 * i + 2]);
      acc[4 * i + 3] = fma(yv, b, acc[4 * i + 3]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 4 * kGramSlots; i++) {
    double t = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[warp][i] = t;
  }
  __syncthreads();
  if (threadIdx.x < 4 * kGramSlots) {
    const int i = threadIdx.x >> 2, c = threadIdx.x & 3;
    if (i < nk) {
      double t = 0.0;
      for (int w = 0; w < kGramThreads / 32; w++) t += red[w][threadIdx.x];
      const int sa = ((ne - (k0 + i)) % mem + mem) % mem;
      if (c == 0) {
        v.syt[(size_t)ne * mem + sa] = t;
        if (sa == ne) v.rho[ne] = 1.0 / fmax(fabs(t), kEps);
      } else if (c == 1) {
        v.yg[(size_t)sa * mem + ne] = t;
        v.yg[(size_t)ne * mem + sa] = t;
      } else if (c == 2) {
        v.ps[sa] = t;
      } else {
        v.py[sa] = t;
      }
    }
  }
}

// slot of age k (0 = oldest) among `used` written slots ending at ne
__device__ __forceinline__ int age_slot(int k, int ne, int used, int mem) {
  const int s = ne - (used - 1 - k);
  return s < 0 ? s + mem : s;
}

// sum over ages kb in [k0, k1) of row[slot(kb)] * x(kb), lanes over kb, on every lane
template <typename F>
__device__ __forceinline__ double warp_row_dot(const double *row, int k0, int k1, int ne, int used,
                                               int mem, F x) {
  double acc = 0.0;
  for (int kb = k0 + (threadIdx.x & 31); kb < k1; kb += 32)
    acc = fma(row[age_slot(kb, ne, used, mem)], x(kb), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// new column of R^-1 (rows older than the newest pair) and its diagonal; gamma
__global__ void __launch_bounds__(32 * kGemvWarps) lbfgs_rinv_kernel(double *state, size_t stride,
                                                                     LbParams P) {
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int mem = P.mem, ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int ka = blockIdx.x * kGemvWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (ka >= used) return;
  const double rho_ne = v.rho[ne];
  if (ka == used - 1) {
    if (lane == 0) {
      v.rinv[(size_t)ne * mem + ne] = rho_ne;
      v.rinvt[(size_t)ne * mem + ne] = rho_ne;
      const int iter = (int)v.sc[SC_ITER];
      v.sc[SC_GAMMA] = iter == 1 ? 1.0
                                 : v.syt[(size_t)ne * mem + ne] /
                                       fmax(v.yg[(size_t)ne * mem + ne], kEps);
    }
    return;
  }
  const int sa = age_slot(ka, ne, used, mem);
  const double *c = v.syt + (size_t)ne * mem;  // c[b] = s_b . y_ne
  const double t = warp_row_dot(v.rinv + (size_t)sa * mem, ka, used - 1, ne, used, mem,
                                [&](int kb) { return c[age_slot(kb, ne, used, mem)]; });
  if (lane == 0) {
    const double x = -t * rho_ne;
    v.rinv[(size_t)sa * mem + ne] = x;
    v.rinvt[(size_t)ne * mem + sa] = x;
  }
}

// v1 = R^-1 (S^T g), kept in alph (by slot)
__global__ void __launch_bounds__(32 * kGemvWarps) lbfgs_v1_kernel(double *state, size_t stride,
                                                                   LbParams P) {
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int mem = P.mem, ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int ka = blockIdx.x * kGemvWarps + (threadIdx.x >> 5);
  if (ka >= used) return;
  const int sa = age_slot(ka, ne, used, mem);
  const double t = warp_row_dot(v.rinv + (size_t)sa * mem, ka, used, ne, used, mem,
                                [&](int kb) { return v.ps[age_slot(kb, ne, used, mem)]; });
  if ((threadIdx.x & 31) == 0) v.alph[sa] = t;
}

// v3 = D v1 + gamma (Y^T Y) v1 - gamma Y^T g
__global__ void __launch_bounds__(32 * kGemvWarps) lbfgs_v2_kernel(double *state, size_t stride,
                                                                   LbParams P) {
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int mem = P.mem, ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int ka = blockIdx.x * kGemvWarps + (threadIdx.x >> 5);
  if (ka >= used) return;
  const int sa = age_slot(ka, ne, used, mem);
  const double gamma = v.sc[SC_GAMMA];
  const double t = warp_row_dot(v.yg + (size_t)sa * mem, 0, used, ne, used, mem,
                                [&](int kb) { return v.alph[age_slot(kb, ne, used, mem)]; });
  if ((threadIdx.x & 31) == 0) {
    const double d = fmax(fabs(v.syt[(size_t)sa * mem + sa]), kEps);
    v.v3[sa] = d * v.alph[sa] + gamma * t - gamma * v.py[sa];
  }
}

// p = R^-T v3; the direction's coefficients cs = -p, cy = gamma v1
__global__ void __launch_bounds__(32 * kGemvWarps) lbfgs_p_kernel(double *state, size_t stride,
                                                                  LbParams P) {
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int mem = P.mem, ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int kb = blockIdx.x * kGemvWarps + (threadIdx.x >> 5);
  if (kb >= used) return;
  const int sb = age_slot(kb, ne, used, mem);
  const double t = warp_row_dot(v.rinvt + (size_t)sb * mem, 0, kb + 1, ne, used, mem,
                                [&](int ka) { return v.v3[age_slot(ka, ne, used, mem)]; });
  if ((threadIdx.x & 31) == 0) {
    v.cs[sb] = -t;
    v.cy[sb] = v.sc[SC_GAMMA] * v.alph[sb];
  }
}

__global__ void __launch_bounds__(kCombThreads) lbfgs_combine_kernel(double *state, size_t stride,
                                                                     LbParams P) {
  __shared__ double cf[2 * (kLbMaxMem / kLbSplit + 1)];
  __shared__ int sl[kLbMaxMem / kLbSplit + 1];
  LbView v = lb_view(state + (size_t)blockIdx.y * stride, P.n, P.mem);
  if ((int)v.sc[SC_PHASE] != 1) return;
  const int64_t n = P.n;
  const int mem = P.mem;
  const int ne = (int)v.sc[SC_NE], used = (int)v.sc[SC_USED];
  const int z = blockIdx.z;
  const int k0 = (int)((int64_t)used * z / kLbSplit), k1 = (int)((int64_t)used * (z + 1) / kLbSplit);
  for (int k = k0 + threadIdx.x; k < k1; k += kCombThreads) {
    const int sk = ((ne - k) % mem + mem) % mem;
    sl[k - k0] = sk;
    cf[2 * (k - k0)] = v.cs[sk];
    cf[2 * (k - k0) + 1] = v.cy[sk];
  }
  __syncthreads();
  const int64_t q = (int64_t)blockIdx.x * kCombThreads + threadIdx.x;
  if (q >= n) return;
  double acc = 0.0;
#pragma unroll 4
  for (int k = 0; k < k1 - k0; k++) {
    const size_t o = (size_t)sl[k] * n + q;
    acc = fma(cf[2 * k], v.ss[o], acc);
    acc = fma(cf[2 * k + 1], v.yy[o], acc);
  }
  v.part[(size_t)z * n + q] = acc;
}

__global__ void lbfgs_post_kernel(double *state, size_t stride, double *params, const double *grad,
                                  LbParams P) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  LbView v = lb_view(state + (size_t)s * stride, P.n, P.mem);
  const int phase = (int)v.sc[SC_PHASE];
  if (phase == 0) return;
  const double *dx = grad + (size_t)s * P.n;
  double *xnew = params + (size_t)s * P.n;
  const int64_t n = P.n;
  const double fx = 0.0;
  if (phase == 1) {
    const double gamma = v.sc[SC_GAMMA];
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
      double d = -gamma * v.dxt[q];
#pragma unroll
      for (int z = 0; z < kLbSplit; z++) d += v.part[(size_t)z * n + q];
      v.dir[q] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) v.sc[SC_ITER] = v.sc[SC_ITER] + 1;
    __syncthreads();
  }
  if (P.linesearch) {
    lm_reset(v, P, v.xx, v.dir, 1.0, sh);
    lm_next(v, P, fx, dx, v.xx, sh);
  } else {
    if (P.qn_maxdisp > 0.0) {
      const double dmax = bmaxabs(v.dir, n, sh);
      if (dmax > P.qn_maxdisp)
        for (int64_t q = threadIdx.x; q < n; q += blockDim.x)
          v.dir[q] = v.dir[q] * P.qn_maxdisp / dmax;
      __syncthreads();
    }
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) v.xx[q] = v.xx[q] + v.dir[q];
    __syncthreads();
  }
  bcopy(xnew, v.xx, n);
  if (threadIdx.x == 0) v.sc[SC_PHASE] = 0;
}

// ---------------------------------------------------------------- conjugate gradients
// conjGrad_next / next_local (conjgrad.F90:142-260).  State per species in the L-BFGS layout
// with mem = 1: xx = uu, gg = gg, dir = hh, qq = scratch; SC_ITER = 0 before the first call
// (st_1), 1 after; SC_CONVERGED sticky.
__global__ void cg_kernel(double *state, size_t stride, double *params, const double *grad,
                          LbParams P, int *conv_flags) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  LbView v = lb_view(state + (size_t)s * stride, P.n, 1);
  const double *du = grad + (size_t)s * P.n;
  double *xnew = params + (size_t)s * P.n;
  const int64_t n = P.n;
  const double fu = 0.0;  // stored by the line minimiser only
  if (v.sc[SC_CONVERGED] == 0.0) {
    if (v.sc[SC_ITER] == 0.0) {
      const double gmax = bmaxabs(du, n, sh);
      if (gmax < P.tol) {
        for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
          v.gg[q] = du[q];
          v.dir[q] = q == 0 ? fu : 0.0;
        }
        __syncthreads();
        if (threadIdx.x == 0) v.sc[SC_CONVERGED] = 1;
      } else {
        for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
          v.gg[q] = -du[q];
          v.dir[q] = v.gg[q];
        }
        __syncthreads();
      }
      const double first = 5.0 * sqrt(bdot(v.gg, v.gg, n, sh));
      if (v.sc[SC_CONVERGED] == 0.0) lm_reset(v, P, v.xx, v.dir, first, sh);
      if (threadIdx.x == 0) v.sc[SC_ITER] = 1;
      __syncthreads();
    }
    bool conv_line = true;
    while (v.sc[SC_CONVERGED] == 0.0 && conv_line) {
      conv_line = lm_next(v, P, fu, du, v.xx, sh);
      if (conv_line) {
        const double *xi = v.d0;  // the line minimum's gradient
        const double xmax = bmaxabs(xi, n, sh);
        if (xmax < P.tol) {
          if (threadIdx.x == 0) v.sc[SC_CONVERGED] = 1;
          __syncthreads();
        } else {
          const double gg_abs = bdot(v.gg, v.gg, n, sh);
          double acc = 0.0;
          for (int64_t q = threadIdx.x; q < n; q += blockDim.x) acc += (xi[q] + v.gg[q]) * xi[q];
          const double dg_abs = block_sum<kOptThreads>(acc, sh);
          if (gg_abs < kEps) {
            if (threadIdx.x == 0) v.sc[SC_CONVERGED] = 1;
            __syncthreads();
          } else {
            for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
              v.gg[q] = -xi[q];
              v.dir[q] = v.gg[q] + (dg_abs / gg_abs) * v.dir[q];
            }
            __syncthreads();
            bcopy(v.xx, v.x0, n);
            lm_reset(v, P, v.xx, v.dir, v.sc[SC_XX1], sh);
          }
        }
      }
    }
    if (v.sc[SC_CONVERGED] != 0.0) bcopy(v.xx, v.x0, n);
  }
  if (threadIdx.x == 0) conv_flags[s] = v.sc[SC_CONVERGED] != 0.0 ? 1 : 0;
  bcopy(xnew, v.xx, n);
}

// ---------------------------------------------------------------- FIRE
// TFire next / fireModifyVelocity (fire.F90:128-190).  State per species: xx = x, dir =
// velocity; scalars SC_ITER = iter, SC_STATE = resetStep, SC_XX0 = a, SC_XX1 = dt.
struct FireParams {
  int64_t n;
  double tol, dt_max;
};

__global__ void fire_kernel(double *state, size_t stride, double *params, const double *grad,
                            FireParams P, int *conv_flags) {
  __shared__ double sh[kOptThreads];
  const int s = blockIdx.x;
  LbView v = lb_view(state + (size_t)s * stride, P.n, 1);
  const double *dx = grad + (size_t)s * P.n;
  double *xnew = params + (size_t)s * P.n;
  const int64_t n = P.n;
  const double gmax = bmaxabs(dx, n, sh);
  const int iter = (int)v.sc[SC_ITER];
  if (gmax < P.tol) {
    if (threadIdx.x == 0) conv_flags[s] = 1;
  } else {
    const double p = -1.0 * bdot(v.dir, dx, n, sh);
    const double mv = sqrt(bdot(v.dir, v.dir, n, sh));
    const double md = sqrt(bdot(dx, dx, n, sh));
    double a = v.sc[SC_XX0], dt = v.sc[SC_XX1];
    const int reset_step = (int)v.sc[SC_STATE];
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x)
      v.dir[q] = (1.0 - a) * v.dir[q] - a * dx[q] * mv / md;
    __syncthreads();
    int new_reset = reset_step;
    if (p < 0.0) {
      for (int64_t q = threadIdx.x; q < n; q += blockDim.x) v.dir[q] = 0.0;
      new_reset = iter;
      dt = dt * 0.5;
      a = 0.1;
    } else if (iter - reset_step > 5) {
      dt = fmin(dt * 1.1, P.dt_max);
      a = a * 0.99;
    }
    __syncthreads();
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
      v.dir[q] = v.dir[q] - dt * dx[q];
      v.xx[q] = v.xx[q] + v.dir[q] * dt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      v.sc[SC_STATE] = new_reset;
      v.sc[SC_XX0] = a;
      v.sc[SC_XX1] = dt;
      conv_flags[s] = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) v.sc[SC_ITER] = iter + 1;
  bcopy(xnew, v.xx, n);
}

// FIRE reset (fire.F90:113-126) on top of the zeroed block: a = a_start = 0.1,
// dt = dt_init = 0.1 dt_max (x = x0 and v = 0 come from lbfgs_reset_kernel)
__global__ void fire_reset_kernel(double *state, size_t stride, int64_t n, double dt_max) {
  if (threadIdx.x != 0) return;
  LbView v = lb_view(state + (size_t)blockIdx.x * stride, n, 1);
  v.sc[SC_XX0] = 0.1;
  v.sc[SC_XX1] = 0.1 * dt_max;
}

// after the whole state block was zeroed
__global__ void lbfgs_reset_kernel(double *state, size_t stride, const double *params,
                                   int64_t n, int mem) {
  const int s = blockIdx.x;
  double *base = state + (size_t)s * stride;
  LbView v = lb_view(base, n, mem);
  for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
    v.xx[q] = params[(size_t)s * n + q];
    v.xold[q] = params[(size_t)s * n + q];
  }
}

}  // namespace

int run_train_gradients(fnetg_ctx *ctx, int loss, const int32_t *order, bool need_predict) {
  (void)order;  // only the accumulation order changes with the reference's shuffle
  if (ctx->batch_train) return run_batch_gradients(ctx, loss);      // tensor-core passes
  if (ctx->fl_weight > 0.0) return run_force_gradients(ctx, loss);  // energy + force loss
  const int64_t N = ctx->N;
  const int S = ctx->S;
  const int nout = ctx->dims.back();
  int rc;
  if (need_predict) {
    rc = run_predict(ctx);
    if (rc) return rc;
  }
  FNETG_CUDA(ctx->d_lossgrad.ensure(sizeof(double) * std::max<int64_t>(N, 1) * nout));
  FNETG_CUDA(ctx->d_losspart.ensure(sizeof(double) * 2 * std::max(S, 1)));
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  LossArgs a{};
  a.S = S;
  a.off = ctx->d_off.as<int64_t>();
  a.out = ctx->d_out.as<double>();
  a.nout = nout;
  a.ngt = ctx->ngt;
  a.nat = ctx->nat;
  a.gt = ctx->d_gt.as<double>();
  a.at = ctx->d_at.as<double>();
  a.aw = ctx->d_aw.as<double>();
  a.saw = ctx->d_struct_aw.as<double>();
  a.w = ctx->d_w.as<int32_t>();
  a.loss = loss;
  a.delta = ctx->d_lossgrad.as<double>();
  a.part = ctx->d_losspart.as<double>();
  if (S > 0) {
    LaunchScope ls(ctx, "loss");
    loss_cta_kernel<<<S, kLossThreads, 0, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  {
    LaunchScope ls(ctx, "loss");
    loss_reduce_kernel<<<1, 1024, 0, ctx->stream>>>(ctx->d_losspart.as<double>(), S,
                                                     ctx->d_scalars.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  return run_mlp_backward(ctx);
}

// The loss kernel over structures [s0, s0 + count) only (a mini-batch): their atoms' scaled
// output gradients and their per-structure loss parts.
int launch_loss_range(fnetg_ctx *ctx, int s0, int count, int loss) {
  // the buffers every loss evaluation writes (no-ops once sized, as during graph capture)
  FNETG_CUDA(ctx->d_lossgrad.ensure(sizeof(double) * std::max<int64_t>(ctx->N, 1) *
                                    ctx->dims.back()));
  FNETG_CUDA(ctx->d_losspart.ensure(sizeof(double) * 2 * std::max(ctx->S, 1)));
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  if (count <= 0) return FNETG_OK;
  LossArgs a{};
  a.S = count;
  a.off = ctx->d_off.as<int64_t>() + s0;
  a.out = ctx->d_out.as<double>();
  a.nout = ctx->dims.back();
  a.ngt = ctx->ngt;
  a.nat = ctx->nat;
  a.gt = ctx->d_gt.as<double>() + (int64_t)s0 * ctx->ngt;
  a.at = ctx->d_at.as<double>();
  a.aw = ctx->d_aw.as<double>();
  a.saw = ctx->d_struct_aw.as<double>() + s0;
  a.w = ctx->d_w.as<int32_t>() + s0;
  a.loss = loss;
  a.delta = ctx->d_lossgrad.as<double>();
  a.part = ctx->d_losspart.as<double>() + 2 * (int64_t)s0;
  LaunchScope ls(ctx, "loss");
  loss_cta_kernel<<<count, kLossThreads, 0, ctx->stream>>>(a);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

// dataset loss from the per-structure parts of every structure
int launch_loss_reduce(fnetg_ctx *ctx) {
  FNETG_CUDA(ctx->d_losspart.ensure(sizeof(double) * 2 * std::max(ctx->S, 1)));
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  LaunchScope ls(ctx, "loss");
  loss_reduce_kernel<<<1, 1024, 0, ctx->stream>>>(ctx->d_losspart.as<double>(), ctx->S,
                                                   ctx->d_scalars.as<double>());
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

int run_update_prepare(fnetg_ctx *ctx, double strength, double alpha) {
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  FNETG_CUDA(ctx->d_conv.ensure(sizeof(int) * 64 + sizeof(double) * 64));
  double *sq = reinterpret_cast<double *>(ctx->d_conv.as<int>() + 64);
  const int64_t nw = ctx->boff[0];
  {
    LaunchScope ls(ctx, "optimizer");
    update_prepare_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        ctx->d_params64.as<double>(), ctx->d_grad64.as<double>(), ctx->nparams, nw, strength,
        alpha, ctx->sum_weights, sq);
  }
  {
    LaunchScope ls(ctx, "optimizer");
    norm_finish_kernel<<<1, 1, 0, ctx->stream>>>(sq, ctx->nsp, ctx->d_scalars.as<double>());
  }
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

int run_optimizer_step(fnetg_ctx *ctx) {
  int *conv = ctx->d_conv.as<int>();
  if (ctx->opt_kind == FNETG_OPT_SD) {
    SdState st{ctx->opt_threshold, ctx->opt_max_disp, ctx->opt_lr};
    LaunchScope ls(ctx, "optimizer");
    sd_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(ctx->d_params64.as<double>(),
                                                          ctx->d_grad64.as<double>(),
                                                          ctx->nparams, st, conv);
  } else if (ctx->opt_kind == FNETG_OPT_CG) {
    LbParams P{ctx->nparams, 1, ctx->opt_threshold, ctx->opt_max_disp, 1, -1.0, 10000.0};
    LaunchScope ls(ctx, "optimizer");
    cg_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        ctx->d_opt.as<double>(), ctx->opt_stride, ctx->d_params64.as<double>(),
        ctx->d_grad64.as<double>(), P, conv);
  } else if (ctx->opt_kind == FNETG_OPT_FIRE) {
    FireParams P{ctx->nparams, ctx->opt_threshold, ctx->opt_max_disp};
    LaunchScope ls(ctx, "optimizer");
    fire_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        ctx->d_opt.as<double>(), ctx->opt_stride, ctx->d_params64.as<double>(),
        ctx->d_grad64.as<double>(), P, conv);
  } else {
    LbParams P{ctx->nparams, ctx->opt_mem, ctx->opt_threshold, ctx->opt_max_disp,
               ctx->opt_linemin, ctx->opt_qn ? ctx->opt_max_disp : -1.0, ctx->opt_threshold};
    double *st = ctx->d_opt.as<double>();
    const size_t stride = ctx->opt_stride;
    const int mem = ctx->opt_mem;
    const dim3 gemv(ceil_div(mem, kGemvWarps), ctx->nsp);
    LaunchScope ls(ctx, "optimizer");
    lbfgs_pre_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        st, stride, ctx->d_params64.as<double>(), ctx->d_grad64.as<double>(), P, conv);
    lbfgs_gram_kernel<<<dim3(ceil_div(mem, kGramSlots), ctx->nsp), kGramThreads, 0,
                        ctx->stream>>>(st, stride, P);
    lbfgs_rinv_kernel<<<gemv, 32 * kGemvWarps, 0, ctx->stream>>>(st, stride, P);
    lbfgs_v1_kernel<<<gemv, 32 * kGemvWarps, 0, ctx->stream>>>(st, stride, P);
    lbfgs_v2_kernel<<<gemv, 32 * kGemvWarps, 0, ctx->stream>>>(st, stride, P);
    lbfgs_p_kernel<<<gemv, 32 * kGemvWarps, 0, ctx->stream>>>(st, stride, P);
    lbfgs_combine_kernel<<<dim3((unsigned)ceil_div(ctx->nparams, (int64_t)kCombThreads),
                                ctx->nsp, kLbSplit),
                           kCombThreads, 0, ctx->stream>>>(st, stride, P);
    lbfgs_post_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        st, stride, ctx->d_params64.as<double>(), ctx->d_grad64.as<double>(), P);
  }
  FNETG_CUDA(cudaGetLastError());
  return run_params_to_compute(ctx);
}

}  // namespace fnetg

using namespace fnetg;

extern "C" {

int fnetg_optimizer_init(fnetg_ctx *ctx, int32_t kind, double threshold, double min_disp,
                         double max_disp, double learning_rate, int32_t memory, int32_t linemin,
                         int32_t qn_max_disp) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "optimizer_init: no network");
  FNETG_CHECK(kind == FNETG_OPT_SD || kind == FNETG_OPT_LBFGS || kind == FNETG_OPT_CG ||
                  kind == FNETG_OPT_FIRE,
              FNETG_E_INVALID, "optimiser kind");
  FNETG_CHECK(threshold > 0.0 && max_disp > 0.0, FNETG_E_INVALID,
              "threshold and maximal displacement must be > 0");
  ctx->opt_kind = kind;
  ctx->opt_threshold = threshold;
  ctx->opt_min_disp = min_disp;
  ctx->opt_max_disp = max_disp;
  ctx->opt_lr = learning_rate;
  ctx->opt_mem = std::max(1, memory);
  ctx->opt_linemin = linemin ? 1 : 0;
  ctx->opt_qn = qn_max_disp ? 1 : 0;
  FNETG_CUDA(ctx->d_conv.ensure(sizeof(int) * 64 + sizeof(double) * 64));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_conv.p, 0, sizeof(int) * 64, ctx->stream));
  if (kind != FNETG_OPT_SD) {
    // L-BFGS, CG and FIRE keep their state in the L-BFGS block layout (mem = 1 for CG/FIRE)
    const int mem = kind == FNETG_OPT_LBFGS ? ctx->opt_mem : 1;
    FNETG_CHECK(mem <= kLbMaxMem, FNETG_E_UNSUPPORTED,
                "optimizer_init: L-BFGS memory above 8192 slots");
    ctx->opt_stride = lb_stride(ctx->nparams, mem);
    FNETG_CUDA(ctx->d_opt.ensure(sizeof(double) * ctx->opt_stride * ctx->nsp));
    FNETG_CUDA(cudaMemsetAsync(ctx->d_opt.p, 0, sizeof(double) * ctx->opt_stride * ctx->nsp,
                               ctx->stream));
    LaunchScope ls(ctx, "optimizer");
    lbfgs_reset_kernel<<<ctx->nsp, kOptThreads, 0, ctx->stream>>>(
        ctx->d_opt.as<double>(), ctx->opt_stride, ctx->d_params64.as<double>(), ctx->nparams,
        mem);
    if (kind == FNETG_OPT_FIRE)
      fire_reset_kernel<<<ctx->nsp, 32, 0, ctx->stream>>>(ctx->d_opt.as<double>(),
                                                          ctx->opt_stride, ctx->nparams, max_disp);
    FNETG_CUDA(cudaGetLastError());
  }
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->opt_set = true;
  ctx->opt_started = false;
  return FNETG_OK;
}

int fnetg_train_iteration(fnetg_ctx *ctx, int32_t loss, double regu_strength, double regu_alpha,
                          const int32_t *order, double *loss_out, double *grad_norm_out,
                          int32_t *converged) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->opt_set, FNETG_E_INVALID, "train_iteration: optimizer not initialised");
  FNETG_CHECK(ctx->targets_set, FNETG_E_INVALID, "train_iteration: no targets");
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "train_iteration: no features");
  FNETG_CHECK(ctx->nf == ctx->dims[0], FNETG_E_SHAPE, "network input width");
  FNETG_CHECK(ctx->ngt + ctx->nat == ctx->dims.back(), FNETG_E_SHAPE,
              "network outputs must equal the number of targets");
  FNETG_CHECK(loss >= 0 && loss <= 3, FNETG_E_INVALID, "loss code");
  int rc;
  if (!ctx->opt_started) {
    rc = run_train_gradients(ctx, loss, order, true);
    if (rc) return rc;
    ctx->opt_started = true;
  }
  rc = run_update_prepare(ctx, regu_strength, regu_alpha);
  if (rc) return rc;
  // the gradient norm of this update is reported like the reference's tmpGradients
  double *pin = static_cast<double *>(ctx->h_pinned);
  FNETG_CUDA(cudaMemcpyAsync(pin + 1, ctx->d_scalars.as<double>() + 1, sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
  rc = run_optimizer_step(ctx);
  if (rc) return rc;
  rc = run_train_gradients(ctx, loss, order, true);
  if (rc) return rc;
  FNETG_CUDA(cudaMemcpyAsync(pin, ctx->d_scalars.as<double>(), sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
  int *pconv = reinterpret_cast<int *>(pin + 8);
  FNETG_CUDA(cudaMemcpyAsync(pconv, ctx->d_conv.p, sizeof(int) * ctx->nsp, cudaMemcpyDeviceToHost,
                             ctx->stream));
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (loss_out) *loss_out = pin[0];
  if (grad_norm_out) *grad_norm_out = pin[1];
  if (converged) *converged = pconv[ctx->nsp - 1];  // the last sub-network's flag (bpnn.F90:774)
  return FNETG_OK;
}

}  // extern "C"
