// Directional derivative (forward mode) of every atom's standardised network inputs along a
// per-atom displacement field w:
//     u[a][g] = sum_b dx_a[g]/dR_b . w_b = sum_{pairs (a, j)} dG_a[g]/dd_aj . (w_j - w_a) / s_g,
// with x = (G - mean) / s the z-scored ACSF values (s = 1 where the reference skips the
// standardisation) and d_aj the displacement of neighbour j (image included) from atom a.
// This is the matrix-free form of TAcsf_calculatePrime's dense dG/dR
// (lib_descriptors/acsf.F90:643-717, gFuncGrad 1496-1670) contracted with w, the product that
// the gradient of a force loss needs (the force kernel computes the other contraction,
// sum_a dE/dx_a . dx_a/dR).  Periodic self images of the centre move with it (d fixed), so
// they enter only as triplet partners.
//
// One warp per centre atom: its pairs are staged in shared memory (displacement, w_j - w_a,
// species code, self flag, cutoff classes), radial functions run lanes-over-pairs, angular
// G5 functions lanes-over-first-neighbour with a loop over the second, in the reference's
// formula (acsf.F90:1440-1492: ordered pairs including j = k, both orders for equal lists).
// G4 and functions with atom ids are not supported here.
#include <algorithm>
#include <array>

#include "internal.cuh"

namespace fnetg {

const int64_t *pair_end(fnetg_ctx *ctx);

namespace {

constexpr int kJvpWarps = 4;
constexpr int kJvpCap = 256;  // pairs of one atom staged in shared memory
constexpr int kJvpGroup = 16; // angular functions evaluated together (same lists and eta)
constexpr int kJvpMaxXi = 4;  // integer xi of the shared-power path
constexpr double kPi = 3.14159265358979323846;

template <typename T> struct JvpArgs {
  int64_t natoms;
  const int64_t *poff, *pend;
  const int32_t *pj;
  const uint32_t *pmeta;
  const V4<T> *rij;
  const int8_t *code;
  const T *w;             // [N][3]
  const GDesc *rad, *ang;     // radial functions; angular functions in group order
  int nrad, nang;
  const int4 *grp;            // angular groups: (chan1, chan2, rclass | eclass << 8, first | count << 16)
  int ngrp;
  const double *zsd;      // z-score deviations [ng] (FP64 path) or null
  const float *zinv;      // inverse deviations [ng], 0 = not standardised (FP32 path) or null
  T *u;                   // [N][nf] atom order
  int nf;
  int *err;
};

template <typename T> __device__ __forceinline__ T jsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T> __device__ __forceinline__ void fcut(T r, T rc, T &fc, T &dfc) {
  const T x = (T)kPi * r / rc;
  fc = (T)0.5 * (cos(x) + (T)1);
  dfc = (T)-0.5 * ((T)kPi / rc) * sin(x);
}
template <> __device__ __forceinline__ void fcut<float>(float r, float rc, float &fc, float &dfc) {
  float s, c;
  sincosf(3.14159265f * r / rc, &s, &c);
  fc = 0.5f * (c + 1.f);
  dfc = -0.5f * (3.14159265f / rc) * s;
}

template <typename T> __device__ __forceinline__ T ipow(T b, int n) {
  T r = (T)1;
  for (int k = 0; k < n; k++) r *= b;
  return r;
}

template <typename T>
__device__ __forceinline__ T zscale(const JvpArgs<T> &a, int g) {
  if (a.zsd) {
    const double sd = a.zsd[g];
    return sd < 1e-08 ? (T)1 : (T)(1.0 / sd);
  }
  if (a.zinv) {
    const float inv = a.zinv[g];
    return inv == 0.f ? (T)1 : (T)inv;
  }
  return (T)1;
}

// pair q belongs to list channel c (-1: every neighbour); self images are in every channel
__device__ __forceinline__ bool in_chan(uint32_t info, int c) {
  return c < 0 || (int)(info & 0xff) == c || ((info >> 8) & 1u);
}

template <typename T>
__global__ void __launch_bounds__(32 * kJvpWarps) jvp_kernel(JvpArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per warp: d (x, y, z, r) and (w_j - w_a, r dot) of every pair, then per angular group the
  // pair's E = exp(-eta r^2) fc and its derivative along w, and the two lists (pair indices)
  V4<T> *D = reinterpret_cast<V4<T> *>(smem) + (size_t)wid * 2 * kJvpCap;
  V4<T> *Wd = D + kJvpCap;
  T *Ep = reinterpret_cast<T *>(reinterpret_cast<V4<T> *>(smem) + (size_t)kJvpWarps * 2 * kJvpCap) +
          (size_t)wid * 2 * kJvpCap;
  T *Edp = Ep + kJvpCap;
  uint32_t *info = reinterpret_cast<uint32_t *>(reinterpret_cast<T *>(
                       reinterpret_cast<V4<T> *>(smem) + (size_t)kJvpWarps * 2 * kJvpCap) +
                                                (size_t)kJvpWarps * 2 * kJvpCap) +
                   (size_t)wid * kJvpCap;
  uint16_t *L1 = reinterpret_cast<uint16_t *>(info + (size_t)(kJvpWarps - wid) * kJvpCap) +
                 (size_t)wid * 2 * kJvpCap;
  uint16_t *L2 = L1 + kJvpCap;
  const int64_t i = (int64_t)blockIdx.x * kJvpWarps + wid;
  if (i >= a.natoms) return;
  const int64_t p0 = a.poff[i];
  const int np = (int)(a.pend[i] - p0);
  T *ui = a.u + i * a.nf;
  if (np > kJvpCap) {
    if (lane == 0) atomicExch(a.err, 1);
    return;
  }
  const T wi0 = a.w[3 * i], wi1 = a.w[3 * i + 1], wi2 = a.w[3 * i + 2];
  for (int q = lane; q < np; q += 32) {
    const V4<T> d = a.rij[p0 + q];
    const int32_t j = a.pj[p0 + q];
    const bool self = j == i;
    const T w0 = self ? (T)0 : a.w[3 * j] - wi0, w1 = self ? (T)0 : a.w[3 * j + 1] - wi1,
            w2 = self ? (T)0 : a.w[3 * j + 2] - wi2;
    D[q] = d;
    Wd[q] = V4<T>{w0, w1, w2, (d.x * w0 + d.y * w1 + d.z * w2) / d.w};
    info[q] = (uint32_t)(uint8_t)a.code[j] | ((uint32_t)self << 8) | ((a.pmeta[p0 + q] >> 24) << 16);
  }
  __syncwarp();
  // ---- radial: dG/dr along r dot
  for (int f = 0; f < a.nrad; f++) {
    const GDesc g = a.rad[f];
    const T rc = (T)g.rcut;
    T acc = (T)0;
    for (int q = lane; q < np; q += 32) {
      const uint32_t inf = info[q];
      if (!in_chan(inf, g.chan1) || !((inf >> (16 + g.rclass)) & 1u)) continue;
      const T r = D[q].w;
      T fc, dfc;
      fcut<T>(r, rc, fc, dfc);
      T dg;
      if (g.type == 1) {
        dg = dfc;
      } else if (g.type == 2) {
        const T x = r - (T)g.rs;
        dg = exp(-(T)g.eta * x * x) * (dfc - (T)2 * (T)g.eta * x * fc);
      } else {
        const T kr = (T)g.kappa * r;
        dg = cos(kr) * dfc - (T)g.kappa * sin(kr) * fc;
      }
      acc += dg * Wd[q].w;
    }
    acc = jsum(acc);
    if (lane == 0) ui[g.out] = acc * zscale(a, g.out);
  }
  // ---- angular G5 by groups of functions sharing both lists, cutoff and eta: per ordered
  // pair (j in list 1, k in list 2, j = k included) the cosine and its derivative once
  const unsigned below = (1u << lane) - 1u;
  for (int gi = 0; gi < a.ngrp; gi++) {
    const int4 gr = a.grp[gi];
    const int rcl = gr.z & 0xff, fcount = gr.w >> 16, first = gr.w & 0xffff;
    const GDesc g0 = a.ang[first];
    const T rc = (T)g0.rcut, eta = (T)g0.eta;
    // E and its derivative of every pair in the cutoff class; the two lists in pair order
    int n1 = 0, n2 = 0;
    for (int q0 = 0; q0 < np; q0 += 32) {
      const int q = q0 + lane;
      bool in1 = false, in2 = false;
      if (q < np) {
        const uint32_t inf = info[q];
        const bool inr = (inf >> (16 + rcl)) & 1u;
        in1 = inr && in_chan(inf, gr.x);
        in2 = inr && in_chan(inf, gr.y);
        if (in1 || in2) {
          const T r = D[q].w;
          T fc, dfc;
          fcut<T>(r, rc, fc, dfc);
          const T e = exp(-eta * r * r);
          Ep[q] = e * fc;
          Edp[q] = e * (dfc - (T)2 * eta * r * fc) * Wd[q].w;
        }
      }
      const unsigned m1 = __ballot_sync(0xffffffffu, in1), m2 = __ballot_sync(0xffffffffu, in2);
      if (in1) L1[n1 + __popc(m1 & below)] = (uint16_t)q;
      if (in2) L2[n2 + __popc(m2 & below)] = (uint16_t)q;
      n1 += __popc(m1);
      n2 += __popc(m2);
    }
    __syncwarp();
    T acc[kJvpGroup];
#pragma unroll
    for (int f = 0; f < kJvpGroup; f++) acc[f] = (T)0;
    // the group's functions in registers: lambda = +-1 with integer xi <= kJvpMaxXi take the
    // powers of (1 +- cos) computed once per pair of neighbours
    T lamf[kJvpGroup], xif[kJvpGroup];
    int xin[kJvpGroup];
    bool fast = true;
#pragma unroll
    for (int f = 0; f < kJvpGroup; f++) {
      lamf[f] = (T)0;
      xif[f] = (T)1;
      xin[f] = 1;
      if (f < fcount) {
        const GDesc &g = a.ang[first + f];
        lamf[f] = (T)g.lambda;
        xif[f] = (T)g.xi;
        xin[f] = g.xi_int;
        fast = fast && g.xi_int >= 1 && g.xi_int <= kJvpMaxXi && (g.lambda == 1.0 || g.lambda == -1.0);
      }
    }
    for (int t = lane; t < n1 * n2; t += 32) {
      const int qj = L1[t / n2], qk = L2[t % n2];
      const V4<T> dj = D[qj], wj = Wd[qj], dk = D[qk], wk = Wd[qk];
      const T Ej = Ep[qj], Ek = Ep[qk], Edj = Edp[qj], Edk = Edp[qk];
      T c = (T)1, cd = (T)0;  // cos(theta) and its derivative; exactly (1, 0) for j = k
      if (qj != qk) {
        const T rr = dj.w * dk.w;
        c = (dj.x * dk.x + dj.y * dk.y + dj.z * dk.z) / rr;
        c = c > (T)1 ? (T)1 : (c < (T)-1 ? (T)-1 : c);
        cd = (wj.x * dk.x + wj.y * dk.y + wj.z * dk.z + dj.x * wk.x + dj.y * wk.y +
              dj.z * wk.z) / rr -
             c * (wj.w / dj.w + wk.w / dk.w);
      }
      const T EE = Ej * Ek, dEE = Edj * Ek + Ej * Edk;
      if (fast) {
        T pp[kJvpMaxXi + 1], pm[kJvpMaxXi + 1];  // (1 + c)^m, (1 - c)^m
        pp[0] = pm[0] = (T)1;
#pragma unroll
        for (int m = 1; m <= kJvpMaxXi; m++) {
          pp[m] = pp[m - 1] * ((T)1 + c);
          pm[m] = pm[m - 1] * ((T)1 - c);
        }
#pragma unroll
        for (int f = 0; f < kJvpGroup; f++) {
          if (f >= fcount) break;
          T p = (T)0, b1 = (T)0;
#pragma unroll
          for (int m = 1; m <= kJvpMaxXi; m++)
            if (m == xin[f]) {
              p = lamf[f] > (T)0 ? pp[m] : pm[m];
              b1 = lamf[f] > (T)0 ? pp[m - 1] : pm[m - 1];
            }
          acc[f] += xif[f] * b1 * lamf[f] * cd * EE + p * dEE;
        }
      } else {
#pragma unroll
        for (int f = 0; f < kJvpGroup; f++) {
          if (f >= fcount) break;
          const T lam = lamf[f], base = (T)1 + lam * c;
          T p, pd;  // base^xi and xi base^(xi - 1)
          if (xin[f] > 0) {
            const T b1 = ipow(base, xin[f] - 1);
            p = b1 * base;
            pd = xif[f] * b1;
          } else {
            p = pow(base, xif[f]);
            pd = base > (T)0 ? xif[f] * pow(base, xif[f] - (T)1) : (T)0;
          }
          acc[f] += pd * lam * cd * EE + p * dEE;
        }
      }
    }
#pragma unroll
    for (int f = 0; f < kJvpGroup; f++) {
      if (f >= fcount) break;
      const T v = jsum(acc[f]);
      if (lane == 0) {
        const GDesc &g = a.ang[first + f];
        ui[g.out] = v * (T)g.pref * zscale(a, g.out);
      }
    }
    __syncwarp();
  }
}

template <typename T> int do_jvp(fnetg_ctx *ctx, const T *d_w, T *d_u) {
  for (auto &g : ctx->h_rad) {
    FNETG_CHECK(g.atomid == 0, FNETG_E_UNSUPPORTED, "features_jvp: atom-id weighted functions");
  }
  for (auto &g : ctx->h_ang_all) {
    FNETG_CHECK(g.type == 5 && g.atomid == 0, FNETG_E_UNSUPPORTED,
                "features_jvp: G4 and atom-id weighted angular functions");
  }
  FNETG_CHECK(ctx->max_pairs <= kJvpCap, FNETG_E_UNSUPPORTED,
              "features_jvp: more than 256 neighbours of one atom");
  // angular functions grouped by (lists, cutoff class, eta class), at most kJvpGroup each
  std::vector<GDesc> ord;
  std::vector<int4> grp;
  {
    std::vector<std::array<int, 4>> keys;
    for (auto &g : ctx->h_ang_all) {
      const std::array<int, 4> k{g.chan1, g.chan2, g.rclass, g.eclass};
      if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
    }
    for (auto &k : keys) {
      std::vector<GDesc> mem;
      for (auto &g : ctx->h_ang_all)
        if (g.chan1 == k[0] && g.chan2 == k[1] && g.rclass == k[2] && g.eclass == k[3]) mem.push_back(g);
      for (size_t q0 = 0; q0 < mem.size(); q0 += kJvpGroup) {
        const int cnt = (int)std::min<size_t>(kJvpGroup, mem.size() - q0);
        grp.push_back(make_int4(k[0], k[1], k[2] | (k[3] << 8), (int)ord.size() | (cnt << 16)));
        ord.insert(ord.end(), mem.begin() + q0, mem.begin() + q0 + cnt);
      }
    }
  }
  FNETG_CUDA(ctx->d_jvp_ang.ensure(sizeof(GDesc) * std::max<size_t>(ord.size(), 1)));
  FNETG_CUDA(ctx->d_jvp_grp.ensure(sizeof(int4) * std::max<size_t>(grp.size(), 1)));
  if (!ord.empty()) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_jvp_ang.p, ord.data(), sizeof(GDesc) * ord.size(),
                          cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_jvp_grp.p, grp.data(), sizeof(int4) * grp.size(),
                          cudaMemcpyHostToDevice));
  }
  JvpArgs<T> a{};
  a.natoms = ctx->N;
  a.poff = ctx->d_poff.as<int64_t>();
  a.pend = pair_end(ctx);
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = ctx->d_rij.as<V4<T>>();
  a.code = ctx->d_code.as<int8_t>();
  a.w = d_w;
  a.rad = ctx->d_rad.as<GDesc>();
  a.ang = ctx->d_jvp_ang.as<GDesc>();
  a.nrad = (int)ctx->h_rad.size();
  a.nang = (int)ord.size();
  a.grp = ctx->d_jvp_grp.as<int4>();
  a.ngrp = (int)grp.size();
  if (ctx->zprec_valid) {
    if (sizeof(T) == 8) a.zsd = ctx->d_zprec.as<double>() + ctx->gf.size();
    else a.zinv = ctx->d_zprec_f.as<float>() + ctx->gf.size();
  }
  a.u = d_u;
  a.nf = ctx->nf;
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  a.err = reinterpret_cast<int *>(ctx->d_scalars.as<double>() + 15);
  FNETG_CUDA(cudaMemsetAsync(a.err, 0, sizeof(int), ctx->stream));
  FNETG_CUDA(cudaMemsetAsync(d_u, 0, sizeof(T) * std::max<int64_t>(ctx->N, 1) * ctx->nf, ctx->stream));
  const size_t smem = (size_t)kJvpWarps * kJvpCap *
                      (2 * sizeof(V4<T>) + 2 * sizeof(T) + sizeof(uint32_t) + 2 * sizeof(uint16_t));
  FNETG_CUDA(raise_smem_limit((const void *)jvp_kernel<T>, smem));
  if (ctx->N > 0) {
    LaunchScope ls(ctx, "features_jvp");
    jvp_kernel<T><<<ceil_div(ctx->N, kJvpWarps), 32 * kJvpWarps, smem, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

}  // namespace

// device entry: w [N][3], u [N][nf] in the context's arithmetic
int run_features_jvp(fnetg_ctx *ctx, const void *d_w, void *d_u) {
  return ctx->prec == FNETG_FP64
             ? do_jvp<double>(ctx, static_cast<const double *>(d_w), static_cast<double *>(d_u))
             : do_jvp<float>(ctx, static_cast<const float *>(d_w), static_cast<float *>(d_u));
}

}  // namespace fnetg

using namespace fnetg;

extern "C" int fnetg_features_jvp(fnetg_ctx *ctx, const double *w, double *u) {
  if (!ctx || !w || !u) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->nb_valid && ctx->feats_valid, FNETG_E_INVALID,
              "features_jvp: neighbour list and features are needed");
  const int64_t N = ctx->N;
  const int nf = ctx->nf;
  const size_t es = ctx->prec == FNETG_FP64 ? 8 : 4;
  DBuf dw, du;
  FNETG_CUDA(dw.ensure(es * std::max<int64_t>(3 * N, 1)));
  FNETG_CUDA(du.ensure(es * std::max<int64_t>(N * nf, 1)));
  if (ctx->prec == FNETG_FP64) {
    FNETG_CUDA(copy_sync(ctx, dw.p, w, sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> wf(3 * N);
    for (int64_t q = 0; q < 3 * N; q++) wf[q] = (float)w[q];
    FNETG_CUDA(copy_sync(ctx, dw.p, wf.data(), sizeof(float) * 3 * N, cudaMemcpyHostToDevice));
  }
  int rc = run_features_jvp(ctx, dw.p, du.p);
  if (rc) return rc;
  int err = 0;
  FNETG_CUDA(copy_sync(ctx, &err, ctx->d_scalars.as<double>() + 15, sizeof(int), cudaMemcpyDeviceToHost));
  FNETG_CHECK(err == 0, FNETG_E_UNSUPPORTED, "features_jvp: an atom has more than 256 neighbours");
  if (ctx->prec == FNETG_FP64) {
    FNETG_CUDA(copy_sync(ctx, u, du.p, sizeof(double) * N * nf, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> uf((size_t)N * nf);
    FNETG_CUDA(copy_sync(ctx, uf.data(), du.p, sizeof(float) * uf.size(), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < uf.size(); q++) u[q] = uf[q];
  }
  return FNETG_OK;
}
