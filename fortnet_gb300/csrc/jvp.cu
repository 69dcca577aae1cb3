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
//
// The integer-xi G5 functions that the value kernel evaluates through moment tensors
// (G_f = sum_m pc_f(m) sum_{|alpha| = m} mult(alpha) M_k1(alpha) M_k2(alpha), with
// M_k(alpha) = sum_{j in list k} E(r_j) u_j^alpha) are differentiated in that form: the
// tangent of every moment, dM_k(alpha) = sum_j d/dt [E(r_j) u_j^alpha] along w, costs one pass
// over the pairs (the monomials and their tangents carried as products, child = parent * u_c,
// dchild = dparent * u_c + parent * du_c), and dG_f = sum_m pc_f(m) sum_alpha mult(alpha)
// (dM_k1 M_k2 + M_k1 dM_k2) with the moments themselves from the value kernel's cache.  That
// kernel (jvp_tile_kernel) also takes the radial functions; the triplet kernel (jvp_kernel)
// then runs only for the angular functions outside the moment form.
#define FNETG_FILE_CODE 6  // site codes of the bounds-checked build
#include <algorithm>
#include <array>

#include "internal.cuh"
#include "tile.cuh"

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

// ---- moment-form tangents (and the radial functions) ---------------------------------------
constexpr int kJtWarps = 4;
constexpr int kJtKD = kMaxMomentDegree + 1;

template <typename T> struct JtArgs {
  int64_t natoms;
  const int64_t *poff, *pend;
  const int32_t *pj;
  const uint32_t *pmeta;
  const V4<T> *rij;
  const int8_t *code;
  const T *w;
  const GDesc *rad;
  int nrad;
  T ecls_eta[kMaxEtaClasses];
  int ecls_rclass[kMaxEtaClasses];
  int necls;
  T rcls[kMaxRcutClasses];
  int nrcls;
  int nz, cap;
  const int32_t *combo;  // [ncombo][2] (list code or -1, eta class)
  int ncombo, n_mono;
  const T *mom;          // moment cache [N][ncombo][n_mono], or null: computed here
  const int32_t *mpair;  // [nmpair][2]
  int nmpair;
  const MFunc *mfunc;
  int nmf;
  const T *fpc;          // [nmf][kJtKD]
  const double *zsd;
  const float *zinv;
  T *u;
  int nf;
  int *err;
};

// per-warp shared memory of jvp_tile_kernel
template <typename T> __host__ __device__ inline size_t jt_warp_bytes(const JtArgs<T> &a) {
  size_t b = sizeof(V4<T>) * 2 * (size_t)a.cap;                 // U, Wd
  b += sizeof(T) * (size_t)a.cap * 2 * (a.nrcls + a.necls);      // fc, dfc; E, dE (along w)
  b += sizeof(T) * (size_t)a.ncombo * a.n_mono * 2;               // M, dM
  b += sizeof(T) * (size_t)a.nmpair * kJtKD;                      // degree-sum tangents
  b = (b + 15) / 16 * 16;
  b += sizeof(uint32_t) * a.cap + sizeof(uint16_t) * (size_t)a.cap * a.nz + sizeof(int) * 8;
  return (b + 127) / 128 * 128;
}

template <typename T> __device__ __forceinline__ T jt_zscale(const JtArgs<T> &a, int g) {
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

// Tangent (and, when VAL, value) moments of nk <= 32 / S consecutive combos k0.. of one list:
// lane (group g, slot s) walks pairs s, s + S, ...; a transposing butterfly over the S slots
// leaves C = ceil(NM / S) consecutive sums on each lane.
template <typename T, int D, int S, bool VAL>
__device__ __forceinline__ void jt_moment_pass(const JtArgs<T> &a, const V4<T> *U, const V4<T> *Wd,
                                               const T *Eb, const T *dEb, const uint16_t *lst,
                                               int n, int k0, int nk, T *M, T *dM, int lane) {
  constexpr int NM = n_mono_of(D);
  constexpr int C = (NM + S - 1) / S;
  constexpr int V = C * S;
  const int grp = lane / S, slot = lane % S;
  const bool on = grp < nk;
  const int e = on ? a.combo[2 * (k0 + grp) + 1] : 0;
  const T *E = Eb + e * a.cap, *dE = dEb + e * a.cap;
  T acc[V], vac[VAL ? V : 1];
#pragma unroll
  for (int al = 0; al < V; al++) acc[al] = 0;
#pragma unroll
  for (int al = 0; al < (VAL ? V : 1); al++) vac[al] = 0;
  for (int kk = slot; kk < n; kk += S) {
    const int q = lst ? lst[kk] : kk;
    const V4<T> u = U[q], wd = Wd[q];
    const T rinv = (T)1 / u.w;
    const T dux = (wd.x - u.x * wd.w) * rinv, duy = (wd.y - u.y * wd.w) * rinv,
            duz = (wd.z - u.z * wd.w) * rinv;
    T m[NM], dm[NM];
    m[0] = on ? E[q] : (T)0;
    dm[0] = on ? dE[q] : (T)0;
#pragma unroll
    for (int al = 1; al < NM; al++) {
      const int ax = kMonoLinks.axis[al], par = kMonoLinks.parent[al];
      const T c = ax == 0 ? u.x : (ax == 1 ? u.y : u.z);
      const T dc = ax == 0 ? dux : (ax == 1 ? duy : duz);
      m[al] = m[par] * c;
      dm[al] = dm[par] * c + m[par] * dc;
    }
#pragma unroll
    for (int al = 0; al < NM; al++) {
      acc[al] += dm[al];
      if (VAL) vac[al] += m[al];
    }
  }
#pragma unroll
  for (int sh = S / 2, L = V; sh >= 1; sh >>= 1, L >>= 1) {
    const bool upper = (lane & sh) != 0;
#pragma unroll
    for (int k = 0; k < L / 2; k++) {
      const T send = upper ? acc[k] : acc[k + L / 2];
      const T keep = upper ? acc[k + L / 2] : acc[k];
      acc[k] = keep + __shfl_xor_sync(0xffffffffu, send, sh);
      if (VAL) {
        const T vs = upper ? vac[k] : vac[k + L / 2];
        const T vk = upper ? vac[k + L / 2] : vac[k];
        vac[k] = vk + __shfl_xor_sync(0xffffffffu, vs, sh);
      }
    }
  }
  if (on) {
#pragma unroll
    for (int c = 0; c < C; c++)
      if (slot * C + c < NM) {
        dM[(k0 + grp) * NM + slot * C + c] = acc[c];
        if (VAL) M[(k0 + grp) * NM + slot * C + c] = vac[c];
      }
  }
}

template <typename T, int D>
__global__ void __launch_bounds__(32 * kJtWarps) jvp_tile_kernel(JtArgs<T> a) {
  extern __shared__ __align__(128) unsigned char jsm[];
  constexpr int NM = n_mono_of(D);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kJtWarps + wid;
  if (i >= a.natoms) return;
  unsigned char *p = jsm + jt_warp_bytes(a) * wid;
  V4<T> *U = reinterpret_cast<V4<T> *>(p);
  V4<T> *Wd = U + a.cap;
  T *fc = reinterpret_cast<T *>(Wd + a.cap);
  T *dfc = fc + (size_t)a.nrcls * a.cap;
  T *E = dfc + (size_t)a.nrcls * a.cap;
  T *dE = E + (size_t)a.necls * a.cap;
  T *M = dE + (size_t)a.necls * a.cap;
  T *dM = M + (size_t)a.ncombo * a.n_mono;
  T *Sd = dM + (size_t)a.ncombo * a.n_mono;
  unsigned char *pi = reinterpret_cast<unsigned char *>(Sd + (size_t)a.nmpair * kJtKD);
  pi = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(pi) + 15) & ~uintptr_t(15));
  uint32_t *info = reinterpret_cast<uint32_t *>(pi);
  uint16_t *lists = reinterpret_cast<uint16_t *>(info + a.cap);
  int *cnt = reinterpret_cast<int *>(lists + (size_t)a.cap * a.nz);
  const int64_t p0 = a.poff[i];
  const int np = (int)(a.pend[i] - p0);
  if (np > a.cap) {
    if (lane == 0) atomicExch(a.err, 1);
    return;
  }
  T *ui = a.u + i * a.nf;
  const T wi0 = a.w[3 * i], wi1 = a.w[3 * i + 1], wi2 = a.w[3 * i + 2];
  // ---- stage: unit vector and r, w_j - w_i and r dot, flags, cutoff and E tables
  for (int q = lane; q < np; q += 32) {
    const V4<T> d = a.rij[p0 + q];
    const int32_t j = a.pj[p0 + q];
    const uint32_t meta = a.pmeta[p0 + q];
    const bool self = j == i;
    const T w0 = self ? (T)0 : a.w[3 * j] - wi0, w1 = self ? (T)0 : a.w[3 * j + 1] - wi1,
            w2 = self ? (T)0 : a.w[3 * j + 2] - wi2;
    const T rinv = (T)1 / d.w;
    const V4<T> u{d.x * rinv, d.y * rinv, d.z * rinv, d.w};
    const T rdot = u.x * w0 + u.y * w1 + u.z * w2;
    U[q] = u;
    Wd[q] = V4<T>{w0, w1, w2, rdot};
    const uint32_t rmask = meta >> 24;
    info[q] = (uint32_t)(uint8_t)a.code[j] | ((uint32_t)self << 8) | (rmask << 16);
    for (int rc = 0; rc < a.nrcls; rc++) {
      const T rcut = a.rcls[rc];
      const bool in = (rmask >> rc) & 1u;
      T f, df;
      cutoff_fc<T>(in ? d.w : rcut, rcut, f, df);
      fc[rc * a.cap + q] = in ? f : (T)0;
      dfc[rc * a.cap + q] = in ? df : (T)0;
    }
    for (int e = 0; e < a.necls; e++) {
      const T eta = a.ecls_eta[e];
      const int rc = a.ecls_rclass[e];
      const T ex = m_exp2<T>((-eta * (T)kLog2e) * (d.w * d.w));
      const T f = fc[rc * a.cap + q];
      E[e * a.cap + q] = ex * f;
      dE[e * a.cap + q] = ex * (dfc[rc * a.cap + q] - (T)2 * eta * d.w * f) * rdot;
    }
  }
  __syncwarp();
  for (int z = 0; z < a.nz; z++) {
    int base = 0;
    for (int q0 = 0; q0 < np; q0 += 32) {
      const int q = q0 + lane;
      bool in = false;
      if (q < np) {
        const uint32_t inf = info[q];
        in = ((int)(inf & 0xff) == z) || ((inf >> 8) & 1u);
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) lists[z * a.cap + base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
      base += __popc(m);
    }
    if (lane == 0) cnt[z] = base;
  }
  __syncwarp();
  // ---- radial functions: dG/dr along r dot, lanes over pairs
  for (int f = 0; f < a.nrad; f++) {
    const GDesc g = a.rad[f];
    const T *fcr = fc + g.rclass * a.cap, *dfcr = dfc + g.rclass * a.cap;
    const uint16_t *lst = g.chan1 >= 0 ? lists + g.chan1 * a.cap : nullptr;
    const int n = g.chan1 >= 0 ? cnt[g.chan1] : np;
    T acc = (T)0;
    for (int k = lane; k < n; k += 32) {
      const int q = lst ? lst[k] : k;
      const T r = U[q].w, fcv = fcr[q], dfv = dfcr[q];
      T dg;
      if (g.type == 1) {
        dg = dfv;
      } else if (g.type == 2) {
        const T x = r - (T)g.rs;
        dg = m_exp2<T>((-(T)g.eta * (T)kLog2e) * (x * x)) * (dfv - (T)2 * (T)g.eta * x * fcv);
      } else {
        const T kr = (T)g.kappa * r;
        dg = m_cos<T>(kr) * dfv - (T)g.kappa * m_sin<T>(kr) * fcv;
      }
      acc += dg * Wd[q].w;
    }
    acc = jsum(acc);
    if (lane == 0 && FNETG_GUARD(g.out >= 0 && g.out < a.nf)) ui[g.out] = acc * jt_zscale(a, g.out);
  }
  if (a.nmf == 0) return;
  // ---- moments (from the cache when it holds them) and their tangents
  const bool cached = a.mom != nullptr;
  if (cached) {
    const T *src = a.mom + i * (int64_t)a.ncombo * a.n_mono;
    for (int k = lane; k < a.ncombo * a.n_mono; k += 32) M[k] = src[k];
  }
  for (int k = 0; k < a.ncombo;) {
    const int z = a.combo[2 * k];
    int nk = 1;
    while (k + nk < a.ncombo && nk < 4 && a.combo[2 * (k + nk)] == z) nk++;
    const uint16_t *lst = z >= 0 ? lists + z * a.cap : nullptr;
    const int n = z >= 0 ? cnt[z] : np;
    if (cached) {
      if (nk == 1) jt_moment_pass<T, D, 32, false>(a, U, Wd, E, dE, lst, n, k, 1, M, dM, lane);
      else if (nk == 2) jt_moment_pass<T, D, 16, false>(a, U, Wd, E, dE, lst, n, k, 2, M, dM, lane);
      else jt_moment_pass<T, D, 8, false>(a, U, Wd, E, dE, lst, n, k, nk, M, dM, lane);
    } else {
      if (nk == 1) jt_moment_pass<T, D, 32, true>(a, U, Wd, E, dE, lst, n, k, 1, M, dM, lane);
      else if (nk == 2) jt_moment_pass<T, D, 16, true>(a, U, Wd, E, dE, lst, n, k, 2, M, dM, lane);
      else jt_moment_pass<T, D, 8, true>(a, U, Wd, E, dE, lst, n, k, nk, M, dM, lane);
    }
    k += nk;
  }
  __syncwarp();
  // ---- degree-sum tangents of every combo pair, then the functions
  for (int it = lane; it < a.nmpair * kJtKD; it += 32) {
    const int pr = it / kJtKD, m = it - pr * kJtKD;
    const int k1 = a.mpair[2 * pr], k2 = a.mpair[2 * pr + 1];
    const T *M1 = M + k1 * NM, *M2 = M + k2 * NM, *dM1 = dM + k1 * NM, *dM2 = dM + k2 * NM;
    const int a0 = m * (m + 1) * (m + 2) / 6, a1 = min(NM, (m + 1) * (m + 2) * (m + 3) / 6);
    T acc = 0;
    for (int al = a0; al < a1; al++)
      acc += (T)kMonoMult[al] * (dM1[al] * M2[al] + M1[al] * dM2[al]);
    Sd[it] = acc;
  }
  __syncwarp();
  for (int f = lane; f < a.nmf; f += 32) {
    const MFunc mf = a.mfunc[f];
    const T *pc = a.fpc + f * kJtKD, *S = Sd + mf.pair * kJtKD;
    T acc = 0;
#pragma unroll
    for (int m = 0; m < kJtKD; m++) acc += pc[m] * S[m];
    if (FNETG_GUARD(mf.out >= 0 && mf.out < a.nf)) ui[mf.out] = acc * jt_zscale(a, mf.out);
  }
}

template <typename T, int D> int launch_jvp_tile(fnetg_ctx *ctx, JtArgs<T> &a) {
  const size_t smem = jt_warp_bytes(a) * kJtWarps;
  FNETG_CHECK(smem <= 227 * 1024, FNETG_E_UNSUPPORTED,
              "features_jvp: the neighbour tile of one atom exceeds shared memory");
  FNETG_CUDA(raise_smem_limit((const void *)jvp_tile_kernel<T, D>, smem));
  LaunchScope ls(ctx, "features_jvp");
  jvp_tile_kernel<T, D><<<ceil_div(ctx->N, kJtWarps), 32 * kJtWarps, smem, ctx->stream>>>(a);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

template <typename T> int do_jvp(fnetg_ctx *ctx, const T *d_w, T *d_u) {
  for (auto &g : ctx->h_rad) {
    FNETG_CHECK(g.atomid == 0, FNETG_E_UNSUPPORTED, "features_jvp: atom-id weighted functions");
  }
  for (auto &g : ctx->h_ang_all) {
    FNETG_CHECK(g.type == 5 && g.atomid == 0, FNETG_E_UNSUPPORTED,
                "features_jvp: G4 and atom-id weighted angular functions");
  }
  // the triplet kernel's angular functions: those outside the moment form
  FNETG_CHECK(ctx->h_ang.empty() || ctx->max_pairs <= kJvpCap, FNETG_E_UNSUPPORTED,
              "features_jvp: more than 256 neighbours of one atom");
  // angular functions grouped by (lists, cutoff class, eta class), at most kJvpGroup each
  std::vector<GDesc> ord;
  std::vector<int4> grp;
  {
    std::vector<std::array<int, 4>> keys;
    for (auto &g : ctx->h_ang) {
      const std::array<int, 4> k{g.chan1, g.chan2, g.rclass, g.eclass};
      if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
    }
    for (auto &k : keys) {
      std::vector<GDesc> mem;
      for (auto &g : ctx->h_ang)
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
  a.nrad = 0;  // the radial functions run in the tile kernel
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
  if (ctx->N == 0) return FNETG_OK;
  // radial and moment-form functions
  {
    JtArgs<T> t{};
    t.natoms = ctx->N;
    t.poff = a.poff;
    t.pend = a.pend;
    t.pj = a.pj;
    t.pmeta = a.pmeta;
    t.rij = a.rij;
    t.code = a.code;
    t.w = d_w;
    t.rad = ctx->d_rad.as<GDesc>();
    t.nrad = (int)ctx->h_rad.size();
    t.necls = (int)ctx->ecls_eta.size();
    for (int e = 0; e < kMaxEtaClasses; e++) {
      const bool on = e < t.necls;
      t.ecls_eta[e] = on ? (T)ctx->ecls_eta[e] : (T)0;
      t.ecls_rclass[e] = on ? ctx->ecls_rclass[e] : 0;
    }
    t.nrcls = (int)ctx->rcut_classes.size();
    for (int c = 0; c < kMaxRcutClasses; c++)
      t.rcls[c] = c < t.nrcls ? (T)ctx->rcut_classes[c] : (T)0;
    t.nz = (int)ctx->zcodes.size();
    t.cap = std::max(32, (ctx->max_pairs + 31) / 32 * 32);
    FNETG_CHECK(t.cap <= 65535, FNETG_E_UNSUPPORTED, "features_jvp: more than 65535 neighbours");
    t.nmf = (int)ctx->h_mfunc.size();
    t.ncombo = t.nmf > 0 ? ctx->n_combo : 0;
    t.n_mono = t.nmf > 0 ? ctx->n_mono : 0;
    t.combo = ctx->d_combo.as<int32_t>();
    t.mom = (t.nmf > 0 && ctx->mom_valid) ? ctx->d_mom.as<T>() : nullptr;
    t.mpair = ctx->d_mpair.as<int32_t>();
    t.nmpair = t.nmf > 0 ? (int)ctx->h_mpair.size() / 2 : 0;
    t.mfunc = ctx->d_mfunc.as<MFunc>();
    t.fpc = static_cast<const T *>(sizeof(T) == 8 ? ctx->d_fpc_d.p : ctx->d_fpc_f.p);
    t.zsd = a.zsd;
    t.zinv = a.zinv;
    t.u = d_u;
    t.nf = ctx->nf;
    t.err = a.err;
    int rc;
    switch (t.nmf > 0 ? ctx->mom_degree : 1) {
      case 1: rc = launch_jvp_tile<T, 1>(ctx, t); break;
      case 2: rc = launch_jvp_tile<T, 2>(ctx, t); break;
      case 3: rc = launch_jvp_tile<T, 3>(ctx, t); break;
      default: rc = launch_jvp_tile<T, 4>(ctx, t); break;
    }
    if (rc) return rc;
  }
  if (a.ngrp > 0) {
    const size_t smem = (size_t)kJvpWarps * kJvpCap *
                        (2 * sizeof(V4<T>) + 2 * sizeof(T) + sizeof(uint32_t) + 2 * sizeof(uint16_t));
    FNETG_CUDA(raise_smem_limit((const void *)jvp_kernel<T>, smem));
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

FNETG_CHECK_READER(check_site_jvp)

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
