// K4 + K9: analytical forces F = -dE/dR (forceAnalysis_analytical,
// lib_analysis/forces.F90:317-425, on the ACSF derivatives of gFuncGrad / iGeoAcsfGrad,
// lib_descriptors/acsf.F90:870-939, 1496-1697) as a fused adjoint contraction.
//
// Instead of materialising the dense [3, nG, N, N] derivative array, every centre atom i
// contracts dE/dG_i (the network Jacobian divided by the z-score deviations) with the
// derivatives of its own G-values on the fly: one warp per atom stages the pair tile,
// accumulates w_p = sum_g dE/dG_ig * dG_ig/dv_p for every neighbour image p (radial terms
// lanes-over-pairs, angular terms lanes-over-(row, column-chunk) of the triplet matrix with
// shared-memory accumulation), and scatters F_j -= w_p, F_i += w_p with FP64 atomics.
// Each periodic image contributes its own derivative (physical forces).
#include <algorithm>

#include "internal.cuh"

namespace fnetg {

namespace {

constexpr double kPi = 3.14159265358979323846;

template <typename T> struct ForceArgs {
  int64_t natoms;
  const int64_t *poff;
  const int32_t *pj;
  const uint32_t *pmeta;
  const V4<T> *rij;
  const int8_t *code;
  const double *ext;
  int next;
  const GDesc *rad;
  int nrad;
  const GDesc *ang;
  const AGroup *groups;
  int ngroups;
  const double *ecls_eta;
  const int *ecls_rclass;
  const int *ecls_atomid;
  int necls;
  const double *rcls;
  int nrcls;
  int nz;
  int cap;
  int ng;
  const T *J;   // [N][nf] atom order, dE/dG (raw features)
  int nf;
  double *F;    // [N][nout][3]
  int out_index, nout;
};

template <typename T> struct FTile {
  V4<T> *v;
  V4<T> *w;        // pair force accumulators (x, y, z)
  T *fc, *dfc;     // [nrcls][cap]
  T *E, *D;        // [necls][cap]
  uint32_t *info;
  int32_t *pj;
  uint16_t *lists;
  int *cnt;
  T *jv;           // [ng] dE/dG of the centre atom
  T *gpar;         // [5][32] lambda, xi, eta, Jw, rcut
  int *gint;       // [3][32] xi_int, eclass, type
  T *idv;          // [cap] atom ids of the group's column (G4 third cutoff)
};

template <typename T> __host__ __device__ size_t ftile_bytes(int cap, int nrcls, int necls, int nz, int ng) {
  size_t b = 0;
  b += 2 * sizeof(V4<T>) * cap;
  b += sizeof(T) * (size_t)cap * 2 * (nrcls + necls);
  b += (sizeof(uint32_t) + sizeof(int32_t)) * cap;
  b += sizeof(T) * (ng + 5 * 32);
  b += sizeof(int) * (3 * 32 + 8);
  b += sizeof(uint16_t) * (size_t)cap * nz;
  b += sizeof(T) * cap;
  return (b + 127) / 128 * 128;
}

template <typename T>
__device__ FTile<T> fcarve(unsigned char *p, int cap, int nrcls, int necls, int nz, int ng) {
  FTile<T> t;
  t.v = reinterpret_cast<V4<T> *>(p);
  p += sizeof(V4<T>) * cap;
  t.w = reinterpret_cast<V4<T> *>(p);
  p += sizeof(V4<T>) * cap;
  t.fc = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * nrcls;
  t.dfc = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * nrcls;
  t.E = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * necls;
  t.D = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * necls;
  t.jv = reinterpret_cast<T *>(p);
  p += sizeof(T) * ng;
  t.gpar = reinterpret_cast<T *>(p);
  p += sizeof(T) * 5 * 32;
  t.idv = reinterpret_cast<T *>(p);
  p += sizeof(T) * cap;
  t.info = reinterpret_cast<uint32_t *>(p);
  p += sizeof(uint32_t) * cap;
  t.pj = reinterpret_cast<int32_t *>(p);
  p += sizeof(int32_t) * cap;
  t.gint = reinterpret_cast<int *>(p);
  p += sizeof(int) * 3 * 32;
  t.cnt = reinterpret_cast<int *>(p);
  p += sizeof(int) * 8;
  t.lists = reinterpret_cast<uint16_t *>(p);
  return t;
}

template <typename T> __device__ __forceinline__ T f_exp(T x);
template <> __device__ __forceinline__ float f_exp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double f_exp<double>(double x) { return exp(x); }
template <typename T> __device__ __forceinline__ T f_cos(T x);
template <> __device__ __forceinline__ float f_cos<float>(float x) { return cosf(x); }
template <> __device__ __forceinline__ double f_cos<double>(double x) { return cos(x); }
template <typename T> __device__ __forceinline__ T f_sin(T x);
template <> __device__ __forceinline__ float f_sin<float>(float x) { return sinf(x); }
template <> __device__ __forceinline__ double f_sin<double>(double x) { return sin(x); }
template <typename T> __device__ __forceinline__ T f_pow(T b, T e);
template <> __device__ __forceinline__ float f_pow<float>(float b, float e) { return powf(b, e); }
template <> __device__ __forceinline__ double f_pow<double>(double b, double e) { return pow(b, e); }
template <typename T> __device__ __forceinline__ T f_sqrt(T x);
template <> __device__ __forceinline__ float f_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double f_sqrt<double>(double x) { return sqrt(x); }

template <typename T> __device__ __forceinline__ T ipow_or_pow(T base, int n, T e) {
  // base^e where n = e if e is a small positive integer (n == 0: general power)
  if (n > 0) {
    T r = 1;
    for (int k = 0; k < n; k++) r *= base;
    return r;
  }
  return f_pow<T>(base, e);
}

template <typename T>
__device__ __forceinline__ T aid(const double *ext, int next, int atomid, int64_t a) {
  return atomid > 0 ? (T)ext[a * next + (atomid - 1)] : (T)1;
}

template <typename T> __device__ __forceinline__ void sh_add(T *p, T v) { atomicAdd(p, v); }

// rows over list R, columns over list C: w[row] += fac * d/dv_row of sum_f Jw_f t_f(row, col)
template <typename T>
__device__ void angular_side(const ForceArgs<T> &a, FTile<T> &tl, const AGroup &G,
                             const uint16_t *lr, int nr, const uint16_t *lc, int nc, T fac,
                             int lane) {
  if (nr == 0 || nc == 0) return;
  const int S = nr >= 32 ? 1 : min(nc, (32 + nr - 1) / nr);
  const int cs = (nc + S - 1) / S;
  const int items = nr * S;
  const T rcut4 = tl.gpar[4 * 32];
  for (int it = lane; it < items; it += 32) {
    const int jj = it / S, ch = it % S;
    const int p = lr ? lr[jj] : jj;
    const V4<T> vp = tl.v[p];
    const T rp = vp.w;
    const T upx = vp.x / rp, upy = vp.y / rp, upz = vp.z / rp;
    T wx = 0, wy = 0, wz = 0;
    const int k0 = ch * cs, k1 = min(nc, k0 + cs);
    for (int kk = k0; kk < k1; kk++) {
      const int q = lc ? lc[kk] : kk;
      const V4<T> vq = tl.v[q];
      const T rq = vq.w;
      const T uqx = vq.x / rq, uqy = vq.y / rq, uqz = vq.z / rq;
      T c = (vp.x * vq.x + vp.y * vq.y + vp.z * vq.z) / (rp * rq + (T)1e-13);
      c = c > (T)1 ? (T)1 : (c < (T)-1 ? (T)-1 : c);
      T g = 1, gd = 0, rpq = 0, ex = 0, ey = 0, ez = 0;
      if (G.has_g4) {
        ex = vp.x - vq.x;
        ey = vp.y - vq.y;
        ez = vp.z - vq.z;
        rpq = f_sqrt<T>(ex * ex + ey * ey + ez * ez);
      }
      T A = 0, B = 0, C = 0;
#pragma unroll 4
      for (int f = 0; f < G.count; f++) {
        const T lam = tl.gpar[f], xi = tl.gpar[32 + f], Jw = tl.gpar[96 + f];
        const int xn = tl.gint[f], e = tl.gint[32 + f], ty = tl.gint[64 + f];
        const T base = (T)1 + lam * c;
        const T angm1 = xn > 1 ? ipow_or_pow<T>(base, xn - 1, xi - (T)1)
                               : (xn == 1 ? (T)1 : f_pow<T>(base, xi - (T)1));
        const T ang = angm1 * base;
        const T angd = xi * lam * angm1;
        const T Ep = tl.E[e * a.cap + p], Eq = tl.E[e * a.cap + q], Dp = tl.D[e * a.cap + p];
        T gg = 1, ggd = 0;
        if (ty == 4) {
          const T eta = tl.gpar[64 + f];
          if (rpq > rcut4) {
            gg = 0;
            ggd = 0;
          } else {
            const T ee = f_exp<T>(-(eta * rpq * rpq));
            const T fcq = (T)0.5 * (f_cos<T>((T)kPi * rpq / rcut4) + (T)1);
            const T dfq = (T)-0.5 * ((T)kPi / rcut4) * f_sin<T>((T)kPi * rpq / rcut4);
            gg = ee * fcq;
            ggd = ee * (dfq - (T)2 * eta * rpq * fcq);
            if (G.atomid > 0) {
              const T ii = tl.idv[p] * tl.idv[q];
              gg *= ii;
              ggd *= ii;
            }
          }
        }
        A += Jw * angd * Ep * Eq * gg;
        B += Jw * ang * Dp * Eq * gg;
        C += Jw * ang * Ep * Eq * ggd;
      }
      // d c / d v_p = (u_q - c u_p) / r_p
      const T s = A / rp;
      wx += s * (uqx - c * upx) + B * upx;
      wy += s * (uqy - c * upy) + B * upy;
      wz += s * (uqz - c * upz) + B * upz;
      if (G.has_g4 && rpq > (T)0) {
        const T sc = C / rpq;
        wx += sc * ex;
        wy += sc * ey;
        wz += sc * ez;
      }
      (void)g;
      (void)gd;
    }
    sh_add<T>(&tl.w[p].x, fac * wx);
    sh_add<T>(&tl.w[p].y, fac * wy);
    sh_add<T>(&tl.w[p].z, fac * wz);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) forces_kernel(ForceArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const size_t tb = ftile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, a.ng);
  FTile<T> tl = fcarve<T>(smem + tb * warp, a.cap, a.nrcls, a.necls, a.nz, a.ng);
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < a.natoms; i += (int64_t)gridDim.x * wpb) {
    const int64_t p0 = a.poff[i];
    const int np = (int)(a.poff[i + 1] - p0);
    for (int g = lane; g < a.ng; g += 32) tl.jv[g] = a.J[i * a.nf + g];
    for (int q = lane; q < np; q += 32) {
      const V4<T> v = a.rij[p0 + q];
      tl.v[q] = v;
      tl.w[q] = V4<T>{0, 0, 0, 0};
      const int32_t j = a.pj[p0 + q];
      tl.pj[q] = j;
      const uint32_t rmask = a.pmeta[p0 + q] >> 24;
      const int c = a.code[j];
      tl.info[q] = (uint32_t)(c & 0xff) | ((uint32_t)(j == i) << 8) | (rmask << 16);
      for (int rc = 0; rc < a.nrcls; rc++) {
        const T rcut = (T)a.rcls[rc];
        const bool in = (rmask >> rc) & 1u;
        tl.fc[rc * a.cap + q] = in ? (T)0.5 * (f_cos<T>((T)kPi * v.w / rcut) + (T)1) : (T)0;
        tl.dfc[rc * a.cap + q] =
            in ? (T)-0.5 * ((T)kPi / rcut) * f_sin<T>((T)kPi * v.w / rcut) : (T)0;
      }
      for (int e = 0; e < a.necls; e++) {
        const T eta = (T)a.ecls_eta[e];
        const int rc = a.ecls_rclass[e];
        const T ex = f_exp<T>(-(eta * (v.w * v.w)));
        T ids = (T)1;
        if (a.ecls_atomid[e] > 0)
          ids = aid<T>(a.ext, a.next, a.ecls_atomid[e], i) * aid<T>(a.ext, a.next, a.ecls_atomid[e], j);
        const T f = tl.fc[rc * a.cap + q], df = tl.dfc[rc * a.cap + q];
        tl.E[e * a.cap + q] = ex * f * ids;
        tl.D[e * a.cap + q] = ex * (df - (T)2 * eta * v.w * f) * ids;
      }
    }
    __syncwarp();
    for (int z = 0; z < a.nz; z++) {
      int base = 0;
      for (int q0 = 0; q0 < np; q0 += 32) {
        const int q = q0 + lane;
        bool in = false;
        if (q < np) {
          const uint32_t inf = tl.info[q];
          in = ((int)(inf & 0xff) == z) || ((inf >> 8) & 1u);
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) tl.lists[z * a.cap + base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
        base += __popc(m);
      }
      if (lane == 0) tl.cnt[z] = base;
    }
    __syncwarp();
    // ---- radial: lanes over pairs
    for (int q = lane; q < np; q += 32) {
      const uint32_t inf = tl.info[q];
      const int code = (int)(inf & 0xff);
      const bool self = (inf >> 8) & 1u;
      const T r = tl.v[q].w;
      T dsum = 0;
      for (int g = 0; g < a.nrad; g++) {
        const GDesc d = a.rad[g];
        if (d.chan1 >= 0 && code != d.chan1 && !self) continue;
        if (!((inf >> (16 + d.rclass)) & 1u)) continue;
        T fc = tl.fc[d.rclass * a.cap + q], dfc = tl.dfc[d.rclass * a.cap + q];
        if (d.atomid > 0) {
          const T ids = aid<T>(a.ext, a.next, d.atomid, i) * aid<T>(a.ext, a.next, d.atomid, tl.pj[q]);
          fc *= ids;
          dfc *= ids;
        }
        T dg;
        if (d.type == 1) {
          dg = dfc;
        } else if (d.type == 2) {
          const T x = r - (T)d.rs;
          dg = f_exp<T>(-((T)d.eta * (x * x))) * (dfc - (T)2 * (T)d.eta * x * fc);
        } else {
          const T kr = (T)d.kappa * r;
          dg = f_cos<T>(kr) * dfc - (T)d.kappa * f_sin<T>(kr) * fc;
        }
        dsum += tl.jv[d.out] * dg;
      }
      const V4<T> v = tl.v[q];
      const T s = dsum / r;
      tl.w[q].x += s * v.x;
      tl.w[q].y += s * v.y;
      tl.w[q].z += s * v.z;
    }
    __syncwarp();
    // ---- angular groups
    for (int gi = 0; gi < a.ngroups; gi++) {
      const AGroup G = a.groups[gi];
      __syncwarp();
      if (lane < G.count) {
        const GDesc d = a.ang[G.first + lane];
        tl.gpar[lane] = (T)d.lambda;
        tl.gpar[32 + lane] = (T)d.xi;
        tl.gpar[64 + lane] = (T)d.eta;
        tl.gpar[96 + lane] = tl.jv[d.out] * (T)d.pref;
        tl.gint[lane] = d.xi_int;
        tl.gint[32 + lane] = d.eclass;
        tl.gint[64 + lane] = d.type;
        if (lane == 0) tl.gpar[128] = (T)d.rcut;
      }
      if (G.has_g4 && G.atomid > 0)
        for (int q = lane; q < np; q += 32) tl.idv[q] = aid<T>(a.ext, a.next, G.atomid, tl.pj[q]);
      __syncwarp();
      const uint16_t *l1 = G.chan1 >= 0 ? tl.lists + G.chan1 * a.cap : nullptr;
      const uint16_t *l2 = G.chan2 >= 0 ? tl.lists + G.chan2 * a.cap : nullptr;
      const int n1 = G.chan1 >= 0 ? tl.cnt[G.chan1] : np;
      const int n2 = G.chan2 >= 0 ? tl.cnt[G.chan2] : np;
      if (G.same) {
        angular_side<T>(a, tl, G, l1, n1, l1, n1, (T)2, lane);
      } else {
        angular_side<T>(a, tl, G, l1, n1, l2, n2, (T)1, lane);
        __syncwarp();
        angular_side<T>(a, tl, G, l2, n2, l1, n1, (T)1, lane);
      }
    }
    __syncwarp();
    // ---- scatter: F_j -= w_p, F_i += sum_p w_p (self images cancel)
    double sx = 0, sy = 0, sz = 0;
    for (int q = lane; q < np; q += 32) {
      if ((tl.info[q] >> 8) & 1u) continue;
      const V4<T> w = tl.w[q];
      const int64_t j = tl.pj[q];
      double *Fj = a.F + (j * a.nout + a.out_index) * 3;
      atomicAdd(Fj + 0, -(double)w.x);
      atomicAdd(Fj + 1, -(double)w.y);
      atomicAdd(Fj + 2, -(double)w.z);
      sx += (double)w.x;
      sy += (double)w.y;
      sz += (double)w.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if (lane == 0) {
      double *Fi = a.F + (i * a.nout + a.out_index) * 3;
      atomicAdd(Fi + 0, sx);
      atomicAdd(Fi + 1, sy);
      atomicAdd(Fi + 2, sz);
    }
    __syncwarp();
  }
}

template <typename T> int launch_forces(fnetg_ctx *ctx) {
  const int64_t N = ctx->N;
  const int nout = ctx->dims.back();
  const int nf = ctx->nf;
  const int ng = (int)ctx->gf.size();
  FNETG_CUDA(ctx->d_forces.ensure(sizeof(double) * std::max<int64_t>(N, 1) * nout * 3));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_forces.p, 0, sizeof(double) * std::max<int64_t>(N, 1) * nout * 3,
                             ctx->stream));
  FNETG_CUDA(ctx->d_jacT.ensure(sizeof(T) * std::max<int64_t>(N, 1) * nf));
  if (N == 0) return FNETG_OK;
  ForceArgs<T> a{};
  a.natoms = N;
  a.poff = ctx->d_poff.as<int64_t>();
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = static_cast<const V4<T> *>(ctx->d_rij.p);
  a.code = ctx->d_code.as<int8_t>();
  a.ext = ctx->d_ext.as<double>();
  a.next = ctx->next;
  a.rad = ctx->d_rad.as<GDesc>();
  a.nrad = (int)ctx->h_rad.size();
  a.ang = ctx->d_ang.as<GDesc>();
  a.groups = ctx->d_groups.as<AGroup>();
  a.ngroups = (int)ctx->h_groups.size();
  a.ecls_eta = ctx->d_ecls_eta.as<double>();
  a.ecls_rclass = ctx->d_ecls_rclass.as<int>();
  a.ecls_atomid = ctx->d_ecls_atomid.as<int>();
  a.necls = (int)ctx->ecls_eta.size();
  a.rcls = ctx->d_rcls.as<double>();
  a.nrcls = (int)ctx->rcut_classes.size();
  a.nz = (int)ctx->zcodes.size();
  a.cap = std::max(32, (ctx->max_pairs + 31) / 32 * 32);
  a.ng = ng;
  a.J = ctx->d_jacT.as<T>();
  a.nf = nf;
  a.F = ctx->d_forces.as<double>();
  a.nout = nout;
  const size_t tb = ftile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, ng);
  int wpb = 8;
  while (wpb > 1 && tb * wpb > 200 * 1024) wpb >>= 1;
  FNETG_CHECK(tb * wpb <= 227 * 1024, FNETG_E_UNSUPPORTED,
              "neighbour tile of one atom exceeds shared memory");
  const size_t smem = tb * wpb;
  FNETG_CUDA(cudaFuncSetAttribute(forces_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, forces_kernel<T>, wpb * 32, smem);
  const int64_t want = (N + wpb - 1) / wpb;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>(want, (int64_t)num_sms() * std::max(per_sm, 1) * 8));
  for (int o = 0; o < nout; o++) {
    int rc = run_jacobian(ctx, o, ctx->d_jacT.p);
    if (rc) return rc;
    a.out_index = o;
    LaunchScope ls(ctx, "forces");
    forces_kernel<T><<<blocks, wpb * 32, smem, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

}  // namespace

int run_forces(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? launch_forces<double>(ctx) : launch_forces<float>(ctx);
}

}  // namespace fnetg
