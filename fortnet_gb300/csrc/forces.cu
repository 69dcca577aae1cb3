// K4 + K9: analytical forces F = -dE/dR (forceAnalysis_analytical,
// lib_analysis/forces.F90:317-425, on the ACSF derivatives of gFuncGrad / iGeoAcsfGrad,
// lib_descriptors/acsf.F90:870-939, 1496-1697) as a fused adjoint contraction.
//
// The dense [3, nG, N, N] derivative array is never formed: every centre atom contracts
// dE/dG_i (network Jacobian divided by the z-score deviations) with the derivatives of its own
// G-values on the fly.  One warp per atom over the shared neighbour tile (tile.cuh) accumulates
// w_p = sum_g dE/dG_ig * dG_ig/dv_p for every neighbour image p:
//   radial terms     lanes over pairs;
//   integer-xi G5    adjoint moments Q_k(alpha) = sum_f J_f coef_f(alpha) M_other(alpha), then per
//                    pair w_p += sum_k Q_k(alpha) d(E u^alpha)/dv_p — O(N_nb) per atom;
//   G4 / other xi    lanes over (row, column chunk) of the triplet matrix with shared-memory
//                    accumulation.
// Forces are scattered as F_j -= w_p, F_i += w_p with FP64 atomics; every periodic image
// contributes its own derivative (physical forces), self images cancel.
#define FNETG_FILE_CODE 3  // site codes of the bounds-checked build
#include <algorithm>

#include "tile.cuh"

namespace fnetg {

namespace {

template <typename T> __device__ __forceinline__ T ipow_or_pow(T base, int n, T e) {
  // base^e where n = e if e is a small positive integer (n == 0: general power)
  if (n > 0) {
    T r = 1;
    for (int k = 0; k < n; k++) r *= base;
    return r;
  }
  return m_pow<T>(base, e);
}

template <typename T> __device__ __forceinline__ void sh_add(T *p, T v) { atomicAdd(p, v); }

// rows over list R, columns over list C: w[row] += fac * d/dv_row of sum_f Jw_f t_f(row, col)
template <typename T>
__device__ void angular_side(const TileArgs<T> &a, Tile<T> &tl, const AGroup &G,
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
      if (sizeof(T) == 4 && p == q) c = (T)1;  // j = k exactly (see the ACSF kernel)
      T g = 1, gd = 0, rpq = 0, ex = 0, ey = 0, ez = 0;
      if (G.has_g4) {
        ex = vp.x - vq.x;
        ey = vp.y - vq.y;
        ez = vp.z - vq.z;
        rpq = m_sqrt<T>(ex * ex + ey * ey + ez * ez);
      }
      T A = 0, B = 0, C = 0;
#pragma unroll 4
      for (int f = 0; f < G.count; f++) {
        const T lam = tl.gpar[f], xi = tl.gpar[32 + f], Jw = tl.gpar[96 + f];
        const int xn = tl.gint[f], e = tl.gint[32 + f], ty = tl.gint[64 + f];
        const T base = (T)1 + lam * c;
        const T angm1 = xn > 1 ? ipow_or_pow<T>(base, xn - 1, xi - (T)1)
                               : (xn == 1 ? (T)1 : m_pow<T>(base, xi - (T)1));
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
            const T ee = m_exp<T>(-(eta * rpq * rpq));
            // rpq <= rcut4: the argument lies in [0, pi]
            T fcq, dfq;
            cutoff_fc<T>(rpq, rcut4, fcq, dfq);
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


// E_e(r) = exp(-eta_e r^2) fc(r) [id_i id_j] and D_e = dE_e/dr of pair q, from the tables when
// the tile keeps them, else from the cutoff tables (the same operations as stage_tile).
template <typename T>
__device__ __forceinline__ void pair_e_d(const TileArgs<T> &a, const Tile<T> &tl, int q, int e,
                                         T r, int64_t i, T &E, T &Dv) {
  if (tl.E) {
    E = tl.E[e * a.cap + q];
    Dv = tl.D[e * a.cap + q];
    return;
  }
  const T eta = a.ecls_eta[e];
  const int rc = a.ecls_rclass[e];
  const int aid = a.ecls_atomid[e];
  const T f = tl.fc[rc * a.cap + q], df = tl.dfc[rc * a.cap + q];
  T ids = (T)1;
  if (aid > 0) ids = atom_id<T>(a.ext, a.next, aid, i) * atom_id<T>(a.ext, a.next, aid, tl.pj[q]);
  const T ex = m_exp2<T>((-eta * (T)kLog2e) * (r * r));
  E = ex * f * ids;
  Dv = ex * (df - (T)2 * eta * r * f) * ids;
}

// Per-pair derivative of the moment terms, degree D and (for NE > 0) the eta-class count known at
// compile time.  Linear in the adjoint moments, so with c_D(alpha) = sum_e D_e Qc_e(alpha) and
// c_E(alpha) = sum_e E_e Qc_e(alpha)
//   w += P_D(u) u + (grad P_E(u) - (grad P_E(u) . u) u) / r,   P_c(u) = sum_alpha c(alpha) u^alpha.
// The monomials are built as products (child = parent * coordinate) and the gradient takes
// d/dx u^alpha = a u^(alpha - e_x) from the same registers.  NE = 0: any class count, one
// polynomial pass per class.
template <typename T, int D, int NE>
__device__ __forceinline__ void moment_pair_force(const TileArgs<T> &a, Tile<T> &tl, int q,
                                                  int zz, int64_t i) {
  constexpr int NM = n_mono_of(D);
  const V4<T> u = tl.u[q];
  const T r = u.w;
  T m[NM];
  m[0] = (T)1;
#pragma unroll
  for (int al = 1; al < NM; al++) {
    const int ax = kMonoLinks.axis[al];
    m[al] = m[kMonoLinks.parent[al]] * (ax == 0 ? u.x : (ax == 1 ? u.y : u.z));
  }
  T P = 0, gx = 0, gy = 0, gz = 0;
  const T *Qz = tl.Qc + (int64_t)zz * a.necls * NM;
  auto add = [&](int al, T cd, T ce) {
    P += cd * m[al];
    const int ea = kMonoTab[al][0], eb = kMonoTab[al][1], ec = kMonoTab[al][2];
    if (ea > 0) gx += (ea == 1 ? ce : (T)ea * ce) * m[kMonoDown.idx[al][0] < 0 ? 0 : kMonoDown.idx[al][0]];
    if (eb > 0) gy += (eb == 1 ? ce : (T)eb * ce) * m[kMonoDown.idx[al][1] < 0 ? 0 : kMonoDown.idx[al][1]];
    if (ec > 0) gz += (ec == 1 ? ce : (T)ec * ce) * m[kMonoDown.idx[al][2] < 0 ? 0 : kMonoDown.idx[al][2]];
  };
  if constexpr (NE > 0) {
    T Ee[NE], De[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) pair_e_d<T>(a, tl, q, e, r, i, Ee[e], De[e]);
#pragma unroll
    for (int al = 0; al < NM; al++) {
      T cd = 0, ce = 0;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        const T qv = Qz[e * NM + al];
        cd += De[e] * qv;
        ce += Ee[e] * qv;
      }
      add(al, cd, ce);
    }
  } else {
    for (int e = 0; e < a.necls; e++) {
      T Ev, Dv;
      pair_e_d<T>(a, tl, q, e, r, i, Ev, Dv);
      const T *Qe = Qz + e * NM;
#pragma unroll
      for (int al = 0; al < NM; al++) {
        const T qv = Qe[al];
        add(al, Dv * qv, Ev * qv);
      }
    }
  }
  const T gu = gx * u.x + gy * u.y + gz * u.z;
  const T ir = (T)1 / r;
  tl.w[q].x += P * u.x + ir * (gx - gu * u.x);
  tl.w[q].y += P * u.y + ir * (gy - gu * u.y);
  tl.w[q].z += P * u.z + ir * (gz - gu * u.z);
}

// All pairs of the tile through moment_pair_force (self images do not move relative to the
// centre; pairs of a species outside the lists take the all-atom row nz).
template <typename T, int D, int NE>
__device__ __forceinline__ void moment_pairs(const TileArgs<T> &a, Tile<T> &tl, int np, int lane,
                                             int64_t i) {
  for (int q = lane; q < np; q += 32) {
    const uint32_t inf = tl.info[q];
    if ((inf >> 8) & 1u) continue;
    const int z = (int)(inf & 0xff);
    moment_pair_force<T, D, NE>(a, tl, q, z < a.nz ? z : a.nz, i);
  }
}

// Radial function parameters staged once per CTA: p0 = rs (G2) or kappa (G3), p1 = eta,
// meta = type | rclass << 4 | atomid << 8.
template <typename T> struct RadEntry {
  T p0, p1;
  int out, meta;
};

template <typename T> __host__ __device__ inline size_t radtab_bytes(int nrad) {
  return ((size_t)sizeof(RadEntry<T>) * nrad + 127) / 128 * 128;
}

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) / 16 * 16; }

// per-CTA copies of the factorised-adjoint tables: the group pack, the combo index and the
// degree coefficients (read in dependent chains per atom: kept out of global memory)
template <typename T> __host__ __device__ inline size_t adjtab_bytes(const TileArgs<T> &a) {
  if (a.ncombo <= 0) return 0;
  const size_t b = align16(sizeof(int32_t) * a.nqg_pack) +
                   align16(sizeof(int32_t) * (a.nz + 1) * a.necls) +
                   align16(sizeof(T) * a.nqg_ent * (kMaxMomentDegree + 1));
  return (b + 127) / 128 * 128;  // the tiles that follow stay 128-byte aligned
}

// per-warp radial coefficient table of the fast path: (rs, eta, J, J eta) per function
template <typename T> __host__ __device__ inline size_t radw_bytes(const TileArgs<T> &a) {
  return a.rad_fast >= 0 ? (sizeof(V4<T>) * a.nrad + 127) / 128 * 128 : 0;
}

// FP32: CTAs of at most 4 warps, 5 per SM (the shared-memory limit of the tiles) at up to 96
// registers a thread; FP64: up to 8 warps a CTA, registers unbounded.
template <typename T> constexpr int kForcesThreads = sizeof(T) == 4 ? 128 : 256;

template <typename T, int D>
__global__ void __launch_bounds__(kForcesThreads<T>, sizeof(T) == 4 ? 5 : 1)
    forces_kernel(const __grid_constant__ TileArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const size_t tb = tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, a.ncombo, a.n_mono, a.ng, true, a.ngroups > 0,
                    tile_etab(a, true), tile_qwords(a));
  RadEntry<T> *rt = reinterpret_cast<RadEntry<T> *>(smem);
  for (int g = threadIdx.x; g < a.nrad; g += blockDim.x) {
    const GDesc d = a.rad[g];
    const T *P = a.radp + 8 * g;
    rt[g] = RadEntry<T>{d.type == 3 ? P[1] : P[2], P[3], d.out,
                        d.type | (d.rclass << 4) | (d.atomid << 8)};
  }
  constexpr int KD = kMaxMomentDegree + 1;
  unsigned char *adj = smem + radtab_bytes<T>(a.nrad);
  int32_t *s_qg = reinterpret_cast<int32_t *>(adj);
  int32_t *s_cidx = reinterpret_cast<int32_t *>(adj + align16(sizeof(int32_t) * a.nqg_pack));
  T *s_mpc = reinterpret_cast<T *>(adj + align16(sizeof(int32_t) * a.nqg_pack) +
                                   align16(sizeof(int32_t) * (a.nz + 1) * a.necls));
  if (a.ncombo > 0) {
    for (int t = threadIdx.x; t < a.nqg_pack; t += blockDim.x) s_qg[t] = a.qg[t];
    for (int t = threadIdx.x; t < (a.nz + 1) * a.necls; t += blockDim.x) s_cidx[t] = a.cidx[t];
    for (int t = threadIdx.x; t < a.nqg_ent * KD; t += blockDim.x) s_mpc[t] = a.mpc[t];
  }
  __syncthreads();
  const size_t fixed = radtab_bytes<T>(a.nrad) + adjtab_bytes<T>(a);
  unsigned char *mine = smem + fixed + (tb + radw_bytes<T>(a)) * warp;
  Tile<T> tl = carve_tile<T>(mine, a, true);
  V4<T> *wt = reinterpret_cast<V4<T> *>(mine + tb);
  // degrees and multinomial weights of this lane's monomials (lane, lane + 32)
  const int mdeg0 = lane < kMaxMono ? kMonoTab[lane][0] + kMonoTab[lane][1] + kMonoTab[lane][2] : 0;
  const int mdeg1 = lane + 32 < kMaxMono
                        ? kMonoTab[lane + 32][0] + kMonoTab[lane + 32][1] + kMonoTab[lane + 32][2]
                        : 0;
  const T mmult0 = lane < kMaxMono ? (T)kMonoMult[lane] : (T)0;
  const T mmult1 = lane + 32 < kMaxMono ? (T)kMonoMult[lane + 32] : (T)0;
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < a.natoms; i += (int64_t)gridDim.x * wpb) {
    const int64_t p0 = a.poff[i];
    const int np = (int)(a.pend[i] - p0);
    if (!FNETG_GUARD(np >= 0 && np <= a.cap)) continue;
    // this atom's dE/dG row and cached moments: asynchronous copies overlapping the staging
    // (the previous atom's readers finished at the loop's closing warp barrier)
    async_copy<T>(tl.jv, a.J + i * a.nf, a.ng, lane);
    if (D > 0 && a.ncombo > 0 && a.mom_cached)
      async_copy<T>(tl.M, a.mom + i * (a.ncombo * n_mono_of(D > 0 ? D : 1)),
                    a.ncombo * n_mono_of(D > 0 ? D : 1), lane);
    stage_tile<T>(a, tl, i, p0, np, lane, true);
    async_copy_wait();
    if (a.rad_fast >= 0) {
      // ---- radial, fast path (G2 only, one cutoff class, no atom ids): per pair
      //   dE/dr = dfc sum_g J_g e_g - 2 fc sum_g J_g eta_g x_g e_g,  x_g = r - rs_g,
      //   e_g = exp(-eta_g x_g^2), over the all-atom functions and the pair's species' own;
      // the table holds (rs, -eta log2 e, J, J eta)
      for (int g = lane; g < a.nrad; g += 32) {
        const RadEntry<T> re = rt[g];
        const T J = tl.jv[re.out];
        wt[g] = V4<T>{re.p0, -re.p1 * (T)kLog2e, J, J * re.p1};
      }
      __syncwarp();
      const int rcl = a.rad_fast;
      for (int q = lane; q < np; q += 32) {
        const uint32_t inf = tl.info[q];
        const int code = (int)(inf & 0xff);
        if ((inf >> 8) & 1u) continue;  // self images do not move relative to the centre
        const T r = tl.u[q].w;
        T s1a = 0, s1b = 0, s2a = 0, s2b = 0;
        const int nseg = code < a.nz ? 2 : 1;
        for (int sg = 0; sg < nseg; sg++) {
          const int g0 = sg == 0 ? 0 : a.rad_seg[code + 1];
          const int g1 = sg == 0 ? a.rad_seg[1] : a.rad_seg[code + 2];
          int g = g0;
          for (; g + 2 <= g1; g += 2) {
            const V4<T> w0 = wt[g], w1 = wt[g + 1];
            const T x0 = r - w0.x, x1 = r - w1.x;
            const T e0 = m_exp2<T>(w0.y * (x0 * x0)), e1 = m_exp2<T>(w1.y * (x1 * x1));
            s1a += w0.z * e0;
            s2a += w0.w * (x0 * e0);
            s1b += w1.z * e1;
            s2b += w1.w * (x1 * e1);
          }
          if (g < g1) {
            const V4<T> w0 = wt[g];
            const T x0 = r - w0.x;
            const T e0 = m_exp2<T>(w0.y * (x0 * x0));
            s1a += w0.z * e0;
            s2a += w0.w * (x0 * e0);
          }
        }
        const T fc = tl.fc[rcl * a.cap + q], dfc = tl.dfc[rcl * a.cap + q];
        const T dsum = dfc * (s1a + s1b) - (T)2 * fc * (s2a + s2b);
        const V4<T> u = tl.u[q];
        tl.w[q].x += dsum * u.x;
        tl.w[q].y += dsum * u.y;
        tl.w[q].z += dsum * u.z;
      }
    } else
    // ---- radial: lanes over pairs, each over the all-atom functions and its species' own
    for (int q = lane; q < np; q += 32) {
      const uint32_t inf = tl.info[q];
      const int code = (int)(inf & 0xff);
      const bool self = (inf >> 8) & 1u;
      if (self) continue;  // self images do not move relative to the centre
      const T r = tl.u[q].w;
      // dE/dr of the radial functions: the cutoff tables are zero outside a function's
      // cutoff class; two independent partial sums per segment
      auto dterm = [&](int g) -> T {
        const RadEntry<T> re = rt[g];
        const int rcl = (re.meta >> 4) & 15;
        T fc = tl.fc[rcl * a.cap + q], dfc = tl.dfc[rcl * a.cap + q];
        const int aid = re.meta >> 8;
        if (aid > 0) {
          const T ids = atom_id<T>(a.ext, a.next, aid, i) * atom_id<T>(a.ext, a.next, aid, tl.pj[q]);
          fc *= ids;
          dfc *= ids;
        }
        const int ty = re.meta & 15;
        T dg;
        if (ty == 1) {
          dg = dfc;
        } else if (ty == 2) {
          const T x = r - re.p0, eta = re.p1;
          dg = m_exp<T>(-(eta * (x * x))) * (dfc - (T)2 * eta * x * fc);
        } else {
          const T kr = re.p0 * r;
          dg = m_cos<T>(kr) * dfc - re.p0 * m_sin<T>(kr) * fc;
        }
        return tl.jv[re.out] * dg;
      };
      T ds0 = 0, ds1 = 0;
      const int nseg = code < a.nz ? 2 : 1;
      for (int sg = 0; sg < nseg; sg++) {
        const int g0 = sg == 0 ? 0 : a.rad_seg[code + 1];
        const int g1 = sg == 0 ? a.rad_seg[1] : a.rad_seg[code + 2];
        int g = g0;
        for (; g + 2 <= g1; g += 2) {
          ds0 += dterm(g);
          ds1 += dterm(g + 1);
        }
        if (g < g1) ds0 += dterm(g);
      }
      const T dsum = ds0 + ds1;
      const V4<T> u = tl.u[q];
      tl.w[q].x += dsum * u.x;
      tl.w[q].y += dsum * u.y;
      tl.w[q].z += dsum * u.z;
    }
    // ---- integer-xi G5 through adjoint moments
    if (D > 0 && a.ncombo > 0) {
      constexpr int NM = n_mono_of(D > 0 ? D : 1);
      // cached moments arrived with the dE/dG row; otherwise they are formed here
      if (!a.mom_cached) compute_moments<T, (D > 0 ? D : 1)>(a, tl, np, lane);
      // Adjoint moments, factorised: coef_f(alpha) = mult(alpha) pc_f(|alpha|), so for every
      // partner group g (combo k receiving M of combo ko through functions F_g)
      //   h_g(m) = sum_{f in F_g} J_out(f) pc_f(m),
      //   Qc[z][e](alpha) = mult(alpha) sum_{k in {list z, all atoms}} sum_{g of k}
      //                     h_g(|alpha|) M_{ko(g)}(alpha).
      const int32_t *qg_ko = s_qg + a.ncombo + 1;
      const int32_t *qg_eoff = qg_ko + a.nqg, *qg_out = qg_eoff + a.nqg + 1;
      const int32_t *row_off = qg_out + a.nqg_ent, *row_term = row_off + (a.nz + 1) * a.necls + 1;
      T *H = tl.Q;
      // h_g(m) with lanes over groups: an entry's dE/dG weight read once for every degree
      for (int g = lane; g < a.nqg; g += 32) {
        T h[KD];
#pragma unroll
        for (int m = 0; m < KD; m++) h[m] = 0;
        const int e1 = qg_eoff[g + 1];
#pragma unroll 2
        for (int e = qg_eoff[g]; e < e1; e++) {
          const T jw = tl.jv[qg_out[e]];
#pragma unroll
          for (int m = 0; m < KD; m++) h[m] += jw * s_mpc[e * KD + m];
        }
#pragma unroll
        for (int m = 0; m < KD; m++) H[g * KD + m] = h[m];
      }
      __syncwarp();
      // Qc rows from their flat term lists (partner group g, partner combo ko); this lane's
      // monomials lane and lane + 32 (degree and weight fixed per kernel)
      const int nrows = (a.nz + 1) * a.necls;
      for (int r = 0; r < nrows; r++) {
        T v0 = 0, v1 = 0;
        const int t1 = row_off[r + 1];
        for (int t = row_off[r]; t < t1; t++) {
          const int tg = row_term[t];
          const T *Mk = tl.M + (tg >> 16) * NM;
          const T *Hg = H + (tg & 0xffff) * KD;
          if (lane < NM) v0 += Hg[mdeg0] * Mk[lane];
          if (lane + 32 < NM) v1 += Hg[mdeg1] * Mk[lane + 32];
        }
        T *dst = tl.Qc + (int64_t)r * NM;
        if (lane < NM) dst[lane] = mmult0 * v0;
        if (lane + 32 < NM) dst[lane + 32] = mmult1 * v1;
      }
      __syncwarp();
      constexpr int DD = D > 0 ? D : 1;
      switch (a.necls) {
        case 1: moment_pairs<T, DD, 1>(a, tl, np, lane, i); break;
        case 2: moment_pairs<T, DD, 2>(a, tl, np, lane, i); break;
        case 3: moment_pairs<T, DD, 3>(a, tl, np, lane, i); break;
        case 4: moment_pairs<T, DD, 4>(a, tl, np, lane, i); break;
        default: moment_pairs<T, DD, 0>(a, tl, np, lane, i); break;
      }
    }
    __syncwarp();
    // ---- remaining angular groups (triplet sweep)
    for (int gi = 0; gi < a.ngroups; gi++) {
      const AGroup G = a.groups[gi];
      __syncwarp();
      if (lane < G.count) {
        const GDesc d = a.ang[G.first + lane];
        const T *P = a.angp + 8 * (G.first + lane);
        tl.gpar[lane] = P[4];
        tl.gpar[32 + lane] = P[5];
        tl.gpar[64 + lane] = P[3];
        tl.gpar[96 + lane] = tl.jv[d.out] * P[6];
        tl.gint[lane] = d.xi_int;
        tl.gint[32 + lane] = d.eclass;
        tl.gint[64 + lane] = d.type;
        if (lane == 0) tl.gpar[128] = P[0];
      }
      if (G.has_g4 && G.atomid > 0)
        for (int q = lane; q < np; q += 32) tl.idv[q] = atom_id<T>(a.ext, a.next, G.atomid, tl.pj[q]);
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
    // ---- scatter: F_j -= w_p, F_i += sum_p w_p (self images cancel).  A lane sums its own
    // pairs (two or three) in T and the warp sums the lanes.  FP32: one vector atomic per pair
    // into the float4 accumulators; FP64: three FP64 atomics.
    T lx = 0, ly = 0, lz = 0;
    for (int q = lane; q < np; q += 32) {
      if ((tl.info[q] >> 8) & 1u) continue;
      const V4<T> w = tl.w[q];
      const int64_t j = tl.pj[q];
      if (!FNETG_GUARD(j >= 0 && j < a.natoms)) continue;
      if constexpr (sizeof(T) == 4) {
        atomicAdd(a.F4 + j * a.nout + a.out_index, make_float4(-w.x, -w.y, -w.z, 0.f));
      } else {
        double *Fj = a.F + (j * a.nout + a.out_index) * 3;
        atomicAdd(Fj + 0, -(double)w.x);
        atomicAdd(Fj + 1, -(double)w.y);
        atomicAdd(Fj + 2, -(double)w.z);
      }
      lx += w.x;
      ly += w.y;
      lz += w.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lx += __shfl_xor_sync(0xffffffffu, lx, o);
      ly += __shfl_xor_sync(0xffffffffu, ly, o);
      lz += __shfl_xor_sync(0xffffffffu, lz, o);
    }
    if (lane == 0) {
      if constexpr (sizeof(T) == 4) {
        atomicAdd(a.F4 + i * a.nout + a.out_index, make_float4(lx, ly, lz, 0.f));
      } else {
        double *Fi = a.F + (i * a.nout + a.out_index) * 3;
        atomicAdd(Fi + 0, (double)lx);
        atomicAdd(Fi + 1, (double)ly);
        atomicAdd(Fi + 2, (double)lz);
      }
    }
    __syncwarp();
  }
}

template <typename T> void fill_tile_args_forces(fnetg_ctx *ctx, TileArgs<T> &a) {
  a = TileArgs<T>{};
  a.natoms = ctx->N;
  a.poff = ctx->d_poff.as<int64_t>();
  a.pend = pair_end(ctx);
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = static_cast<const V4<T> *>(ctx->d_rij.p);
  a.code = ctx->d_code.as<int8_t>();
  a.bpos = ctx->d_bpos.as<int32_t>();
  a.ext = ctx->d_ext.as<double>();
  a.next = ctx->next;
  a.rad = ctx->d_rad.as<GDesc>();
  a.nrad = (int)ctx->h_rad.size();
  for (int c = 0; c < kMaxSpeciesCodes + 2; c++)
    a.rad_seg[c] = c < (int)ctx->rad_seg.size() ? ctx->rad_seg[c] : 0;
  a.ang = ctx->d_ang.as<GDesc>();
  const bool dbl = sizeof(T) == 8;
  a.radp = static_cast<const T *>(dbl ? ctx->d_radpar_d.p : ctx->d_radpar_f.p);
  a.angp = static_cast<const T *>(dbl ? ctx->d_angpar_d.p : ctx->d_angpar_f.p);
  a.groups = ctx->d_groups.as<AGroup>();
  a.ngroups = (int)ctx->h_groups.size();
  fill_class_tables<T>(ctx, a);
  a.nz = (int)ctx->zcodes.size();
  a.cap = std::max(32, (ctx->max_pairs + 31) / 32 * 32);
  a.mfunc = ctx->d_mfunc.as<MFunc>();
  a.nmf = (int)ctx->h_mfunc.size();
  a.qg = ctx->d_qgroups.as<int32_t>();
  a.nqg = ctx->n_qgroups;
  a.nqg_pack = ctx->n_qgpack;
  a.nqg_ent = ctx->n_qgent;
  a.rad_fast = ctx->rad_fast;
  a.mpc = static_cast<const T *>(dbl ? ctx->d_mpc_d.p : ctx->d_mpc_f.p);
  a.combo = ctx->d_combo.as<int32_t>();
  a.ncombo = ctx->n_combo;
  a.cidx = ctx->d_cidx.as<int32_t>();
  a.n_mono = ctx->n_mono;
  a.nf = ctx->nf;
  a.ng = (int)ctx->gf.size();
}

// FP32 force accumulators [N][nout] (float4) into the FP64 force array [N][nout][3]
__global__ void forces4_to_f64_kernel(const float4 *f4, double *F, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 v = f4[k];
  F[3 * k + 0] = (double)v.x;
  F[3 * k + 1] = (double)v.y;
  F[3 * k + 2] = (double)v.z;
}

template <typename T, int D> int launch_forces_d(fnetg_ctx *ctx, TileArgs<T> &a, int nout) {
  const int64_t N = ctx->N;
  const size_t tb = tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, a.ncombo, a.n_mono, a.ng, true, a.ngroups > 0,
                    tile_etab(a, true), tile_qwords(a));
  const size_t fixed = radtab_bytes<T>(a.nrad) + adjtab_bytes<T>(a);
  int wpb = 1, per_sm = 1;
  size_t smem = 0;
  const cudaError_t err =
      pick_warps(forces_kernel<T, D>, fixed, tb + radw_bytes<T>(a), wpb, smem, per_sm,
                 kForcesThreads<T> / 32);
  FNETG_CHECK(err != cudaErrorInvalidValue, FNETG_E_UNSUPPORTED,
              "neighbour tile of one atom exceeds shared memory");
  FNETG_CUDA(err);
  const int64_t want = (N + wpb - 1) / wpb;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>(want, (int64_t)num_sms() * per_sm * 8));
  for (int o = 0; o < nout; o++) {
    if (!(ctx->jac_ready && nout == 1)) {
      int rc = run_jacobian(ctx, o, ctx->d_jacT.p);
      if (rc) return rc;
    }
    a.out_index = o;
    LaunchScope ls(ctx, "forces");
    forces_kernel<T, D><<<blocks, wpb * 32, smem, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  if (sizeof(T) == 4) {
    const int64_t n = N * nout;
    LaunchScope ls(ctx, "forces_out");
    forces4_to_f64_kernel<<<(int)ceil_div(n, 256), 256, 0, ctx->stream>>>(
        ctx->d_forces4.as<float4>(), ctx->d_forces.as<double>(), n);
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

template <typename T> int launch_forces(fnetg_ctx *ctx) {
  const int64_t N = ctx->N;
  const int nout = ctx->dims.back();
  const int nf = ctx->nf;
  FNETG_CUDA(ctx->d_forces.ensure(sizeof(double) * std::max<int64_t>(N, 1) * nout * 3));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_forces.p, 0, sizeof(double) * std::max<int64_t>(N, 1) * nout * 3,
                             ctx->stream));
  FNETG_CUDA(ctx->d_jacT.ensure(sizeof(T) * std::max<int64_t>(N, 1) * nf));
  if (N == 0) return FNETG_OK;
  TileArgs<T> a;
  fill_tile_args_forces<T>(ctx, a);
  a.J = ctx->d_jacT.as<T>();
  a.F = ctx->d_forces.as<double>();
  if (sizeof(T) == 4) {
    FNETG_CUDA(ctx->d_forces4.ensure(sizeof(float4) * (size_t)N * nout));
    FNETG_CUDA(cudaMemsetAsync(ctx->d_forces4.p, 0, sizeof(float4) * (size_t)N * nout, ctx->stream));
    a.F4 = ctx->d_forces4.as<float4>();
  }
  if (ctx->mom_valid) {
    a.mom = ctx->d_mom.as<T>();
    a.mom_cached = 1;
  }
  a.nout = nout;
  switch (ctx->mom_degree) {
    case 0: return launch_forces_d<T, 0>(ctx, a, nout);
    case 1: return launch_forces_d<T, 1>(ctx, a, nout);
    case 2: return launch_forces_d<T, 2>(ctx, a, nout);
    case 3: return launch_forces_d<T, 3>(ctx, a, nout);
    default: return launch_forces_d<T, 4>(ctx, a, nout);
  }
}

}  // namespace

int run_forces(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? launch_forces<double>(ctx) : launch_forces<float>(ctx);
}

FNETG_CHECK_READER(check_site_forces)

}  // namespace fnetg
