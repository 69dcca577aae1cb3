// K2/K3: ACSF values G1..G5 (lib_descriptors/acsf.F90:1287-1492 driven by iGeoAcsf
// 797-866) and K5: z-score statistics / standardisation (acsf.F90:445-511).
//
// One warp per centre atom over the shared neighbour tile (tile.cuh).  Radial functions run
// lanes-over-functions, each lane summing one function over its species list in list order.
// G5 functions with an integer xi <= 4 use the moment form
//   sum_{j,k} (1 + lambda cos t_jk)^xi E_j E_k
//     = sum_{m <= xi} C(xi, m) lambda^m sum_{|alpha| = m} m!/alpha! M1(alpha) M2(alpha),
// an exact identity (cos t_jk = u_j . u_k) that turns the O(N_nb^2) triplet sum of g5
// (acsf.F90:1480-1488) into O(N_nb) moments.  G4 and other xi run a lanes-over-triplets sweep
// for a group of up to 32 functions sharing two lists, with exp(-eta r^2) fc(r) tabulated per
// pair and eta class.
#define FNETG_FILE_CODE 2  // site codes of the bounds-checked build
#include <algorithm>

#include "tile.cuh"

namespace fnetg {

namespace {

// Per-CTA copy of the radial descriptors in shape order: parameters (kappa, rs, -eta log2 e)
// and (list-channel bit, cutoff class, atom id, type | output column << 8).  The channel bit
// is 1 << species code, or bit 31 for the all-atom list.
template <typename T> struct RadDesc {
  V4<T> p;
  int4 m;
};

template <typename T> __host__ __device__ inline size_t raddesc_bytes(int nrad) {
  return (sizeof(RadDesc<T>) * (size_t)nrad + 127) / 128 * 128;
}

constexpr int kKD = kMaxMomentDegree + 1;

// Per-CTA tables of the factorised G5 evaluation: combo pairs (int2), functions (pair, output
// column) and degree coefficients pc_f(m).
template <typename T> __host__ __device__ inline size_t g5tab_bytes(const TileArgs<T> &a) {
  if (a.nmf <= 0) return 0;
  const size_t b = sizeof(int32_t) * 2 * (size_t)(a.nmpair + a.nmf) +
                   sizeof(T) * (size_t)a.nmf * kKD;
  return (b + 127) / 128 * 128;
}

// per-warp degree sums S_p(m) = sum_{|alpha| = m} mult(alpha) M_k1(alpha) M_k2(alpha)
template <typename T> __host__ __device__ inline size_t g5sum_bytes(const TileArgs<T> &a) {
  return a.nmf > 0 ? (sizeof(T) * (size_t)a.nmpair * kKD + 127) / 128 * 128 : 0;
}

template <typename T> struct RvDesc {
  T rs, c2;       // rs, -eta log2 e
  uint32_t bits;  // list-channel bit
};

// List-channel bits of tile pair q: its species and the all-atom list; every list for a self
// image; none for lanes past the end.
template <typename T>
__device__ __forceinline__ uint32_t pair_channels(const Tile<T> &t, int q, bool live) {
  const uint32_t inf = t.info[q];
  const int code = (int)(inf & 0xff);
  return !live ? 0u
         : ((inf >> 8) & 1u) ? kRvAllChannels
                             : (0x80000000u | (code < kMaxSpeciesCodes ? 1u << code : 0u));
}

// One batch of up to 32 radial G2 functions (one cutoff class, no atom ids), lanes over pairs,
// each function evaluated per pair without branches and added where its list holds the pair.
// A transposing butterfly returns function f's sum on lane f.
template <typename T, typename Desc>
__device__ __forceinline__ T radial_batch(const Tile<T> &t, const T *fcr, int np, int nb, int lane,
                                          Desc desc) {
  T acc[32];
#pragma unroll
  for (int f = 0; f < 32; f++) acc[f] = 0;
  for (int q0 = 0; q0 < np; q0 += 32) {
    const int q = q0 + lane;
    const bool live = q < np;
    const int qq = live ? q : q0;
    const uint32_t cm = pair_channels<T>(t, qq, live);
    const T r = t.u[qq].w;
    const T fc = fcr[qq];
#pragma unroll
    for (int f = 0; f < 32; f++) {
      if (f < nb) {
        const RvDesc<T> d = desc(f);
        const T x = r - d.rs;
        const T v = m_exp2<T>(d.c2 * (x * x)) * fc;
        if (cm & d.bits) acc[f] += v;
      }
    }
  }
  return transpose_reduce32<T>(acc, lane);
}

// The grid form of the radial G2 set: every shape (rs, eta) on the same rv_nc list channels
// (the species expansion of the reference's radial functions), output column of (shape sh,
// channel c) at rv_out[sh * rv_nc + c].  Walked list by list: for channel c, lane (group g,
// slot s) sums shapes g SPG .. g SPG + SPG - 1 over the channel list's pairs s, s + S, ...
// (S slots, 32 / S groups); a transposing butterfly over the slots leaves shape g SPG + s on
// lane (g, s).  Each (pair, shape) term of a channel is evaluated once and added without
// predication, and the per-lane shape parameters stay in registers.  Needs
// rv_nshape <= 32 / S x SPG.
template <typename T, int S, int SPG>
__device__ __forceinline__ void radial_lists(const TileArgs<T> &a, const Tile<T> &t, const T *fcr,
                                             int np, int lane, int64_t row) {
  constexpr int C = (SPG + S - 1) / S;
  constexpr int V = C * S;
  const int grp = lane / S, slot = lane % S;
  const int nc = a.rv_nc, ns = a.rv_nshape;
  T rs[SPG], c2[SPG];
#pragma unroll
  for (int k = 0; k < SPG; k++) {
    const int sh = min(grp * SPG + k, ns - 1);  // lanes past the last shape repeat it, unused
    rs[k] = a.rv_rs[sh];
    c2[k] = a.rv_c2[sh];
  }
  for (int c = 0; c < nc; c++) {
    const uint32_t bits = a.rv_chan[c];
    const bool all = bits == 0x80000000u;  // the all-atom list: every pair of the tile
    const int z = all ? 0 : __ffs((int)bits) - 1;
    const uint16_t *lst = all ? nullptr : t.lists + z * a.cap;
    const int n = all ? np : t.cnt[z];
    T acc[V];
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = 0;
    for (int k = slot; k < n; k += S) {
      const int q = lst ? lst[k] : k;
      const T r = t.u[q].w;
      const T fc = fcr[q];
#pragma unroll
      for (int kk = 0; kk < SPG; kk++) {
        const T x = r - rs[kk];
        acc[kk] += m_exp2<T>(c2[kk] * (x * x)) * fc;
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
      }
    }
#pragma unroll
    for (int cc = 0; cc < C; cc++) {
      const int k = slot * C + cc, shp = grp * SPG + k;
      if (k < SPG && shp < ns)
        a.feat[row * a.nf + a.rv_out[shp * nc + c]] = acc[cc];
    }
  }
}

template <typename T, int D>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1)
    acsf_kernel(const __grid_constant__ TileArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const size_t tb =
      tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, a.ncombo, a.n_mono, a.ng, false, a.ngroups > 0,
                    tile_etab(a, false));
  RadDesc<T> *rd = reinterpret_cast<RadDesc<T> *>(smem);
  for (int g = threadIdx.x; g < a.nrad; g += blockDim.x) {
    const int src = a.radv[g];
    const GDesc d = a.rad[src];
    const T *P = a.radp + 8 * src;
    const uint32_t bits = d.chan1 < 0 ? 0x80000000u : (1u << d.chan1);
    rd[g] = RadDesc<T>{V4<T>{P[1], P[2], -P[3] * (T)kLog2e, (T)0},
                       make_int4((int)bits, d.rclass, d.atomid, d.type | (d.out << 8))};
  }
  // int2 tables first (8-byte aligned from the 128-byte aligned start), then the T tables
  unsigned char *g5 = smem + raddesc_bytes<T>(a.nrad);
  int2 *s_pair = reinterpret_cast<int2 *>(g5);
  int2 *s_mf = s_pair + a.nmpair;
  T *s_fpc = reinterpret_cast<T *>(s_mf + a.nmf);
  if (D > 0 && a.nmf > 0) {
    for (int t2 = threadIdx.x; t2 < a.nmf * kKD; t2 += blockDim.x) s_fpc[t2] = a.fpc[t2];
    for (int t2 = threadIdx.x; t2 < a.nmpair; t2 += blockDim.x)
      s_pair[t2] = make_int2(a.mpair[2 * t2], a.mpair[2 * t2 + 1]);
    for (int t2 = threadIdx.x; t2 < a.nmf; t2 += blockDim.x)
      s_mf[t2] = make_int2(a.mfunc[t2].pair, a.mfunc[t2].out);
  }
  __syncthreads();
  const size_t fixed = raddesc_bytes<T>(a.nrad) + g5tab_bytes<T>(a);
  unsigned char *mine = smem + fixed + (tb + g5sum_bytes<T>(a)) * warp;
  Tile<T> t = carve_tile<T>(mine, a, false);
  T *S = reinterpret_cast<T *>(mine + tb);
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < a.natoms; i += (int64_t)gridDim.x * wpb) {
    const int64_t p0 = a.poff[i];
    const int np = (int)(a.pend[i] - p0);
    const int64_t row = a.bpos[i];
    if (!FNETG_GUARD(np >= 0 && np <= a.cap && row >= 0 && row < a.natoms)) continue;
    // the next atom of this warp: its pair range requested now, its records prefetched into
    // L2 once the range has arrived (after the staging)
    const int64_t inext = i + (int64_t)gridDim.x * wpb;
    int64_t nx0 = 0, nx1 = 0;
    if (inext < a.natoms) {
      nx0 = a.poff[inext];
      nx1 = a.pend[inext];
    }
    stage_tile<T>(a, t, i, p0, np, lane, false);
    prefetch_pairs<T>(a, nx0, nx1, lane);
    if (D > 0 && a.ncombo > 0) {
      compute_moments<T, (D > 0 ? D : 1)>(a, t, np, lane);
      if (a.mom) {
        const int nm = a.ncombo * a.n_mono;
        T *dst = a.mom + i * nm;
        for (int k = lane; k < nm; k += 32) dst[k] = t.M[k];
      }
    }
    if (a.rad_fast >= 0) {
      // ---- radial functions, all G2 of one cutoff class without atom ids: lanes over pairs,
      // the functions in batches of 32 (radial_batch); descriptors from the kernel parameters
      // when they fit there, else from the per-CTA table
      const T *fcr = t.fc + a.rad_fast * a.cap;
      if (a.rv_nc > 0 && a.rv_nshape <= 12) {
        radial_lists<T, 8, 3>(a, t, fcr, np, lane, row);
      } else if (a.rv_nc > 0 && a.rv_nshape <= 24) {
        radial_lists<T, 4, 3>(a, t, fcr, np, lane, row);
      } else if (a.rv_nc > 0) {
        radial_lists<T, 4, 4>(a, t, fcr, np, lane, row);
      } else if (a.rv_param) {
#pragma unroll 1
        for (int b = 0; b < kRadParam / 32; b++) {
          if (b * 32 < a.nrad) {
            const int nb = min(32, a.nrad - b * 32);
            const T tot = radial_batch<T>(t, fcr, np, nb, lane, [&](int f) {
              return RvDesc<T>{a.rv_rs[b * 32 + f], a.rv_c2[b * 32 + f], a.rv_bits[b * 32 + f]};
            });
            if (lane < nb) a.feat[row * a.nf + a.rv_out[b * 32 + lane]] = tot;
          }
        }
      } else {
        for (int b0 = 0; b0 < a.nrad; b0 += 32) {
          const int nb = min(32, a.nrad - b0);
          const RadDesc<T> *rb = rd + b0;
          const T tot = radial_batch<T>(t, fcr, np, nb, lane, [&](int f) {
            return RvDesc<T>{rb[f].p.y, rb[f].p.z, (uint32_t)rb[f].m.x};
          });
          if (lane < nb) a.feat[row * a.nf + (rb[lane].m.w >> 8)] = tot;
        }
      }
    } else {
      // ---- radial functions, general: items (function, part) over lanes; a function's list
      // is split into rad_split contiguous parts on adjacent lanes (full lanes when the
      // function count is not a multiple of 32), each part walked with four independent
      // partial sums, the parts combined by shuffles.  The cutoff table is zero outside a
      // function's class.
      const int S = a.rad_split;
      const int sh = S == 4 ? 2 : (S == 2 ? 1 : 0);  // S is a power of two: no divisions
      const int items = a.nrad * S;
      for (int base = 0; base < items; base += 32) {
        const int it = base + lane;
        const int g = it >> sh, part = it - (g << sh);
        T acc = 0;
        if (it < items) {
          const RadDesc<T> rdg = rd[g];
          const T kappa = rdg.p.x, rs = rdg.p.y, c2 = rdg.p.z;
          const uint32_t fbit = (uint32_t)rdg.m.x;
          const int chan1 = fbit == 0x80000000u ? -1 : __ffs((int)fbit) - 1;
          const int rclass = rdg.m.y, atomid = rdg.m.z, type = rdg.m.w & 15;
          const uint16_t *lst = chan1 >= 0 ? t.lists + chan1 * a.cap : nullptr;
          const int n = chan1 >= 0 ? t.cnt[chan1] : np;
          const int chunk = (((n + S - 1) >> sh) + 3) & ~3;
          const int k0 = min(n, part * chunk), k1 = min(n, k0 + chunk);
          const T *fcr = t.fc + rclass * a.cap;
          const T idi = atom_id<T>(a.ext, a.next, atomid, i);
          auto term = [&](int q) -> T {
            const T r = t.u[q].w;
            T fc = fcr[q];
            if (atomid > 0) fc *= idi * atom_id<T>(a.ext, a.next, atomid, t.pj[q]);
            if (type == 1) return fc;
            if (type == 2) {
              const T x = r - rs;
              return m_exp2<T>(c2 * (x * x)) * fc;
            }
            return m_cos<T>(kappa * r) * fc;
          };
          T acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
          int k = k0;
          for (; k + 4 <= k1; k += 4) {
            int q0 = k, q1 = k + 1, q2 = k + 2, q3 = k + 3;
            if (lst) {
              const uint2 w = *reinterpret_cast<const uint2 *>(lst + k);
              q0 = (int)(w.x & 0xffffu);
              q1 = (int)(w.x >> 16);
              q2 = (int)(w.y & 0xffffu);
              q3 = (int)(w.y >> 16);
            }
            acc0 += term(q0);
            acc1 += term(q1);
            acc2 += term(q2);
            acc3 += term(q3);
          }
          for (; k < k1; k++) acc0 += term(lst ? lst[k] : k);
          acc = (acc0 + acc1) + (acc2 + acc3);
        }
        for (int o = 1; o < S; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (it < items && part == 0) a.feat[row * a.nf + (rd[g].m.w >> 8)] = acc;
      }
    }
    // ---- integer-xi G5 through moments, factorised: coef_f(alpha) = mult(alpha) pc_f(|alpha|),
    // so G_f = sum_m pc_f(m) S_p(m) with the degree sums S_p of the function's combo pair
    if (D > 0 && a.nmf > 0) {
      // one combo pair per lane: its monomials unrolled, each added to its degree's sum with
      // the multinomial weight as a constant (the same order within a degree as a loop over
      // the degree's monomials)
      constexpr int NM = n_mono_of(D > 0 ? D : 1);
      for (int p = lane; p < a.nmpair; p += 32) {
        const int2 kk = s_pair[p];
        const T *M1 = t.M + kk.x * NM, *M2 = t.M + kk.y * NM;
        T sm[kKD];
#pragma unroll
        for (int m = 0; m < kKD; m++) sm[m] = 0;
#pragma unroll
        for (int al = 0; al < NM; al++)
          sm[kMonoTab[al][0] + kMonoTab[al][1] + kMonoTab[al][2]] +=
              (T)kMonoMult[al] * (M1[al] * M2[al]);
#pragma unroll
        for (int m = 0; m < kKD; m++) S[p * kKD + m] = sm[m];
      }
      __syncwarp();
      for (int f = lane; f < a.nmf; f += 32) {
        const int2 mf = s_mf[f];
        const T *pc = s_fpc + f * kKD, *Sp = S + mf.x * kKD;
        T acc = 0;
#pragma unroll
        for (int m = 0; m < kKD; m++) acc += pc[m] * Sp[m];
        a.feat[row * a.nf + mf.y] = acc;
      }
    }
    // ---- remaining angular groups: lanes over triplets
    for (int gi = 0; gi < a.ngroups; gi++) {
      const AGroup G = a.groups[gi];
      __syncwarp();
      if (lane < G.count) {
        const GDesc d = a.ang[G.first + lane];
        const T *P = a.angp + 8 * (G.first + lane);
        t.gpar[lane] = P[4];
        t.gpar[32 + lane] = P[5];
        t.gpar[64 + lane] = P[3];
        t.gpar[96 + lane] = P[6];
        t.gint[lane] = d.xi_int;
        t.gint[32 + lane] = d.eclass;
        t.gint[64 + lane] = d.type;
        if (lane == 0) t.gpar[128] = P[0];
      }
      if (G.has_g4 && G.atomid > 0)
        for (int q = lane; q < np; q += 32) t.idv[q] = atom_id<T>(a.ext, a.next, G.atomid, t.pj[q]);
      __syncwarp();
      const uint16_t *l1 = G.chan1 >= 0 ? t.lists + G.chan1 * a.cap : nullptr;
      const uint16_t *l2 = G.chan2 >= 0 ? t.lists + G.chan2 * a.cap : nullptr;
      const int n1 = G.chan1 >= 0 ? t.cnt[G.chan1] : np;
      const int n2 = G.chan2 >= 0 ? t.cnt[G.chan2] : np;
      const int64_t ntrip = (int64_t)n1 * n2;
      T acc[kMaxGroupFuncs];
#pragma unroll
      for (int f = 0; f < kMaxGroupFuncs; f++) acc[f] = 0;
      const T rcut_g4 = t.gpar[128];
      if (n2 > 0) {
        const int dj = 32 / n2, dk = 32 % n2;
        int jj = lane / n2, kk = lane % n2;
        for (int64_t tr = lane; tr < ntrip; tr += 32) {
          const int p = l1 ? l1[jj] : jj;
          const int q = l2 ? l2[kk] : kk;
          const V4<T> vp = t.v[p], vq = t.v[q];
          const T dot = vp.x * vq.x + vp.y * vq.y + vp.z * vq.z;
          // theta of acsf.F90:1173-1174; cos(acos(x)) == x up to rounding, clamped to the
          // domain of acos
          T c = dot / (vp.w * vq.w + (T)1e-13);
          c = c > (T)1 ? (T)1 : (c < (T)-1 ? (T)-1 : c);
          // j = k: the reference's 1 - cos is ~1e-13 / r^2; float division lands a few ulp
          // off 1, which (1 - c)-type terms weighted by E_j^2 would turn into noise
          if (sizeof(T) == 4 && p == q) c = (T)1;
          T fjk = 1, rjk2 = 0;
          if (G.has_g4) {
            const T ex = vp.x - vq.x, ey = vp.y - vq.y, ez = vp.z - vq.z;
            rjk2 = ex * ex + ey * ey + ez * ez;
            const T rjk = m_sqrt<T>(rjk2);
            T fcv, dfv;
            cutoff_fc<T>(min(rjk, rcut_g4), rcut_g4, fcv, dfv);
            fjk = rjk > rcut_g4 ? (T)0 : fcv;
            if (G.atomid > 0) fjk *= t.idv[p] * t.idv[q];
          }
#pragma unroll
          for (int f = 0; f < kMaxGroupFuncs; f++) {
            if (f < G.count) {
              const T base = (T)1 + t.gpar[f] * c;
              const T ang = int_pow<T>(base, t.gint[f], t.gpar[32 + f]);
              const int e = t.gint[32 + f];
              T rad = t.E[e * a.cap + p] * t.E[e * a.cap + q];
              if (t.gint[64 + f] == 4) rad *= m_exp<T>(-(t.gpar[64 + f] * rjk2)) * fjk;
              acc[f] += ang * rad;
            }
          }
          jj += dj;
          kk += dk;
          if (kk >= n2) {
            kk -= n2;
            jj += 1;
          }
        }
      }
      T mine = 0;
#pragma unroll
      for (int f = 0; f < kMaxGroupFuncs; f++) {
        if (f < G.count) {
          const T s = warp_sum<T>(acc[f]);
          if (lane == f) mine = s;
        }
      }
      if (lane < G.count) {
        const GDesc d = a.ang[G.first + lane];
        a.feat[row * a.nf + d.out] = mine * t.gpar[96 + lane];
      }
    }
    __syncwarp();
  }
}

// ---- external network inputs gathered behind the ACSF columns --------------------------
template <typename T>
__global__ void ext_inputs_kernel(T *feat, int nf, int col0, const double *ext, int next,
                                  const int32_t *idx, int nidx, const int32_t *bpos, int64_t N) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * nidx) return;
  const int64_t a = t / nidx;
  const int k = (int)(t % nidx);
  feat[(int64_t)bpos[a] * nf + col0 + k] = (T)ext[a * next + idx[k] - 1];
}

// ---- z-score: per-CTA FP64 partial sums over atom chunks, deterministic final sums -----
template <typename T>
__global__ void zsum_kernel(const T *feat, int nf, int ng, const int32_t *bpos,
                            const int32_t *astruct, const int32_t *w, int64_t N,
                            const double *mean, double *part, int64_t chunk) {
  const int64_t a0 = (int64_t)blockIdx.x * chunk;
  const int64_t a1 = min(N, a0 + chunk);
  for (int f = threadIdx.x; f < ng; f += blockDim.x) {
    double acc = 0.0;
    for (int64_t a = a0; a < a1; a++) {
      const double wt = w ? (double)w[astruct[a]] : 1.0;
      const double x = (double)feat[(int64_t)bpos[a] * nf + f];
      if (mean) {
        const double d = x - mean[f];
        acc += wt * (d * d);
      } else {
        acc += wt * x;
      }
    }
    part[(int64_t)blockIdx.x * ng + f] = acc;
  }
}

__global__ void zfinish_kernel(const double *part, int nparts, int ng, double denom, double *out,
                               int is_std) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= ng) return;
  double acc = 0.0;
  for (int p = 0; p < nparts; p++) acc += part[(int64_t)p * ng + f];
  out[f] = is_std ? sqrt(acc / denom) : acc / denom;
}

// FP64 contexts: the reference's (x - mean) / sd in FP64 for bit-level parity
__global__ void zapply_kernel_d(double *feat, int nf, int ng, int64_t N, const double *zprec) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * ng) return;
  const int64_t r = t / ng;
  const int f = (int)(t % ng);
  const double sd = zprec[ng + f];
  if (sd < 1e-08) return;
  double *x = feat + r * nf + f;
  *x = (*x - zprec[f]) / sd;
}

// FP32 contexts: float mean and inverse deviation (zf[f], zf[ng + f]; inverse 0 = column
// left as it is), one row per thread group, all float arithmetic
__global__ void zapply_kernel_f(float *feat, int nf, int ng, int64_t N, const float *zf) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * ng) return;
  const int64_t r = t / ng;
  const int f = (int)(t - r * ng);
  const float inv = zf[ng + f];
  if (inv == 0.f) return;
  float *x = feat + r * nf + f;
  *x = (*x - zf[f]) * inv;
}

// The same on float4 groups of four columns (ng and nf multiples of four, fewer than 2^31
// groups): one 32-bit division per four features instead of a 64-bit one per feature.
__global__ void zapply_kernel_f4(float *feat, int nf4, int ng4, int n4, const float *zf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n4) return;
  const int r = t / ng4;
  const int c = t - r * ng4;
  const float4 mu = reinterpret_cast<const float4 *>(zf)[c];
  const float4 inv = reinterpret_cast<const float4 *>(zf + 4 * ng4)[c];
  float4 *x = reinterpret_cast<float4 *>(feat) + (int64_t)r * nf4 + c;
  float4 v = *x;
  if (inv.x != 0.f) v.x = (v.x - mu.x) * inv.x;
  if (inv.y != 0.f) v.y = (v.y - mu.y) * inv.y;
  if (inv.z != 0.f) v.z = (v.z - mu.z) * inv.z;
  if (inv.w != 0.f) v.w = (v.w - mu.w) * inv.w;
  *x = v;
}

// float copies of the statistics for the FP32 kernels
__global__ void zfloat_kernel(const double *zprec, int ng, float *zf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= ng) return;
  const double sd = zprec[ng + f];
  zf[f] = (float)zprec[f];
  zf[ng + f] = sd < 1e-08 ? 0.f : (float)(1.0 / sd);
}

template <typename T> void fill_tile_args(fnetg_ctx *ctx, TileArgs<T> &a) {
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
  a.radv = ctx->d_radv.as<int32_t>();
  a.rad_fast = ctx->rad_fast;
  a.nrad = (int)ctx->h_rad.size();
  a.rv_param = a.rv_nc = a.rv_nshape = 0;
  if (ctx->rad_fast >= 0 && a.nrad <= kRadParam) {
    a.rv_param = 1;
    auto chanbit = [](const GDesc &d) { return d.chan1 < 0 ? 0x80000000u : (1u << d.chan1); };
    for (int g = 0; g < a.nrad; g++) {
      const GDesc &d = ctx->h_rad[ctx->h_radv[g]];
      a.rv_rs[g] = (T)d.rs;
      a.rv_c2[g] = -(T)d.eta * (T)kLog2e;
      a.rv_bits[g] = chanbit(d);
      a.rv_out[g] = d.out;
    }
    // grid form: the first shape's channel run repeated, shape by shape, with distinct shapes;
    // at most 32 shapes (the list-by-list walk's lanes)
    int nc = 0;
    const GDesc &d0 = ctx->h_rad[ctx->h_radv[0]];
    while (nc < a.nrad && ctx->h_rad[ctx->h_radv[nc]].rs == d0.rs &&
           ctx->h_rad[ctx->h_radv[nc]].eta == d0.eta)
      nc++;
    bool grid = nc >= 1 && nc <= kMaxSpeciesCodes + 1 && a.nrad % nc == 0 && a.nrad / nc <= 32;
    for (int g = 0; grid && g < a.nrad; g++) {
      const GDesc &d = ctx->h_rad[ctx->h_radv[g]];
      const GDesc &h = ctx->h_rad[ctx->h_radv[g - g % nc]];  // the shape's first function
      grid = chanbit(d) == chanbit(ctx->h_rad[ctx->h_radv[g % nc]]) && d.rs == h.rs && d.eta == h.eta &&
             (g % nc != 0 || g == 0 ||
              d.rs != ctx->h_rad[ctx->h_radv[g - 1]].rs || d.eta != ctx->h_rad[ctx->h_radv[g - 1]].eta);
    }
    if (grid) {
      const int ns = a.nrad / nc;
      a.rv_nc = nc;
      a.rv_nshape = ns;
      T rs[kRadParam] = {}, c2[kRadParam] = {};
      int32_t out[kRadParam] = {};
      for (int sh = 0; sh < ns; sh++) {
        const GDesc &d = ctx->h_rad[ctx->h_radv[sh * nc]];
        rs[sh] = (T)d.rs;
        c2[sh] = -(T)d.eta * (T)kLog2e;
        for (int c = 0; c < nc; c++) out[sh * nc + c] = ctx->h_rad[ctx->h_radv[sh * nc + c]].out;
      }
      for (int g = 0; g < kRadParam; g++) {
        a.rv_rs[g] = rs[g];
        a.rv_c2[g] = c2[g];
        a.rv_out[g] = out[g];
      }
      for (int c = 0; c < nc; c++) a.rv_chan[c] = chanbit(ctx->h_rad[ctx->h_radv[c]]);
    }
  }
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
  a.mpair = ctx->d_mpair.as<int32_t>();
  a.nmpair = (int)ctx->h_mpair.size() / 2;
  a.fpc = static_cast<const T *>(sizeof(T) == 8 ? ctx->d_fpc_d.p : ctx->d_fpc_f.p);
  a.combo = ctx->d_combo.as<int32_t>();
  a.ncombo = ctx->n_combo;
  a.cidx = ctx->d_cidx.as<int32_t>();
  a.n_mono = ctx->n_mono;
  a.feat = ctx->d_feat.as<T>();
  a.nf = ctx->nf;
  a.ng = (int)ctx->gf.size();
}

template <typename T, int D> int launch_acsf_d(fnetg_ctx *ctx, TileArgs<T> &a) {
  const int64_t N = ctx->N;
  const size_t tb =
      tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz, a.ncombo, a.n_mono, a.ng, false, a.ngroups > 0,
                    tile_etab(a, false));
  int wpb = 1, per_sm = 1;
  size_t smem = 0;
  const cudaError_t err = pick_warps(acsf_kernel<T, D>, raddesc_bytes<T>(a.nrad) + g5tab_bytes<T>(a),
                                     tb + g5sum_bytes<T>(a), wpb, smem, per_sm);
  FNETG_CHECK(err != cudaErrorInvalidValue, FNETG_E_UNSUPPORTED,
              "neighbour tile of one atom exceeds shared memory");
  FNETG_CUDA(err);
  const int64_t want = (N + wpb - 1) / wpb;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>(want, (int64_t)num_sms() * per_sm * 8));
  LaunchScope ls(ctx, "acsf");
  acsf_kernel<T, D><<<blocks, wpb * 32, smem, ctx->stream>>>(a);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

template <typename T> int launch_acsf(fnetg_ctx *ctx) {
  const int64_t N = ctx->N;
  FNETG_CUDA(ctx->d_feat.ensure(sizeof(T) * std::max<int64_t>(N, 1) * std::max(ctx->nf, 1)));
  if (N == 0) return FNETG_OK;
  TileArgs<T> a;
  fill_tile_args<T>(ctx, a);
  FNETG_CHECK(a.cap <= 65535, FNETG_E_UNSUPPORTED, "more than 65535 neighbours of one atom");
  // general radial path: the split S in {1, 2, 4} with the fewest lane passes per list
  // element (ceil(nrad S / 32) / S, ties to the smaller S)
  a.rad_split = 1;
  for (int S = 2; S <= 4; S <<= 1)
    if ((double)ceil_div((int64_t)a.nrad * S, 32) / S <
        (double)ceil_div((int64_t)a.nrad * a.rad_split, 32) / a.rad_split)
      a.rad_split = S;
  if (a.ncombo > 0) {
    FNETG_CUDA(ctx->d_mom.ensure(sizeof(T) * (size_t)N * a.ncombo * a.n_mono));
    a.mom = ctx->d_mom.as<T>();
  }
  switch (ctx->mom_degree) {
    case 0: return launch_acsf_d<T, 0>(ctx, a);
    case 1: return launch_acsf_d<T, 1>(ctx, a);
    case 2: return launch_acsf_d<T, 2>(ctx, a);
    case 3: return launch_acsf_d<T, 3>(ctx, a);
    default: return launch_acsf_d<T, 4>(ctx, a);
  }
}

template <typename T> int launch_zscore(fnetg_ctx *ctx, const int32_t *weights, bool compute) {
  const int ng = (int)ctx->gf.size();
  const int nf = ctx->nf;
  const int64_t N = ctx->N;
  FNETG_CUDA(ctx->d_zprec.ensure(sizeof(double) * 2 * std::max(ng, 1)));
  double *z = ctx->d_zprec.as<double>();
  if (compute) {
    FNETG_CHECK(N > 0, FNETG_E_INVALID, "z-score of an empty dataset");
    int32_t *dw = nullptr;
    double denom = 0.0;
    if (weights) {
      FNETG_CUDA(ctx->d_w.ensure(sizeof(int32_t) * std::max(ctx->S, 1)));
      FNETG_CUDA(cudaMemcpyAsync(ctx->d_w.p, weights, sizeof(int32_t) * ctx->S,
                                 cudaMemcpyHostToDevice, ctx->stream));
      dw = ctx->d_w.as<int32_t>();
      for (int s = 0; s < ctx->S; s++)
        denom += (double)weights[s] * (double)(ctx->h_off[s + 1] - ctx->h_off[s]);
    } else {
      denom = (double)N;
    }
    FNETG_CHECK(denom > 0.0, FNETG_E_INVALID, "z-score: zero total weight");
    const int64_t chunk = 256;
    const int nparts = ceil_div(N, chunk);
    FNETG_CUDA(ctx->d_zpart.ensure(sizeof(double) * (size_t)nparts * ng));
    double *part = ctx->d_zpart.as<double>();
    const int thr = std::min(256, std::max(32, (ng + 31) / 32 * 32));
    {
      LaunchScope ls(ctx, "zscore");
      zsum_kernel<T><<<nparts, thr, 0, ctx->stream>>>(ctx->d_feat.as<T>(), nf, ng,
                                                       ctx->d_bpos.as<int32_t>(),
                                                       ctx->d_atom_struct.as<int32_t>(), dw, N,
                                                       nullptr, part, chunk);
    }
    {
      LaunchScope ls(ctx, "zscore");
      zfinish_kernel<<<ceil_div(ng, 128), 128, 0, ctx->stream>>>(part, nparts, ng, denom, z, 0);
    }
    {
      LaunchScope ls(ctx, "zscore");
      zsum_kernel<T><<<nparts, thr, 0, ctx->stream>>>(ctx->d_feat.as<T>(), nf, ng,
                                                       ctx->d_bpos.as<int32_t>(),
                                                       ctx->d_atom_struct.as<int32_t>(), dw, N, z,
                                                       part, chunk);
    }
    {
      LaunchScope ls(ctx, "zscore");
      zfinish_kernel<<<ceil_div(ng, 128), 128, 0, ctx->stream>>>(part, nparts, ng, denom, z + ng,
                                                                 1);
    }
    FNETG_CUDA(cudaGetLastError());
    ctx->h_zprec.resize(2 * ng);
    FNETG_CUDA(cudaMemcpyAsync(ctx->h_zprec.data(), z, sizeof(double) * 2 * ng,
                               cudaMemcpyDeviceToHost, ctx->stream));
    FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  } else {
    FNETG_CHECK((int)ctx->h_zprec.size() == 2 * ng, FNETG_E_SHAPE, "zprec size");
    FNETG_CUDA(cudaMemcpyAsync(z, ctx->h_zprec.data(), sizeof(double) * 2 * ng,
                               cudaMemcpyHostToDevice, ctx->stream));
  }
  if (ng > 0) {
    FNETG_CUDA(ctx->d_zprec_f.ensure(sizeof(float) * 2 * ng));
    LaunchScope ls(ctx, "zscore");
    zfloat_kernel<<<ceil_div(ng, 128), 128, 0, ctx->stream>>>(z, ng, ctx->d_zprec_f.as<float>());
    FNETG_CUDA(cudaGetLastError());
  }
  if (N > 0 && ng > 0) {
    LaunchScope ls(ctx, "zscore");
    if (sizeof(T) == 8)
      zapply_kernel_d<<<ceil_div(N * ng, 256), 256, 0, ctx->stream>>>(ctx->d_feat.as<double>(),
                                                                      nf, ng, N, z);
    else if (ng % 4 == 0 && nf % 4 == 0 && N * (ng / 4) < ((int64_t)1 << 31))
      zapply_kernel_f4<<<ceil_div(N * (ng / 4), 256), 256, 0, ctx->stream>>>(
          ctx->d_feat.as<float>(), nf / 4, ng / 4, (int)(N * (ng / 4)), ctx->d_zprec_f.as<float>());
    else
      zapply_kernel_f<<<ceil_div(N * ng, 256), 256, 0, ctx->stream>>>(
          ctx->d_feat.as<float>(), nf, ng, N, ctx->d_zprec_f.as<float>());
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
}

template <typename T> int launch_ext(fnetg_ctx *ctx) {
  const int nidx = (int)ctx->ext_idx.size();
  if (nidx == 0 || ctx->N == 0) return FNETG_OK;
  DBuf &idxbuf = ctx->d_extidx;
  FNETG_CUDA(idxbuf.ensure(sizeof(int32_t) * nidx));
  FNETG_CUDA(cudaMemcpyAsync(idxbuf.p, ctx->ext_idx.data(), sizeof(int32_t) * nidx,
                             cudaMemcpyHostToDevice, ctx->stream));
  LaunchScope ls(ctx, "ext_inputs");
  ext_inputs_kernel<T><<<ceil_div(ctx->N * nidx, 256), 256, 0, ctx->stream>>>(
      ctx->d_feat.as<T>(), ctx->nf, (int)ctx->gf.size(), ctx->d_ext.as<double>(), ctx->next,
      idxbuf.as<int32_t>(), nidx, ctx->d_bpos.as<int32_t>(), ctx->N);
  FNETG_CUDA(cudaGetLastError());
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FNETG_OK;
}

}  // namespace

int run_acsf(fnetg_ctx *ctx) {
  ctx->feat_gen++;
  ctx->nf = (int)ctx->gf.size() + (int)ctx->ext_idx.size();
  int rc = ctx->prec == FNETG_FP64 ? launch_acsf<double>(ctx) : launch_acsf<float>(ctx);
  if (rc) return rc;
  ctx->feats_valid = true;
  ctx->mom_valid = ctx->n_combo > 0 && ctx->N > 0;
  return FNETG_OK;
}

int run_ext_inputs(fnetg_ctx *ctx) {
  ctx->feat_gen++;
  return ctx->prec == FNETG_FP64 ? launch_ext<double>(ctx) : launch_ext<float>(ctx);
}

int run_zscore(fnetg_ctx *ctx, const int32_t *weights, bool compute) {
  ctx->feat_gen++;
  return ctx->prec == FNETG_FP64 ? launch_zscore<double>(ctx, weights, compute)
                                 : launch_zscore<float>(ctx, weights, compute);
}

FNETG_CHECK_READER(check_site_acsf)

}  // namespace fnetg
