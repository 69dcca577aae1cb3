// Per-atom neighbour tile shared by the ACSF value and force kernels.
//
// One warp owns one centre atom.  Its neighbour images are staged in shared memory once:
// displacement and distance, unit vector, neighbour index, species code / self-image flag /
// cutoff-class mask, the cutoff functions of every cutoff class and, per angular eta class,
// E(r) = exp(-eta r^2) fc(r) [id_i id_j] and (forces) dE/dr.  The per-species lists of
// buildGFunctionNeighborlists (lib_descriptors/acsf.F90:943-1066) become ordered index lists
// over the tile — the centre atom's periodic self-images belong to every species list, as in
// the reference's species-reduced geometries.  Moments M_k(alpha) = sum_{j in list} E_j u_j^alpha
// of every (list, eta class) combo feed the integer-xi G5 functions.
#pragma once

#include <algorithm>

#include "internal.cuh"

namespace fnetg {

constexpr double kPi = 3.14159265358979323846;  // lib_dftbp/constants.F90:15

// monomial exponents (x, y, z), ordered by degree then descending x and y exponents
__device__ constexpr int kMonoTab[kMaxMono][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0},
    {0, 1, 1}, {0, 0, 2}, {3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {1, 1, 1}, {1, 0, 2},
    {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}, {4, 0, 0}, {3, 1, 0}, {3, 0, 1}, {2, 2, 0},
    {2, 1, 1}, {2, 0, 2}, {1, 3, 0}, {1, 2, 1}, {1, 1, 2}, {1, 0, 3}, {0, 4, 0}, {0, 3, 1},
    {0, 2, 2}, {0, 1, 3}, {0, 0, 4}};

__host__ __device__ constexpr int n_mono_of(int D) { return (D + 1) * (D + 2) * (D + 3) / 6; }

// multinomial weights m! / (a! b! c!) of the monomials above
__device__ constexpr int kMonoMult[kMaxMono] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 1, 1, 3, 3, 3, 6, 3, 1, 3,
                                                3, 1, 1, 4, 4, 6, 12, 6, 4, 12, 12, 4, 1, 4, 6, 4, 1};
constexpr int mono_fact(int n) { return n <= 1 ? 1 : n * mono_fact(n - 1); }
constexpr bool mono_mult_table_ok() {
  for (int al = 0; al < kMaxMono; al++) {
    const int a = kMonoTab[al][0], b = kMonoTab[al][1], c = kMonoTab[al][2];
    if (kMonoMult[al] * mono_fact(a) * mono_fact(b) * mono_fact(c) != mono_fact(a + b + c))
      return false;
  }
  return true;
}
static_assert(mono_mult_table_ok(), "multinomial table");

// Each monomial of degree >= 1 as its parent (one exponent lower) times one coordinate, the
// first of x, y, z with a nonzero exponent.
struct MonoLinks {
  int parent[kMaxMono];
  int axis[kMaxMono];
};
constexpr int mono_index(int a, int b, int c) {
  for (int al = 0; al < kMaxMono; al++)
    if (kMonoTab[al][0] == a && kMonoTab[al][1] == b && kMonoTab[al][2] == c) return al;
  return -1;
}
constexpr MonoLinks make_mono_links() {
  MonoLinks l{};
  for (int al = 1; al < kMaxMono; al++) {
    const int a = kMonoTab[al][0], b = kMonoTab[al][1], c = kMonoTab[al][2];
    l.axis[al] = a > 0 ? 0 : (b > 0 ? 1 : 2);
    l.parent[al] = a > 0 ? mono_index(a - 1, b, c) : (b > 0 ? mono_index(a, b - 1, c) : mono_index(a, b, c - 1));
  }
  return l;
}
__device__ constexpr MonoLinks kMonoLinks = make_mono_links();

// Each monomial's derivative partner per coordinate: the index of alpha - e_axis, -1 when that
// exponent is zero (d/dx u^alpha = a u^(alpha - e_x)).
struct MonoDown {
  int idx[kMaxMono][3];
};
constexpr MonoDown make_mono_down() {
  MonoDown d{};
  for (int al = 0; al < kMaxMono; al++) {
    const int a = kMonoTab[al][0], b = kMonoTab[al][1], c = kMonoTab[al][2];
    d.idx[al][0] = a > 0 ? mono_index(a - 1, b, c) : -1;
    d.idx[al][1] = b > 0 ? mono_index(a, b - 1, c) : -1;
    d.idx[al][2] = c > 0 ? mono_index(a, b, c - 1) : -1;
  }
  return d;
}
__device__ constexpr MonoDown kMonoDown = make_mono_down();
constexpr bool mono_links_ok() {
  const MonoLinks l = make_mono_links();
  for (int al = 1; al < kMaxMono; al++)
    if (l.parent[al] < 0 || l.parent[al] >= al) return false;
  return true;
}
static_assert(mono_links_ok(), "monomial parents precede their children");

// Float exp through the hardware base-2 exponential: exp(x) = 2^(x log2 e) with the product
// x log2 e carried as hi + lo (log2 e split into a float head and tail, the rounding of x * head
// recovered by an FMA), ex2.approx on hi and the first-order factor 1 + lo ln 2 for the tail.
// Inputs below -87.3 flush to zero (ftz), as the FP32 kernels need for exp(-eta r^2).
__device__ __forceinline__ float exp_ex2(float x) {
  constexpr float kL2eHi = 1.44269502162933349609375f;  // log2 e rounded to float
  constexpr float kL2eLo = 1.925963033500011e-08f;      // log2 e - kL2eHi
  const float hi = x * kL2eHi;
  const float lo = fmaf(x, kL2eLo, fmaf(x, kL2eHi, -hi));
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(hi));
  return fmaf(r * lo, 0.693147180559945309f, r);
}

template <typename T> __device__ __forceinline__ T m_exp(T x);
template <> __device__ __forceinline__ float m_exp<float>(float x) { return exp_ex2(x); }
template <> __device__ __forceinline__ double m_exp<double>(double x) { return exp(x); }
// 2^x: ex2.approx (flushing results below 2^-126 to zero) for float, exp2 for double.  Callers
// fold log2 e into their coefficients, exp(-eta x^2) = 2^(-eta log2(e) x^2): the rounding of
// the folded coefficient is of the size of the rounding of eta x^2 itself.
template <typename T> __device__ __forceinline__ T m_exp2(T x);
template <> __device__ __forceinline__ float m_exp2<float>(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
template <> __device__ __forceinline__ double m_exp2<double>(double x) { return exp2(x); }
constexpr double kLog2e = 1.44269504088896340736;
template <typename T> __device__ __forceinline__ T m_cos(T x);
template <> __device__ __forceinline__ float m_cos<float>(float x) { return cosf(x); }
template <> __device__ __forceinline__ double m_cos<double>(double x) { return cos(x); }
template <typename T> __device__ __forceinline__ T m_sin(T x);
template <> __device__ __forceinline__ float m_sin<float>(float x) { return sinf(x); }
template <> __device__ __forceinline__ double m_sin<double>(double x) { return sin(x); }
// Cutoff function fc(r) = (cos(pi r / rc) + 1) / 2 and its derivative -(pi / 2rc) sin(pi r / rc)
// for r <= rc.  FP64: the reference's formulas (acsf.F90:1240-1262).  FP32: the same values
// through half angles, fc = sin^2 phi and dfc = -(pi / rc) sin phi cos phi with
// phi = (pi / 2)(rc - r) / rc, which keeps full relative accuracy as r -> rc where the
// reference form cancels; sin and cos from their Taylor series (through u^13 / u^12, Horner in
// u^2) on an angle u in [0, pi/4] (truncation below 1e-13).
template <typename T> __device__ __forceinline__ void cutoff_fc(T r, T rc, T &fc, T &dfc);
template <>
__device__ __forceinline__ void cutoff_fc<double>(double r, double rc, double &fc, double &dfc) {
  fc = 0.5 * (cos(kPi * r / rc) + 1.0);
  dfc = -0.5 * (kPi / rc) * sin(kPi * r / rc);
}
__device__ __forceinline__ void sincos_taylor(float u, float &s, float &c) {
  const float w = u * u;
  float ps = 1.f / 6227020800.f;   // 1/13!
  ps = fmaf(ps, w, -1.f / 39916800.f);
  ps = fmaf(ps, w, 1.f / 362880.f);
  ps = fmaf(ps, w, -1.f / 5040.f);
  ps = fmaf(ps, w, 1.f / 120.f);
  ps = fmaf(ps, w, -1.f / 6.f);
  ps = fmaf(ps, w, 1.f);
  float pc = 1.f / 479001600.f;    // 1/12!
  pc = fmaf(pc, w, -1.f / 3628800.f);
  pc = fmaf(pc, w, 1.f / 40320.f);
  pc = fmaf(pc, w, -1.f / 720.f);
  pc = fmaf(pc, w, 1.f / 24.f);
  pc = fmaf(pc, w, -0.5f);
  pc = fmaf(pc, w, 1.f);
  s = u * ps;
  c = pc;
}
template <>
__device__ __forceinline__ void cutoff_fc<float>(float r, float rc, float &fc, float &dfc) {
  // sin phi = cos theta and cos phi = sin theta for theta = (pi / 2) r / rc: the series run on
  // the smaller of the two angles (<= pi/4), so both ends of [0, rc] keep relative accuracy
  const float irc = 1.f / rc;
  const float phi = (float)(kPi / 2.0) * ((rc - r) * irc);
  const float theta = (float)(kPi / 2.0) * (r * irc);
  float sm, cm;
  sincos_taylor(fminf(phi, theta), sm, cm);
  const float s = phi <= theta ? sm : cm, c = phi <= theta ? cm : sm;
  fc = s * s;
  dfc = -((float)kPi * irc) * (s * c);
}

template <typename T> __device__ __forceinline__ T m_pow(T b, T e);
template <> __device__ __forceinline__ float m_pow<float>(float b, float e) { return powf(b, e); }
template <> __device__ __forceinline__ double m_pow<double>(double b, double e) { return pow(b, e); }
template <typename T> __device__ __forceinline__ T m_sqrt(T x);
template <> __device__ __forceinline__ float m_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double m_sqrt<double>(double x) { return sqrt(x); }

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T atom_id(const double *ext, int next, int atomid, int64_t a) {
  return atomid > 0 ? (T)ext[a * next + (atomid - 1)] : (T)1;
}

// base^n for a small positive integer n (exact repeated multiplication), else pow(base, e)
template <typename T> __device__ __forceinline__ T int_pow(T base, int n, T e) {
  if (n > 0) {
    T r = base;
    for (int k = 1; k < n; k++) r *= base;
    return r;
  }
  return m_pow<T>(base, e);
}

// Everything the per-atom kernels read (one struct for both kernels).
constexpr int kRadParam = 128;                 // radial descriptors carried as kernel parameters
constexpr uint32_t kRvAllChannels = 0x800000ffu;  // channel bits of a self image: every list

template <typename T> struct TileArgs {
  int64_t natoms;
  const int64_t *poff;     // pairs of atom i: [poff[i], pend[i])
  const int64_t *pend;
  const int32_t *pj;
  const uint32_t *pmeta;
  const V4<T> *rij;
  const int8_t *code;
  const int32_t *bpos;
  const double *ext;
  int next;
  const GDesc *rad;
  const T *radp;          // [nrad][8] parameters in the kernel's width
  int nrad;
  int rad_seg[kMaxSpeciesCodes + 2];  // radial functions by list channel (see the context)
  const int32_t *radv;    // value kernel: radial functions in shape order
  int rad_split;          // value kernel, general radial path: lanes per function (1, 2 or 4)
  // value kernel, radial fast path with at most kRadParam functions: the descriptors held in
  // the kernel parameters.  Grid form (rv_nc > 0: every shape, at most 32, on the same rv_nc
  // list channels): per shape rs and -eta log2 e, per channel its bit, per function (shape sh,
  // channel c) its output column at sh * rv_nc + c.  Otherwise per function rs, -eta log2 e,
  // channel bit and output column.
  int rv_param, rv_nc, rv_nshape;
  T rv_rs[kRadParam], rv_c2[kRadParam];
  uint32_t rv_bits[kRadParam];
  int32_t rv_out[kRadParam];
  uint32_t rv_chan[kMaxSpeciesCodes + 1];
  const GDesc *ang;       // triplet-sweep functions
  const T *angp;          // [nang][8]
  const AGroup *groups;
  int ngroups;
  // eta classes and cutoff classes as kernel parameters (read per pair by the staging)
  T ecls_eta[kMaxEtaClasses];
  int ecls_rclass[kMaxEtaClasses];
  int ecls_atomid[kMaxEtaClasses];
  int necls;
  T rcls[kMaxRcutClasses];
  int nrcls;
  int nz;
  int cap;
  // moment form
  const MFunc *mfunc;
  int nmf;
  const int32_t *combo;   // [ncombo][2]
  int ncombo;
  const int32_t *cidx;    // [(nz+1)*necls]
  int n_mono;
  // factorised adjoint (forces): partner groups packed as [ncombo + 1] group offsets, [nqg]
  // partner combos, [nqg + 1] entry offsets, [entries] output columns; degree coefficients
  // mpc[entry][kMaxMomentDegree + 1]
  const int32_t *qg;
  int nqg;
  const T *mpc;
  int nqg_pack, nqg_ent;  // ints of the pack, entries of mpc (both staged per CTA)
  // value kernel, factorised G5: distinct combo pairs [nmpair][2], coefficients
  // fpc[nmf][kMaxMomentDegree + 1]
  const int32_t *mpair;
  int nmpair;
  const T *fpc;
  int rad_fast;           // forces: every radial function a G2 without atom id in this
                          // cutoff class (per-warp coefficient table), else -1
  // moment cache [natoms][ncombo][n_mono]: written by the ACSF kernel (mom != null), read by
  // the force kernel when mom_cached
  T *mom;
  int mom_cached;
  // values
  T *feat;
  int nf;
  // forces
  int ng;
  const T *J;
  double *F;     // FP64 kernels: [N][nout][3]
  float4 *F4;    // FP32 kernels: [N][nout] (x, y, z, unused), converted into F afterwards
  int out_index, nout;
};

template <typename T> struct Tile {
  V4<T> *v;         // dx, dy, dz, r (neighbour minus centre)
  V4<T> *u;         // unit vector, r
  V4<T> *w;         // pair force accumulators (forces kernel only)
  T *fc, *dfc;      // [nrcls][cap]
  T *E, *D;         // [necls][cap]
  uint32_t *info;   // code | self << 8 | rmask << 16
  int32_t *pj;
  T *idv;           // [cap] atom ids of a group's column
  T *gpar;          // [5][32]
  int *gint;        // [3][32]
  int *cnt;         // [8]
  T *M;             // [ncombo][n_mono] moments
  T *Q;             // [nqg][kMaxMomentDegree + 1] per-group degree sums h_g(m) (forces)
  T *Qc;            // [nz + 1][necls][n_mono] adjoint moments of a pair's species list plus
                    // the all-atom list, per eta class (forces; row nz: all-atom list only)
  T *jv;            // [ng] dE/dG of the centre atom (forces)
  uint16_t *lists;  // [nz][cap]
};

// Length of the force tile's adjoint scratch: the per-group degree sums h_g(m).
template <typename T> __host__ __device__ inline int tile_qwords(const TileArgs<T> &a) {
  return a.ncombo > 0 ? a.nqg * (kMaxMomentDegree + 1) : 0;
}

// Whether a tile keeps per-pair E/D tables: the value kernel always; the force kernel for
// triplet groups or when the moments are recomputed rather than read from the cache.
template <typename T> __host__ __device__ inline bool tile_etab(const TileArgs<T> &a, bool forces) {
  return !forces || a.ngroups > 0 || !a.mom_cached;
}

template <typename T>
__host__ __device__ inline size_t tile_bytes(int cap, int nrcls, int necls, int nz, int ncombo,
                                             int nmono, int ng, bool forces, bool trip,
                                             bool etab, int qwords = 0) {
  // v and idv serve the triplet sweep only; the E (and, for forces, D) tables are kept when
  // etab (values, triplets, or moments not taken from the cache)
  size_t b = 0;
  b += sizeof(V4<T>) * cap * ((forces ? 2 : 1) + (trip ? 1 : 0));
  b += sizeof(T) * (size_t)cap * (nrcls + (etab ? necls : 0)) * (forces ? 2 : 1);
  if (trip) b += sizeof(T) * cap;             // idv
  b += sizeof(T) * 5 * 32;                    // gpar
  b += sizeof(T) * (size_t)ncombo * nmono;
  if (forces) b += sizeof(T) * (size_t)qwords;
  if (forces && ncombo > 0) b += sizeof(T) * (size_t)(nz + 1) * necls * nmono;
  b += forces ? sizeof(T) * ng : 0;
  b = (b + 7) / 8 * 8;
  b += sizeof(uint32_t) * cap + sizeof(int32_t) * cap;
  b += sizeof(int) * (3 * 32 + 8);
  b += sizeof(uint16_t) * (size_t)cap * nz;
  return (b + 127) / 128 * 128;
}

template <typename T>
__device__ Tile<T> carve_tile(unsigned char *p, const TileArgs<T> &a, bool forces) {
  Tile<T> t;
  const int cap = a.cap;
  const bool trip = a.ngroups > 0;
  t.v = nullptr;
  if (trip) {
    t.v = reinterpret_cast<V4<T> *>(p);
    p += sizeof(V4<T>) * cap;
  }
  t.u = reinterpret_cast<V4<T> *>(p);
  p += sizeof(V4<T>) * cap;
  t.w = nullptr;
  if (forces) {
    t.w = reinterpret_cast<V4<T> *>(p);
    p += sizeof(V4<T>) * cap;
  }
  const bool etab = tile_etab(a, forces);
  t.fc = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * a.nrcls;
  t.E = nullptr;
  if (etab) {
    t.E = reinterpret_cast<T *>(p);
    p += sizeof(T) * (size_t)cap * a.necls;
  }
  t.dfc = t.D = nullptr;
  if (forces) {
    t.dfc = reinterpret_cast<T *>(p);
    p += sizeof(T) * (size_t)cap * a.nrcls;
    if (etab) {
      t.D = reinterpret_cast<T *>(p);
      p += sizeof(T) * (size_t)cap * a.necls;
    }
  }
  t.idv = nullptr;
  if (trip) {
    t.idv = reinterpret_cast<T *>(p);
    p += sizeof(T) * cap;
  }
  t.gpar = reinterpret_cast<T *>(p);
  p += sizeof(T) * 5 * 32;
  t.M = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)a.ncombo * a.n_mono;
  t.Q = t.jv = t.Qc = nullptr;
  if (forces) {
    t.Q = reinterpret_cast<T *>(p);
    p += sizeof(T) * (size_t)tile_qwords(a);
    if (a.ncombo > 0) {
      t.Qc = reinterpret_cast<T *>(p);
      p += sizeof(T) * (size_t)(a.nz + 1) * a.necls * a.n_mono;
    }
    t.jv = reinterpret_cast<T *>(p);
    p += sizeof(T) * a.ng;
  }
  p = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 7) & ~uintptr_t(7));
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

// Asynchronous global -> shared copy of n elements (cp.async, lanes striding): 16-byte pieces
// when both ends are 16-byte aligned and the length a multiple of 16 bytes, else element-sized
// pieces.  One commit group per call; async_copy_wait completes every group of the lane and
// synchronises the warp.
template <typename T>
__device__ __forceinline__ void async_copy(T *dst, const T *src, int n, int lane) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "element size");
  const uintptr_t da = reinterpret_cast<uintptr_t>(dst), sa = reinterpret_cast<uintptr_t>(src);
  const size_t bytes = sizeof(T) * (size_t)n;
  if (((da | sa) & 15u) == 0 && (bytes & 15u) == 0) {
    const int n16 = (int)(bytes / 16);
    for (int k = lane; k < n16; k += 32) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(reinterpret_cast<char *>(dst) + 16 * (size_t)k);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d),
                   "l"(reinterpret_cast<const char *>(src) + 16 * (size_t)k)
                   : "memory");
    }
  } else {
    for (int k = lane; k < n; k += 32) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(dst + k);
      asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src + k),
                   "n"((int)sizeof(T))
                   : "memory");
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void async_copy_wait() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncwarp();
}

// L2 prefetch of [p, p + bytes): one 128-byte line per lane and instruction.
__device__ __forceinline__ void prefetch_l2(const void *p, size_t bytes, int lane) {
  const uintptr_t b = reinterpret_cast<uintptr_t>(p);
  const uintptr_t end = b + bytes;
  for (uintptr_t l = (b & ~uintptr_t(127)) + 128u * (uintptr_t)lane; l < end; l += 128u * 32u)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(l));
}

// Pair records of a later atom [p0, p1) brought into L2 while the current atom is processed.
template <typename T>
__device__ __forceinline__ void prefetch_pairs(const TileArgs<T> &a, int64_t p0, int64_t p1,
                                               int lane) {
  if (p1 <= p0) return;
  const size_t n = (size_t)(p1 - p0);
  prefetch_l2(a.rij + p0, sizeof(V4<T>) * n, lane);
  prefetch_l2(a.pj + p0, sizeof(int32_t) * n, lane);
  prefetch_l2(a.pmeta + p0, sizeof(uint32_t) * n, lane);
}

// The eta-class and cutoff-class tables of the context, in the kernels' width.
template <typename T> inline void fill_class_tables(const fnetg_ctx *ctx, TileArgs<T> &a) {
  a.necls = (int)ctx->ecls_eta.size();
  for (int e = 0; e < kMaxEtaClasses; e++) {
    const bool on = e < a.necls;
    a.ecls_eta[e] = on ? (T)ctx->ecls_eta[e] : (T)0;
    a.ecls_rclass[e] = on ? ctx->ecls_rclass[e] : 0;
    a.ecls_atomid[e] = on ? ctx->ecls_atomid[e] : 0;
  }
  a.nrcls = (int)ctx->rcut_classes.size();
  for (int c = 0; c < kMaxRcutClasses; c++)
    a.rcls[c] = c < a.nrcls ? (T)ctx->rcut_classes[c] : (T)0;
}

// Warps per CTA for a warp-per-atom kernel whose CTA needs `fixed` + wpb * `per_warp` bytes of
// dynamic shared memory: the choice among 8, 4, 2, 1 (at most max_w, the kernel's launch bound)
// with the most resident warps per SM (ties go to the larger CTA).  Raises the kernel's
// shared-memory limit to cover that choice.
template <typename K>
inline cudaError_t pick_warps(K kernel, size_t fixed, size_t per_warp, int &wpb, size_t &smem,
                              int &ctas_per_sm, int max_w = 8) {
  cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int best_w = 0, best_warps = -1, best_ctas = 0;
  for (int w = 8; w >= 1; w >>= 1) {
    if (w > max_w) continue;
    const size_t bytes = fixed + per_warp * (size_t)w;
    if (bytes > 227 * 1024) continue;
    err = raise_smem_limit(reinterpret_cast<const void *>(kernel), bytes);
    if (err != cudaSuccess) return err;
    int ctas = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, kernel, w * 32, bytes);
    if (err != cudaSuccess) return err;
    if (ctas * w > best_warps) {
      best_warps = ctas * w;
      best_w = w;
      best_ctas = ctas;
    }
  }
  if (best_w == 0) return cudaErrorInvalidValue;
  wpb = best_w;
  smem = fixed + per_warp * (size_t)best_w;
  ctas_per_sm = std::max(best_ctas, 1);
  return raise_smem_limit(reinterpret_cast<const void *>(kernel), smem);
}

// One pair of the tile: displacement, unit vector, neighbour, flags, cutoff tables and (when
// the tile keeps them) the eta-class tables.
template <typename T>
__device__ __forceinline__ void stage_pair(const TileArgs<T> &a, Tile<T> &t, int64_t i, int q,
                                           const V4<T> v, int32_t j, uint32_t meta, int c,
                                           bool forces) {
  {
    if (t.v) t.v[q] = v;
    const T rinv = (T)1 / v.w;
    t.u[q] = V4<T>{v.x * rinv, v.y * rinv, v.z * rinv, v.w};
    if (forces) t.w[q] = V4<T>{0, 0, 0, 0};
    t.pj[q] = j;
    const uint32_t rmask = meta >> 24;
    t.info[q] = (uint32_t)(c & 0xff) | ((uint32_t)(j == i) << 8) | (rmask << 16);
    for (int rc = 0; rc < a.nrcls; rc++) {
      const T rcut = a.rcls[rc];
      const bool in = (rmask >> rc) & 1u;
      T fcv, dfv;
      cutoff_fc<T>(in ? v.w : rcut, rcut, fcv, dfv);
      t.fc[rc * a.cap + q] = in ? fcv : (T)0;
      if (forces) t.dfc[rc * a.cap + q] = in ? dfv : (T)0;
    }
    for (int e = 0; t.E && e < a.necls; e++) {
      const T eta = a.ecls_eta[e];
      const int aid = a.ecls_atomid[e];
      const int rc = a.ecls_rclass[e];
      const T ex = m_exp2<T>((-eta * (T)kLog2e) * (v.w * v.w));
      T ids = (T)1;
      if (aid > 0) ids = atom_id<T>(a.ext, a.next, aid, i) * atom_id<T>(a.ext, a.next, aid, j);
      const T f = t.fc[rc * a.cap + q];
      t.E[e * a.cap + q] = ex * f * ids;
      if (forces) t.D[e * a.cap + q] = ex * (t.dfc[rc * a.cap + q] - (T)2 * eta * v.w * f) * ids;
    }
  }
}

// Stage the pair tile of atom i (all lanes), build the ordered species lists.  A lane takes
// pairs q and q + 32 together: both pair records and both neighbour species are requested
// before either is used, so the two memory round trips overlap.
template <typename T>
__device__ void stage_tile(const TileArgs<T> &a, Tile<T> &t, int64_t i, int64_t p0, int np,
                           int lane, bool forces) {
  for (int q0 = 0; q0 < np; q0 += 64) {
    const int qa = q0 + lane, qb = q0 + 32 + lane;
    const bool ha = qa < np, hb = qb < np;
    V4<T> va{}, vb{};
    int32_t ja = 0, jb = 0;
    uint32_t ma = 0, mb = 0;
    if (ha) {
      va = a.rij[p0 + qa];
      ja = a.pj[p0 + qa];
      ma = a.pmeta[p0 + qa];
    }
    if (hb) {
      vb = a.rij[p0 + qb];
      jb = a.pj[p0 + qb];
      mb = a.pmeta[p0 + qb];
    }
    const int ca = ha ? a.code[ja] : 0, cb = hb ? a.code[jb] : 0;
    if (ha) stage_pair<T>(a, t, i, qa, va, ja, ma, ca, forces);
    if (hb) stage_pair<T>(a, t, i, qb, vb, jb, mb, cb, forces);
  }
  __syncwarp();
  for (int z = 0; z < a.nz; z++) {
    int base = 0;
    for (int q0 = 0; q0 < np; q0 += 32) {
      const int q = q0 + lane;
      bool in = false;
      if (q < np) {
        const uint32_t inf = t.info[q];
        in = ((int)(inf & 0xff) == z) || ((inf >> 8) & 1u);
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in && FNETG_GUARD(base + __popc(m & ((1u << lane) - 1u)) < a.cap))
        t.lists[z * a.cap + base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
      base += __popc(m);
    }
    if (lane == 0) t.cnt[z] = base;
  }
  __syncwarp();
}


// Sum of v[0..31] over the warp's lanes, returned on lane l for index l: each of the five
// butterfly steps exchanges half of the remaining values (31 shuffles instead of 160).
template <typename T>
__device__ __forceinline__ T transpose_reduce32(T *v, int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for (int k = 0; k < s; k++) {
      const T send = upper ? v[k] : v[k + s];
      const T keep = upper ? v[k + s] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  return v[0];
}

// One pass of the moment sums M_k(alpha) = sum over list(k) of E_e(k)(j) u_j^alpha for nk <= 32 / S
// consecutive combos k0.. of one list (the combos are ordered by list, then eta class).  Lane
// (group g, slot s) walks the list's pairs s, s + S, ... with the weight of combo k0 + g, the
// monomials carried as products (child = parent * coordinate); a transposing butterfly over the
// S slots then leaves C = ceil(NM / S) consecutive sums on each lane.
template <typename T, int D, int S>
__device__ __forceinline__ void moment_pass(const TileArgs<T> &a, Tile<T> &t, const uint16_t *lst,
                                            int n, int k0, int nk, int lane) {
  constexpr int NM = n_mono_of(D);
  constexpr int C = (NM + S - 1) / S;
  constexpr int V = C * S;
  const int grp = lane / S, slot = lane % S;
  const bool on = grp < nk;
  const int e = on ? a.combo[2 * (k0 + grp) + 1] : 0;
  const T *E = t.E + e * a.cap;
  T acc[V];
#pragma unroll
  for (int al = 0; al < V; al++) acc[al] = 0;
  for (int kk = slot; kk < n; kk += S) {
    const int q = lst ? lst[kk] : kk;
    const V4<T> u = t.u[q];
    T m[NM];
    m[0] = on ? E[q] : (T)0;
#pragma unroll
    for (int al = 1; al < NM; al++) {
      const int ax = kMonoLinks.axis[al];
      m[al] = m[kMonoLinks.parent[al]] * (ax == 0 ? u.x : (ax == 1 ? u.y : u.z));
    }
#pragma unroll
    for (int al = 0; al < NM; al++) acc[al] += m[al];
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
  if (on) {
    T *M = t.M + (k0 + grp) * NM;
#pragma unroll
    for (int c = 0; c < C; c++)
      if (slot * C + c < NM) M[slot * C + c] = acc[c];
  }
}

// M_k(alpha) for every (list, eta class) combo k: runs of one list's combos taken up to four
// at a time (8 slots per combo for three or four, 16 for two, 32 for one).
template <typename T, int D>
__device__ void compute_moments(const TileArgs<T> &a, Tile<T> &t, int np, int lane) {
  for (int k = 0; k < a.ncombo;) {
    const int z = a.combo[2 * k];
    int nk = 1;
    while (k + nk < a.ncombo && nk < 4 && a.combo[2 * (k + nk)] == z) nk++;
    const uint16_t *lst = z >= 0 ? t.lists + z * a.cap : nullptr;
    const int n = z >= 0 ? t.cnt[z] : np;
    if (nk == 1) moment_pass<T, D, 32>(a, t, lst, n, k, 1, lane);
    else if (nk == 2) moment_pass<T, D, 16>(a, t, lst, n, k, 2, lane);
    else moment_pass<T, D, 8>(a, t, lst, n, k, nk, lane);
    k += nk;
  }
  __syncwarp();
}

}  // namespace fnetg
