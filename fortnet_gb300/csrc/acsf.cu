// K2/K3: ACSF values G1..G5 (lib_descriptors/acsf.F90:1287-1492 driven by iGeoAcsf
// 797-866) and K5: z-score statistics / standardisation (acsf.F90:445-511).
//
// One warp per centre atom.  The atom's pair tile (displacements, distances, species code,
// self-image flag, cutoff-class mask) is staged in shared memory once; the per-species
// neighbour lists of buildGFunctionNeighborlists (acsf.F90:943-1066) become ordered index
// lists built with ballots — the centre atom's periodic self-images are members of every
// species list, as in the reference's species-reduced geometries.  Radial functions run
// lanes-over-functions (each lane sums one function over its list in list order); angular
// functions run lanes-over-triplets for a group of up to 32 functions sharing two lists,
// with exp(-eta r^2) * fc(r) tabulated per pair and eta class so that every triplet costs
// one cos(theta), one power and two multiplies per function.
#include <algorithm>

#include "internal.cuh"

namespace fnetg {

namespace {

constexpr double kPi = 3.14159265358979323846;  // lib_dftbp/constants.F90:15

template <typename T> struct AcsfArgs {
  int64_t natoms;
  const int64_t *poff;
  const int32_t *pj;
  const uint32_t *pmeta;
  const V4<T> *rij;
  const int8_t *code;
  const int32_t *bpos;
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
  T *feat;
  int nf;
  int cap;
};

// per-warp shared-memory tile
template <typename T> struct Tile {
  V4<T> *v;        // dx, dy, dz, r
  T *fc;           // [nrcls][cap] 0.5*(cos(pi r/rc)+1) (0 outside the class)
  T *E;            // [necls][cap] exp(-eta r^2) * fc * id_i * id_j
  uint32_t *info;  // code | self << 8 | rmask << 16
  int32_t *pj;     // global neighbour index
  uint16_t *lists; // [nz][cap]
  int *cnt;        // [nz]
  T *gpar;         // group parameters [4][32]: lambda, xi, eta, pref
  int *gint;       // [3][32]: xi_int, eclass, type
  T *idv;          // [cap] atom ids of the group's column (G4 third cutoff)
};

template <typename T> __host__ __device__ size_t tile_bytes(int cap, int nrcls, int necls, int nz) {
  size_t b = 0;
  b += sizeof(V4<T>) * cap;
  b += sizeof(T) * (size_t)cap * (nrcls + necls);
  b += sizeof(uint32_t) * cap + sizeof(int32_t) * cap;
  b += sizeof(uint16_t) * (size_t)cap * nz;
  b += sizeof(int) * 8;
  b += sizeof(T) * 4 * 32 + sizeof(int) * 3 * 32;
  b += sizeof(T) * cap;
  return (b + 127) / 128 * 128;
}

template <typename T>
__device__ Tile<T> carve(unsigned char *base, int cap, int nrcls, int necls, int nz) {
  Tile<T> t;
  unsigned char *p = base;
  t.v = reinterpret_cast<V4<T> *>(p);
  p += sizeof(V4<T>) * cap;
  t.fc = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * nrcls;
  t.E = reinterpret_cast<T *>(p);
  p += sizeof(T) * (size_t)cap * necls;
  t.gpar = reinterpret_cast<T *>(p);
  p += sizeof(T) * 4 * 32;
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

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T> __device__ __forceinline__ T t_exp(T x);
template <> __device__ __forceinline__ float t_exp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double t_exp<double>(double x) { return exp(x); }
template <typename T> __device__ __forceinline__ T t_cos(T x);
template <> __device__ __forceinline__ float t_cos<float>(float x) { return cosf(x); }
template <> __device__ __forceinline__ double t_cos<double>(double x) { return cos(x); }
template <typename T> __device__ __forceinline__ T t_pow(T b, T e);
template <> __device__ __forceinline__ float t_pow<float>(float b, float e) { return powf(b, e); }
template <> __device__ __forceinline__ double t_pow<double>(double b, double e) { return pow(b, e); }
template <typename T> __device__ __forceinline__ T t_sqrt(T x);
template <> __device__ __forceinline__ float t_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double t_sqrt<double>(double x) { return sqrt(x); }

// base^n for a small positive integer n (exact repeated multiplication), else pow
template <typename T> __device__ __forceinline__ T xi_pow(T base, int n, T xi) {
  if (n > 0) {
    T r = base;
    for (int k = 1; k < n; k++) r *= base;
    return r;
  }
  return t_pow<T>(base, xi);
}

template <typename T>
__device__ __forceinline__ T atom_id(const double *ext, int next, int atomid, int64_t a) {
  return atomid > 0 ? (T)ext[a * next + (atomid - 1)] : (T)1;
}

template <typename T>
__global__ void __launch_bounds__(256) acsf_kernel(AcsfArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const size_t tb = tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz);
  Tile<T> tile = carve<T>(smem + tb * warp, a.cap, a.nrcls, a.necls, a.nz);
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < a.natoms; i += (int64_t)gridDim.x * wpb) {
    const int64_t p0 = a.poff[i];
    const int np = (int)(a.poff[i + 1] - p0);
    const int64_t row = a.bpos[i];
    // ---- stage the pair tile
    for (int q = lane; q < np; q += 32) {
      V4<T> v = a.rij[p0 + q];
      tile.v[q] = v;
      const int32_t j = a.pj[p0 + q];
      tile.pj[q] = j;
      const uint32_t meta = a.pmeta[p0 + q];
      const uint32_t rmask = meta >> 24;
      const int c = a.code[j];
      tile.info[q] = (uint32_t)(c & 0xff) | ((uint32_t)(j == i) << 8) | (rmask << 16);
      for (int rc = 0; rc < a.nrcls; rc++) {
        const T rcut = (T)a.rcls[rc];
        tile.fc[rc * a.cap + q] =
            ((rmask >> rc) & 1u) ? (T)0.5 * (t_cos<T>((T)kPi * v.w / rcut) + (T)1) : (T)0;
      }
      for (int e = 0; e < a.necls; e++) {
        const T eta = (T)a.ecls_eta[e];
        const int aid = a.ecls_atomid[e];
        T val = t_exp<T>(-(eta * (v.w * v.w))) * tile.fc[a.ecls_rclass[e] * a.cap + q];
        if (aid > 0) val *= atom_id<T>(a.ext, a.next, aid, i) * atom_id<T>(a.ext, a.next, aid, j);
        tile.E[e * a.cap + q] = val;
      }
    }
    __syncwarp();
    // ---- ordered species lists (self images belong to every list)
    for (int z = 0; z < a.nz; z++) {
      int base = 0;
      for (int q0 = 0; q0 < np; q0 += 32) {
        const int q = q0 + lane;
        bool in = false;
        if (q < np) {
          const uint32_t inf = tile.info[q];
          in = ((int)(inf & 0xff) == z) || ((inf >> 8) & 1u);
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) tile.lists[z * a.cap + base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
        base += __popc(m);
      }
      if (lane == 0) tile.cnt[z] = base;
    }
    __syncwarp();
    // ---- radial functions: lanes over functions, list order
    for (int g = lane; g < a.nrad; g += 32) {
      const GDesc d = a.rad[g];
      const uint16_t *lst = d.chan1 >= 0 ? tile.lists + d.chan1 * a.cap : nullptr;
      const int n = d.chan1 >= 0 ? tile.cnt[d.chan1] : np;
      const T *fcr = tile.fc + d.rclass * a.cap;
      const T idi = atom_id<T>(a.ext, a.next, d.atomid, i);
      T acc = 0;
      for (int k = 0; k < n; k++) {
        const int q = lst ? lst[k] : k;
        if (!((tile.info[q] >> (16 + d.rclass)) & 1u)) continue;
        const T r = tile.v[q].w;
        T fc = fcr[q];
        if (d.atomid > 0) fc *= idi * atom_id<T>(a.ext, a.next, d.atomid, tile.pj[q]);
        T term;
        if (d.type == 1) {
          term = fc;
        } else if (d.type == 2) {
          const T x = r - (T)d.rs;
          term = t_exp<T>(-((T)d.eta * (x * x))) * fc;
        } else {
          term = t_cos<T>((T)d.kappa * r) * fc;
        }
        acc += term;
      }
      a.feat[row * a.nf + d.out] = acc;
    }
    // ---- angular groups: lanes over triplets
    for (int gi = 0; gi < a.ngroups; gi++) {
      const AGroup G = a.groups[gi];
      __syncwarp();
      if (lane < G.count) {
        const GDesc d = a.ang[G.first + lane];
        tile.gpar[lane] = (T)d.lambda;
        tile.gpar[32 + lane] = (T)d.xi;
        tile.gpar[64 + lane] = (T)d.eta;
        tile.gpar[96 + lane] = (T)d.pref;
        tile.gint[lane] = d.xi_int;
        tile.gint[32 + lane] = d.eclass;
        tile.gint[64 + lane] = d.type;
      }
      if (G.has_g4 && G.atomid > 0)
        for (int q = lane; q < np; q += 32)
          tile.idv[q] = atom_id<T>(a.ext, a.next, G.atomid, tile.pj[q]);
      __syncwarp();
      const uint16_t *l1 = G.chan1 >= 0 ? tile.lists + G.chan1 * a.cap : nullptr;
      const uint16_t *l2 = G.chan2 >= 0 ? tile.lists + G.chan2 * a.cap : nullptr;
      const int n1 = G.chan1 >= 0 ? tile.cnt[G.chan1] : np;
      const int n2 = G.chan2 >= 0 ? tile.cnt[G.chan2] : np;
      const int64_t ntrip = (int64_t)n1 * n2;
      T acc[kMaxGroupFuncs];
#pragma unroll
      for (int f = 0; f < kMaxGroupFuncs; f++) acc[f] = 0;
      const double rcut_g4 = a.ang[G.first].rcut;
      if (n2 > 0) {
        const int dj = 32 / n2, dk = 32 % n2;
        int jj = lane / n2, kk = lane % n2;
        for (int64_t t = lane; t < ntrip; t += 32) {
          const int p = l1 ? l1[jj] : jj;
          const int q = l2 ? l2[kk] : kk;
          const V4<T> vp = tile.v[p], vq = tile.v[q];
          const T dot = vp.x * vq.x + vp.y * vq.y + vp.z * vq.z;
          // theta of acsf.F90:1173-1174; cos(acos(x)) == x up to rounding, clamped to the
          // domain of acos
          T c = dot / (vp.w * vq.w + (T)1e-13);
          c = c > (T)1 ? (T)1 : (c < (T)-1 ? (T)-1 : c);
          T fjk = 1, rjk2 = 0;
          if (G.has_g4) {
            const T ex = vp.x - vq.x, ey = vp.y - vq.y, ez = vp.z - vq.z;
            rjk2 = ex * ex + ey * ey + ez * ez;
            const T rjk = t_sqrt<T>(rjk2);
            fjk = rjk > (T)rcut_g4 ? (T)0 : (T)0.5 * (t_cos<T>((T)kPi * rjk / (T)rcut_g4) + (T)1);
            if (G.atomid > 0) fjk *= tile.idv[p] * tile.idv[q];
          }
#pragma unroll
          for (int f = 0; f < kMaxGroupFuncs; f++) {
            if (f < G.count) {
              const T base = (T)1 + tile.gpar[f] * c;
              const T ang = xi_pow<T>(base, tile.gint[f], tile.gpar[32 + f]);
              const int e = tile.gint[32 + f];
              T rad = tile.E[e * a.cap + p] * tile.E[e * a.cap + q];
              if (tile.gint[64 + f] == 4) rad *= t_exp<T>(-(tile.gpar[64 + f] * rjk2)) * fjk;
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
        a.feat[row * a.nf + d.out] = mine * tile.gpar[96 + lane];
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

template <typename T>
__global__ void zapply_kernel(T *feat, int nf, int ng, int64_t N, const double *zprec) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * ng) return;
  const int64_t r = t / ng;
  const int f = (int)(t % ng);
  const double sd = zprec[ng + f];
  if (sd < 1e-08) return;
  T *x = feat + r * nf + f;
  *x = (T)(((double)*x - zprec[f]) / sd);
}

template <typename T> int launch_acsf(fnetg_ctx *ctx) {
  const int ng = (int)ctx->gf.size();
  const int nf = ctx->nf;
  const int64_t N = ctx->N;
  FNETG_CUDA(ctx->d_feat.ensure(sizeof(T) * std::max<int64_t>(N, 1) * std::max(nf, 1)));
  if (N == 0) return FNETG_OK;
  AcsfArgs<T> a{};
  a.natoms = N;
  a.poff = ctx->d_poff.as<int64_t>();
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = static_cast<const V4<T> *>(ctx->d_rij.p);
  a.code = ctx->d_code.as<int8_t>();
  a.bpos = ctx->d_bpos.as<int32_t>();
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
  a.feat = ctx->d_feat.as<T>();
  a.nf = nf;
  a.cap = std::max(32, (ctx->max_pairs + 31) / 32 * 32);
  FNETG_CHECK(a.cap <= 65535, FNETG_E_UNSUPPORTED, "more than 65535 neighbours of one atom");
  const size_t tb = tile_bytes<T>(a.cap, a.nrcls, a.necls, a.nz);
  int wpb = 8;
  while (wpb > 1 && tb * wpb > 200 * 1024) wpb >>= 1;
  FNETG_CHECK(tb * wpb <= 227 * 1024, FNETG_E_UNSUPPORTED,
              "neighbour tile of one atom exceeds shared memory");
  const size_t smem = tb * wpb;
  FNETG_CUDA(cudaFuncSetAttribute(acsf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, acsf_kernel<T>, wpb * 32, smem);
  const int64_t want = (N + wpb - 1) / wpb;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)num_sms() * std::max(per_sm, 1) * 8));
  {
    LaunchScope ls(ctx, "acsf");
    acsf_kernel<T><<<blocks, wpb * 32, smem, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  return FNETG_OK;
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
  if (N > 0 && ng > 0) {
    LaunchScope ls(ctx, "zscore");
    zapply_kernel<T><<<ceil_div(N * ng, 256), 256, 0, ctx->stream>>>(ctx->d_feat.as<T>(), nf, ng,
                                                                     N, z);
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
  ctx->nf = (int)ctx->gf.size() + (int)ctx->ext_idx.size();
  int rc = ctx->prec == FNETG_FP64 ? launch_acsf<double>(ctx) : launch_acsf<float>(ctx);
  if (rc) return rc;
  ctx->feats_valid = true;
  return FNETG_OK;
}

int run_ext_inputs(fnetg_ctx *ctx) {
  return ctx->prec == FNETG_FP64 ? launch_ext<double>(ctx) : launch_ext<float>(ctx);
}

int run_zscore(fnetg_ctx *ctx, const int32_t *weights, bool compute) {
  return ctx->prec == FNETG_FP64 ? launch_zscore<double>(ctx, weights, compute)
                                 : launch_zscore<float>(ctx, weights, compute);
}

}  // namespace fnetg
