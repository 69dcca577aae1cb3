// K1: periodic cutoff neighbour search whose pair sets and per-atom order equal the
// reference's dynamic neighbour iterator (lib_dftbp/dynneighlist.F90:233-320 over
// lib_dftbp/latpointiter.F90:121-253).
//
// One warp per centre atom.  Images are visited in the iterator's order (central cell
// first, then lattice points n1 outer .. n3 inner, origin excluded); within an image the
// atoms are visited cyclically starting after (central cell) or at (images) the centre.
// Lanes test 32 consecutive candidates; a float pre-filter with a safety margin rejects the
// far candidates and survivors are decided by the reference's FP64 arithmetic
// (nc = c_j + L n, d = c_i - nc, d2 = (d0^2 + d1^2) + d2^2, d2 <= rc^2) with every
// operation rounded separately (no FMA contraction).  A ballot keeps the accepted pairs in
// iterator order, so the fill pass reproduces the reference's neighbour order exactly.
#define FNETG_FILE_CODE 1  // site codes of the bounds-checked build
#include <algorithm>
#include <cstring>

#include "internal.cuh"

int fnetg_lattice_ranges(const double *L, double rcut, int32_t *lohi);

namespace fnetg {

namespace {

struct NbArgs {
  const int64_t *off;
  const int32_t *astruct;
  const double *coords;
  const V4<float> *cf;     // [N] high parts of the relative float coordinates
  const V4<float> *cl;     // [N] low parts
  const double *lat;
  const int64_t *img_off;  // [S+1] per-structure range into the image table
  const V4<double> *imgs;  // cell vectors (x, y, z, packed n1/n2/n3) in the iterator's order
  const V4<float> *imgf;   // [2 * images] float high parts (w: packed n1/n2/n3), low parts
  const float *bbox;      // [S*6] lo, hi (relative frame)
  int64_t natoms;
  double rc2;             // rcut*rcut (exact decision)
  float rc2_lo, rc2_hi;   // float distances below / above are decided without FP64
  const double *rcls;     // cutoff classes (ascending)
  const float *rcls2_lo, *rcls2_hi;
  int nrcls;
  int exact_geometry;     // FP64 displacement / distance for every accepted pair
  // fill pass
  const int64_t *poff;
  int64_t *count;
  int32_t *pj;
  uint32_t *pmeta;
  void *rij;              // V4<T>
  double *d2out;          // optional
  int *maxp;
  // slab fill (slab_cap > 0): atom i's pairs at [i * slab_cap, i * slab_cap + count), the pass
  // counts as well; begin/end offsets, overflow flag (count > slab_cap) and the pair total
  int64_t slab_cap;
  int64_t *pbeg, *pend;
  int *overflow;
  unsigned long long *total;
  // cell lists of the structures that use them (cgrid[s].w != 0): per structure the grid
  // dimensions and its first cell, per cell the range of its atoms in catom (structure-local
  // indices)
  const int4 *cgrid;
  const int64_t *coff;
  const int64_t *cstart;
  const V4<float> *cpos;  // per cell slot: relative float position, w = structure-local index
  int64_t nslots;  // pair slots of pj / pmeta / rij (bounds-checked build)
  float inv_cs;   // 1 / cell edge (relative float frame)
  float rbox;     // half-width of a centre's candidate box, >= the float pre-filter's reach
};

constexpr int kCellMin = 96;         // structures with fewer atoms test every atom
constexpr int kCellMaxAtoms = 4096;  // per-warp bitmask of accepted neighbours per image
constexpr int kCellDimMax = 32;      // cells per axis

__device__ __forceinline__ double exact_d2(const double *ci, const double *cj, const double *cv,
                                           double *d) {
  // the reference's arithmetic: nc = c_j + cellVec, d2 = sum((c_i - nc)**2) in index order
  const double nc0 = __dadd_rn(cj[0], cv[0]);
  const double nc1 = __dadd_rn(cj[1], cv[1]);
  const double nc2 = __dadd_rn(cj[2], cv[2]);
  d[0] = __dsub_rn(nc0, ci[0]);  // neighbour - centre; (c_i - nc)^2 == (nc - c_i)^2 exactly
  d[1] = __dsub_rn(nc1, ci[1]);
  d[2] = __dsub_rn(nc2, ci[2]);
  double s = __dmul_rn(d[0], d[0]);
  s = __dadd_rn(s, __dmul_rn(d[1], d[1]));
  s = __dadd_rn(s, __dmul_rn(d[2], d[2]));
  return s;
}

// the reference's FP64 squared distance of centre ci and atom j shifted by image img
// (-1: central cell); d receives the displacement
__device__ __forceinline__ double exact_pair(const NbArgs &a, const double *ci, int64_t j,
                                             int64_t img, double (&d)[3]) {
  double cv[3] = {0.0, 0.0, 0.0};
  if (img >= 0) {
    const V4<double> iv = a.imgs[img];
    cv[0] = iv.x;
    cv[1] = iv.y;
    cv[2] = iv.z;
  }
  const double cj[3] = {a.coords[3 * j], a.coords[3 * j + 1], a.coords[3 * j + 2]};
  return exact_d2(ci, cj, cv, d);
}

__device__ __forceinline__ void cell_vector(const double *L, int n1, int n2, int n3, double *cv) {
  // matmul(latVecs, n) summed in index order
  for (int c = 0; c < 3; c++) {
    double v = __dmul_rn(L[c + 0], (double)n1);
    v = __dadd_rn(v, __dmul_rn(L[c + 3], (double)n2));
    v = __dadd_rn(v, __dmul_rn(L[c + 6], (double)n3));
    cv[c] = v;
  }
}

// (a + b) - c for a = ah + al, b = bh + bl, c = ch + cl, each part a float: error-free
// transformations (Knuth's TwoSum) of the two high-part operations plus the low parts, so the
// result is the float rounding of the double-float value, all on the FP32 pipe.
__device__ __forceinline__ float two_sum(float a, float b, float &err) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

__device__ __forceinline__ float disp_df(float ah, float al, float bh, float bl, float ch,
                                         float cl) {
  float e1, e2;
  const float s = two_sum(ah, bh, e1);
  const float t = two_sum(s, -ch, e2);
  return __fadd_rn(t, __fadd_rn(__fadd_rn(e1, e2), __fsub_rn(__fadd_rn(al, bl), cl)));
}

constexpr int kNbWarps = 8;  // warps per CTA of the neighbour kernel
constexpr int kNbQueue = 128;  // ring of accepted pairs per warp (a power of two)

// Store accepted pair (centre i, structure-local neighbour jl, image img or im0 - 1 for the
// central cell) as the rank-th pair of atom i, at wpos + rank (within the slab capacity).
template <typename T>
__device__ __forceinline__ void store_pair(const NbArgs &a, const double *ci, const V4<float> &cif,
                                           const V4<float> &cil, int64_t i, int64_t a0, int jl,
                                           int img_i, int64_t im0, int64_t wpos, int64_t rank) {
  if (a.slab_cap > 0 && rank >= a.slab_cap) return;
  const int64_t img = img_i;
  const int64_t j = a0 + jl;
  const int64_t q = wpos + rank;
  if (!FNETG_GUARD(q >= 0 && q < a.nslots && jl >= 0)) return;
  V4<float> ch{0.f, 0.f, 0.f, 0.f}, cvl{0.f, 0.f, 0.f, 0.f};
  uint32_t packed = 0;
  if (img >= im0) {
    ch = a.imgf[2 * img];
    cvl = a.imgf[2 * img + 1];
    packed = __float_as_uint(ch.w);
  }
  const V4<float> cjf = a.cf[j];
  a.pj[q] = (int32_t)j;
  uint32_t mask = 0;
  V4<T> v;
  if (a.exact_geometry || a.d2out) {
    double d[3];
    const double dist2 = exact_pair(a, ci, j, img >= im0 ? img : -1, d);
    for (int c = 0; c < a.nrcls; c++)
      if (dist2 <= __dmul_rn(a.rcls[c], a.rcls[c])) mask |= 1u << c;
    if (a.d2out) a.d2out[q] = dist2;
    v.x = (T)d[0];
    v.y = (T)d[1];
    v.z = (T)d[2];
    v.w = (T)sqrt(dist2);
  } else {
    // the pre-filter's float distance decides the cutoff classes outside their error bands
    const float e0 = (cjf.x + ch.x) - cif.x, e1 = (cjf.y + ch.y) - cif.y,
                e2 = (cjf.z + ch.z) - cif.z;
    const float df = e0 * e0 + e1 * e1 + e2 * e2;
    // displacement in double-float arithmetic from the split coordinates, rounded once to
    // float; distance in float
    const V4<float> cjl = a.cl[j];
    const float fx = disp_df(cjf.x, cjl.x, ch.x, cvl.x, cif.x, cil.x);
    const float fy = disp_df(cjf.y, cjl.y, ch.y, cvl.y, cif.y, cil.y);
    const float fz = disp_df(cjf.z, cjl.z, ch.z, cvl.z, cif.z, cil.z);
    v.x = (T)fx;
    v.y = (T)fy;
    v.z = (T)fz;
    v.w = (T)sqrtf(fx * fx + fy * fy + fz * fz);
    for (int c = 0; c < a.nrcls; c++) {
      if (df <= a.rcls2_lo[c]) {
        mask |= 1u << c;
      } else if (df <= a.rcls2_hi[c]) {
        double d[3];
        if (exact_pair(a, ci, j, img >= im0 ? img : -1, d) <= __dmul_rn(a.rcls[c], a.rcls[c]))
          mask |= 1u << c;
      }
    }
  }
  a.pmeta[q] = (packed & 0xffffffu) | (mask << 24);
  reinterpret_cast<V4<T> *>(a.rij)[q] = v;
}

// Four CTAs of 256 threads per SM: at most 64 registers a thread (80 unbounded, 3 CTAs)
template <typename T, bool kFill>
__global__ void __launch_bounds__(256, 4) nb_kernel(NbArgs a) {
  __shared__ int blk_max;
  __shared__ unsigned long long blk_sum;
  __shared__ int2 queue_all[kNbWarps][kNbQueue];  // accepted pairs waiting to be stored
  __shared__ uint32_t bits_all[kNbWarps][kCellMaxAtoms / 32];  // accepted atoms of one image
  if (threadIdx.x == 0) {
    blk_max = 0;
    blk_sum = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i < a.natoms) {
    const int s = a.astruct[i];
    const int64_t a0 = a.off[s];
    const int n = (int)(a.off[s + 1] - a0);
    const int il = (int)(i - a0);
    const double ci[3] = {a.coords[3 * i], a.coords[3 * i + 1], a.coords[3 * i + 2]};
    const V4<float> cif = a.cf[i];
    const V4<float> cil = a.cl[i];
    int64_t wpos = 0;
    if (kFill) wpos = a.slab_cap > 0 ? i * a.slab_cap : a.poff[i];
    int2 *queue = queue_all[threadIdx.x >> 5];
    uint32_t *bits = bits_all[threadIdx.x >> 5];
    const int4 cg = a.cgrid ? a.cgrid[s] : make_int4(0, 0, 0, 0);
    const int64_t cbase = cg.w ? a.coff[s] : 0;
    int qh = 0, qn = 0;   // head and length of the ring of queued pairs (uniform)
    int64_t stored = 0;   // accepted candidates already stored
    int64_t cnt = 0;
    const float *bb = a.bbox + 6 * s;
    const int64_t im0 = a.img_off[s], im1 = a.img_off[s + 1];
    // the ring's first 32 pairs stored by the 32 lanes, at consecutive slots
    auto drain32 = [&]() {
      const int2 e = queue[(qh + lane) & (kNbQueue - 1)];
      store_pair<T>(a, ci, cif, cil, i, a0, e.x, e.y, im0, wpos, stored + lane);
      __syncwarp();
      qh = (qh + 32) & (kNbQueue - 1);
      qn -= 32;
      stored += 32;
    };
    // image -1 is the central cell, then the lattice points of the table (n1 outer .. n3 inner).
    // The images are tested 32 at a time, one per lane, against the reach of the structure's
    // shifted bounding box; the warp then walks the reachable ones in order.
    for (int64_t ibase = im0 - 1; ibase < im1; ibase += 32) {
      bool reach = false;
      const int64_t mine = ibase + lane;
      if (mine < im0) {
        reach = true;
      } else if (mine < im1) {
        const V4<float> chm = a.imgf[2 * mine];
        const float p[3] = {cif.x, cif.y, cif.z};
        const float cvf[3] = {chm.x, chm.y, chm.z};
        float dd = 0.f;
        for (int c = 0; c < 3; c++) {
          const float lo = bb[c] + cvf[c], hi = bb[3 + c] + cvf[c];
          const float e = p[c] < lo ? lo - p[c] : (p[c] > hi ? p[c] - hi : 0.f);
          dd += e * e;
        }
        reach = !(dd > a.rc2_hi);
      }
      for (unsigned pend = __ballot_sync(0xffffffffu, reach); pend; pend &= pend - 1u) {
        const int64_t img = ibase + (__ffs(pend) - 1);
        V4<float> ch{0.f, 0.f, 0.f, 0.f};
        int tstart = 1, tcount = n - 1;
        if (img >= im0) {
          ch = a.imgf[2 * img];
          tstart = 0;
          tcount = n;
        }
        // candidates 64 at a time, two per lane: the shifted centre is formed once per image
        const float px = cif.x - ch.x, py = cif.y - ch.y, pz = cif.z - ch.z;
        // the reference's decision for structure-local atom jl of this image
        auto decide = [&](int jl, const V4<float> &cjf) -> bool {
          const float e0 = cjf.x - px, e1 = cjf.y - py, e2 = cjf.z - pz;
          const float df = e0 * e0 + e1 * e1 + e2 * e2;
          if (df <= a.rc2_lo) return true;
          if (df > a.rc2_hi) return false;
          double d[3];
          return exact_pair(a, ci, a0 + jl, img >= im0 ? img : -1, d) <= a.rc2;
        };
        if (cg.w) {
          // cell list: only the cells of the box around the shifted centre are tested; the
          // accepted atoms are marked in a bitmask and leave in the iterator's cyclic order
          int lo[3], hi[3];
          const float pc[3] = {px, py, pz};
          const int gd[3] = {cg.x, cg.y, cg.z};
          bool empty = false;
          for (int c = 0; c < 3; c++) {
            lo[c] = max(0, (int)floorf((pc[c] - a.rbox) * a.inv_cs));
            hi[c] = min(gd[c] - 1, (int)floorf((pc[c] + a.rbox) * a.inv_cs));
            empty = empty || lo[c] > hi[c];
          }
          if (empty) continue;
          const int nwd = (n + 31) >> 5;
          for (int w = lane; w < nwd; w += 32) bits[w] = 0u;
          __syncwarp();
          // lanes over the (x, y) columns of the box: the cells lo[2]..hi[2] of a column are
          // consecutive in the cell order, so a column's atoms are one contiguous run
          const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1;
          for (int c = lane; c < nx * ny; c += 32) {
            const int cx = lo[0] + c / ny, cy = lo[1] + c % ny;
            const int64_t kcol = cbase + ((int64_t)cx * cg.y + cy) * cg.z;
            const int64_t q0 = a.cstart[kcol + lo[2]], q1 = a.cstart[kcol + hi[2] + 1];
            // the column's atoms are stored contiguously with their positions: two at a time,
            // both loads issued before either test
            for (int64_t q = q0; q < q1; q += 2) {
              const V4<float> pa = a.cpos[q];
              const bool two = q + 1 < q1;
              const V4<float> pb = two ? a.cpos[q + 1] : pa;
              const int ja = (int)__float_as_int(pa.w), jb = (int)__float_as_int(pb.w);
              if (!(ja == il && img < im0) && decide(ja, pa) && FNETG_GUARD(ja >= 0 && ja < n))
                atomicOr(&bits[ja >> 5], 1u << (ja & 31));
              if (two && !(jb == il && img < im0) && decide(jb, pb) &&
                  FNETG_GUARD(jb >= 0 && jb < n))
                atomicOr(&bits[jb >> 5], 1u << (jb & 31));
            }
          }
          __syncwarp();
          // slots of the cyclic order: the start word from the start bit, the other words, the
          // start word below the start bit
          const int start = img < im0 ? (il + 1 == n ? 0 : il + 1) : il;
          const int sw = start >> 5, sb = start & 31;
          const int nslot = nwd + (sb > 0 ? 1 : 0);
          for (int base = 0; base < nslot; base += 32) {
            const int t = base + lane;
            uint32_t m = 0u;
            int widx = 0;
            if (t < nslot) {
              widx = t == nwd ? sw : (sw + t) % nwd;
              m = bits[widx];
              if (t == 0) m &= sb > 0 ? ~((1u << sb) - 1u) : 0xffffffffu;
              else if (t == nwd) m &= (1u << sb) - 1u;
            }
            if (!kFill) {
              int c = __popc(m);
#pragma unroll
              for (int k = 16; k > 0; k >>= 1) c += __shfl_xor_sync(0xffffffffu, c, k);
              cnt += c;
              continue;
            }
            // ranks of the accepted atoms in the cyclic order: the slots' popcounts scanned over
            // the lanes; the pairs join the ring in that order and leave it 32 at a time
            const int pc = __popc(m);
            int off = pc;
#pragma unroll
            for (int k = 1; k < 32; k <<= 1) {
              const int v = __shfl_up_sync(0xffffffffu, off, k);
              if (lane >= k) off += v;
            }
            const int total = __shfl_sync(0xffffffffu, off, 31);
            off -= pc;
            if (qn + total <= kNbQueue) {
              int pos = qh + qn + off;
              for (uint32_t mm = m; mm; mm &= mm - 1u)
                queue[(pos++) & (kNbQueue - 1)] = make_int2(widx * 32 + __ffs(mm) - 1, (int)img);
              qn += total;
              __syncwarp();
              while (qn >= 32) drain32();
            } else {
              // more than the ring holds: the ring's pairs first, then this round's directly
              for (int k = lane; k < qn; k += 32) {
                const int2 e = queue[(qh + k) & (kNbQueue - 1)];
                store_pair<T>(a, ci, cif, cil, i, a0, e.x, e.y, im0, wpos, stored + k);
              }
              __syncwarp();
              stored += qn;
              qh = qn = 0;
              for (uint32_t mm = m; mm; mm &= mm - 1u) {
                store_pair<T>(a, ci, cif, cil, i, a0, widx * 32 + __ffs(mm) - 1, (int)img, im0,
                              wpos, stored + off);
                off++;
              }
              stored += total;
            }
            cnt += total;
          }
          continue;
        }
        auto test = [&](int k, bool &ok, int &jl) {
          ok = false;
          jl = 0;
          if (k < tcount) {
            jl = il + tstart + k;
            if (jl >= n) jl -= n;
            const V4<float> cjf = a.cf[a0 + jl];
            const float e0 = cjf.x - px, e1 = cjf.y - py, e2 = cjf.z - pz;
            const float df = e0 * e0 + e1 * e1 + e2 * e2;
            if (df <= a.rc2_lo) {
              ok = true;
            } else if (df <= a.rc2_hi) {
              // within the float error bound of the cutoff: the reference's FP64 decision
              double d[3];
              ok = exact_pair(a, ci, a0 + jl, img >= im0 ? img : -1, d) <= a.rc2;
            }
          }
        };
        for (int base = 0; base < tcount; base += 64) {
          bool ok0, ok1;
          int j0, j1;
          test(base + lane, ok0, j0);
          test(base + 32 + lane, ok1, j1);
          const unsigned m0 = __ballot_sync(0xffffffffu, ok0), m1 = __ballot_sync(0xffffffffu, ok1);
          const int n0 = __popc(m0), n1 = __popc(m1);
          if (kFill) {
            // queue the accepted candidates in iterator order; store them 32 at a time
            // (at most 31 waiting + 64 new: within the ring)
            const unsigned below = (1u << lane) - 1u;
            const int r0 = qn + __popc(m0 & below), r1 = qn + n0 + __popc(m1 & below);
            if (ok0 && FNETG_GUARD(r0 < kNbQueue))
              queue[(qh + r0) & (kNbQueue - 1)] = make_int2(j0, (int)img);
            if (ok1 && FNETG_GUARD(r1 < kNbQueue))
              queue[(qh + r1) & (kNbQueue - 1)] = make_int2(j1, (int)img);
            qn += n0 + n1;
            __syncwarp();
            while (qn >= 32) drain32();
          }
          cnt += n0 + n1;
        }
      }
    }
    if (kFill && lane < qn) {
      const int2 e = queue[(qh + lane) & (kNbQueue - 1)];
      store_pair<T>(a, ci, cif, cil, i, a0, e.x, e.y, im0, wpos, stored + lane);
    }
    if ((!kFill || a.slab_cap > 0) && lane == 0) {
      a.count[i] = cnt;
      atomicMax(&blk_max, (int)cnt);
      if (kFill) {
        a.pbeg[i] = wpos;
        a.pend[i] = wpos + min(cnt, a.slab_cap);
        if (cnt > a.slab_cap) atomicExch(a.overflow, 1);
        atomicAdd(&blk_sum, (unsigned long long)cnt);
      }
    }
  }
  if (!kFill || a.slab_cap > 0) {
    __syncthreads();
    if (threadIdx.x == 0) {
      atomicMax(a.maxp, blk_max);
      if (kFill) atomicAdd(a.total, blk_sum);
    }
  }
}

// exact squared distances of every stored pair (parity downloads only)
__global__ void pair_d2_kernel(const int64_t *poff, const int64_t *pend, const int32_t *pj,
                               const uint32_t *pmeta, const int32_t *astruct,
                               const double *coords, const double *lat, int64_t natoms,
                               double *d2out) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= natoms) return;
  const double ci[3] = {coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]};
  const double *L = lat + 9 * astruct[i];
  for (int64_t q = poff[i] + lane; q < pend[i]; q += 32) {
    const uint32_t m = pmeta[q];
    const int n1 = (int8_t)(m & 0xff), n2 = (int8_t)((m >> 8) & 0xff), n3 = (int8_t)((m >> 16) & 0xff);
    double cv[3] = {0.0, 0.0, 0.0};
    if (n1 || n2 || n3) cell_vector(L, n1, n2, n3, cv);
    const int64_t j = pj[q];
    const double cj[3] = {coords[3 * j], coords[3 * j + 1], coords[3 * j + 2]};
    double d[3];
    d2out[q] = exact_d2(ci, cj, cv, d);
  }
}

// ---- exclusive scan of int64 (three phases) ----------------------------------------------
constexpr int kScanBlock = 1024;

__global__ void scan_block_kernel(const int64_t *in, int64_t *out, int64_t *sums, int64_t n) {
  __shared__ int64_t sh[kScanBlock];
  const int64_t g = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  int64_t v = g < n ? in[g] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (g < n) out[g] = sh[threadIdx.x] - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void scan_sums_kernel(int64_t *sums, int64_t nb, int64_t *total) {
  // single block: sequential chunks per thread, then a block scan of chunk totals
  __shared__ int64_t sh[kScanBlock];
  const int64_t per = (nb + kScanBlock - 1) / kScanBlock;
  const int64_t b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
  int64_t acc = 0;
  for (int64_t b = b0; b < b1; b++) acc += sums[b];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int64_t run = sh[threadIdx.x] - acc;
  for (int64_t b = b0; b < b1; b++) {
    int64_t v = sums[b];
    sums[b] = run;
    run += v;
  }
  if (threadIdx.x == kScanBlock - 1) *total = sh[threadIdx.x];
}

__global__ void scan_add_kernel(int64_t *out, const int64_t *sums, int64_t n, int64_t *total) {
  const int64_t g = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (g < n) out[g] += sums[blockIdx.x];
  if (g == 0) out[n] = *total;
}

// Float copies of the coordinates relative to each structure's bounding-box corner (the float
// pre-filter's rounding then does not depend on where a structure sits) and the boxes.
__global__ void prep_coords_kernel(const double *coords, const int64_t *off, V4<float> *cf,
                                   V4<float> *cl, float *bbox, int S) {
  __shared__ double lo[3][256], hi[3][256];
  const int s = blockIdx.x;
  if (s >= S) return;
  const int64_t a0 = off[s], a1 = off[s + 1];
  double l[3] = {1e300, 1e300, 1e300}, h[3] = {-1e300, -1e300, -1e300};
  for (int64_t a = a0 + threadIdx.x; a < a1; a += blockDim.x)
    for (int c = 0; c < 3; c++) {
      l[c] = fmin(l[c], coords[3 * a + c]);
      h[c] = fmax(h[c], coords[3 * a + c]);
    }
  for (int c = 0; c < 3; c++) {
    lo[c][threadIdx.x] = l[c];
    hi[c][threadIdx.x] = h[c];
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; c++) {
        lo[c][threadIdx.x] = fmin(lo[c][threadIdx.x], lo[c][threadIdx.x + o]);
        hi[c][threadIdx.x] = fmax(hi[c][threadIdx.x], hi[c][threadIdx.x + o]);
      }
    __syncthreads();
  }
  double ref[3];
  for (int c = 0; c < 3; c++) ref[c] = (double)(float)lo[c][0];
  for (int64_t a = a0 + threadIdx.x; a < a1; a += blockDim.x) {
    // high part = float rounding of the FP64 relative coordinate, low part = float rounding
    // of the remainder: together they hold the relative coordinate to about 2^-48 of itself
    const double r0 = coords[3 * a] - ref[0], r1 = coords[3 * a + 1] - ref[1],
                 r2 = coords[3 * a + 2] - ref[2];
    const float h0 = (float)r0, h1 = (float)r1, h2 = (float)r2;
    cf[a] = V4<float>{h0, h1, h2, 0.f};
    cl[a] = V4<float>{(float)(r0 - (double)h0), (float)(r1 - (double)h1), (float)(r2 - (double)h2),
                      0.f};
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; c++) {
      bbox[6 * s + c] = 0.f;
      bbox[6 * s + 3 + c] = (float)(hi[c][0] - ref[c]);
    }
}

// Per structure: the FP64 bounding-box diagonal sqrt((hi - lo)_x^2 + (hi - lo)_y^2 +
// (hi - lo)_z^2), in that operation order, into a running maximum (the bits of a non-negative
// double order like the value), and a flag for any coordinate that is not finite.
__global__ void coords_summary_kernel(const double *coords, const int64_t *off, int S,
                                      unsigned long long *max_bits, int *nonfinite) {
  __shared__ double lo[3][256], hi[3][256];
  __shared__ int bad;
  const int s = blockIdx.x;
  if (s >= S) return;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int64_t a0 = off[s], a1 = off[s + 1];
  double l[3] = {1e300, 1e300, 1e300}, h[3] = {-1e300, -1e300, -1e300};
  bool fin = true;
  for (int64_t a = a0 + threadIdx.x; a < a1; a += blockDim.x)
    for (int c = 0; c < 3; c++) {
      const double x = coords[3 * a + c];
      fin = fin && isfinite(x);
      l[c] = fmin(l[c], x);
      h[c] = fmax(h[c], x);
    }
  if (!fin) atomicOr(&bad, 1);
  for (int c = 0; c < 3; c++) {
    lo[c][threadIdx.x] = l[c];
    hi[c][threadIdx.x] = h[c];
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; c++) {
        lo[c][threadIdx.x] = fmin(lo[c][threadIdx.x], lo[c][threadIdx.x + o]);
        hi[c][threadIdx.x] = fmax(hi[c][threadIdx.x], hi[c][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (bad) atomicOr(nonfinite, 1);
    if (a1 > a0) {
      const double d0 = hi[0][0] - lo[0][0], d1 = hi[1][0] - lo[1][0], d2 = hi[2][0] - lo[2][0];
      const double e =
          sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
      atomicMax(max_bits, (unsigned long long)__double_as_longlong(e));
    }
  }
}

// Cell grid of every structure that uses one: edge 1 / inv_cs over its bounding box (relative
// float frame), at most kCellDimMax cells per axis.
__global__ void cell_grid_kernel(const float *bbox, const int64_t *off, int S, float inv_cs,
                                 int4 *cgrid, int64_t *ncell) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int64_t n = off[s + 1] - off[s];
  const bool on = n >= kCellMin && n <= kCellMaxAtoms;
  int g[3] = {0, 0, 0};
  if (on)
    for (int c = 0; c < 3; c++)
      g[c] = min(kCellDimMax, max(1, (int)(bbox[6 * s + 3 + c] * inv_cs) + 1));
  cgrid[s] = make_int4(g[0], g[1], g[2], on ? 1 : 0);
  ncell[s] = on ? (int64_t)g[0] * g[1] * g[2] : 0;
}

__device__ __forceinline__ int64_t cell_key(const V4<float> &p, const int4 &g, int64_t base,
                                            float inv_cs) {
  const int cx = min(g.x - 1, max(0, (int)floorf(p.x * inv_cs)));
  const int cy = min(g.y - 1, max(0, (int)floorf(p.y * inv_cs)));
  const int cz = min(g.z - 1, max(0, (int)floorf(p.z * inv_cs)));
  return base + ((int64_t)cx * g.y + cy) * g.z + cz;
}

__global__ void cell_count_kernel(const V4<float> *cf, const int32_t *astruct, int64_t N,
                                  const int4 *cgrid, const int64_t *coff, float inv_cs,
                                  int64_t *akey, int64_t *ccount) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const int s = astruct[a];
  const int4 g = cgrid[s];
  if (!g.w) {
    akey[a] = -1;
    return;
  }
  const int64_t key = cell_key(cf[a], g, coff[s], inv_cs);
  akey[a] = key;
  atomicAdd(reinterpret_cast<unsigned long long *>(ccount + key), 1ull);
}

__global__ void cell_fill_kernel(const int64_t *akey, const int32_t *astruct, const int64_t *off,
                                 int64_t N, const int64_t *cstart, int64_t *cfill,
                                 const V4<float> *cf, V4<float> *cpos) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const int64_t key = akey[a];
  if (key < 0) return;
  const int64_t pos =
      cstart[key] + (int64_t)atomicAdd(reinterpret_cast<unsigned long long *>(cfill + key), 1ull);
  V4<float> p = cf[a];
  p.w = __int_as_float((int)(a - off[astruct[a]]));
  cpos[pos] = p;
}

}  // namespace

// Cell lists of the structures with kCellMin..kCellMaxAtoms atoms for the given cutoff (cells of
// half the cutoff): counted, scanned and filled on the device.
int build_cells(fnetg_ctx *ctx, double rcut, float &inv_cs) {
  const int S = ctx->S;
  const int64_t N = ctx->N;
  inv_cs = (float)(2.0 / rcut);
  FNETG_CUDA(ctx->d_cgrid.ensure(sizeof(int4) * std::max(S, 1)));
  FNETG_CUDA(ctx->d_cnum.ensure(sizeof(int64_t) * std::max(S, 1)));
  FNETG_CUDA(ctx->d_coff.ensure(sizeof(int64_t) * (S + 1)));
  if (S == 0) return FNETG_OK;
  {
    LaunchScope ls(ctx, "neighbors");
    cell_grid_kernel<<<ceil_div(S, 128), 128, 0, ctx->stream>>>(
        ctx->d_bbox.as<float>(), ctx->d_off.as<int64_t>(), S, inv_cs, ctx->d_cgrid.as<int4>(),
        ctx->d_cnum.as<int64_t>());
    FNETG_CUDA(cudaGetLastError());
  }
  int rc = exclusive_scan_i64(ctx, ctx->d_cnum.as<int64_t>(), ctx->d_coff.as<int64_t>(), S);
  if (rc) return rc;
  int64_t ncells = 0;
  FNETG_CUDA(copy_sync(ctx, &ncells, ctx->d_coff.as<int64_t>() + S, sizeof(int64_t),
                        cudaMemcpyDeviceToHost));
  FNETG_CUDA(ctx->d_ccount.ensure(sizeof(int64_t) * std::max<int64_t>(ncells, 1)));
  FNETG_CUDA(ctx->d_cstart.ensure(sizeof(int64_t) * (ncells + 1)));
  FNETG_CUDA(ctx->d_cfill.ensure(sizeof(int64_t) * std::max<int64_t>(ncells, 1)));
  FNETG_CUDA(ctx->d_akey.ensure(sizeof(int64_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_cpos.ensure(sizeof(V4<float>) * std::max<int64_t>(N, 1)));
  if (ncells == 0 || N == 0) {
    ctx->ncells = 0;
    return FNETG_OK;
  }
  FNETG_CUDA(cudaMemsetAsync(ctx->d_ccount.p, 0, sizeof(int64_t) * ncells, ctx->stream));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_cfill.p, 0, sizeof(int64_t) * ncells, ctx->stream));
  {
    LaunchScope ls(ctx, "neighbors");
    cell_count_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(
        ctx->d_coordsf.as<V4<float>>(), ctx->d_atom_struct.as<int32_t>(), N,
        ctx->d_cgrid.as<int4>(), ctx->d_coff.as<int64_t>(), inv_cs, ctx->d_akey.as<int64_t>(),
        ctx->d_ccount.as<int64_t>());
    FNETG_CUDA(cudaGetLastError());
  }
  rc = exclusive_scan_i64(ctx, ctx->d_ccount.as<int64_t>(), ctx->d_cstart.as<int64_t>(), ncells);
  if (rc) return rc;
  {
    LaunchScope ls(ctx, "neighbors");
    cell_fill_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(
        ctx->d_akey.as<int64_t>(), ctx->d_atom_struct.as<int32_t>(), ctx->d_off.as<int64_t>(), N,
        ctx->d_cstart.as<int64_t>(), ctx->d_cfill.as<int64_t>(), ctx->d_coordsf.as<V4<float>>(),
        ctx->d_cpos.as<V4<float>>());
    FNETG_CUDA(cudaGetLastError());
  }
  ctx->ncells = ncells;
  return FNETG_OK;
}

int prepare_coords(fnetg_ctx *ctx) {
  if (ctx->S == 0) return FNETG_OK;
  LaunchScope ls(ctx, "coords");
  prep_coords_kernel<<<ctx->S, 256, 0, ctx->stream>>>(
      ctx->d_coords.as<double>(), ctx->d_off.as<int64_t>(), ctx->d_coordsf.as<V4<float>>(),
      ctx->d_coordsf.as<V4<float>>() + std::max<int64_t>(ctx->N, 1), ctx->d_bbox.as<float>(),
      ctx->S);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

int coords_summary(fnetg_ctx *ctx, const double *d_xyz, double *max_extent, bool *nonfinite) {
  *max_extent = 0.0;
  *nonfinite = false;
  if (ctx->S == 0 || ctx->N == 0) return FNETG_OK;
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(ctx->d_scalars.p) + 8;
  FNETG_CUDA(cudaMemsetAsync(acc, 0, 16, ctx->stream));
  {
    LaunchScope ls(ctx, "coords");
    coords_summary_kernel<<<ctx->S, 256, 0, ctx->stream>>>(
        d_xyz, ctx->d_off.as<int64_t>(), ctx->S, acc, reinterpret_cast<int *>(acc + 1));
    FNETG_CUDA(cudaGetLastError());
  }
  unsigned long long h[2] = {0, 0};
  FNETG_CUDA(cudaMemcpyAsync(h, acc, 16, cudaMemcpyDeviceToHost, ctx->stream));
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(max_extent, &h[0], sizeof(double));
  *nonfinite = (h[1] & 0xffffffffull) != 0;
  return FNETG_OK;
}

// out has n+1 entries (out[n] = total)
int exclusive_scan_i64(fnetg_ctx *ctx, const int64_t *in, int64_t *out, int64_t n) {
  const int64_t nb = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  FNETG_CUDA(ctx->d_scan_tmp.ensure(sizeof(int64_t) * (nb + 2)));
  int64_t *sums = ctx->d_scan_tmp.as<int64_t>();
  int64_t *total = sums + nb + 1;
  {
    LaunchScope ls(ctx, "scan");
    scan_block_kernel<<<nb, kScanBlock, 0, ctx->stream>>>(in, out, sums, n);
  }
  {
    LaunchScope ls(ctx, "scan");
    scan_sums_kernel<<<1, kScanBlock, 0, ctx->stream>>>(sums, nb, total);
  }
  {
    LaunchScope ls(ctx, "scan");
    scan_add_kernel<<<nb, kScanBlock, 0, ctx->stream>>>(out, sums, n, total);
  }
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

int run_neighbors(fnetg_ctx *ctx, double rcut) {
  const int64_t N = ctx->N;
  const int S = ctx->S;
  FNETG_CHECK(rcut > 0.0, FNETG_E_INVALID, "neighbour cutoff must be > 0");
  // the lattice-point tables and the cutoff-class uploads depend on the lattices, periodic
  // flags, cutoff and cutoff classes only: rebuilt when one of them changed
  const bool reuse = ctx->nbimg_valid && ctx->nbimg_rcut == rcut && ctx->nbimg_lat == ctx->h_lat &&
                     ctx->nbimg_periodic == ctx->h_periodic && ctx->nbimg_rcls == ctx->rcut_classes;
  if (!reuse) {
    ctx->nbimg_valid = false;
    std::vector<int32_t> ranges((size_t)6 * std::max(S, 1), 0);
    for (int s = 0; s < S; s++) {
      if (!ctx->h_periodic[s]) continue;
      if (fnetg_lattice_ranges(ctx->h_lat.data() + 9 * s, rcut, ranges.data() + 6 * s))
        return fail(ctx, FNETG_E_GEOMETRY, "dependent lattice vectors");
      for (int c = 0; c < 6; c++)
        FNETG_CHECK(std::abs(ranges[6 * s + c]) <= 127, FNETG_E_UNSUPPORTED,
                    "more than 127 periodic images along a lattice vector");
    }
    // lattice points of every structure in the iterator's order (latpointiter.F90:121-174,
    // origin excluded) with the cell vector matmul(latVecs, n) summed in index order
    std::vector<int64_t> img_off(S + 1, 0);
    std::vector<V4<double>> imgs;
    std::vector<V4<float>> imgs_f;
    for (int s = 0; s < S; s++) {
      img_off[s] = (int64_t)imgs.size();
      if (!ctx->h_periodic[s]) continue;
      const int32_t *r = ranges.data() + 6 * s;
      const double *L = ctx->h_lat.data() + 9 * s;
      for (int n1 = r[0]; n1 <= r[1]; n1++)
        for (int n2 = r[2]; n2 <= r[3]; n2++)
          for (int n3 = r[4]; n3 <= r[5]; n3++) {
            if (n1 == 0 && n2 == 0 && n3 == 0) continue;
            double cv[3];
            for (int c = 0; c < 3; c++) {
              double v = L[c + 0] * (double)n1;
              v = v + L[c + 3] * (double)n2;
              v = v + L[c + 6] * (double)n3;
              cv[c] = v;
            }
            const uint64_t packed = (uint64_t)((uint32_t)(uint8_t)(int8_t)n1 |
                                               ((uint32_t)(uint8_t)(int8_t)n2 << 8) |
                                               ((uint32_t)(uint8_t)(int8_t)n3 << 16));
            double w;
            std::memcpy(&w, &packed, sizeof w);
            imgs.push_back(V4<double>{cv[0], cv[1], cv[2], w});
            float h[3], l[3];
            for (int c = 0; c < 3; c++) {
              h[c] = (float)cv[c];
              l[c] = (float)(cv[c] - (double)h[c]);
            }
            float pw;
            const uint32_t p32 = (uint32_t)packed;
            std::memcpy(&pw, &p32, sizeof pw);
            imgs_f.push_back(V4<float>{h[0], h[1], h[2], pw});
            imgs_f.push_back(V4<float>{l[0], l[1], l[2], 0.f});
          }
    }
    img_off[S] = (int64_t)imgs.size();
    FNETG_CUDA(ctx->d_img_off.ensure(sizeof(int64_t) * (S + 1)));
    FNETG_CUDA(ctx->d_imgs.ensure(sizeof(V4<double>) * std::max<size_t>(imgs.size(), 1)));
    FNETG_CUDA(ctx->d_imgs_f.ensure(sizeof(V4<float>) * std::max<size_t>(imgs_f.size(), 1)));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_img_off.p, img_off.data(), sizeof(int64_t) * (S + 1),
                               cudaMemcpyHostToDevice, ctx->stream));
    if (!imgs.empty()) {
      FNETG_CUDA(cudaMemcpyAsync(ctx->d_imgs.p, imgs.data(), sizeof(V4<double>) * imgs.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
      FNETG_CUDA(cudaMemcpyAsync(ctx->d_imgs_f.p, imgs_f.data(), sizeof(V4<float>) * imgs_f.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    }
    // cutoff classes must contain the search cutoff's membership for the G-functions
    FNETG_CUDA(ctx->d_rcls.ensure(sizeof(double) * kMaxRcutClasses));
    if (!ctx->rcut_classes.empty())
      FNETG_CUDA(cudaMemcpyAsync(ctx->d_rcls.p, ctx->rcut_classes.data(),
                                 sizeof(double) * ctx->rcut_classes.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    // the farthest image translation over all structures
    double shift_max = 0.0;
    for (int s = 0; s < S; s++) {
      double shift = 0.0;
      if (ctx->h_periodic[s]) {
        for (int k = 0; k < 3; k++) {
          const double *col = ctx->h_lat.data() + 9 * s + 3 * k;
          const double len = std::sqrt(col[0] * col[0] + col[1] * col[1] + col[2] * col[2]);
          const int nmax = std::max(std::abs(ranges[6 * s + 2 * k]), std::abs(ranges[6 * s + 2 * k + 1]));
          shift += len * nmax;
        }
      }
      shift_max = std::max(shift_max, shift);
    }
    ctx->nbimg_shift = shift_max;
    ctx->nbimg_rcut = rcut;
    ctx->nbimg_lat = ctx->h_lat;
    ctx->nbimg_periodic = ctx->h_periodic;
    ctx->nbimg_rcls = ctx->rcut_classes;
    ctx->nbimg_valid = true;
  }
  FNETG_CUDA(ctx->d_pcount.ensure(sizeof(int64_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_poff.ensure(sizeof(int64_t) * (N + 1)));
  FNETG_CUDA(ctx->d_maxp.ensure(sizeof(int) * 4));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_maxp.p, 0, sizeof(int) * 4, ctx->stream));
  const std::vector<double> &rcls = ctx->rcut_classes;
  NbArgs a{};
  a.off = ctx->d_off.as<int64_t>();
  a.astruct = ctx->d_atom_struct.as<int32_t>();
  a.coords = ctx->d_coords.as<double>();
  a.cf = ctx->d_coordsf.as<V4<float>>();
  a.cl = ctx->d_coordsf.as<V4<float>>() + std::max<int64_t>(N, 1);
  a.imgf = ctx->d_imgs_f.as<V4<float>>();
  a.img_off = ctx->d_img_off.as<int64_t>();
  a.imgs = ctx->d_imgs.as<V4<double>>();
  a.bbox = ctx->d_bbox.as<float>();
  a.natoms = N;
  a.rc2 = rcut * rcut;
  // Float error bound of the pre-filter: coordinates relative to each structure's box corner
  // are at most `reach` in magnitude (box extent plus the farthest image translation); each of
  // the few float roundings of a component difference is below 2^-23 * reach, so the squared
  // distance is off by less than 8 * 2^-23 * reach * rcut + 2^-20 * rcut^2.
  const double reach = ctx->nbimg_shift + ctx->max_extent + rcut;
  auto margin = [&](double rc) { return 16.0 * 1.2e-7 * reach * rc + 1e-6 * rc * rc + 1e-6; };
  a.rc2_lo = (float)(rcut * rcut - margin(rcut));
  a.rc2_hi = (float)(rcut * rcut + margin(rcut));
  std::vector<float> rlo(kMaxRcutClasses, 0.f), rhi(kMaxRcutClasses, 0.f);
  for (size_t c = 0; c < rcls.size(); c++) {
    rlo[c] = (float)(rcls[c] * rcls[c] - margin(rcls[c]));
    rhi[c] = (float)(rcls[c] * rcls[c] + margin(rcls[c]));
  }
  FNETG_CUDA(ctx->d_rcls2.ensure(sizeof(float) * 2 * kMaxRcutClasses));
  FNETG_CUDA(cudaMemcpyAsync(ctx->d_rcls2.p, rlo.data(), sizeof(float) * kMaxRcutClasses,
                             cudaMemcpyHostToDevice, ctx->stream));
  FNETG_CUDA(cudaMemcpyAsync(ctx->d_rcls2.as<float>() + kMaxRcutClasses, rhi.data(),
                             sizeof(float) * kMaxRcutClasses, cudaMemcpyHostToDevice, ctx->stream));
  a.rcls = ctx->d_rcls.as<double>();
  a.rcls2_lo = ctx->d_rcls2.as<float>();
  a.rcls2_hi = ctx->d_rcls2.as<float>() + kMaxRcutClasses;
  a.nrcls = (int)rcls.size();
  a.exact_geometry = ctx->prec == FNETG_FP64 ? 1 : 0;
  a.count = ctx->d_pcount.as<int64_t>();
  a.maxp = ctx->d_maxp.as<int>();
  // cell lists (the candidate boxes reach past the float pre-filter's outer bound)
  {
    float inv_cs = 0.f;
    int rc = build_cells(ctx, rcut, inv_cs);
    if (rc) return rc;
    a.cgrid = ctx->ncells > 0 ? ctx->d_cgrid.as<int4>() : nullptr;
    a.coff = ctx->d_coff.as<int64_t>();
    a.cstart = ctx->d_cstart.as<int64_t>();
    a.cpos = ctx->d_cpos.as<V4<float>>();
    a.inv_cs = inv_cs;
    a.rbox = (float)(std::sqrt((double)a.rc2_hi) * (1.0 + 1e-5) + 1e-5);
  }
  const int threads = kNbWarps * 32, wpb = kNbWarps;
  const int blocks = std::max(1, ceil_div(N, wpb));
  const size_t es = ctx->prec == FNETG_FP64 ? 8 : 4;
  // Slab pass: with a per-atom capacity from the previous build of this dataset, one pass
  // finds, counts and stores the pairs; an atom beyond the capacity sends the build down the
  // counted path below.
  if (N > 0 && ctx->nb_cap_hint > 0 && ctx->nb_hint_n == N) {
    const int64_t cap = ctx->nb_cap_hint, slots = N * cap;
    FNETG_CUDA(ctx->d_pj.ensure(sizeof(int32_t) * slots));
    FNETG_CUDA(ctx->d_pmeta.ensure(sizeof(uint32_t) * slots));
    FNETG_CUDA(ctx->d_rij.ensure(4 * es * slots));
    FNETG_CUDA(ctx->d_pend.ensure(sizeof(int64_t) * N));
    a.slab_cap = cap;
    a.nslots = slots;
    a.poff = nullptr;
    a.pbeg = ctx->d_poff.as<int64_t>();
    a.pend = ctx->d_pend.as<int64_t>();
    a.overflow = ctx->d_maxp.as<int>() + 1;
    a.total = reinterpret_cast<unsigned long long *>(ctx->d_maxp.as<int>() + 2);
    a.pj = ctx->d_pj.as<int32_t>();
    a.pmeta = ctx->d_pmeta.as<uint32_t>();
    a.rij = ctx->d_rij.p;
    a.d2out = nullptr;
    {
      LaunchScope ls(ctx, "neighbors");
      if (ctx->prec == FNETG_FP64)
        nb_kernel<double, true><<<blocks, threads, 0, ctx->stream>>>(a);
      else
        nb_kernel<float, true><<<blocks, threads, 0, ctx->stream>>>(a);
      FNETG_CUDA(cudaGetLastError());
    }
    int flags[4] = {0, 0, 0, 0};
    FNETG_CUDA(cudaMemcpyAsync(flags, ctx->d_maxp.p, sizeof(int) * 4, cudaMemcpyDeviceToHost,
                               ctx->stream));
    FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (flags[1] == 0) {
      unsigned long long total = 0;
      std::memcpy(&total, flags + 2, sizeof total);
      ctx->P = (int64_t)total;
      ctx->pslots = slots;
      ctx->pslab = true;
      ctx->d2_valid = false;
      ctx->max_pairs = flags[0];
      ctx->nb_rcut = rcut;
      ctx->nb_valid = true;
      ctx->feats_valid = false;
      ctx->mom_valid = false;
      return FNETG_OK;
    }
    FNETG_CUDA(cudaMemsetAsync(ctx->d_maxp.p, 0, sizeof(int) * 4, ctx->stream));
    a.slab_cap = 0;
  }
  if (N > 0) {
    LaunchScope ls(ctx, "neighbors");
    if (ctx->prec == FNETG_FP64)
      nb_kernel<double, false><<<blocks, threads, 0, ctx->stream>>>(a);
    else
      nb_kernel<float, false><<<blocks, threads, 0, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  int rc = exclusive_scan_i64(ctx, a.count, ctx->d_poff.as<int64_t>(), N);
  if (rc) return rc;
  int64_t P = 0;
  int maxp = 0;
  FNETG_CUDA(cudaMemcpyAsync(&P, ctx->d_poff.as<int64_t>() + N, sizeof(int64_t),
                             cudaMemcpyDeviceToHost, ctx->stream));
  FNETG_CUDA(cudaMemcpyAsync(&maxp, ctx->d_maxp.p, sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream));
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (N == 0) P = 0;
  FNETG_CUDA(ctx->d_pj.ensure(sizeof(int32_t) * std::max<int64_t>(P, 1)));
  FNETG_CUDA(ctx->d_pmeta.ensure(sizeof(uint32_t) * std::max<int64_t>(P, 1)));
  FNETG_CUDA(ctx->d_rij.ensure(4 * es * std::max<int64_t>(P, 1)));
  a.poff = ctx->d_poff.as<int64_t>();
  a.nslots = P;
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = ctx->d_rij.p;
  a.d2out = nullptr;
  if (N > 0 && P > 0) {
    LaunchScope ls(ctx, "neighbors");
    if (ctx->prec == FNETG_FP64)
      nb_kernel<double, true><<<blocks, threads, 0, ctx->stream>>>(a);
    else
      nb_kernel<float, true><<<blocks, threads, 0, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  ctx->P = P;
  ctx->pslots = P;
  ctx->pslab = false;
  // capacity for the next build of this dataset: an eighth above the largest count
  ctx->nb_cap_hint = N > 0 ? ((int64_t)maxp + maxp / 8 + 8 + 7) / 8 * 8 : 0;
  ctx->nb_hint_n = N;
  ctx->d2_valid = false;
  ctx->max_pairs = maxp;
  ctx->nb_rcut = rcut;
  ctx->nb_valid = true;
  ctx->feats_valid = false;
  ctx->mom_valid = false;
  return FNETG_OK;
}

const int64_t *pair_end(fnetg_ctx *ctx) {
  return ctx->pslab ? ctx->d_pend.as<int64_t>() : ctx->d_poff.as<int64_t>() + 1;
}

int pair_d2(fnetg_ctx *ctx) {
  if (ctx->d2_valid) return FNETG_OK;
  FNETG_CUDA(ctx->d_d2.ensure(sizeof(double) * std::max<int64_t>(ctx->pslots, 1)));
  if (ctx->N > 0 && ctx->P > 0) {
    LaunchScope ls(ctx, "neighbors");
    pair_d2_kernel<<<ceil_div(ctx->N, 8), 256, 0, ctx->stream>>>(
        ctx->d_poff.as<int64_t>(), pair_end(ctx), ctx->d_pj.as<int32_t>(),
        ctx->d_pmeta.as<uint32_t>(),
        ctx->d_atom_struct.as<int32_t>(), ctx->d_coords.as<double>(), ctx->d_lat.as<double>(),
        ctx->N, ctx->d_d2.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  ctx->d2_valid = true;
  return FNETG_OK;
}

FNETG_CHECK_READER(check_site_neighbors)

}  // namespace fnetg
