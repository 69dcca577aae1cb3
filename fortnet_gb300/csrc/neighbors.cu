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
#include <algorithm>

#include "internal.cuh"

int fnetg_lattice_ranges(const double *L, double rcut, int32_t *lohi);

namespace fnetg {

namespace {

struct NbArgs {
  const int64_t *off;
  const int32_t *astruct;
  const double *coords;
  const V4<float> *cf;
  const double *lat;
  const int32_t *ranges;  // [S*6] lo0,hi0,lo1,hi1,lo2,hi2 (periodic) — zeros otherwise
  const int32_t *periodic;
  const float *bbox;      // [S*6] lo, hi
  int64_t natoms;
  double rc2;             // rcut*rcut (exact decision)
  float rc2_filter;       // generous float bound for the pre-filter
  float rc_filter;
  const double *rcls;     // cutoff classes (ascending)
  int nrcls;
  // fill pass
  const int64_t *poff;
  int64_t *count;
  int32_t *pj;
  uint32_t *pmeta;
  void *rij;              // V4<T>
  double *d2out;
  int *maxp;
};

__device__ __forceinline__ double exact_d2(const double *ci, const double *cj, const double *cv,
                                           double *d) {
  double nc0 = __dadd_rn(cj[0], cv[0]);
  double nc1 = __dadd_rn(cj[1], cv[1]);
  double nc2 = __dadd_rn(cj[2], cv[2]);
  d[0] = __dsub_rn(nc0, ci[0]);  // neighbour - centre (sign irrelevant for d2)
  d[1] = __dsub_rn(nc1, ci[1]);
  d[2] = __dsub_rn(nc2, ci[2]);
  double e0 = __dsub_rn(ci[0], nc0), e1 = __dsub_rn(ci[1], nc1), e2 = __dsub_rn(ci[2], nc2);
  double s = __dmul_rn(e0, e0);
  s = __dadd_rn(s, __dmul_rn(e1, e1));
  s = __dadd_rn(s, __dmul_rn(e2, e2));
  return s;
}

template <typename T, bool kFill>
__global__ void __launch_bounds__(256) nb_kernel(NbArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= a.natoms) return;
  const int s = a.astruct[i];
  const int64_t a0 = a.off[s];
  const int n = (int)(a.off[s + 1] - a0);
  const int il = (int)(i - a0);
  double ci[3] = {a.coords[3 * i], a.coords[3 * i + 1], a.coords[3 * i + 2]};
  const V4<float> cif = a.cf[i];
  int64_t wpos = 0;
  if (kFill) wpos = a.poff[i];
  int64_t cnt = 0;
  const bool per = a.periodic[s] != 0;
  int lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0, lo2 = 0, hi2 = 0;
  if (per) {
    lo0 = a.ranges[6 * s + 0]; hi0 = a.ranges[6 * s + 1];
    lo1 = a.ranges[6 * s + 2]; hi1 = a.ranges[6 * s + 3];
    lo2 = a.ranges[6 * s + 4]; hi2 = a.ranges[6 * s + 5];
  }
  const double *L = a.lat + 9 * s;
  const float *bb = a.bbox + 6 * s;
  // image index -1 is the central cell
  const int n1span = hi0 - lo0 + 1, n2span = hi1 - lo1 + 1, n3span = hi2 - lo2 + 1;
  const int nimg = per ? n1span * n2span * n3span : 0;
  for (int img = -1; img < nimg; img++) {
    int n1 = 0, n2 = 0, n3 = 0;
    double cv[3] = {0.0, 0.0, 0.0};
    int tstart = 1, tcount = n - 1;
    if (img >= 0) {
      n1 = lo0 + img / (n2span * n3span);
      n2 = lo1 + (img / n3span) % n2span;
      n3 = lo2 + img % n3span;
      if (n1 == 0 && n2 == 0 && n3 == 0) continue;
      for (int c = 0; c < 3; c++) {
        double v = __dmul_rn(L[c + 0], (double)n1);
        v = __dadd_rn(v, __dmul_rn(L[c + 3], (double)n2));
        v = __dadd_rn(v, __dmul_rn(L[c + 6], (double)n3));
        cv[c] = v;
      }
      tstart = 0;
      tcount = n;
      // prune the whole image when the shifted bounding box is out of reach
      float dd = 0.f;
      const float cvf[3] = {(float)cv[0], (float)cv[1], (float)cv[2]};
      const float p[3] = {cif.x, cif.y, cif.z};
      for (int c = 0; c < 3; c++) {
        float lo = bb[c] + cvf[c], hi = bb[3 + c] + cvf[c];
        float e = p[c] < lo ? lo - p[c] : (p[c] > hi ? p[c] - hi : 0.f);
        dd += e * e;
      }
      if (dd > a.rc2_filter) continue;
    }
    const float cvf0 = (float)cv[0], cvf1 = (float)cv[1], cvf2 = (float)cv[2];
    for (int base = 0; base < tcount; base += 32) {
      const int t = tstart + base + lane;
      bool ok = false;
      double d[3] = {0, 0, 0}, dist2 = 0.0;
      int64_t j = 0;
      if (base + lane < tcount) {
        j = a0 + (il + t) % n;
        const V4<float> cjf = a.cf[j];
        float e0 = cif.x - (cjf.x + cvf0), e1 = cif.y - (cjf.y + cvf1), e2 = cif.z - (cjf.z + cvf2);
        float df = e0 * e0 + e1 * e1 + e2 * e2;
        if (df <= a.rc2_filter) {
          double cj[3] = {a.coords[3 * j], a.coords[3 * j + 1], a.coords[3 * j + 2]};
          dist2 = exact_d2(ci, cj, cv, d);
          ok = dist2 <= a.rc2;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, ok);
      if (kFill && ok) {
        const int64_t q = wpos + cnt + __popc(m & ((1u << lane) - 1u));
        a.pj[q] = (int32_t)j;
        uint32_t mask = 0;
        for (int c = 0; c < a.nrcls; c++)
          if (dist2 <= __dmul_rn(a.rcls[c], a.rcls[c])) mask |= 1u << c;
        a.pmeta[q] = ((uint32_t)(uint8_t)(int8_t)n1) | ((uint32_t)(uint8_t)(int8_t)n2 << 8) |
                     ((uint32_t)(uint8_t)(int8_t)n3 << 16) | (mask << 24);
        V4<T> v;
        v.x = (T)d[0];
        v.y = (T)d[1];
        v.z = (T)d[2];
        v.w = (T)sqrt(dist2);
        reinterpret_cast<V4<T> *>(a.rij)[q] = v;
        a.d2out[q] = dist2;
      }
      cnt += __popc(m);
    }
  }
  if (!kFill && lane == 0) {
    a.count[i] = cnt;
    atomicMax(a.maxp, (int)cnt);
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

}  // namespace

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
  std::vector<int32_t> ranges((size_t)6 * std::max(S, 1), 0);
  for (int s = 0; s < S; s++) {
    if (!ctx->h_periodic[s]) continue;
    if (fnetg_lattice_ranges(ctx->h_lat.data() + 9 * s, rcut, ranges.data() + 6 * s))
      return fail(ctx, FNETG_E_GEOMETRY, "dependent lattice vectors");
    for (int c = 0; c < 6; c++)
      FNETG_CHECK(std::abs(ranges[6 * s + c]) <= 127, FNETG_E_UNSUPPORTED,
                  "more than 127 periodic images along a lattice vector");
  }
  FNETG_CUDA(ctx->d_ranges.ensure(sizeof(int32_t) * ranges.size()));
  FNETG_CUDA(cudaMemcpyAsync(ctx->d_ranges.p, ranges.data(), sizeof(int32_t) * ranges.size(),
                             cudaMemcpyHostToDevice, ctx->stream));
  FNETG_CUDA(ctx->d_pcount.ensure(sizeof(int64_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_poff.ensure(sizeof(int64_t) * (N + 1)));
  FNETG_CUDA(ctx->d_maxp.ensure(sizeof(int) * 4));
  FNETG_CUDA(cudaMemsetAsync(ctx->d_maxp.p, 0, sizeof(int) * 4, ctx->stream));
  // cutoff classes must contain the search cutoff's membership for the G-functions
  std::vector<double> rcls = ctx->rcut_classes;
  FNETG_CUDA(ctx->d_rcls.ensure(sizeof(double) * kMaxRcutClasses));
  if (!rcls.empty())
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_rcls.p, rcls.data(), sizeof(double) * rcls.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  NbArgs a{};
  a.off = ctx->d_off.as<int64_t>();
  a.astruct = ctx->d_atom_struct.as<int32_t>();
  a.coords = ctx->d_coords.as<double>();
  a.cf = ctx->d_coordsf.as<V4<float>>();
  a.lat = ctx->d_lat.as<double>();
  a.ranges = ctx->d_ranges.as<int32_t>();
  a.periodic = ctx->d_periodic.as<int32_t>();
  a.bbox = ctx->d_bbox.as<float>();
  a.natoms = N;
  a.rc2 = rcut * rcut;
  // float pre-filter bound: generous relative and absolute margins over the exact bound
  const double rcf = rcut * (1.0 + 1e-4) + 1e-3;
  a.rc2_filter = (float)(rcf * rcf);
  a.rc_filter = (float)rcf;
  a.rcls = ctx->d_rcls.as<double>();
  a.nrcls = (int)rcls.size();
  a.count = ctx->d_pcount.as<int64_t>();
  a.maxp = ctx->d_maxp.as<int>();
  const int threads = 256, wpb = threads / 32;
  const int blocks = std::max(1, ceil_div(N, wpb));
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
  const size_t es = ctx->prec == FNETG_FP64 ? 8 : 4;
  FNETG_CUDA(ctx->d_pj.ensure(sizeof(int32_t) * std::max<int64_t>(P, 1)));
  FNETG_CUDA(ctx->d_pmeta.ensure(sizeof(uint32_t) * std::max<int64_t>(P, 1)));
  FNETG_CUDA(ctx->d_rij.ensure(4 * es * std::max<int64_t>(P, 1)));
  FNETG_CUDA(ctx->d_d2.ensure(sizeof(double) * std::max<int64_t>(P, 1)));
  a.poff = ctx->d_poff.as<int64_t>();
  a.pj = ctx->d_pj.as<int32_t>();
  a.pmeta = ctx->d_pmeta.as<uint32_t>();
  a.rij = ctx->d_rij.p;
  a.d2out = ctx->d_d2.as<double>();
  if (N > 0 && P > 0) {
    LaunchScope ls(ctx, "neighbors");
    if (ctx->prec == FNETG_FP64)
      nb_kernel<double, true><<<blocks, threads, 0, ctx->stream>>>(a);
    else
      nb_kernel<float, true><<<blocks, threads, 0, ctx->stream>>>(a);
    FNETG_CUDA(cudaGetLastError());
  }
  ctx->P = P;
  ctx->max_pairs = maxp;
  ctx->nb_rcut = rcut;
  ctx->nb_valid = true;
  ctx->feats_valid = false;
  return FNETG_OK;
}

}  // namespace fnetg
