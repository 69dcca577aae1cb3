// Context management and the C-ABI entry points of libfnetg.
#include <algorithm>
#include <tuple>
#include <cstdio>
#include <array>
#include <set>

#include <mutex>

#include "internal.cuh"

using namespace fnetg;

namespace fnetg {

int fail(fnetg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(fnetg_ctx *c, cudaError_t e, const char *where) {
  char buf[512];
  snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), where);
  if (c) c->err = buf;
  return e == cudaErrorMemoryAllocation ? FNETG_E_NOMEM : FNETG_E_CUDA;
}

int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

cudaError_t raise_smem_limit(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{dev, kernel}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

static cudaEvent_t pool_event(fnetg_ctx *c) {
  if (c->ev_free.empty()) {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t e = c->ev_free.back();
  c->ev_free.pop_back();
  return e;
}

LaunchScope::LaunchScope(fnetg_ctx *ctx, const char *n) : c(ctx), name(n) {
  c->launches++;
  if (c->prof) {
    e0 = pool_event(c);
    cudaEventRecord(e0, c->stream);
  }
}

LaunchScope::~LaunchScope() {
  if (!c->prof) return;
  cudaEvent_t e1 = pool_event(c);
  cudaEventRecord(e1, c->stream);
  c->ev_pending.push_back({name, e0, e1});
}

// resolves recorded launch events into the per-kernel table (after the stream has drained)
void resolve_profile(fnetg_ctx *c) {
  if (c->ev_pending.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto &p : c->ev_pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.e0, p.e1);
    auto &e = c->prof_tab[p.name];
    e.ms += ms;
    e.launches += 1;
    c->ev_free.push_back(p.e0);
    c->ev_free.push_back(p.e1);
  }
  c->ev_pending.clear();
}

}  // namespace fnetg

// ---------------------------------------------------------------------------------------
// Reciprocal lattice exactly as the reference derives it (fnetdata.F90:1141-1148 with
// determinant33 / invert33 of lib_dftbp/simplealgebra.F90:41-125, then a transpose).
// This file is compiled with -ffp-contract=off so the host arithmetic is not fused.
static int recvecs2p(const double *L, double *R) {
#define M(i, j) L[((i)-1) + 3 * ((j)-1)]
  double tmp = M(1, 1) * (M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3));
  tmp = tmp - M(1, 2) * (M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3));
  tmp = tmp + M(1, 3) * (M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2));
  const double det = tmp;
  if (!(std::fabs(det) >= 1e-12)) return -1;
  double inv[9];
#define INV(i, j) inv[((i)-1) + 3 * ((j)-1)]
  INV(1, 1) = -(M(2, 3) * M(3, 2)) + M(2, 2) * M(3, 3);
  INV(2, 1) = M(2, 3) * M(3, 1) - M(2, 1) * M(3, 3);
  INV(3, 1) = -(M(2, 2) * M(3, 1)) + M(2, 1) * M(3, 2);
  INV(1, 2) = M(1, 3) * M(3, 2) - M(1, 2) * M(3, 3);
  INV(2, 2) = -(M(1, 3) * M(3, 1)) + M(1, 1) * M(3, 3);
  INV(3, 2) = M(1, 2) * M(3, 1) - M(1, 1) * M(3, 2);
  INV(1, 3) = -(M(1, 3) * M(2, 2)) + M(1, 2) * M(2, 3);
  INV(2, 3) = M(1, 3) * M(2, 1) - M(1, 1) * M(2, 3);
  INV(3, 3) = -(M(1, 2) * M(2, 1)) + M(1, 1) * M(2, 2);
  for (int k = 0; k < 9; k++) inv[k] = inv[k] / det;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i + 3 * j] = inv[j + 3 * i];
#undef M
#undef INV
  return 0;
}

// image ranges of TLatPointIter_init / getRanges (latpointiter.F90:226-253), extension 1
int fnetg_lattice_ranges(const double *L, double rcut, int32_t *lohi) {
  double R[9];
  if (recvecs2p(L, R)) return -1;
  for (int ii = 0; ii < 3; ii++) {
    const double *col = R + 3 * ii;
    double s = col[0] * col[0];
    s = s + col[1] * col[1];
    s = s + col[2] * col[2];
    int itmp = (int)std::floor(rcut * std::sqrt(s));
    lohi[2 * ii] = -(itmp + 1);
    lohi[2 * ii + 1] = itmp + 1;
  }
  return 0;
}

// ---------------------------------------------------------------------------------------
namespace fnetg {
// Per-structure sums of the atomic outputs, one thread per (structure, output), atoms in order
// (the host loop's order and operations: the same FP64 result)
__global__ void struct_sum_kernel(const double *out, const int64_t *off, int S, int nout,
                                  double *gsum) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)S * nout) return;
  const int s = (int)(t / nout), o = (int)(t - (int64_t)s * nout);
  double acc = 0.0;
  for (int64_t a = off[s]; a < off[s + 1]; a++) acc += out[a * nout + o];
  gsum[t] = acc;
}
}  // namespace fnetg

extern "C" {

int fnetg_abi_version(void) { return FNETG_ABI_VERSION; }

int fnetg_create(fnetg_ctx **out, int32_t precision, int32_t device) {
  if (!out) return FNETG_E_INVALID;
  *out = nullptr;
  if (precision != FNETG_FP32 && precision != FNETG_FP64) return FNETG_E_INVALID;
  fnetg_ctx *ctx = new fnetg_ctx();
  ctx->prec = precision;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_pinned, 4096);
  if (e != cudaSuccess) {
    delete ctx;
    return e == cudaErrorMemoryAllocation ? FNETG_E_NOMEM : FNETG_E_CUDA;
  }
  *out = ctx;
  return FNETG_OK;
}

int fnetg_destroy(fnetg_ctx *ctx) {
  if (!ctx) return FNETG_E_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  for (auto &p : ctx->ev_pending) {
    cudaEventDestroy(p.e0);
    cudaEventDestroy(p.e1);
  }
  for (auto e : ctx->ev_free) cudaEventDestroy(e);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->batch) fnetg::batch_free(ctx->batch);
  cudaStream_t s = ctx->stream;
  delete ctx;  // DBuf destructors free device memory
  if (s) cudaStreamDestroy(s);
  return FNETG_OK;
}

const char *fnetg_last_error(const fnetg_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fnetg_get_stream(fnetg_ctx *ctx, void **stream) {
  if (!ctx || !stream) return FNETG_E_INVALID;
  *stream = (void *)ctx->stream;
  return FNETG_OK;
}

int fnetg_synchronize(fnetg_ctx *ctx) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FNETG_OK;
}

int fnetg_check_status(fnetg_ctx *ctx, int32_t *site) {
  if (!ctx || !site) return FNETG_E_INVALID;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  int first = 0;
  for (int v : {check_site_neighbors(), check_site_acsf(), check_site_forces(), check_site_mlp(),
                check_site_batch(), check_site_jvp()}) {
    FNETG_CHECK(v >= 0, FNETG_E_CUDA, "check_status: reading a check word failed");
    if (first == 0) first = v;
  }
  *site = first;
  return FNETG_OK;
}

int fnetg_profile_enable(fnetg_ctx *ctx, int32_t enable) {
  if (!ctx) return FNETG_E_INVALID;
  ctx->prof = enable != 0;
  return FNETG_OK;
}

int fnetg_profile_read(fnetg_ctx *ctx, const char *name, double *ms, int64_t *launches) {
  if (!ctx || !name) return FNETG_E_INVALID;
  resolve_profile(ctx);
  auto it = ctx->prof_tab.find(name);
  if (it == ctx->prof_tab.end()) {
    if (ms) *ms = 0.0;
    if (launches) *launches = 0;
    return -1;
  }
  if (ms) *ms = it->second.ms;
  if (launches) *launches = it->second.launches;
  return FNETG_OK;
}

int fnetg_profile_reset(fnetg_ctx *ctx) {
  if (!ctx) return FNETG_E_INVALID;
  resolve_profile(ctx);
  ctx->prof_tab.clear();
  ctx->launches = 0;
  return FNETG_OK;
}

int64_t fnetg_launch_count(fnetg_ctx *ctx) { return ctx ? ctx->launches : -1; }

// ---------------------------------------------------------------------------------------
static void invalidate_geometry(fnetg_ctx *ctx) {
  ctx->nb_valid = false;
  ctx->feats_valid = false;
  ctx->mom_valid = false;
}

static int rebuild_buckets(fnetg_ctx *ctx, bool order_changes);

// per-atom species code (index into the atomic numbers the G-functions reference, -1 none)
static int refresh_codes(fnetg_ctx *ctx) {
  std::vector<int8_t> code(std::max<int64_t>(ctx->N, 1), -1);
  for (int64_t a = 0; a < ctx->N; a++)
    for (size_t z = 0; z < ctx->zcodes.size(); z++)
      if (ctx->h_atnum[a] == ctx->zcodes[z]) code[a] = (int8_t)z;
  FNETG_CUDA(ctx->d_code.ensure(std::max<int64_t>(ctx->N, 1)));
  if (ctx->N > 0)
    FNETG_CUDA(copy_sync(ctx, ctx->d_code.p, code.data(), ctx->N, cudaMemcpyHostToDevice));
  return FNETG_OK;
}

int fnetg_upload_structures(fnetg_ctx *ctx, int32_t nstruct, const int64_t *atom_offsets,
                            const int32_t *atnum, const double *coords, const int32_t *periodic,
                            const double *latvecs, const double *ext, int32_t next) {
  if (!ctx) return FNETG_E_INVALID;
  ctx->feat_gen++;
  FNETG_CHECK(nstruct >= 0 && atom_offsets && (nstruct == 0 || (atnum && coords)),
              FNETG_E_INVALID, "upload_structures: null array");
  FNETG_CHECK(atom_offsets[0] == 0, FNETG_E_SHAPE, "atom_offsets[0] must be 0");
  for (int s = 0; s < nstruct; s++)
    FNETG_CHECK(atom_offsets[s + 1] >= atom_offsets[s], FNETG_E_SHAPE,
                "atom_offsets must be non-decreasing");
  const int64_t N = atom_offsets[nstruct];
  FNETG_CHECK(N < (int64_t(1) << 31), FNETG_E_UNSUPPORTED, "more than 2^31 atoms");
  FNETG_CHECK(next >= 0 && (next == 0 || ext), FNETG_E_INVALID, "external features");
  for (int64_t q = 0; q < 3 * N; q++)
    FNETG_CHECK(std::isfinite(coords[q]), FNETG_E_GEOMETRY, "non-finite coordinate");
  cudaSetDevice(ctx->device);
  ctx->S = nstruct;
  ctx->N = N;
  ctx->next = next;
  ctx->h_off.assign(atom_offsets, atom_offsets + nstruct + 1);
  ctx->h_atnum.assign(atnum, atnum + N);
  ctx->h_periodic.assign(nstruct, 0);
  ctx->h_lat.assign((size_t)9 * nstruct, 0.0);
  for (int s = 0; s < nstruct; s++) {
    ctx->h_periodic[s] = periodic ? (periodic[s] != 0) : 0;
    if (ctx->h_periodic[s]) {
      FNETG_CHECK(latvecs, FNETG_E_INVALID, "periodic structure without lattice vectors");
      for (int k = 0; k < 9; k++) ctx->h_lat[9 * s + k] = latvecs[9 * s + k];
      double R[9];
      if (recvecs2p(latvecs + 9 * s, R))
        return fail(ctx, FNETG_E_GEOMETRY,
                    "dependent lattice vectors in structure " + std::to_string(s));
    }
  }
  std::vector<int32_t> astruct(N);
  for (int s = 0; s < nstruct; s++)
    for (int64_t a = atom_offsets[s]; a < atom_offsets[s + 1]; a++) astruct[a] = s;
  FNETG_CUDA(ctx->d_off.ensure(sizeof(int64_t) * (nstruct + 1)));
  FNETG_CUDA(ctx->d_atom_struct.ensure(sizeof(int32_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_coords.ensure(sizeof(double) * 3 * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_coordsf.ensure(sizeof(V4<float>) * 2 * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_atnum.ensure(sizeof(int32_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_lat.ensure(sizeof(double) * 9 * std::max(nstruct, 1)));
  FNETG_CUDA(ctx->d_bbox.ensure(sizeof(float) * 6 * std::max(nstruct, 1)));
  FNETG_CUDA(ctx->d_periodic.ensure(sizeof(int32_t) * std::max(nstruct, 1)));
  cudaStream_t st = ctx->stream;
  FNETG_CUDA(cudaMemcpyAsync(ctx->d_off.p, atom_offsets, sizeof(int64_t) * (nstruct + 1),
                             cudaMemcpyHostToDevice, st));
  if (N > 0) {
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_atom_struct.p, astruct.data(), sizeof(int32_t) * N,
                               cudaMemcpyHostToDevice, st));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_coords.p, coords, sizeof(double) * 3 * N,
                               cudaMemcpyHostToDevice, st));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_atnum.p, atnum, sizeof(int32_t) * N,
                               cudaMemcpyHostToDevice, st));
  }
  if (nstruct > 0) {
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_lat.p, ctx->h_lat.data(), sizeof(double) * 9 * nstruct,
                               cudaMemcpyHostToDevice, st));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_periodic.p, ctx->h_periodic.data(),
                               sizeof(int32_t) * nstruct, cudaMemcpyHostToDevice, st));
  }
  if (next > 0 && N > 0) {
    FNETG_CUDA(ctx->d_ext.ensure(sizeof(double) * N * next));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_ext.p, ext, sizeof(double) * N * next,
                               cudaMemcpyHostToDevice, st));
  }
  {
    int rc = prepare_coords(ctx);
    if (rc) return rc;
  }
  ctx->max_extent = 0.0;
  for (int s = 0; s < nstruct; s++) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t a = atom_offsets[s]; a < atom_offsets[s + 1]; a++)
      for (int c = 0; c < 3; c++) {
        lo[c] = std::min(lo[c], coords[3 * a + c]);
        hi[c] = std::max(hi[c], coords[3 * a + c]);
      }
    if (atom_offsets[s + 1] > atom_offsets[s])
      ctx->max_extent = std::max(ctx->max_extent, std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) +
                                                             (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                                             (hi[2] - lo[2]) * (hi[2] - lo[2])));
  }
  FNETG_CUDA(cudaStreamSynchronize(st));
  invalidate_geometry(ctx);
  ctx->targets_set = false;
  // default: every atom in sub-network 0 until fnetg_set_species
  ctx->h_species.assign(N, 0);
  ctx->layout_gen++;
  ctx->species_set = false;
  int rc = refresh_codes(ctx);
  if (rc) return rc;
  return rebuild_buckets(ctx, true);
}

int fnetg_update_coords(fnetg_ctx *ctx, const double *coords) {
  if (!ctx || (!coords && ctx->N > 0)) return FNETG_E_INVALID;
  ctx->feat_gen++;
  const int64_t N = ctx->N;
  // the new coordinates land in a staging buffer; the device checks them and measures the
  // structures' extents (no pass over them on the host), and only checked coordinates replace
  // the context's: a refused update leaves the context as it was
  double ext = 0.0;
  if (N > 0) {
    FNETG_CUDA(ctx->d_coords_in.ensure(sizeof(double) * 3 * N));
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_coords_in.p, coords, sizeof(double) * 3 * N,
                               cudaMemcpyHostToDevice, ctx->stream));
    bool bad = false;
    int rc = coords_summary(ctx, ctx->d_coords_in.as<double>(), &ext, &bad);
    if (rc) return rc;
    FNETG_CHECK(!bad, FNETG_E_GEOMETRY, "non-finite coordinate");
    FNETG_CUDA(cudaMemcpyAsync(ctx->d_coords.p, ctx->d_coords_in.p, sizeof(double) * 3 * N,
                               cudaMemcpyDeviceToDevice, ctx->stream));
  }
  int rc = prepare_coords(ctx);
  if (rc) return rc;
  ctx->max_extent = ext;
  invalidate_geometry(ctx);
  return FNETG_OK;
}

// species buckets: rows of every sub-network contiguous, tiles never straddle species
static int rebuild_buckets(fnetg_ctx *ctx, bool order_changes) {
  const int64_t N = ctx->N;
  int nsp = 1;
  for (int64_t a = 0; a < N; a++) nsp = std::max(nsp, ctx->h_species[a] + 1);
  if (ctx->net_set) nsp = std::max(nsp, ctx->nsp);
  std::vector<int64_t> cnt(nsp + 1, 0);
  for (int64_t a = 0; a < N; a++) cnt[ctx->h_species[a] + 1]++;
  for (int s = 0; s < nsp; s++) cnt[s + 1] += cnt[s];
  ctx->h_bucket_off = cnt;
  std::vector<int32_t> bpos(std::max<int64_t>(N, 1)), bperm(std::max<int64_t>(N, 1));
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int64_t a = 0; a < N; a++) {
    int64_t r = fill[ctx->h_species[a]]++;
    bpos[a] = (int32_t)r;
    bperm[r] = (int32_t)a;
  }
  ctx->tile_rows = ctx->prec == FNETG_FP64 ? 32 : 64;
  std::vector<int32_t> tiles;
  for (int s = 0; s < nsp; s++)
    for (int64_t r = cnt[s]; r < cnt[s + 1]; r += ctx->tile_rows) {
      tiles.push_back(s);
      tiles.push_back((int32_t)r);
      tiles.push_back((int32_t)std::min<int64_t>(ctx->tile_rows, cnt[s + 1] - r));
      tiles.push_back(0);
    }
  ctx->ntiles = (int64_t)tiles.size() / 4;
  // first tile of every species (tiles are grouped by species in order)
  std::vector<int64_t> t0(nsp + 1, 0);
  for (int64_t t = 0; t < ctx->ntiles; t++) t0[tiles[4 * t] + 1]++;
  for (int s = 0; s < nsp; s++) t0[s + 1] += t0[s];
  ctx->h_sp_tile0 = t0;
  FNETG_CUDA(ctx->d_sp_tile0.ensure(sizeof(int64_t) * (nsp + 1)));
  FNETG_CUDA(copy_sync(ctx, ctx->d_sp_tile0.p, t0.data(), sizeof(int64_t) * (nsp + 1),
                        cudaMemcpyHostToDevice));
  FNETG_CUDA(ctx->d_species.ensure(sizeof(int32_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_bpos.ensure(sizeof(int32_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_bperm.ensure(sizeof(int32_t) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_tiles.ensure(sizeof(int32_t) * std::max<size_t>(tiles.size(), 4)));
  if (N > 0) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_species.p, ctx->h_species.data(), sizeof(int32_t) * N,
                          cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_bpos.p, bpos.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_bperm.p, bperm.data(), sizeof(int32_t) * N,
                          cudaMemcpyHostToDevice));
  }
  if (!tiles.empty())
    FNETG_CUDA(copy_sync(ctx, ctx->d_tiles.p, tiles.data(), sizeof(int32_t) * tiles.size(),
                          cudaMemcpyHostToDevice));
  if (order_changes) ctx->feats_valid = false;
  return FNETG_OK;
}

int fnetg_set_species(fnetg_ctx *ctx, const int32_t *species) {
  if (!ctx || (!species && ctx->N > 0)) return FNETG_E_INVALID;
  ctx->feat_gen++;
  for (int64_t a = 0; a < ctx->N; a++)
    FNETG_CHECK(species[a] >= 0 && species[a] < 1024, FNETG_E_INVALID, "species index");
  if (ctx->net_set)
    for (int64_t a = 0; a < ctx->N; a++)
      FNETG_CHECK(species[a] < ctx->nsp, FNETG_E_SHAPE, "species index >= number of networks");
  ctx->h_species.assign(species, species + ctx->N);
  ctx->layout_gen++;
  ctx->species_set = true;
  // features are stored in bucket order; a new order needs a fresh featurisation
  return rebuild_buckets(ctx, true);
}

// ---------------------------------------------------------------------------------------
int fnetg_set_gfunctions(fnetg_ctx *ctx, int32_t ng, const fnetg_gfunc *g) {
  if (!ctx || ng < 0 || (ng > 0 && !g)) return FNETG_E_INVALID;
  FNETG_CHECK(ng <= 4096, FNETG_E_UNSUPPORTED, "more than 4096 G-functions");
  std::vector<int32_t> zs;
  std::set<double> rset;
  for (int k = 0; k < ng; k++) {
    const fnetg_gfunc &f = g[k];
    FNETG_CHECK(f.type >= 1 && f.type <= 5, FNETG_E_INVALID, "G-function type must be 1..5");
    FNETG_CHECK(f.rcut > 0.0 && std::isfinite(f.rcut), FNETG_E_INVALID, "cutoff must be > 0");
    FNETG_CHECK(f.atomid >= 0, FNETG_E_INVALID, "atomid must be >= 0");
    if (f.atomid > 0)
      FNETG_CHECK(f.atomid <= ctx->next, FNETG_E_SHAPE, "atomid beyond the external features");
    rset.insert(f.rcut);
    for (int z : {f.z1, f.z2})
      if (z != 0 && std::find(zs.begin(), zs.end(), z) == zs.end()) zs.push_back(z);
  }
  FNETG_CHECK((int)zs.size() <= kMaxSpeciesCodes, FNETG_E_UNSUPPORTED,
              "more than 8 distinct atomic numbers in the G-functions");
  FNETG_CHECK((int)rset.size() <= kMaxRcutClasses, FNETG_E_UNSUPPORTED,
              "more than 8 distinct cutoffs");
  ctx->gf.assign(g, g + ng);
  ctx->zcodes = zs;
  ctx->rcut_classes.assign(rset.begin(), rset.end());
  auto code_of = [&](int z) -> int {
    if (z == 0) return -1;
    return (int)(std::find(zs.begin(), zs.end(), z) - zs.begin());
  };
  auto rclass_of = [&](double r) -> int {
    return (int)(std::find(ctx->rcut_classes.begin(), ctx->rcut_classes.end(), r) -
                 ctx->rcut_classes.begin());
  };
  ctx->h_rad.clear();
  ctx->h_ang.clear();
  ctx->h_groups.clear();
  ctx->ecls_eta.clear();
  ctx->ecls_rclass.clear();
  ctx->ecls_atomid.clear();
  std::vector<GDesc> ang;
  for (int k = 0; k < ng; k++) {
    const fnetg_gfunc &f = g[k];
    GDesc d{};
    d.type = f.type;
    bool resolved = !(f.z1 == 0 && f.z2 == 0);
    d.chan1 = resolved ? code_of(f.z1) : -1;
    d.chan2 = resolved ? (f.type >= 4 ? code_of(f.z2) : d.chan1) : -1;
    d.atomid = f.atomid;
    d.out = k;
    d.rclass = rclass_of(f.rcut);
    d.rcut = f.rcut;
    d.kappa = f.kappa;
    d.rs = f.rs;
    d.eta = f.eta;
    d.lambda = f.lambda;
    d.xi = f.xi;
    d.pref = std::pow(2.0, 1.0 - f.xi);
    d.xi_int = (f.xi >= 1.0 && f.xi <= 16.0 && f.xi == std::floor(f.xi)) ? (int)f.xi : 0;
    d.eclass = -1;
    if (f.type >= 4) {
      int e = -1;
      for (size_t q = 0; q < ctx->ecls_eta.size(); q++)
        if (ctx->ecls_eta[q] == f.eta && ctx->ecls_rclass[q] == d.rclass &&
            ctx->ecls_atomid[q] == f.atomid)
          e = (int)q;
      if (e < 0) {
        FNETG_CHECK((int)ctx->ecls_eta.size() < kMaxEtaClasses, FNETG_E_UNSUPPORTED,
                    "more than 16 distinct (eta, cutoff, atomid) among angular functions");
        e = (int)ctx->ecls_eta.size();
        ctx->ecls_eta.push_back(f.eta);
        ctx->ecls_rclass.push_back(d.rclass);
        ctx->ecls_atomid.push_back(f.atomid);
      }
      d.eclass = e;
      ang.push_back(d);
    } else {
      ctx->h_rad.push_back(d);
    }
  }
  // radial functions grouped by list channel (all atoms first, then species codes in order):
  // a pair visits the all-atom segment and its own species' segment only
  std::stable_sort(ctx->h_rad.begin(), ctx->h_rad.end(),
                   [](const GDesc &x, const GDesc &y) { return x.chan1 < y.chan1; });
  ctx->rad_seg.assign(kMaxSpeciesCodes + 2, 0);
  {
    int nall = 0;
    for (auto &d : ctx->h_rad) nall += d.chan1 < 0 ? 1 : 0;
    ctx->rad_seg[1] = nall;
    int pos = nall;
    for (int c = 0; c < (int)zs.size(); c++) {
      for (auto &d : ctx->h_rad) pos += d.chan1 == c ? 1 : 0;
      ctx->rad_seg[c + 2] = pos;
    }
  }
  // value kernel order: functions of one shape (type, cutoff class, atom id, rs / eta / kappa)
  // adjacent, list channels in ascending order within a shape (the order above is stable), so
  // that a species-expanded set forms a shape x channel grid
  {
    const int nr = (int)ctx->h_rad.size();
    std::vector<int32_t> ord(nr);
    for (int g = 0; g < nr; g++) ord[g] = g;
    auto key = [&](int g) {
      const GDesc &d = ctx->h_rad[g];
      return std::make_tuple(d.type, d.rclass, d.atomid, d.type == 3 ? d.kappa : 0.0,
                             d.type == 2 ? d.rs : 0.0, d.type == 2 ? d.eta : 0.0);
    };
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return key(x) < key(y); });
    ctx->h_radv = ord;
  }
  // force kernel fast path: every radial function a G2 without atom id, one cutoff class
  ctx->rad_fast = ctx->h_rad.empty() ? -1 : ctx->h_rad[0].rclass;
  for (auto &d : ctx->h_rad)
    if (d.type != 2 || d.atomid != 0 || d.rclass != ctx->rad_fast) ctx->rad_fast = -1;
  ctx->h_ang_all = ang;  // every angular function, before the moment form takes its share
  // G5 functions with a small integer xi take the moment form; the rest (G4, other xi) the
  // triplet sweep
  std::vector<GDesc> mom, trip;
  for (auto &d : ang) {
    if (d.type == 5 && d.xi_int >= 1 && d.xi_int <= kMaxMomentDegree) mom.push_back(d);
    else trip.push_back(d);
  }
  ang = trip;
  ctx->h_mfunc.clear();
  ctx->h_combo.clear();
  ctx->mom_degree = 0;
  for (auto &d : mom) ctx->mom_degree = std::max(ctx->mom_degree, d.xi_int);
  const int D = ctx->mom_degree;
  ctx->n_mono = D > 0 ? (D + 1) * (D + 2) * (D + 3) / 6 : 0;
  const int nz = (int)zs.size(), ne = (int)ctx->ecls_eta.size();
  ctx->h_cidx.assign((size_t)(nz + 1) * std::max(ne, 1), -1);
  auto combo_of = [&](int chan, int e) -> int {
    int &slot = ctx->h_cidx[(size_t)(chan + 1) * ne + e];
    if (slot < 0) {
      slot = (int)ctx->h_combo.size() / 2;
      ctx->h_combo.push_back(chan);
      ctx->h_combo.push_back(e);
    }
    return slot;
  };
  auto fact = [](int n) {
    double r = 1.0;
    for (int k = 2; k <= n; k++) r *= k;
    return r;
  };
  for (auto &d : mom) {
    MFunc mf{};
    mf.k1 = combo_of(d.chan1, d.eclass);
    mf.k2 = combo_of(d.chan2, d.eclass);
    mf.out = d.out;
    ctx->h_mfunc.push_back(mf);
  }
  // combos renumbered in (list channel, eta class) order: the moment kernels take runs of one
  // list's eta classes together
  {
    const int nc = (int)ctx->h_combo.size() / 2;
    std::vector<int> ord(nc), pos(nc);
    for (int k = 0; k < nc; k++) ord[k] = k;
    std::sort(ord.begin(), ord.end(), [&](int x, int y) {
      return std::make_pair(ctx->h_combo[2 * x], ctx->h_combo[2 * x + 1]) <
             std::make_pair(ctx->h_combo[2 * y], ctx->h_combo[2 * y + 1]);
    });
    std::vector<int32_t> sorted(2 * nc);
    for (int k = 0; k < nc; k++) {
      pos[ord[k]] = k;
      sorted[2 * k] = ctx->h_combo[2 * ord[k]];
      sorted[2 * k + 1] = ctx->h_combo[2 * ord[k] + 1];
    }
    ctx->h_combo = sorted;
    for (auto &mf : ctx->h_mfunc) {
      mf.k1 = pos[mf.k1];
      mf.k2 = pos[mf.k2];
    }
    for (auto &c : ctx->h_cidx)
      if (c >= 0) c = pos[c];
  }
  ctx->n_combo = (int)ctx->h_combo.size() / 2;
  // Degree coefficients pc_f(m) = 2^(1-xi) C(xi, m) lambda^m (coef_f(alpha) = pc_f(|alpha|)
  // times the multinomial m!/alpha!), and per combo k the partner groups: for each partner
  // combo ko, the functions f whose adjoint sends M_ko into Q_k (listed twice when k1 = k2).
  ctx->h_mpc.assign((size_t)ctx->h_mfunc.size() * (kMaxMomentDegree + 1), 0.0);
  for (size_t f = 0; f < mom.size(); f++) {
    const GDesc &d = mom[f];
    for (int m = 0; m <= d.xi_int; m++)
      ctx->h_mpc[f * (kMaxMomentDegree + 1) + m] =
          d.pref * (fact(d.xi_int) / (fact(m) * fact(d.xi_int - m))) * std::pow(d.lambda, m);
  }
  ctx->h_fpc = ctx->h_mpc;  // per function (h_mpc is regrouped for the adjoint below)
  ctx->h_mpair.clear();
  for (auto &mf : ctx->h_mfunc) {
    const int lo = std::min(mf.k1, mf.k2), hi = std::max(mf.k1, mf.k2);
    int pidx = -1;
    for (size_t q = 0; q + 1 < ctx->h_mpair.size(); q += 2)
      if (ctx->h_mpair[q] == lo && ctx->h_mpair[q + 1] == hi) pidx = (int)(q / 2);
    if (pidx < 0) {
      pidx = (int)ctx->h_mpair.size() / 2;
      ctx->h_mpair.push_back(lo);
      ctx->h_mpair.push_back(hi);
    }
    mf.pair = pidx;
  }
  {
    FNETG_CUDA(ctx->d_mpair.ensure(sizeof(int32_t) * std::max<size_t>(ctx->h_mpair.size(), 2)));
    FNETG_CUDA(ctx->d_fpc_d.ensure(sizeof(double) * std::max<size_t>(ctx->h_fpc.size(), 1)));
    FNETG_CUDA(ctx->d_fpc_f.ensure(sizeof(float) * std::max<size_t>(ctx->h_fpc.size(), 1)));
    if (!ctx->h_mpair.empty()) {
      const std::vector<float> pf(ctx->h_fpc.begin(), ctx->h_fpc.end());
      FNETG_CUDA(copy_sync(ctx, ctx->d_mpair.p, ctx->h_mpair.data(),
                            sizeof(int32_t) * ctx->h_mpair.size(), cudaMemcpyHostToDevice));
      FNETG_CUDA(copy_sync(ctx, ctx->d_fpc_d.p, ctx->h_fpc.data(),
                            sizeof(double) * ctx->h_fpc.size(), cudaMemcpyHostToDevice));
      FNETG_CUDA(copy_sync(ctx, ctx->d_fpc_f.p, pf.data(), sizeof(float) * pf.size(),
                            cudaMemcpyHostToDevice));
    }
  }
  std::vector<int32_t> qg_off(ctx->n_combo + 1, 0), qg_ko, qg_foff(1, 0), qg_f;
  for (int k = 0; k < ctx->n_combo; k++) {
    qg_off[k] = (int32_t)qg_ko.size();
    std::vector<std::pair<int, std::vector<int32_t>>> groups;
    auto add = [&](int ko, int f) {
      for (auto &g : groups)
        if (g.first == ko) {
          g.second.push_back(f);
          return;
        }
      groups.push_back({ko, {f}});
    };
    for (size_t f = 0; f < ctx->h_mfunc.size(); f++) {
      const MFunc &mf = ctx->h_mfunc[f];
      if (mf.k1 == k) add(mf.k2, (int)f);
      if (mf.k2 == k) add(mf.k1, (int)f);
    }
    for (auto &g : groups) {
      qg_ko.push_back(g.first);
      qg_f.insert(qg_f.end(), g.second.begin(), g.second.end());
      qg_foff.push_back((int32_t)qg_f.size());
    }
  }
  qg_off[ctx->n_combo] = (int32_t)qg_ko.size();
  ctx->n_qgroups = (int)qg_ko.size();
  {
    // [n_combo + 1] group offsets, [G] partner combos, [G + 1] entry offsets, [E] output
    // column of each entry's function; the entries' degree coefficients follow in d_mpc_*
    std::vector<int32_t> pack;
    pack.insert(pack.end(), qg_off.begin(), qg_off.end());
    pack.insert(pack.end(), qg_ko.begin(), qg_ko.end());
    pack.insert(pack.end(), qg_foff.begin(), qg_foff.end());
    for (int32_t f : qg_f) pack.push_back(ctx->h_mfunc[f].out);
    // adjoint rows (list channel zz in 0..nz, row nz the all-atom list only; eta class e):
    // [rows + 1] term offsets, then the terms g | ko << 16 over the groups of the row's own
    // combo and of the all-atom combo of the same class
    {
      const int nrows = (nz + 1) * ne;
      std::vector<int32_t> roff(1, 0), terms;
      for (int zz = 0; zz <= nz; zz++)
        for (int e = 0; e < ne; e++) {
          const int ks = zz < nz ? ctx->h_cidx[(size_t)(zz + 1) * ne + e] : -1;
          const int ka = ctx->h_cidx[e];
          for (int k : {ks, ka}) {
            if (k < 0) continue;
            for (int g = qg_off[k]; g < qg_off[k + 1]; g++) terms.push_back(g | (qg_ko[g] << 16));
          }
          roff.push_back((int32_t)terms.size());
        }
      FNETG_CHECK((int)roff.size() == nrows + 1, FNETG_E_CUDA, "adjoint rows");
      FNETG_CHECK(qg_ko.size() < 65536 && ctx->n_combo < 32768, FNETG_E_UNSUPPORTED,
                  "too many moment partner groups");
      pack.insert(pack.end(), roff.begin(), roff.end());
      pack.insert(pack.end(), terms.begin(), terms.end());
    }
    std::vector<double> epc;
    for (int32_t f : qg_f)
      epc.insert(epc.end(), ctx->h_mpc.begin() + (size_t)f * (kMaxMomentDegree + 1),
                 ctx->h_mpc.begin() + (size_t)(f + 1) * (kMaxMomentDegree + 1));
    ctx->h_mpc = epc;
    ctx->n_qgpack = (int)pack.size();
    ctx->n_qgent = (int)qg_f.size();
    FNETG_CUDA(ctx->d_qgroups.ensure(sizeof(int32_t) * std::max<size_t>(pack.size(), 1)));
    FNETG_CUDA(copy_sync(ctx, ctx->d_qgroups.p, pack.data(), sizeof(int32_t) * pack.size(),
                          cudaMemcpyHostToDevice));
    std::vector<float> pcf(ctx->h_mpc.begin(), ctx->h_mpc.end());
    FNETG_CUDA(ctx->d_mpc_d.ensure(sizeof(double) * std::max<size_t>(ctx->h_mpc.size(), 1)));
    FNETG_CUDA(ctx->d_mpc_f.ensure(sizeof(float) * std::max<size_t>(pcf.size(), 1)));
    if (!pcf.empty()) {
      FNETG_CUDA(copy_sync(ctx, ctx->d_mpc_d.p, ctx->h_mpc.data(), sizeof(double) * ctx->h_mpc.size(),
                            cudaMemcpyHostToDevice));
      FNETG_CUDA(copy_sync(ctx, ctx->d_mpc_f.p, pcf.data(), sizeof(float) * pcf.size(),
                            cudaMemcpyHostToDevice));
    }
  }
  // per-combo list of the moment functions whose Q (adjoint moment) it receives
  FNETG_CUDA(ctx->d_mfunc.ensure(sizeof(MFunc) * std::max<size_t>(ctx->h_mfunc.size(), 1)));
  FNETG_CUDA(ctx->d_combo.ensure(sizeof(int32_t) * std::max<size_t>(ctx->h_combo.size(), 2)));
  FNETG_CUDA(ctx->d_cidx.ensure(sizeof(int32_t) * std::max<size_t>(ctx->h_cidx.size(), 1)));
  if (!ctx->h_mfunc.empty()) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_mfunc.p, ctx->h_mfunc.data(), sizeof(MFunc) * ctx->h_mfunc.size(),
                          cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_combo.p, ctx->h_combo.data(),
                          sizeof(int32_t) * ctx->h_combo.size(), cudaMemcpyHostToDevice));
  }
  FNETG_CUDA(copy_sync(ctx, ctx->d_cidx.p, ctx->h_cidx.data(), sizeof(int32_t) * ctx->h_cidx.size(),
                        cudaMemcpyHostToDevice));
  // group the remaining angular functions by list channels, cutoff and atom-id column
  // (stable), at most kMaxGroupFuncs per group
  std::vector<std::array<int, 4>> chans;
  for (auto &d : ang) {
    std::array<int, 4> c{d.chan1, d.chan2, d.rclass, d.atomid};
    if (std::find(chans.begin(), chans.end(), c) == chans.end()) chans.push_back(c);
  }
  for (auto &c : chans) {
    std::vector<GDesc> members;
    for (auto &d : ang)
      if (d.chan1 == c[0] && d.chan2 == c[1] && d.rclass == c[2] && d.atomid == c[3])
        members.push_back(d);
    for (size_t q0 = 0; q0 < members.size(); q0 += kMaxGroupFuncs) {
      AGroup grp{};
      grp.chan1 = c[0];
      grp.chan2 = c[1];
      grp.same = (c[0] == c[1]) ? 1 : 0;
      grp.atomid = c[3];
      grp.first = (int)ctx->h_ang.size();
      grp.count = (int)std::min<size_t>(kMaxGroupFuncs, members.size() - q0);
      grp.has_g4 = 0;
      for (int q = 0; q < grp.count; q++) {
        ctx->h_ang.push_back(members[q0 + q]);
        if (members[q0 + q].type == 4) grp.has_g4 = 1;
      }
      ctx->h_groups.push_back(grp);
    }
  }
  FNETG_CUDA(ctx->d_ang_all.ensure(sizeof(GDesc) * std::max<size_t>(ctx->h_ang_all.size(), 1)));
  if (!ctx->h_ang_all.empty())
    FNETG_CUDA(copy_sync(ctx, ctx->d_ang_all.p, ctx->h_ang_all.data(),
                          sizeof(GDesc) * ctx->h_ang_all.size(), cudaMemcpyHostToDevice));
  FNETG_CUDA(ctx->d_rad.ensure(sizeof(GDesc) * std::max<size_t>(ctx->h_rad.size(), 1)));
  FNETG_CUDA(ctx->d_ang.ensure(sizeof(GDesc) * std::max<size_t>(ctx->h_ang.size(), 1)));
  FNETG_CUDA(ctx->d_groups.ensure(sizeof(AGroup) * std::max<size_t>(ctx->h_groups.size(), 1)));
  FNETG_CUDA(ctx->d_ecls_eta.ensure(sizeof(double) * kMaxEtaClasses));
  FNETG_CUDA(ctx->d_ecls_rclass.ensure(sizeof(int) * kMaxEtaClasses));
  FNETG_CUDA(ctx->d_ecls_atomid.ensure(sizeof(int) * kMaxEtaClasses));
  FNETG_CUDA(ctx->d_rcls.ensure(sizeof(double) * kMaxRcutClasses));
  FNETG_CUDA(ctx->d_radv.ensure(sizeof(int32_t) * std::max<size_t>(ctx->h_radv.size(), 1)));
  if (!ctx->h_rad.empty()) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_rad.p, ctx->h_rad.data(), sizeof(GDesc) * ctx->h_rad.size(),
                          cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_radv.p, ctx->h_radv.data(),
                          sizeof(int32_t) * ctx->h_radv.size(), cudaMemcpyHostToDevice));
  }
  if (!ctx->h_ang.empty())
    FNETG_CUDA(copy_sync(ctx, ctx->d_ang.p, ctx->h_ang.data(), sizeof(GDesc) * ctx->h_ang.size(),
                          cudaMemcpyHostToDevice));
  if (!ctx->h_groups.empty())
    FNETG_CUDA(copy_sync(ctx, ctx->d_groups.p, ctx->h_groups.data(),
                          sizeof(AGroup) * ctx->h_groups.size(), cudaMemcpyHostToDevice));
  if (!ctx->ecls_eta.empty()) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_ecls_eta.p, ctx->ecls_eta.data(),
                          sizeof(double) * ctx->ecls_eta.size(), cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_ecls_rclass.p, ctx->ecls_rclass.data(),
                          sizeof(int) * ctx->ecls_rclass.size(), cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_ecls_atomid.p, ctx->ecls_atomid.data(),
                          sizeof(int) * ctx->ecls_atomid.size(), cudaMemcpyHostToDevice));
  }
  if (!ctx->rcut_classes.empty())
    FNETG_CUDA(copy_sync(ctx, ctx->d_rcls.p, ctx->rcut_classes.data(),
                          sizeof(double) * ctx->rcut_classes.size(), cudaMemcpyHostToDevice));
  {
    auto params = [](const std::vector<GDesc> &v, std::vector<double> &pd, std::vector<float> &pf) {
      pd.clear();
      for (auto &d : v) {
        const double q[8] = {d.rcut, d.kappa, d.rs, d.eta, d.lambda, d.xi, d.pref, 0.0};
        pd.insert(pd.end(), q, q + 8);
      }
      if (pd.empty()) pd.assign(8, 0.0);
      pf.assign(pd.begin(), pd.end());
    };
    std::vector<double> pd;
    std::vector<float> pf;
    params(ctx->h_rad, pd, pf);
    FNETG_CUDA(ctx->d_radpar_d.ensure(sizeof(double) * pd.size()));
    FNETG_CUDA(ctx->d_radpar_f.ensure(sizeof(float) * pf.size()));
    FNETG_CUDA(copy_sync(ctx, ctx->d_radpar_d.p, pd.data(), sizeof(double) * pd.size(), cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_radpar_f.p, pf.data(), sizeof(float) * pf.size(), cudaMemcpyHostToDevice));
    params(ctx->h_ang, pd, pf);
    FNETG_CUDA(ctx->d_angpar_d.ensure(sizeof(double) * pd.size()));
    FNETG_CUDA(ctx->d_angpar_f.ensure(sizeof(float) * pf.size()));
    FNETG_CUDA(copy_sync(ctx, ctx->d_angpar_d.p, pd.data(), sizeof(double) * pd.size(), cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_angpar_f.p, pf.data(), sizeof(float) * pf.size(), cudaMemcpyHostToDevice));
    std::vector<float> ef(kMaxEtaClasses, 0.f), rf(kMaxRcutClasses, 0.f);
    for (size_t q = 0; q < ctx->ecls_eta.size(); q++) ef[q] = (float)ctx->ecls_eta[q];
    for (size_t q = 0; q < ctx->rcut_classes.size(); q++) rf[q] = (float)ctx->rcut_classes[q];
    FNETG_CUDA(ctx->d_ecls_eta_f.ensure(sizeof(float) * kMaxEtaClasses));
    FNETG_CUDA(ctx->d_rcls_f.ensure(sizeof(float) * kMaxRcutClasses));
    FNETG_CUDA(copy_sync(ctx, ctx->d_ecls_eta_f.p, ef.data(), sizeof(float) * kMaxEtaClasses, cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_rcls_f.p, rf.data(), sizeof(float) * kMaxRcutClasses, cudaMemcpyHostToDevice));
  }
  ctx->nb_valid = false;
  ctx->feats_valid = false;
  ctx->mom_valid = false;
  ctx->zprec_valid = false;
  ctx->nf = ng + (int)ctx->ext_idx.size();
  return refresh_codes(ctx);
}

int fnetg_neighbors(fnetg_ctx *ctx, double rcut, int64_t *npairs) {
  if (!ctx) return FNETG_E_INVALID;
  if (rcut <= 0.0) {
    FNETG_CHECK(!ctx->rcut_classes.empty(), FNETG_E_INVALID,
                "neighbors: no cutoff given and no G-functions set");
    rcut = ctx->rcut_classes.back();
  }
  int rc = run_neighbors(ctx, rcut);
  if (rc) return rc;
  if (npairs) *npairs = ctx->P;
  return FNETG_OK;
}

int fnetg_get_neighbors(fnetg_ctx *ctx, int64_t *pair_offsets, int32_t *j, int32_t *shift,
                        double *d2) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->nb_valid, FNETG_E_INVALID, "get_neighbors: no neighbour list");
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  const int64_t N = ctx->N, P = ctx->P, slots = ctx->pslots;
  // device [begin, end) of every atom -> compact offsets
  std::vector<int64_t> beg(std::max<int64_t>(N, 1)), end(std::max<int64_t>(N, 1)), off(N + 1, 0);
  if (N > 0) {
    FNETG_CUDA(copy_sync(ctx, beg.data(), ctx->d_poff.p, sizeof(int64_t) * N, cudaMemcpyDeviceToHost));
    FNETG_CUDA(copy_sync(ctx, end.data(), fnetg::pair_end(ctx), sizeof(int64_t) * N,
                          cudaMemcpyDeviceToHost));
  }
  for (int64_t a = 0; a < N; a++) off[a + 1] = off[a] + (end[a] - beg[a]);
  FNETG_CHECK(off[N] == P, FNETG_E_CUDA, "get_neighbors: inconsistent pair offsets");
  if (pair_offsets) memcpy(pair_offsets, off.data(), sizeof(int64_t) * (N + 1));
  auto compact = [&](const auto *src, auto *dst) {
    for (int64_t a = 0; a < N; a++)
      for (int64_t q = 0; q < end[a] - beg[a]; q++) dst[off[a] + q] = src[beg[a] + q];
  };
  if (j && P > 0) {
    std::vector<int32_t> all(slots);
    FNETG_CUDA(copy_sync(ctx, all.data(), ctx->d_pj.p, sizeof(int32_t) * slots, cudaMemcpyDeviceToHost));
    compact(all.data(), j);
    // convert to structure-local indices
    for (int s = 0; s < ctx->S; s++)
      for (int64_t a = ctx->h_off[s]; a < ctx->h_off[s + 1]; a++)
        for (int64_t q = off[a]; q < off[a + 1]; q++) j[q] -= (int32_t)ctx->h_off[s];
  }
  if (shift && P > 0) {
    std::vector<uint32_t> all(slots), meta(P);
    FNETG_CUDA(copy_sync(ctx, all.data(), ctx->d_pmeta.p, sizeof(uint32_t) * slots,
                          cudaMemcpyDeviceToHost));
    compact(all.data(), meta.data());
    for (int64_t q = 0; q < P; q++)
      for (int c = 0; c < 3; c++) shift[3 * q + c] = (int32_t)(int8_t)((meta[q] >> (8 * c)) & 0xff);
  }
  if (d2 && P > 0) {
    int rc = pair_d2(ctx);
    if (rc) return rc;
    FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> all(slots);
    FNETG_CUDA(copy_sync(ctx, all.data(), ctx->d_d2.p, sizeof(double) * slots, cudaMemcpyDeviceToHost));
    compact(all.data(), d2);
  }
  return FNETG_OK;
}

int fnetg_acsf(fnetg_ctx *ctx, double *vals) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(!ctx->gf.empty(), FNETG_E_INVALID, "acsf: no G-functions set");
  if (!ctx->nb_valid) {
    int rc = run_neighbors(ctx, ctx->rcut_classes.back());
    if (rc) return rc;
  }
  int rc = run_acsf(ctx);
  if (rc) return rc;
  rc = run_ext_inputs(ctx);
  if (rc) return rc;
  ctx->zprec_valid = false;
  if (vals) {
    const int ng = (int)ctx->gf.size();
    int32_t nf = 0;
    std::vector<double> all((size_t)ctx->N * ctx->nf);
    rc = fnetg_get_features(ctx, all.data(), &nf);
    if (rc) return rc;
    for (int64_t a = 0; a < ctx->N; a++)
      for (int k = 0; k < ng; k++) vals[a * ng + k] = all[a * nf + k];
  }
  return FNETG_OK;
}

int fnetg_acsf_zscore(fnetg_ctx *ctx, const int32_t *weights, double *zprec, int32_t compute) {
  if (!ctx || !zprec) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "acsf_zscore: no features computed");
  const int ng = (int)ctx->gf.size();
  if (!compute) ctx->h_zprec.assign(zprec, zprec + 2 * ng);
  int rc = run_zscore(ctx, weights, compute != 0);
  if (rc) return rc;
  if (compute) memcpy(zprec, ctx->h_zprec.data(), sizeof(double) * 2 * ng);
  ctx->zprec_valid = true;
  return FNETG_OK;
}

int fnetg_set_external_inputs(fnetg_ctx *ctx, int32_t n, const int32_t *indices) {
  if (!ctx || n < 0 || (n > 0 && !indices)) return FNETG_E_INVALID;
  for (int k = 0; k < n; k++)
    FNETG_CHECK(indices[k] >= 1 && indices[k] <= ctx->next, FNETG_E_SHAPE,
                "external input index out of range");
  ctx->ext_idx.assign(indices, indices + n);
  ctx->nf = (int)ctx->gf.size() + n;
  ctx->feats_valid = false;
  return FNETG_OK;
}

int fnetg_get_features(fnetg_ctx *ctx, double *feats, int32_t *nf_out) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "get_features: no features computed");
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  const int nf = ctx->nf;
  if (nf_out) *nf_out = nf;
  if (!feats) return FNETG_OK;
  const int64_t N = ctx->N;
  std::vector<int32_t> bpos(N);
  if (N > 0)
    FNETG_CUDA(copy_sync(ctx, bpos.data(), ctx->d_bpos.p, sizeof(int32_t) * N, cudaMemcpyDeviceToHost));
  if (ctx->prec == FNETG_FP64) {
    std::vector<double> buf((size_t)N * nf);
    if (N > 0)
      FNETG_CUDA(copy_sync(ctx, buf.data(), ctx->d_feat.p, sizeof(double) * buf.size(),
                            cudaMemcpyDeviceToHost));
    for (int64_t a = 0; a < N; a++)
      for (int k = 0; k < nf; k++) feats[a * nf + k] = buf[(size_t)bpos[a] * nf + k];
  } else {
    std::vector<float> buf((size_t)N * nf);
    if (N > 0)
      FNETG_CUDA(copy_sync(ctx, buf.data(), ctx->d_feat.p, sizeof(float) * buf.size(),
                            cudaMemcpyDeviceToHost));
    for (int64_t a = 0; a < N; a++)
      for (int k = 0; k < nf; k++) feats[a * nf + k] = buf[(size_t)bpos[a] * nf + k];
  }
  return FNETG_OK;
}

int fnetg_set_features(fnetg_ctx *ctx, int32_t nf, const double *feats) {
  if (!ctx || nf <= 0 || (!feats && ctx->N > 0)) return FNETG_E_INVALID;
  ctx->feat_gen++;
  const int64_t N = ctx->N;
  std::vector<int32_t> bpos(std::max<int64_t>(N, 1));
  if (N > 0)
    FNETG_CUDA(copy_sync(ctx, bpos.data(), ctx->d_bpos.p, sizeof(int32_t) * N, cudaMemcpyDeviceToHost));
  const size_t es = ctx->prec == FNETG_FP64 ? 8 : 4;
  FNETG_CUDA(ctx->d_feat.ensure(es * std::max<int64_t>(N, 1) * nf));
  if (ctx->prec == FNETG_FP64) {
    std::vector<double> buf((size_t)N * nf);
    for (int64_t a = 0; a < N; a++)
      for (int k = 0; k < nf; k++) buf[(size_t)bpos[a] * nf + k] = feats[a * nf + k];
    if (N > 0)
      FNETG_CUDA(copy_sync(ctx, ctx->d_feat.p, buf.data(), 8 * buf.size(), cudaMemcpyHostToDevice));
  } else {
    std::vector<float> buf((size_t)N * nf);
    for (int64_t a = 0; a < N; a++)
      for (int k = 0; k < nf; k++) buf[(size_t)bpos[a] * nf + k] = (float)feats[a * nf + k];
    if (N > 0)
      FNETG_CUDA(copy_sync(ctx, ctx->d_feat.p, buf.data(), 4 * buf.size(), cudaMemcpyHostToDevice));
  }
  ctx->nf = nf;
  ctx->feats_valid = true;
  ctx->zprec_valid = false;
  return FNETG_OK;
}

// ---------------------------------------------------------------------------------------
int64_t fnetg_nparams(int32_t nlayer, const int32_t *dims) {
  if (nlayer < 2 || !dims) return -1;
  int64_t n = 0;
  for (int l = 0; l < nlayer - 1; l++) n += (int64_t)dims[l] * dims[l + 1];
  n += dims[nlayer - 1];
  for (int l = 0; l < nlayer; l++) n += dims[l];
  return n;
}

int fnetg_set_network(fnetg_ctx *ctx, int32_t nspecies, int32_t nlayer, const int32_t *dims,
                      int32_t activation, const double *params) {
  if (!ctx || !dims || !params) return FNETG_E_INVALID;
  FNETG_CHECK(nspecies >= 1 && nspecies <= 64, FNETG_E_INVALID, "1..64 sub-networks");
  FNETG_CHECK(nlayer >= 2 && nlayer <= kMaxLayers, FNETG_E_UNSUPPORTED, "2..16 layers");
  FNETG_CHECK(activation >= 0 && activation <= 9, FNETG_E_INVALID, "activation code");
  for (int l = 0; l < nlayer; l++)
    FNETG_CHECK(dims[l] >= 1 && dims[l] <= kMaxWidth, FNETG_E_UNSUPPORTED,
                "layer widths must be 1..256");
  for (int64_t a = 0; a < ctx->N; a++)
    FNETG_CHECK(ctx->h_species[a] < nspecies, FNETG_E_SHAPE,
                "an atom's species index exceeds the number of sub-networks");
  ctx->nsp = nspecies;
  ctx->nlayer = nlayer;
  ctx->dims.assign(dims, dims + nlayer);
  ctx->act = activation;
  ctx->nparams = fnetg_nparams(nlayer, dims);
  ctx->woff.assign(nlayer, 0);
  ctx->boff.assign(nlayer, 0);
  int64_t ind = 0;
  for (int l = 0; l < nlayer; l++) {
    ctx->woff[l] = ind;
    ind += (int64_t)dims[l] * (l < nlayer - 1 ? dims[l + 1] : 1);
  }
  for (int l = 0; l < nlayer; l++) {
    ctx->boff[l] = ind;
    ind += dims[l];
  }
  const size_t n = (size_t)nspecies * ctx->nparams;
  for (size_t q = 0; q < n; q++)
    FNETG_CHECK(std::isfinite(params[q]), FNETG_E_INVALID, "non-finite network parameter");
  FNETG_CUDA(ctx->d_params64.ensure(sizeof(double) * n));
  FNETG_CUDA(ctx->d_params.ensure((ctx->prec == FNETG_FP64 ? 8 : 4) * n));
  FNETG_CUDA(copy_sync(ctx, ctx->d_params64.p, params, sizeof(double) * n, cudaMemcpyHostToDevice));
  ctx->net_set = true;
  ctx->opt_set = false;
  // the bucket order depends on the species only: features stay valid
  int rc = rebuild_buckets(ctx, false);
  if (rc) return rc;
  return run_params_to_compute(ctx);
}

int fnetg_get_params(fnetg_ctx *ctx, double *params) {
  if (!ctx || !params) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "get_params: no network");
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  FNETG_CUDA(copy_sync(ctx, params, ctx->d_params64.p, sizeof(double) * ctx->nsp * ctx->nparams,
                        cudaMemcpyDeviceToHost));
  return FNETG_OK;
}

static int check_ready_for_network(fnetg_ctx *ctx) {
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "no network set");
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "no features computed");
  FNETG_CHECK(ctx->nf == ctx->dims[0], FNETG_E_SHAPE,
              "network input width differs from the number of features");
  return FNETG_OK;
}

int fnetg_predict(fnetg_ctx *ctx, double *atomic_out, double *global_out) {
  if (!ctx) return FNETG_E_INVALID;
  int rc = check_ready_for_network(ctx);
  if (rc) return rc;
  // the forward at these parameters and inputs is already on the device (a training
  // iteration's gradient evaluation leaves it there): reused
  if (ctx->out_pgen != ctx->param_gen || ctx->out_fgen != ctx->feat_gen) {
    rc = run_predict(ctx);
    if (rc) return rc;
  }
  if (!atomic_out && !global_out) return FNETG_OK;
  const int nout = ctx->dims.back();
  if (atomic_out) {
    // atomic outputs straight into the caller's buffer; the sums over each structure's atoms
    // in atom order on the host
    if (ctx->N > 0)
      FNETG_CUDA(copy_sync(ctx, atomic_out, ctx->d_out.p, sizeof(double) * ctx->N * nout,
                            cudaMemcpyDeviceToHost));
    if (global_out) {
      for (int s = 0; s < ctx->S; s++)
        for (int o = 0; o < nout; o++) {
          double acc = 0.0;
          for (int64_t a = ctx->h_off[s]; a < ctx->h_off[s + 1]; a++)
            acc += atomic_out[a * nout + o];
          global_out[(size_t)s * nout + o] = acc;
        }
    }
    return FNETG_OK;
  }
  // sums only: the same atom-order sums on the device, S * nout values downloaded
  if (ctx->S > 0) {
    FNETG_CUDA(ctx->d_gsum.ensure(sizeof(double) * ctx->S * nout));
    {
      LaunchScope ls(ctx, "struct_sum");
      struct_sum_kernel<<<ceil_div((int64_t)ctx->S * nout, 128), 128, 0, ctx->stream>>>(
          ctx->d_out.as<double>(), ctx->d_off.as<int64_t>(), ctx->S, nout, ctx->d_gsum.as<double>());
      FNETG_CUDA(cudaGetLastError());
    }
    FNETG_CUDA(copy_sync(ctx, global_out, ctx->d_gsum.p, sizeof(double) * ctx->S * nout,
                          cudaMemcpyDeviceToHost));
  }
  return FNETG_OK;
}

int fnetg_jacobian(fnetg_ctx *ctx, double *jac) {
  if (!ctx || !jac) return FNETG_E_INVALID;
  int rc = check_ready_for_network(ctx);
  if (rc) return rc;
  const int nout = ctx->dims.back(), nf = ctx->nf;
  const int64_t N = ctx->N;
  std::vector<double> buf((size_t)std::max<int64_t>(N, 1) * nf);
  for (int o = 0; o < nout; o++) {
    rc = run_jacobian(ctx, o, nullptr);
    if (rc) return rc;
    FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (N > 0)
      FNETG_CUDA(copy_sync(ctx, buf.data(), ctx->d_jac.p, sizeof(double) * N * nf,
                            cudaMemcpyDeviceToHost));
    for (int64_t a = 0; a < N; a++)
      for (int f = 0; f < nf; f++) jac[(a * nout + o) * nf + f] = buf[a * nf + f];
  }
  return FNETG_OK;
}

int fnetg_forces(fnetg_ctx *ctx, double *forces) {
  if (!ctx) return FNETG_E_INVALID;
  int rc = check_ready_for_network(ctx);
  if (rc) return rc;
  FNETG_CHECK(ctx->nb_valid, FNETG_E_INVALID, "forces: no neighbour list");
  rc = run_forces(ctx);
  if (rc) return rc;
  if (forces) {
    FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
    const int nout = ctx->dims.back();
    if (ctx->N > 0)
      FNETG_CUDA(copy_sync(ctx, forces, ctx->d_forces.p, sizeof(double) * ctx->N * nout * 3,
                            cudaMemcpyDeviceToHost));
  }
  return FNETG_OK;
}

// ---------------------------------------------------------------------------------------
int fnetg_set_targets(fnetg_ctx *ctx, int32_t ngt, int32_t nat, const double *gt,
                      const double *at, const double *atomic_w, const int32_t *weights) {
  if (!ctx || ngt < 0 || nat < 0) return FNETG_E_INVALID;
  FNETG_CHECK(ngt + nat > 0, FNETG_E_INVALID, "no targets");
  FNETG_CHECK(ngt == 0 || gt, FNETG_E_INVALID, "global targets missing");
  FNETG_CHECK(nat == 0 || at, FNETG_E_INVALID, "atomic targets missing");
  const int64_t N = ctx->N;
  const int S = ctx->S;
  ctx->ngt = ngt;
  ctx->nat = nat;
  std::vector<double> aw(std::max<int64_t>(N, 1), 1.0);
  if (atomic_w) aw.assign(atomic_w, atomic_w + N);
  std::vector<int32_t> w(std::max(S, 1), 1);
  if (weights) w.assign(weights, weights + S);
  double sw = 0.0;
  for (int s = 0; s < S; s++) sw += (double)w[s];
  ctx->sum_weights = sw;
  // per-structure sum of atomic weights (loss weighting, loss.F90:556-559)
  std::vector<double> saw(std::max(S, 1), 0.0);
  for (int s = 0; s < S; s++) {
    double acc = 0.0;
    for (int64_t a = ctx->h_off[s]; a < ctx->h_off[s + 1]; a++) acc = acc + aw[a];
    saw[s] = acc;
  }
  FNETG_CUDA(ctx->d_gt.ensure(sizeof(double) * std::max<int64_t>((int64_t)S * ngt, 1)));
  FNETG_CUDA(ctx->d_at.ensure(sizeof(double) * std::max<int64_t>(N * nat, 1)));
  FNETG_CUDA(ctx->d_aw.ensure(sizeof(double) * std::max<int64_t>(N, 1)));
  FNETG_CUDA(ctx->d_w.ensure(sizeof(int32_t) * std::max(S, 1)));
  FNETG_CUDA(ctx->d_struct_aw.ensure(sizeof(double) * std::max(S, 1)));
  if (ngt > 0 && S > 0)
    FNETG_CUDA(copy_sync(ctx, ctx->d_gt.p, gt, sizeof(double) * S * ngt, cudaMemcpyHostToDevice));
  if (nat > 0 && N > 0)
    FNETG_CUDA(copy_sync(ctx, ctx->d_at.p, at, sizeof(double) * N * nat, cudaMemcpyHostToDevice));
  if (N > 0)
    FNETG_CUDA(copy_sync(ctx, ctx->d_aw.p, aw.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  if (S > 0) {
    FNETG_CUDA(copy_sync(ctx, ctx->d_w.p, w.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice));
    FNETG_CUDA(copy_sync(ctx, ctx->d_struct_aw.p, saw.data(), sizeof(double) * S,
                          cudaMemcpyHostToDevice));
  }
  ctx->targets_set = true;
  return FNETG_OK;
}

int fnetg_train_gradients(fnetg_ctx *ctx, int32_t loss, const int32_t *order, double *grad,
                          double *loss_out, double *atomic_out) {
  if (!ctx) return FNETG_E_INVALID;
  int rc = check_ready_for_network(ctx);
  if (rc) return rc;
  FNETG_CHECK(ctx->targets_set, FNETG_E_INVALID, "train_gradients: no targets");
  FNETG_CHECK(ctx->ngt + ctx->nat == ctx->dims.back(), FNETG_E_SHAPE,
              "network outputs must equal the number of targets");
  FNETG_CHECK(loss >= 0 && loss <= 3, FNETG_E_INVALID, "loss code");
  rc = run_train_gradients(ctx, loss, order, true);
  if (rc) return rc;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (grad)
    FNETG_CUDA(copy_sync(ctx, grad, ctx->d_grad64.p, sizeof(double) * ctx->nsp * ctx->nparams,
                          cudaMemcpyDeviceToHost));
  if (loss_out)
    FNETG_CUDA(copy_sync(ctx, loss_out, ctx->d_scalars.p, sizeof(double), cudaMemcpyDeviceToHost));
  if (atomic_out && ctx->N > 0)
    FNETG_CUDA(copy_sync(ctx, atomic_out, ctx->d_out.p, sizeof(double) * ctx->N * ctx->dims.back(),
                          cudaMemcpyDeviceToHost));
  return FNETG_OK;
}

int fnetg_update_prepare(fnetg_ctx *ctx, double *grad, double strength, double alpha,
                         double *grad_norm) {
  if (!ctx || !grad) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "update_prepare: no network");
  FNETG_CHECK(ctx->sum_weights > 0.0 || !ctx->targets_set, FNETG_E_INVALID, "sum of weights");
  const size_t n = (size_t)ctx->nsp * ctx->nparams;
  FNETG_CUDA(ctx->d_grad64.ensure(sizeof(double) * n));
  FNETG_CUDA(cudaMemcpyAsync(ctx->d_grad64.p, grad, sizeof(double) * n, cudaMemcpyHostToDevice,
                             ctx->stream));
  if (!ctx->targets_set) ctx->sum_weights = 1.0;
  int rc = run_update_prepare(ctx, strength, alpha);
  if (rc) return rc;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  FNETG_CUDA(copy_sync(ctx, grad, ctx->d_grad64.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (grad_norm)
    FNETG_CUDA(copy_sync(ctx, grad_norm, ctx->d_scalars.as<double>() + 1, sizeof(double),
                          cudaMemcpyDeviceToHost));
  return FNETG_OK;
}

}  // extern "C"
