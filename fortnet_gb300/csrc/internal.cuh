// Internal definitions of the fnetg library (context, device buffers, launch plumbing).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <atomic>
#include <vector>

#include "../../include/fnetg.h"

namespace fnetg {

// ---------------------------------------------------------------------------------------
// Index checks of the bounds-checked build (compiled with -DFNETG_CHECKS, a separate library):
// FNETG_GUARD(ok) records the first failing site (file code x 100000 + line) in the word of
// its translation unit and evaluates to ok, so that the guarded access is skipped; the
// default build compiles every guard to `true`.  fnetg_check_status reads and clears the
// words of every translation unit.
#ifdef FNETG_CHECKS
static __device__ int g_fnetg_check_site;
__device__ __forceinline__ bool fnetg_guard(bool ok, int site) {
  if (!ok) atomicCAS(&g_fnetg_check_site, 0, site);
  return ok;
}
#define FNETG_GUARD(ok) ::fnetg::fnetg_guard((ok), FNETG_FILE_CODE * 100000 + __LINE__)
// host reader of this translation unit's word (read and cleared)
#define FNETG_CHECK_READER(fn)                                                \
  int fn() {                                                                  \
    int v = 0, z = 0;                                                         \
    if (cudaMemcpyFromSymbol(&v, g_fnetg_check_site, sizeof(int)) != cudaSuccess) return -1; \
    if (cudaMemcpyToSymbol(g_fnetg_check_site, &z, sizeof(int)) != cudaSuccess) return -1;   \
    return v;                                                                 \
  }
#else
#define FNETG_GUARD(ok) true
#define FNETG_CHECK_READER(fn) \
  int fn() { return 0; }
#endif

// ---------------------------------------------------------------------------------------
// small vector types with explicit alignment (the deprecated double4 is avoided)
template <typename T> struct __align__(4 * sizeof(T)) V4 { T x, y, z, w; };

constexpr int kMaxSpeciesCodes = 8;   // distinct atomic numbers referenced by G-functions
constexpr int kMaxRcutClasses = 8;    // distinct cutoffs in one G-function set
constexpr int kMaxEtaClasses = 16;    // distinct (eta, rcut, atomid) of angular functions
constexpr int kMaxGroupFuncs = 32;    // angular functions evaluated together per channel
constexpr int kMaxLayers = 16;
constexpr int kMaxWidth = 256;        // widest network layer supported by the SIMT MLP

// G-function descriptor as the kernels see it (prepared on the host).
struct GDesc {
  int type;     // 1..5
  int chan1;    // species code of list 1, -1 = all atoms (unresolved)
  int chan2;    // species code of list 2 (angular), -1 = all atoms
  int atomid;   // 0 or 1-based external-feature column
  int out;      // output column in the feature row
  int rclass;   // cutoff class
  int eclass;   // E-table class (angular), -1 if none
  int xi_int;   // xi as an integer in [1, 16] if integral, else 0
  double rcut, kappa, rs, eta, lambda, xi, pref;  // pref = 2^(1 - xi)
};

// A group of angular functions sharing list channels (evaluated in one triplet sweep).
struct AGroup {
  int chan1, chan2;  // species codes, -1 = all
  int same;          // 1 if the two lists are the same list (Z1 == Z2 or unresolved)
  int first, count;  // range into the angular descriptor array
  int has_g4;
  int atomid;        // shared by every function of the group (0 = none)
};

// Angular G5 function with an integer xi <= kMaxMomentDegree, evaluated through moment tensors:
// sum_{j,k} (1 + lambda u_j.u_k)^xi E_j E_k = sum_alpha coef(alpha) M1(alpha) M2(alpha).
constexpr int kMaxMomentDegree = 4;
constexpr int kMaxMono = 35;  // monomials of degree <= 4 in three variables
struct MFunc {
  int k1, k2;  // moment combos (list, eta class) of the two neighbour lists
  int out;     // output column
  int pair;    // index of the combo pair (min(k1, k2), max(k1, k2)) among the distinct pairs
};

// Stream-ordered allocation from a memory pool, for contexts driven by one host thread each
// (the prediction service's lanes): set per thread through DBuf::pool.
struct PoolAlloc {
  cudaMemPool_t pool;
  cudaStream_t stream;
};

// Device buffer with grow-only reallocation.  A regrowth allocates 1/8 more than asked, so
// that slowly growing sizes do not reallocate.  Plain allocations use cudaMalloc/cudaFree
// (which synchronise the whole device); when the allocating thread has set DBuf::pool, the
// buffer comes from that pool in the order of that stream (no device-wide synchronisation,
// and no new device mappings while the pool holds enough reserved memory).  Allocations made
// by a host thread are added to *account when the thread has set it.
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  bool pooled = false;
  cudaStream_t pool_stream = nullptr;
  inline static thread_local std::atomic<int64_t> *account = nullptr;
  inline static thread_local const PoolAlloc *pool = nullptr;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      if (pooled) cudaFreeAsync(p, pool_stream);
      else cudaFree(p);
    }
    if (p && account) *account -= (int64_t)bytes;
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    const bool regrow = p != nullptr;
    release();
    if (n == 0) n = 16;
    if (regrow) n += n / 8;
    cudaError_t e;
    if (pool) {
      e = cudaMallocFromPoolAsync(&p, n, pool->pool, pool->stream);
      pooled = true;
      pool_stream = pool->stream;
    } else {
      e = cudaMalloc(&p, n);
      pooled = false;
    }
    if (e == cudaSuccess) {
      bytes = n;
      if (account) *account += (int64_t)n;
    } else {
      p = nullptr;
    }
    return e;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

struct ProfEntry {
  double ms = 0.0;
  int64_t launches = 0;
};

struct PendingLaunch {
  const char *name;
  cudaEvent_t e0, e1;
};

// state of the batched mixed-precision form (batch.cu)
struct BatchState;
void batch_free(BatchState *b);

}  // namespace fnetg

struct fnetg_ctx {
  int prec = FNETG_FP32;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // structures
  int32_t S = 0;
  int64_t N = 0;
  std::vector<int64_t> h_off;
  std::vector<int32_t> h_atnum, h_periodic;
  std::vector<double> h_lat;
  int32_t next = 0;
  // d_coordsf: [2N] float coordinates relative to the structure's box corner, high parts then
  // the low parts (coordinate - high part); d_coords_in: coordinates of fnetg_update_coords
  // until they are checked
  fnetg::DBuf d_off, d_atom_struct, d_coords, d_coordsf, d_atnum, d_lat, d_ranges, d_bbox,
      d_ext, d_periodic, d_coords_in;

  // species (sub-network index per atom) and bucketing
  bool species_set = false;
  std::vector<int32_t> h_species;
  // bumped whenever the structures or the atoms' species change (plans built on them compare it)
  uint64_t layout_gen = 0;
  std::vector<int64_t> h_bucket_off;  // [nsp+1] rows of every species bucket
  std::vector<int64_t> h_tiles;       // packed (species, row0, nrows) triples for MLP tiles
  fnetg::DBuf d_species, d_bpos, d_bperm, d_tiles;
  int64_t ntiles = 0;
  int tile_rows = 0;

  // G-functions
  std::vector<fnetg_gfunc> gf;
  std::vector<fnetg::GDesc> h_rad, h_ang;
  std::vector<fnetg::GDesc> h_ang_all;  // every angular function in input order (h_ang holds
                                        // only the triplet-sweep ones)
  fnetg::DBuf d_ang_all, d_jvp_ang, d_jvp_grp;
  std::vector<int> rad_seg;  // [kMaxSpeciesCodes + 2]: all-atom radial functions [0, rad_seg[1]),
                             // species code c in [rad_seg[c + 1], rad_seg[c + 2])
  std::vector<int32_t> h_radv;  // value-kernel order of h_rad: by shape (type, cutoff class,
                                // atom id, rs / eta / kappa), then list channel
  std::vector<fnetg::AGroup> h_groups;
  std::vector<double> rcut_classes;
  std::vector<double> ecls_eta;
  std::vector<int> ecls_rclass, ecls_atomid;
  std::vector<int32_t> zcodes;  // atomic numbers of species codes
  // moment form of the integer-xi G5 functions
  int mom_degree = 0, n_mono = 0, n_combo = 0;
  std::vector<fnetg::MFunc> h_mfunc;
  std::vector<int32_t> h_combo;     // [ncombo][2] (list code or -1 = all, eta class)
  std::vector<int32_t> h_cidx;      // [(nz+1) * necls] combo index, -1 if unused
  fnetg::DBuf d_mfunc, d_combo, d_cidx;
  std::vector<double> h_mpc;    // [entries][kMaxMomentDegree + 1] degree coefficients of the
                                // adjoint group entries
  int n_qgroups = 0;            // adjoint partner groups over all combos
  fnetg::DBuf d_qgroups, d_mpc_d, d_mpc_f;
  // kernel parameter copies in both arithmetic widths: [rcut, kappa, rs, eta, lambda, xi, pref, 0]
  fnetg::DBuf d_radpar_f, d_radpar_d, d_angpar_f, d_angpar_d, d_ecls_eta_f, d_rcls_f;
  fnetg::DBuf d_rad, d_radv, d_ang, d_groups, d_code, d_ecls_eta, d_ecls_rclass, d_ecls_atomid,
      d_rcls;

  // neighbour list
  bool nb_valid = false;
  double nb_rcut = 0.0;
  int64_t P = 0;
  int max_pairs = 0;
  bool d2_valid = false;
  double max_extent = 0.0;  // largest structure bounding-box extent (Bohr)
  fnetg::DBuf d_img_off, d_imgs, d_imgs_f;
  // G5 moments of every atom from the last ACSF launch ([N][ncombo][n_mono], compute width),
  // reused by the force kernel while geometry, pairs and functions are unchanged
  bool mom_valid = false;
  fnetg::DBuf d_mom;
  // Pairs of atom i: [poff[i], pend[i]).  Counted builds store them compactly (CSR, pend =
  // poff + 1); slab builds at [i * cap, i * cap + count) with an explicit end array.
  bool pslab = false;
  int64_t pslots = 0;       // allocated pair slots (P when compact)
  int64_t nb_cap_hint = 0;  // per-atom capacity for the next slab build (0: count first)
  // lattice-point tables of the last build, reused while the lattices, periodic flags, cutoff
  // and cutoff classes are unchanged (coordinates may move)
  bool nbimg_valid = false;
  double nbimg_rcut = 0.0;
  std::vector<double> nbimg_lat, nbimg_rcls;
  std::vector<int32_t> nbimg_periodic, nbimg_ranges;
  double nbimg_shift = 0.0;  // largest translation of an image over all structures
  int64_t nb_hint_n = -1;   // atom count the capacity was measured on
  fnetg::DBuf d_pcount, d_poff, d_pend, d_pj, d_pmeta, d_rij, d_d2, d_scan_tmp, d_maxp, d_rcls2;
  // cell lists of the larger structures (rebuilt with every neighbour search)
  int64_t ncells = 0;
  fnetg::DBuf d_cgrid, d_cnum, d_coff, d_ccount, d_cstart, d_cfill, d_akey, d_cpos;

  // features (bucketed rows, compute precision)
  int nf = 0;
  bool feats_valid = false;
  std::vector<int32_t> ext_idx;
  fnetg::DBuf d_feat, d_zprec, d_zprec_f, d_zpart, d_extidx;
  std::vector<double> h_zprec;
  bool zprec_valid = false;

  // network
  bool net_set = false;
  int nsp = 0, nlayer = 0, act = 0;
  std::vector<int32_t> dims;
  int64_t nparams = 0;
  std::vector<int64_t> woff, boff;
  std::vector<int64_t> h_sp_tile0;  // [nsp+1] first MLP tile of every species
  int n_qgpack = 0, n_qgent = 0;  // ints of the adjoint group pack, entries of its coefficients
  // value kernel: distinct moment-combo pairs (k1 <= k2) of the G5 moment functions and every
  // function's degree coefficients pc_f(m) (MFunc::pad holds the function's pair)
  std::vector<int32_t> h_mpair;
  std::vector<double> h_fpc;
  fnetg::DBuf d_mpair, d_fpc_d, d_fpc_f;
  int rad_fast = -1;  // every radial function a G2 without atom id in this cutoff class (else -1)
  // MLP launch variants picked by timing on first use, per precision and kernel kind
  // (forward, Jacobian, backward), for the network shape mlp_dims
  int mlp_cfg[6] = {-1, -1, -1, -1, -1, -1};
  std::vector<int32_t> mlp_dims;
  fnetg::DBuf d_params64, d_params, d_ref_of_compute, d_sp_tile0;
  std::vector<int64_t> h_ref_of_compute;  // the table last uploaded to d_ref_of_compute
  fnetg::DBuf d_gchunk;  // FP64 gradient sums of tile chunks

  // versions of the network inputs and of the compute parameters; d_out holds the plain form's
  // forward at (out_fgen, out_pgen), -1 when another kernel wrote it
  int64_t feat_gen = 0, param_gen = 0, out_fgen = -1, out_pgen = -1;

  // outputs / training
  int ngt = 0, nat = 0;
  bool targets_set = false;
  fnetg::DBuf d_gt, d_at, d_aw, d_w, d_out, d_gsum, d_lossgrad, d_losspart, d_gpart, d_grad64,
      d_order, d_jac, d_jacT, d_forces, d_forces4, d_scalars, d_struct_aw;
  double sum_weights = 0.0;

  // optimiser state (device)
  bool opt_set = false;
  int opt_kind = 0;
  bool opt_started = false;
  fnetg::DBuf d_opt;        // per-species optimiser state blocks (FP64)
  size_t opt_stride = 0;    // doubles per species block
  double opt_threshold = 0, opt_min_disp = 0, opt_max_disp = 0, opt_lr = 0;
  int opt_mem = 0, opt_linemin = 1, opt_qn = 0;
  fnetg::DBuf d_xnew, d_conv;
  void *h_pinned = nullptr;  // small pinned staging area for scalars

  // force-loss training: weight c of c / (3 N) sum |F - F*|^2 (0 = energies only), FP64
  // target forces [N][3], the loss's force gradient w [N][3], feature tangents u [N][nf],
  // per-tile gradient partials
  double fl_weight = 0.0;
  bool jac_ready = false;  // d_jacT already holds the Jacobian the force kernel needs
  fnetg::DBuf d_fl_target, d_fl_w, d_fl_u, d_fl_part, d_fl_gpart;

  // batched mixed-precision form: mini-batch tiles, packed BF16 features and weights, the
  // captured epoch (owned; freed with the context)
  fnetg::BatchState *batch = nullptr;
  bool batch_train = false;  // training gradients from the tensor-core kernels

  // profiling
  bool prof = false;
  std::map<std::string, fnetg::ProfEntry> prof_tab;
  std::vector<fnetg::PendingLaunch> ev_pending;
  std::vector<cudaEvent_t> ev_free;
  int64_t launches = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace fnetg {

// error helpers -------------------------------------------------------------------------
int fail(fnetg_ctx *c, int code, const std::string &msg);
int cuda_fail(fnetg_ctx *c, cudaError_t e, const char *where);

#define FNETG_CUDA(call)                                        \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return ::fnetg::cuda_fail(ctx, _e, #call); \
  } while (0)

#define FNETG_CHECK(cond, code, msg)                   \
  do {                                                 \
    if (!(cond)) return ::fnetg::fail(ctx, code, msg); \
  } while (0)

// launch accounting: every kernel launch of the library goes through these
struct LaunchScope {
  fnetg_ctx *c;
  const char *name;
  cudaEvent_t e0 = nullptr;
  LaunchScope(fnetg_ctx *ctx, const char *n);
  ~LaunchScope();
};

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
// Raise (never lower) a kernel's dynamic shared-memory limit on the current device.  The
// limit is per kernel, not per launch: contexts on other host threads launch the same kernel
// with other sizes, and lowering it under them would make their launches fail.
cudaError_t raise_smem_limit(const void *kernel, size_t bytes);
// A copy on the context's stream, waited for: ordered after the context's kernels (the
// stream does not synchronise with the legacy default stream), and the host buffer may be
// released on return.  Contexts on other host threads are not waited for.
inline cudaError_t copy_sync(fnetg_ctx *c, void *dst, const void *src, size_t bytes,
                             cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, c->stream);
  return e == cudaSuccess ? cudaStreamSynchronize(c->stream) : e;
}
int num_sms();
void resolve_profile(fnetg_ctx *c);

// Loss functions of lib_common/loss.F90 (217-721) for one prediction p and target t: the
// gradient of the loss term, the term, and the term sums turned into the loss value.
__device__ __forceinline__ double lossgrad(int loss, double p, double t) {
  switch (loss) {
    case FNETG_LOSS_RMS: return (p - t) / sqrt((p - t) * (p - t));
    case FNETG_LOSS_MAE: return (p - t) / fabs(p - t);
    case FNETG_LOSS_MAPE: return 100.0 * (p - t) / (t * t * fabs(p / t - 1.0));
    default: return 2.0 * (p - t);
  }
}
__device__ __forceinline__ double loss_term(int loss, double p, double t) {
  switch (loss) {
    case FNETG_LOSS_MAE: return fabs(t - p);
    case FNETG_LOSS_MAPE: return fabs((t - p) / t);
    default: return (t - p) * (t - p);
  }
}
__device__ __forceinline__ double loss_finish(int loss, double sum, int n) {
  switch (loss) {
    case FNETG_LOSS_RMS: return sqrt(sum / (double)n);
    case FNETG_LOSS_MAPE: return 100.0 * sum / (double)n;
    default: return sum / (double)n;
  }
}

// kernels' host entry points (one per translation unit)
int run_neighbors(fnetg_ctx *ctx, double rcut);
int prepare_coords(fnetg_ctx *ctx);
// Largest structure bounding-box diagonal of the device coordinates d_xyz [N][3] and whether
// any of them is not finite (one reduction on the device, 16 bytes read back, synchronous).
int coords_summary(fnetg_ctx *ctx, const double *d_xyz, double *max_extent, bool *nonfinite);
int pair_d2(fnetg_ctx *ctx);
const int64_t *pair_end(fnetg_ctx *ctx);  // device end offsets of every atom's pairs
int run_acsf(fnetg_ctx *ctx);
int run_zscore(fnetg_ctx *ctx, const int32_t *weights, bool compute);
int run_ext_inputs(fnetg_ctx *ctx);
int run_predict(fnetg_ctx *ctx);
int run_jacobian(fnetg_ctx *ctx, int out_index, void *dst);
int run_forces(fnetg_ctx *ctx);
int run_train_gradients(fnetg_ctx *ctx, int loss, const int32_t *order, bool need_predict);
int run_force_gradients(fnetg_ctx *ctx, int loss);
int run_force_loss_terms(fnetg_ctx *ctx);
int run_batch_gradients(fnetg_ctx *ctx, int loss);
int run_features_jvp(fnetg_ctx *ctx, const void *d_w, void *d_u);
int run_update_prepare(fnetg_ctx *ctx, double strength, double alpha);
int run_optimizer_step(fnetg_ctx *ctx);
int run_params_to_compute(fnetg_ctx *ctx);
int exclusive_scan_i64(fnetg_ctx *ctx, const int64_t *in, int64_t *out, int64_t n);
// check words of the bounds-checked build (0 = no failed check; always 0 in the default build)
int check_site_neighbors();
int check_site_acsf();
int check_site_forces();
int check_site_mlp();
int check_site_batch();
int check_site_jvp();

}  // namespace fnetg
