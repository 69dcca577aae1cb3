// Finite-difference forces (forceAnalysis_finiteDiff, lib_analysis/forces.F90:85-117, 182-306):
// for every atom a and axis c of a structure, the structure is copied twice with coordinate
// (a, c) shifted by -delta and +delta; the ACSF values of each copy (standardised with the
// context's z-score statistics) go through the network and the copies' summed outputs give
//   F[a][o][c] = (P_o(-delta) - P_o(+delta)) / (2 delta).
// The copies run through the same device pipeline in a scratch context, in batches of at
// most kBatchAtoms atoms.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.cuh"

namespace {

constexpr int64_t kBatchAtoms = int64_t(1) << 21;

struct Scratch {
  fnetg_ctx *t = nullptr;
  ~Scratch() {
    if (t) fnetg_destroy(t);
  }
};

}  // namespace

using namespace fnetg;

extern "C" int fnetg_forces_fd(fnetg_ctx *ctx, double delta, double *forces) {
  if (!ctx || !forces) return FNETG_E_INVALID;
  FNETG_CHECK(delta > 0.0, FNETG_E_INVALID, "forces_fd: delta must be > 0");
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "forces_fd: no network");
  FNETG_CHECK(!ctx->gf.empty(), FNETG_E_INVALID, "forces_fd: no G-functions");
  FNETG_CHECK(ctx->species_set, FNETG_E_INVALID, "forces_fd: no species");
  const int64_t N = ctx->N;
  const int S = ctx->S;
  const int nout = ctx->dims.back();
  const int next = ctx->next;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  // host copies of the dataset and the parameters
  std::vector<double> coords((size_t)std::max<int64_t>(N, 1) * 3);
  std::vector<double> ext((size_t)std::max<int64_t>(N, 1) * std::max(next, 1));
  std::vector<double> params((size_t)ctx->nsp * ctx->nparams);
  if (N > 0) {
    FNETG_CUDA(copy_sync(ctx, coords.data(), ctx->d_coords.p, sizeof(double) * 3 * N,
                          cudaMemcpyDeviceToHost));
    if (next > 0)
      FNETG_CUDA(copy_sync(ctx, ext.data(), ctx->d_ext.p, sizeof(double) * N * next,
                            cudaMemcpyDeviceToHost));
  }
  FNETG_CUDA(copy_sync(ctx, params.data(), ctx->d_params64.p, sizeof(double) * params.size(),
                        cudaMemcpyDeviceToHost));
  std::memset(forces, 0, sizeof(double) * (size_t)N * nout * 3);

  Scratch sc;
  int rc = fnetg_create(&sc.t, ctx->prec, ctx->device);
  if (rc) return fail(ctx, rc, "forces_fd: scratch context");
  auto pass = [&](int code) {
    return code ? fail(ctx, code, std::string("forces_fd: ") + fnetg_last_error(sc.t)) : 0;
  };

  // copies in the order (structure, atom, axis, -delta then +delta)
  struct Copy {
    int s;
    int64_t a;
    int c;
    double sign;
  };
  std::vector<Copy> batch;
  int64_t batch_atoms = 0;
  auto run_batch = [&]() -> int {
    const int nb = (int)batch.size();
    if (nb == 0) return 0;
    std::vector<int64_t> off(nb + 1, 0);
    for (int k = 0; k < nb; k++)
      off[k + 1] = off[k] + (ctx->h_off[batch[k].s + 1] - ctx->h_off[batch[k].s]);
    const int64_t M = off[nb];
    std::vector<int32_t> atnum(M), species(M), periodic(nb);
    std::vector<double> xyz(3 * M), lat(9 * (size_t)nb), bext((size_t)M * std::max(next, 1));
    for (int k = 0; k < nb; k++) {
      const Copy &cp = batch[k];
      const int64_t a0 = ctx->h_off[cp.s], n = ctx->h_off[cp.s + 1] - a0;
      for (int64_t q = 0; q < n; q++) {
        atnum[off[k] + q] = ctx->h_atnum[a0 + q];
        species[off[k] + q] = ctx->h_species[a0 + q];
        for (int c = 0; c < 3; c++) xyz[3 * (off[k] + q) + c] = coords[3 * (a0 + q) + c];
        for (int e = 0; e < next; e++) bext[(off[k] + q) * next + e] = ext[(a0 + q) * next + e];
      }
      double &x = xyz[3 * (off[k] + (cp.a - a0)) + cp.c];
      x = cp.sign < 0.0 ? x - delta : x + delta;
      periodic[k] = ctx->h_periodic[cp.s];
      for (int e = 0; e < 9; e++) lat[9 * k + e] = ctx->h_lat[9 * cp.s + e];
    }
    int r = pass(fnetg_upload_structures(sc.t, nb, off.data(), atnum.data(), xyz.data(),
                                         periodic.data(), lat.data(),
                                         next > 0 ? bext.data() : nullptr, next));
    if (!r) r = pass(fnetg_set_species(sc.t, species.data()));
    if (!r) r = pass(fnetg_set_gfunctions(sc.t, (int32_t)ctx->gf.size(), ctx->gf.data()));
    if (!r) r = pass(fnetg_set_external_inputs(sc.t, (int32_t)ctx->ext_idx.size(),
                                               ctx->ext_idx.data()));
    if (!r) r = pass(fnetg_acsf(sc.t, nullptr));
    if (!r && ctx->zprec_valid) {
      std::vector<double> z = ctx->h_zprec;
      r = pass(fnetg_acsf_zscore(sc.t, nullptr, z.data(), 0));
    }
    if (!r) r = pass(fnetg_set_network(sc.t, ctx->nsp, (int32_t)ctx->dims.size(),
                                       ctx->dims.data(), ctx->act, params.data()));
    std::vector<double> glob((size_t)nb * nout);
    if (!r) r = pass(fnetg_predict(sc.t, nullptr, glob.data()));
    if (r) return r;
    // copies come in (-delta, +delta) pairs
    for (int k = 0; k + 1 < nb; k += 2) {
      const Copy &cp = batch[k];
      for (int o = 0; o < nout; o++)
        forces[(cp.a * nout + o) * 3 + cp.c] =
            (glob[(size_t)k * nout + o] - glob[(size_t)(k + 1) * nout + o]) / (2.0 * delta);
    }
    batch.clear();
    batch_atoms = 0;
    return 0;
  };
  for (int s = 0; s < S; s++) {
    const int64_t a0 = ctx->h_off[s], n = ctx->h_off[s + 1] - a0;
    for (int64_t a = a0; a < a0 + n; a++)
      for (int c = 0; c < 3; c++) {
        if (batch_atoms + 2 * n > kBatchAtoms && !batch.empty()) {
          rc = run_batch();
          if (rc) return rc;
        }
        batch.push_back(Copy{s, a, c, -1.0});
        batch.push_back(Copy{s, a, c, 1.0});
        batch_atoms += 2 * n;
      }
  }
  return run_batch();
}
