// Parity of the C++ host layer (fnet::TAcsf, fnet::TBpnn, force analyses, training) run on
// the GPU library against the oracle's C restatement, on seeded periodic cells with self and
// repeated images and on clusters.  Prints one line per check and exits non-zero on failure.
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "fnet_host.hpp"
#include "fnet_oracle.h"

namespace {

int failures = 0;

void check(const std::string &name, const std::vector<double> &got, const std::vector<double> &ref,
           double rtol, double atol) {
  double worst = 0.0;
  bool ok = got.size() == ref.size();
  for (size_t k = 0; ok && k < got.size(); k++) {
    const double err = std::fabs(got[k] - ref[k]);
    const double tol = atol + rtol * std::fabs(ref[k]);
    if (!(err <= tol)) ok = false;
    worst = std::fmax(worst, err / (atol + rtol * std::fabs(ref[k])));
  }
  std::printf("%s %s (%zu values, worst error / tolerance %.3g)\n", ok ? "PASS" : "FAIL",
              name.c_str(), got.size(), worst);
  if (!ok) failures++;
}

// two-species periodic cells (some smaller than the cutoff) and one cluster
fnet::Dataset make_dataset(unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  fnet::Dataset d;
  d.atomicNumbers = {1, 8};
  d.atomOffsets = {0};
  const int sizes[] = {5, 9, 14, 7};
  for (int s = 0; s < 4; s++) {
    const int n = sizes[s];
    const bool periodic = s < 3;
    const double L = 6.0 + 2.5 * s;
    std::vector<double> lat(9, 0.0);
    if (periodic) {
      lat = {L, 0.3, -0.2, 0.1, 1.1 * L, 0.25, -0.3, 0.2, 0.95 * L};
    }
    for (int a = 0; a < n; a++) {
      for (int c = 0; c < 3; c++) d.coords.push_back(u(rng) * (periodic ? L : 9.0));
      const int sp = u(rng) < 0.5 ? 0 : 1;
      d.localAtToGlobalSp.push_back(sp);
      d.localAtToAtNum.push_back(d.atomicNumbers[sp]);
      d.atomicWeights.push_back(1.0);
    }
    d.periodic.push_back(periodic ? 1 : 0);
    d.latVecs.insert(d.latVecs.end(), lat.begin(), lat.end());
    d.weights.push_back(1 + s % 2);
    d.globalTargets.push_back(-1.0 + 0.1 * s);
    d.atomOffsets.push_back(d.atomOffsets.back() + n);
  }
  d.nGlobalTargets = 1;
  return d;
}

std::vector<fnetg_gfunc> make_functions() {
  const double rc = 7.0;
  std::vector<fnetg_gfunc> g;
  for (int z : {1, 8}) {
    for (double eta : {0.05, 0.3}) g.push_back(fnetg_gfunc{2, 0, z, 0, rc, 0.0, 0.5, eta, 0.0, 0.0});
    g.push_back(fnetg_gfunc{3, 0, z, 0, rc, 1.3, 0.0, 0.0, 0.0, 0.0});
  }
  for (int z1 : {1, 8})
    for (int z2 : {1, 8}) {
      if (z2 < z1) continue;
      for (double lam : {1.0, -1.0})
        for (double xi : {1.0, 2.0, 4.0}) g.push_back(fnetg_gfunc{5, 0, z1, z2, rc, 0.0, 0.0, 0.02, lam, xi});
    }
  return g;
}

orc_batch batch_of(const fnet::Dataset &d) {
  orc_batch b{};
  b.nstruct = d.nDatapoints();
  b.atom_offsets = d.atomOffsets.data();
  b.coords = d.coords.data();
  b.atnum = d.localAtToAtNum.data();
  b.periodic = d.periodic.data();
  b.latvecs = d.latVecs.data();
  b.ext = nullptr;
  b.next = 0;
  return b;
}

}  // namespace

int main() {
  const fnet::Dataset data = make_dataset(2024);
  const std::vector<fnetg_gfunc> funcs = make_functions();
  const int ng = (int)funcs.size();
  const int64_t N = data.nTotalAtoms();
  std::vector<orc_gfunc> og;
  for (const auto &g : funcs)
    og.push_back(orc_gfunc{g.type, g.atomid, g.z1, g.z2, g.rcut, g.kappa, g.rs, g.eta, g.lambda, g.xi});
  const orc_batch b = batch_of(data);

  // ---- oracle side
  std::vector<double> vals((size_t)N * ng), zprec(2 * ng);
  orc_acsf(&b, og.data(), ng, 1, vals.data(), 1);
  orc_zscore_stats(vals.data(), N, ng, data.atomOffsets.data(), data.nDatapoints(),
                   data.weights.data(), zprec.data());
  std::vector<double> feats = vals;
  orc_zscore_apply(feats.data(), N, ng, zprec.data());
  const std::vector<int32_t> dims = {ng, 6, 5, 1};
  const orc_net net{(int32_t)dims.size(), dims.data(), ORC_ACT_TANH};
  const int64_t np = orc_nparams(&net);
  std::vector<double> p_ref((size_t)2 * np);
  void *rl = orc_ranlux_new(3, 77);
  orc_init_bpnn_params(rl, &net, 2, p_ref.data());
  orc_ranlux_free(rl);
  std::vector<double> pred_ref((size_t)N), jac_ref((size_t)N * ng), f_ref((size_t)N * 3);
  orc_predict(&net, p_ref.data(), ng, feats.data(), N, data.localAtToGlobalSp.data(), pred_ref.data());
  orc_jacobian(&net, p_ref.data(), ng, feats.data(), N, data.localAtToGlobalSp.data(), jac_ref.data());
  orc_forces_ex(&b, og.data(), ng, zprec.data(), 1, jac_ref.data(), 1, f_ref.data());

  try {
    fnet::Context ctx(FNETG_FP64);
    ctx.upload(data);
    fnet::TAcsf acsf;
    acsf.gFunctions = funcs;
    acsf.calculate(ctx, true);
    check("TAcsf z-score statistics", acsf.zPrec, zprec, 1e-11, 1e-12);
    check("TAcsf standardised values", acsf.vals(ctx), feats, 1e-10, 1e-11);

    fnet::TBpnn bpnn(dims, data.atomicNumbers, FNETG_ACT_TANH);
    bpnn.initRandom(77);
    check("TBpnn RANLUX normalXavier initialisation", bpnn.serializedWeightsAndBiases(), p_ref, 0.0, 0.0);
    bpnn.load(ctx);
    const fnet::Predicts p = bpnn.predictBatch(ctx);
    check("TBpnn predictBatch", p.atomic, pred_ref, 1e-10, 1e-12);
    check("TBpnn nJacobian", bpnn.nJacobian(ctx), jac_ref, 1e-9, 1e-11);
    check("forceAnalysis analytical", fnet::forceAnalysisAnalytical(ctx, bpnn), f_ref, 1e-8, 1e-10);

    // three L-BFGS iterations against the oracle's optimiser on the oracle's gradients
    std::vector<double> params = p_ref;
    std::vector<int32_t> order(data.nDatapoints());
    for (int s = 0; s < data.nDatapoints(); s++) order[s] = s + 1;
    double sumw = 0.0;
    for (int w : data.weights) sumw += w;
    std::vector<void *> opts;
    for (int s = 0; s < 2; s++)
      opts.push_back(orc_lbfgs_new((int32_t)np, 1e-30, 1e-6, 1.0, 20, 1, 0, params.data() + s * np));
    std::vector<double> dd(params.size()), pr((size_t)N);
    for (int it = 0; it < 3; it++) {
      orc_train_gradients(&net, params.data(), 2, ng, feats.data(), data.localAtToGlobalSp.data(),
                          data.nDatapoints(), data.atomOffsets.data(), 1, 0,
                          data.globalTargets.data(), nullptr, data.atomicWeights.data(),
                          data.weights.data(), order.data(), ORC_LOSS_MSE, dd.data(), pr.data());
      orc_update_prepare(&net, params.data(), 2, dd.data(), 0.0, 0.0, sumw);
      for (int s = 0; s < 2; s++)
        orc_lbfgs_next(opts[s], 0.0, dd.data() + s * np, params.data() + s * np);
    }
    for (void *o : opts) orc_opt_free(o);
    fnet::TrainingSettings st;
    st.optimizer = FNETG_OPT_LBFGS;
    st.threshold = 1e-30;
    st.maxDisplacement = 1.0;
    st.memory = 20;
    st.nIterations = 3;
    bpnn.nTrain(ctx, st);
    check("TBpnn nTrain (L-BFGS, 3 iterations)", bpnn.serializedWeightsAndBiases(), params, 1e-8, 1e-10);
  } catch (const fnet::Error &e) {
    std::printf("FAIL exception %d: %s\n", e.code, e.what());
    return 1;
  }
  std::printf("%s\n", failures ? "FAILED" : "ALL PASSED");
  return failures ? 1 : 0;
}
