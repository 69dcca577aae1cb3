// fnetg: the fnet program (prg_fnet/fortnet.F90) on the GPU library, driven by the same
// fortnet_in.hsd input.
//
//   fnetg [INPUT.hsd] [--fp32] [--parse-only]
//
// Relative paths in the input (Dataset, Validset, NetstatFile) are taken relative to the
// input file's directory, and the outputs are written there, as the reference does when run in
// that directory: train mode writes the netstat file (every NSaveNet iterations and at the
// end), validate and predict modes write fnetout.hdf5, a Driver = Socket block runs the i-PI
// client.  --parse-only prints the processed input (settings and the species-expanded
// G-functions) as JSON without touching the GPU.
#include <cmath>
#include <cstdio>
#include <memory>
#include <random>
#include <cstring>
#include <string>
#include <vector>

#include "fnet_input.hpp"

namespace {

std::string dir_of(const std::string &p) {
  const size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string resolve(const std::string &base, const std::string &p) {
  return p.empty() || p[0] == '/' ? p : base + "/" + p;
}

// the dataset's atoms mapped onto the sub-networks of atomicNumbers (the network's order)
fnet::Dataset onto_networks(const fnet::Dataset &data, const std::vector<int32_t> &atomicNumbers) {
  fnet::Dataset d = data;
  for (size_t a = 0; a < d.localAtToAtNum.size(); a++) {
    int sp = -1;
    for (size_t s = 0; s < atomicNumbers.size(); s++)
      if (atomicNumbers[s] == d.localAtToAtNum[a]) sp = (int)s;
    if (sp < 0)
      throw fnet::Error(FNETG_E_INVALID, "BPNN does not contain sub-network of atomic number " +
                                             std::to_string(d.localAtToAtNum[a]) + ".");
    d.localAtToGlobalSp[a] = sp;
  }
  d.atomicNumbers = atomicNumbers;
  return d;
}

void print_functions(const std::vector<fnetg_gfunc> &g) {
  std::printf("\"gfunctions\": [");
  for (size_t k = 0; k < g.size(); k++)
    std::printf("%s[%d, %d, %d, %d, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g]", k ? ", " : "",
                g[k].type, g[k].atomid, g[k].z1, g[k].z2, g[k].rcut, g[k].kappa, g[k].rs,
                g[k].eta, g[k].lambda, g[k].xi);
  std::printf("]");
}

int parse_only(const fnet::InputSettings &in, const std::string &base) {
  std::printf("{\"mode\": \"%s\", \"read_netstat\": %d, \"seed\": %lld, \"seed_given\": %d,\n",
              in.mode.c_str(), in.readNetStats ? 1 : 0, (long long)in.seed, in.seedGiven ? 1 : 0);
  std::printf("\"dataset\": \"%s\", \"validset\": \"%s\", \"netstat\": \"%s\",\n",
              in.dataset.c_str(), in.validset.c_str(), in.netstatFile.c_str());
  std::printf("\"hidden\": [");
  for (size_t k = 0; k < in.hidden.size(); k++) std::printf("%s%d", k ? ", " : "", in.hidden[k]);
  std::printf("], \"activation\": %d, \"standardize\": %d, \"reduce\": %d, \"external\": \"%s\",\n",
              in.activation, in.standardize ? 1 : 0, in.reduce ? 1 : 0, in.extIndexSpec.c_str());
  const fnet::TrainingSettings &t = in.training;
  std::printf("\"training\": %d, \"optimizer\": %d, \"threshold\": %.17g, \"min_disp\": %.17g, "
              "\"max_disp\": %.17g, \"learning_rate\": %.17g, \"memory\": %d, \"linemin\": %d, "
              "\"qn_max_disp\": %d, \"niter\": %d, \"loss\": %d, \"shuffle\": %d, "
              "\"regu_strength\": %.17g, \"regu_alpha\": %.17g, \"nprintout\": %lld, "
              "\"nsavenet\": %lld,\n",
              in.hasTraining ? 1 : 0, t.optimizer, t.threshold, t.minDisplacement,
              t.maxDisplacement, t.learningRate, t.memory, t.lineMin ? 1 : 0,
              t.maxForQNDisplacement ? 1 : 0, t.nIterations, t.loss, in.shuffle ? 1 : 0,
              t.reguStrength, t.reguAlpha, (long long)in.nPrintout, (long long)in.nSaveNet);
  std::printf("\"forces\": \"%s\", \"fd_delta\": %.17g, \"socket\": %d,\n", in.forces.c_str(),
              in.fdDelta, in.socket ? 1 : 0);
  // species expansion over the training dataset's species, as processFeaturesBlock does
  std::vector<fnetg_gfunc> g = in.baseFunctions;
  if (in.hasMapping && !in.readNetStats && !in.socket) {
    const fnet::Dataset d = fnet::readHdfDataset(resolve(base, in.dataset));
    g = fnet::expandFunctions(in.baseFunctions, d.atomicNumbers, in.reduce);
  }
  print_functions(g);
  std::printf("}\n");
  return 0;
}

// loss of the context's current parameters (validation monitoring)
double loss_of(fnet::Context &ctx, int32_t loss) {
  double l = 0.0;
  ctx.check(fnetg_train_gradients(ctx.get(), loss, nullptr, nullptr, &l, nullptr));
  return l;
}

int train(const fnet::InputSettings &in, const std::string &base, int32_t prec) {
  const fnet::Dataset data = fnet::readHdfDataset(resolve(base, in.dataset));
  if (data.nGlobalTargets + data.nAtomicTargets == 0)
    throw fnet::Error(FNETG_E_INVALID, "Selected running mode requires the dataset to hold target information.");
  fnet::Netstat ns;
  std::unique_ptr<fnet::TBpnn> bpnn;
  if (in.readNetStats) {
    ns = fnet::readNetstat(resolve(base, in.netstatFile));
    bpnn.reset(new fnet::TBpnn(fnet::TBpnn::fromNetstat(ns)));
  } else {
    ns.atomicNumbers = data.atomicNumbers;
    if (in.hasMapping) ns.gFunctions = fnet::expandFunctions(in.baseFunctions, data.atomicNumbers, in.reduce);
    if (in.hasExternal) ns.extIndices = fnet::rangeToInt(in.extIndexSpec, data.nExtFeatures);
    const int nf = (int)(ns.gFunctions.size() + ns.extIndices.size());
    ns.dims.push_back(nf);
    ns.dims.insert(ns.dims.end(), in.hidden.begin(), in.hidden.end());
    ns.dims.push_back(data.nGlobalTargets + data.nAtomicTargets);
    ns.activation = in.activation;
    bpnn.reset(new fnet::TBpnn(ns.dims, ns.atomicNumbers, ns.activation));
    // without RandomSeed the reference draws one (initprogram.F90:756-758)
    const int32_t seed = in.seedGiven ? (int32_t)in.seed
                                      : (int32_t)(std::random_device{}() & 0x7fffffff);
    bpnn->initRandom(seed);
  }
  ns.nGlobalTargets = data.nGlobalTargets;
  ns.nAtomicTargets = data.nAtomicTargets;
  const fnet::Dataset d = onto_networks(data, ns.atomicNumbers);
  fnet::Context ctx(prec);
  ctx.upload(d);
  fnet::TAcsf acsf;
  acsf.gFunctions = ns.gFunctions;
  acsf.zPrec = ns.zPrec;
  acsf.extIndices = ns.extIndices;
  if (!acsf.gFunctions.empty()) {
    acsf.calculate(ctx, in.standardize);
  } else {
    std::vector<double> feats;
    for (int64_t a = 0; a < d.nTotalAtoms(); a++)
      for (int32_t col : ns.extIndices) feats.push_back(d.extFeatures[a * d.nExtFeatures + col - 1]);
    ctx.check(fnetg_set_features(ctx.get(), (int32_t)ns.extIndices.size(), feats.data()));
  }
  ns.zPrec = acsf.zPrec;
  bpnn->load(ctx);
  // validation monitoring on a second context
  std::unique_ptr<fnet::Context> vctx;
  std::unique_ptr<fnet::Dataset> vdata;
  if (!in.validset.empty()) {
    vdata.reset(new fnet::Dataset(onto_networks(fnet::readHdfDataset(resolve(base, in.validset)),
                                                ns.atomicNumbers)));
    vctx.reset(new fnet::Context(prec));
    vctx->upload(*vdata);
    fnet::TAcsf va = acsf;
    if (!va.gFunctions.empty()) va.calculate(*vctx, false);
    ctx.check(fnetg_set_targets(vctx->get(), vdata->nGlobalTargets, vdata->nAtomicTargets,
                                vdata->nGlobalTargets > 0 ? vdata->globalTargets.data() : nullptr,
                                vdata->nAtomicTargets > 0 ? vdata->atomicTargets.data() : nullptr,
                                vdata->atomicWeights.data(), vdata->weights.data()));
  }
  const fnet::TrainingSettings &st = in.training;
  ctx.check(fnetg_set_targets(ctx.get(), d.nGlobalTargets, d.nAtomicTargets,
                              d.nGlobalTargets > 0 ? d.globalTargets.data() : nullptr,
                              d.nAtomicTargets > 0 ? d.atomicTargets.data() : nullptr,
                              d.atomicWeights.data(), d.weights.data()));
  ctx.check(fnetg_optimizer_init(ctx.get(), st.optimizer, st.threshold, st.minDisplacement,
                                 st.maxDisplacement, st.learningRate, st.memory, st.lineMin ? 1 : 0,
                                 st.maxForQNDisplacement ? 1 : 0));
  const std::string netstat = resolve(base, in.netstatFile);
  const int64_t np = fnetg_nparams((int32_t)ns.dims.size(), ns.dims.data());
  ns.params.assign((size_t)np * ns.atomicNumbers.size(), 0.0);
  std::printf("Starting training...\n\n%11s      %13s      %13s%s\n", "iTrain", "Loss", "Gradients",
              vctx ? "      V-Loss" : "");
  bool converged = false;
  int it = 0;
  double best = INFINITY;
  int best_it = 0;
  for (it = 1; it <= st.nIterations; it++) {
    double loss = 0.0, grad = 0.0;
    int32_t conv = 0;
    ctx.check(fnetg_train_iteration(ctx.get(), st.loss, st.reguStrength, st.reguAlpha, nullptr, &loss,
                                    &grad, &conv));
    if (loss < best) {
      best = loss;
      best_it = it;
    }
    const bool last = conv || it == st.nIterations;
    if (in.nPrintout > 0 && (it % in.nPrintout == 0 || last)) {
      if (vctx) {
        ctx.check(fnetg_get_params(ctx.get(), ns.params.data()));
        ctx.check(fnetg_set_network(vctx->get(), (int32_t)ns.atomicNumbers.size(), (int32_t)ns.dims.size(),
                                    ns.dims.data(), ns.activation, ns.params.data()));
        std::printf("%11d      %13.6E      %13.6E      %13.6E\n", it, loss, grad,
                    loss_of(*vctx, st.loss));
      } else {
        std::printf("%11d      %13.6E      %13.6E\n", it, loss, grad);
      }
    }
    if ((in.nSaveNet > 0 && it % in.nSaveNet == 0) || last) {
      ctx.check(fnetg_get_params(ctx.get(), ns.params.data()));
      fnet::writeNetstat(netstat, ns);
    }
    if (conv) {
      converged = true;
      break;
    }
  }
  std::printf("\nTraining finished (%s)\n\nLoss Analysis (global min.)\niTrain: %d, Loss: %.6E\n",
              converged ? "gradients converged" : "max. Iterations reached", best_it, best);
  return 0;
}

int predict(const fnet::InputSettings &in, const std::string &base, int32_t prec) {
  const fnet::Netstat ns = fnet::readNetstat(resolve(base, in.netstatFile));
  const fnet::Dataset d = onto_networks(fnet::readHdfDataset(resolve(base, in.dataset)), ns.atomicNumbers);
  if (in.mode == "validate" && d.nGlobalTargets + d.nAtomicTargets == 0)
    throw fnet::Error(FNETG_E_INVALID, "Selected running mode requires the dataset to hold target information.");
  fnet::Context ctx(prec);
  ctx.upload(d);
  fnet::TAcsf acsf;
  acsf.gFunctions = ns.gFunctions;
  acsf.zPrec = ns.zPrec;
  acsf.extIndices = ns.extIndices;
  if (!acsf.gFunctions.empty()) {
    acsf.calculate(ctx, false);
  } else {
    std::vector<double> feats;
    for (int64_t a = 0; a < d.nTotalAtoms(); a++)
      for (int32_t col : ns.extIndices) feats.push_back(d.extFeatures[a * d.nExtFeatures + col - 1]);
    ctx.check(fnetg_set_features(ctx.get(), (int32_t)ns.extIndices.size(), feats.data()));
  }
  fnet::TBpnn bpnn = fnet::TBpnn::fromNetstat(ns);
  bpnn.load(ctx);
  const fnet::Predicts p = bpnn.predictBatch(ctx);
  std::vector<double> f;
  if (in.forces == "analytical") f = fnet::forceAnalysisAnalytical(ctx, bpnn);
  if (in.forces == "finitedifferences") f = fnet::forceAnalysisFiniteDiff(ctx, bpnn, in.fdDelta);
  const int nout = ns.dims.back();
  std::vector<fnet::FnetoutDatapoint> pts(d.nDatapoints());
  double emin = INFINITY, emax = 0.0;
  for (int s = 0; s < d.nDatapoints(); s++) {
    const int64_t a0 = d.atomOffsets[s], a1 = d.atomOffsets[s + 1];
    pts[s].rawPredictions.assign(p.atomic.begin() + a0 * nout, p.atomic.begin() + a1 * nout);
    if (!f.empty()) pts[s].forces.assign(f.begin() + a0 * nout * 3, f.begin() + a1 * nout * 3);
    if (in.mode == "validate") {
      pts[s].globalTargets.assign(d.globalTargets.begin() + (int64_t)s * d.nGlobalTargets,
                                  d.globalTargets.begin() + (int64_t)(s + 1) * d.nGlobalTargets);
      pts[s].atomicTargets.assign(d.atomicTargets.begin() + a0 * d.nAtomicTargets,
                                  d.atomicTargets.begin() + a1 * d.nAtomicTargets);
      for (int o = 0; o < ns.nGlobalTargets; o++) {
        const double e = std::fabs(p.global[(size_t)s * nout + o] - pts[s].globalTargets[o]);
        emin = std::fmin(emin, e);
        emax = std::fmax(emax, e);
      }
    }
  }
  fnet::writeFnetout(resolve(base, "fnetout.hdf5"), in.mode, ns.nGlobalTargets, ns.nAtomicTargets, pts);
  if (in.mode == "validate" && ns.nGlobalTargets > 0)
    std::printf("Validation\n\nmin. absolute error: %15.6E\nmax. absolute error: %15.6E\n", emin, emax);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    std::string input = "fortnet_in.hsd";
    int32_t prec = FNETG_FP64;
    bool parseOnly = false;
    for (int k = 1; k < argc; k++) {
      if (!std::strcmp(argv[k], "--fp32")) prec = FNETG_FP32;
      else if (!std::strcmp(argv[k], "--parse-only")) parseOnly = true;
      else input = argv[k];
    }
    const fnet::InputSettings in = fnet::readInput(fnet::hsd::parseFile(input));
    const std::string base = dir_of(input);
    if (parseOnly) return parse_only(in, base);
    if (in.socket) {
      const fnet::Netstat ns = fnet::readNetstat(resolve(base, in.netstatFile));
      fnet::SocketDriverSettings st = in.socketSettings;
      st.precision = prec;
      std::printf("%lld\n", (long long)fnet::runSocketDriver(ns, st));
      return 0;
    }
    return in.mode == "train" ? train(in, base, prec) : predict(in, base, prec);
  } catch (const fnet::Error &e) {
    std::fprintf(stderr, "fnetg: error %d: %s\n", e.code, e.what());
    return 1;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "fnetg: %s\n", e.what());
    return 1;
  }
}
