// fnetg_run: the validate / predict flow of the fnet program (fortnet.F90:1047-1059) on the
// GPU library, driven from a Fortnet dataset and a netstat file.
//
//   fnetg_run DATASET NETSTAT [--fp32] [--forces analytical | --forces fd DELTA]
//       featurise with the netstat's ACSF mapping and z-score statistics, predict every
//       atom, optionally compute forces; prints one JSON object (atomic and global
//       predictions, forces).
//   fnetg_run --dump DATASET [NETSTAT]
//       read the files only (no GPU) and print what was read as JSON.
//   fnetg_run --copy-netstat NETSTAT OUT
//       read a netstat file and write the model it holds to OUT (no GPU).
//
// With --fnetout FILE [--mode predict|validate] the run also writes the reference's fnetout
// file (predictions, forces, and in validate mode the dataset's targets).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fnet_host.hpp"

namespace {

void print_array(const char *name, const std::vector<double> &v, bool last = false) {
  std::printf("\"%s\": [", name);
  for (size_t k = 0; k < v.size(); k++) std::printf(k ? ", %.17g" : "%.17g", v[k]);
  std::printf("]%s\n", last ? "" : ",");
}

template <typename T> std::vector<double> as_double(const std::vector<T> &v) {
  return std::vector<double>(v.begin(), v.end());
}

int dump(const char *dataset, const char *netstat) {
  const fnet::Dataset d = fnet::readHdfDataset(dataset);
  std::printf("{\n\"ndatapoints\": %d, \"ntotal\": %lld, \"nglobaltargets\": %d, "
              "\"natomictargets\": %d, \"nextfeatures\": %d,\n",
              d.nDatapoints(), (long long)d.nTotalAtoms(), d.nGlobalTargets, d.nAtomicTargets,
              d.nExtFeatures);
  print_array("atom_offsets", as_double(d.atomOffsets));
  print_array("coords", d.coords);
  print_array("atnum", as_double(d.localAtToAtNum));
  print_array("species", as_double(d.localAtToGlobalSp));
  print_array("periodic", as_double(d.periodic));
  print_array("latvecs", d.latVecs);
  print_array("atomic_numbers", as_double(d.atomicNumbers));
  print_array("weights", as_double(d.weights));
  print_array("atomic_weights", d.atomicWeights);
  print_array("global_targets", d.globalTargets);
  print_array("atomic_targets", d.atomicTargets);
  print_array("ext", d.extFeatures, netstat == nullptr);
  if (netstat) {
    const fnet::Netstat ns = fnet::readNetstat(netstat);
    std::vector<double> gf;
    for (const auto &g : ns.gFunctions) {
      const double row[10] = {(double)g.type, g.rcut, g.kappa, g.rs, g.eta, g.lambda, g.xi,
                              (double)g.atomid, (double)g.z1, (double)g.z2};
      gf.insert(gf.end(), row, row + 10);
    }
    print_array("gfunctions", gf);
    print_array("zprec", ns.zPrec);
    print_array("ext_indices", as_double(ns.extIndices));
    print_array("net_atomic_numbers", as_double(ns.atomicNumbers));
    print_array("dims", as_double(ns.dims));
    std::printf("\"activation\": %d, \"nglobal\": %d, \"natomic\": %d,\n", ns.activation,
                ns.nGlobalTargets, ns.nAtomicTargets);
    print_array("params", ns.params, true);
  }
  std::printf("}\n");
  return 0;
}

int run(int argc, char **argv) {
  const char *dataset = argv[1], *netstat = argv[2];
  int32_t prec = FNETG_FP64;
  std::string forces, fnetout, mode = "predict";
  double delta = 0.0;
  for (int k = 3; k < argc; k++) {
    if (!std::strcmp(argv[k], "--fnetout") && k + 1 < argc) {
      fnetout = argv[++k];
    } else if (!std::strcmp(argv[k], "--mode") && k + 1 < argc) {
      mode = argv[++k];
    } else if (!std::strcmp(argv[k], "--fp32")) {
      prec = FNETG_FP32;
    } else if (!std::strcmp(argv[k], "--forces") && k + 1 < argc) {
      forces = argv[++k];
      if (forces == "fd") {
        if (k + 1 >= argc) throw fnet::Error(FNETG_E_INVALID, "--forces fd needs DELTA");
        delta = std::stod(argv[++k]);
      }
    }
  }
  const fnet::Dataset data = fnet::readHdfDataset(dataset);
  const fnet::Netstat ns = fnet::readNetstat(netstat);
  // the dataset's species order follows its own atomicnumbers; the networks follow the
  // netstat's: map every atom to its sub-network
  fnet::Dataset d = data;
  for (size_t a = 0; a < d.localAtToAtNum.size(); a++) {
    int sp = -1;
    for (size_t s = 0; s < ns.atomicNumbers.size(); s++)
      if (ns.atomicNumbers[s] == d.localAtToAtNum[a]) sp = (int)s;
    if (sp < 0) throw fnet::Error(FNETG_E_INVALID, "atom species without a sub-network");
    d.localAtToGlobalSp[a] = sp;
  }
  fnet::Context ctx(prec);
  ctx.upload(d);
  fnet::TAcsf acsf;
  acsf.gFunctions = ns.gFunctions;
  acsf.zPrec = ns.zPrec;
  acsf.extIndices = ns.extIndices;
  if (acsf.gFunctions.empty()) {
    // external features only: the network inputs are the selected dataset columns
    std::vector<double> feats;
    for (int64_t a = 0; a < d.nTotalAtoms(); a++)
      for (int32_t col : ns.extIndices) feats.push_back(d.extFeatures[a * d.nExtFeatures + col - 1]);
    ctx.check(fnetg_set_features(ctx.get(), (int32_t)ns.extIndices.size(), feats.data()));
  } else {
    acsf.calculate(ctx, false);
  }
  fnet::TBpnn bpnn = fnet::TBpnn::fromNetstat(ns);
  bpnn.load(ctx);
  const fnet::Predicts p = bpnn.predictBatch(ctx);
  std::vector<double> f;
  if (forces == "analytical") f = fnet::forceAnalysisAnalytical(ctx, bpnn);
  if (forces == "fd") f = fnet::forceAnalysisFiniteDiff(ctx, bpnn, delta);
  std::printf("{\n");
  print_array("atomic", p.atomic);
  if (!f.empty()) print_array("forces", f);
  print_array("global", p.global, true);
  std::printf("}\n");
  if (!fnetout.empty()) {
    const int nout = ns.dims.back();
    std::vector<fnet::FnetoutDatapoint> pts(d.nDatapoints());
    for (int s = 0; s < d.nDatapoints(); s++) {
      const int64_t a0 = d.atomOffsets[s], a1 = d.atomOffsets[s + 1];
      pts[s].rawPredictions.assign(p.atomic.begin() + a0 * nout, p.atomic.begin() + a1 * nout);
      if (!f.empty()) pts[s].forces.assign(f.begin() + a0 * nout * 3, f.begin() + a1 * nout * 3);
      if (mode == "validate") {
        pts[s].globalTargets.assign(d.globalTargets.begin() + (int64_t)s * d.nGlobalTargets,
                                    d.globalTargets.begin() + (int64_t)(s + 1) * d.nGlobalTargets);
        pts[s].atomicTargets.assign(d.atomicTargets.begin() + a0 * d.nAtomicTargets,
                                    d.atomicTargets.begin() + a1 * d.nAtomicTargets);
      }
    }
    fnet::writeFnetout(fnetout, mode, ns.nGlobalTargets, ns.nAtomicTargets, pts);
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    if (argc >= 3 && !std::strcmp(argv[1], "--dump")) return dump(argv[2], argc > 3 ? argv[3] : nullptr);
    if (argc == 4 && !std::strcmp(argv[1], "--copy-netstat")) {
      fnet::writeNetstat(argv[3], fnet::readNetstat(argv[2]));
      return 0;
    }
    if (argc >= 3) return run(argc, argv);
    std::fprintf(stderr, "usage: fnetg_run DATASET NETSTAT [--fp32] [--forces analytical|fd DELTA]\n"
                         "                 [--fnetout FILE [--mode predict|validate]]\n"
                         "       fnetg_run --dump DATASET [NETSTAT]\n"
                         "       fnetg_run --copy-netstat NETSTAT OUT\n");
    return 2;
  } catch (const fnet::Error &e) {
    std::fprintf(stderr, "fnetg_run: error %d: %s\n", e.code, e.what());
    return 1;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "fnetg_run: %s\n", e.what());
    return 1;
  }
}
