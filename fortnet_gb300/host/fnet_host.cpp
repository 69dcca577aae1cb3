// C++ host side over the fnetg C-ABI (see fnet_host.hpp).
#include "fnet_host.hpp"
#include "h5write.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>

#include "hdf5lite.hpp"

namespace fnet {

namespace {

const char *kElements[] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",
    "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn",
    "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh",
    "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd",
    "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re",
    "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th",
    "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md", "No", "Lr", "Rf", "Db",
    "Sg", "Bh", "Hs", "Mt", "Ds", "Rg", "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};

std::string lower(std::string s) {
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string elementSymbol(int z) {
  if (z < 1 || z > 118) throw Error(FNETG_E_INVALID, "atomic number out of range");
  return kElements[z - 1];
}

// number of parameters of one sub-network in the serialised order (network.F90:126-142)
int64_t nParams(const std::vector<int32_t> &dims) {
  return fnetg_nparams((int32_t)dims.size(), dims.data());
}

}  // namespace

int32_t activationCode(const std::string &name) {
  static const char *names[] = {"tanh", "sigmoid", "relu", "lrelu", "softplus",
                                "bent", "atan",    "gaussian", "heaviside", "linear"};
  const std::string n = lower(name);
  for (int k = 0; k < 10; k++)
    if (n == names[k]) return k;
  throw Error(FNETG_E_INVALID, "unknown activation '" + name + "'");
}

// ---------------------------------------------------------------- files

Dataset readHdfDataset(const std::string &path) {
  auto root = h5::read(path);
  const h5::Node &ds = (*root)["fnetdata/dataset"];
  const h5::Node &tr = ds["training"];
  const int npts = (int)ds.attr("ndatapoints").as_int();
  Dataset d;
  d.nExtFeatures = (int)ds.attr("nextfeatures").as_int();
  if (ds.attr("withstructures").as_int() != 1)
    throw Error(FNETG_E_INVALID, "datasets without structures carry no geometry for ACSF");
  d.nGlobalTargets = (int)tr.attr("nglobaltargets").as_int();
  d.nAtomicTargets = (int)tr.attr("natomictargets").as_int();
  for (auto z : ds["atomicnumbers"].value.integers()) d.atomicNumbers.push_back((int32_t)z);
  d.atomOffsets.push_back(0);
  for (int i = 1; i <= npts; i++) {
    const h5::Node &dp = ds["datapoint" + std::to_string(i)];
    const h5::Node &geo = dp["geometry"];
    d.weights.push_back((int32_t)dp.attr("weight").as_int());
    std::vector<double> c = geo["coordinates"].value.doubles();
    const int64_t n = (int64_t)c.size() / 3;
    const bool periodic = geo.attr("periodic").as_int() == 1;
    const bool frac = geo.attr("fractional").as_int() == 1;
    std::vector<double> L(9, 0.0);
    if (periodic) {
      L = geo["basis"].value.doubles();
      if (L.size() != 9) throw Error(FNETG_E_SHAPE, "lattice basis must hold 9 values");
      if (frac) {
        // cartesian = latVecs . fractional, summed in index order
        std::vector<double> cart(c.size());
        for (int64_t a = 0; a < n; a++)
          for (int r = 0; r < 3; r++) {
            double acc = L[r + 0] * c[3 * a + 0];
            acc = acc + L[r + 3] * c[3 * a + 1];
            acc = acc + L[r + 6] * c[3 * a + 2];
            cart[3 * a + r] = acc;
          }
        c = cart;
      }
    }
    d.coords.insert(d.coords.end(), c.begin(), c.end());
    for (auto z : geo["localattoatnum"].value.integers()) d.localAtToAtNum.push_back((int32_t)z);
    for (auto sp : geo["localattoglobalsp"].value.integers())
      d.localAtToGlobalSp.push_back((int32_t)sp - 1);
    d.periodic.push_back(periodic ? 1 : 0);
    d.latVecs.insert(d.latVecs.end(), L.begin(), L.end());
    if (dp.has("atomicweights")) {
      auto w = dp["atomicweights"].value.doubles();
      d.atomicWeights.insert(d.atomicWeights.end(), w.begin(), w.end());
    } else {
      d.atomicWeights.insert(d.atomicWeights.end(), (size_t)n, 1.0);
    }
    if (d.nGlobalTargets > 0) {
      auto g = dp["globaltargets"].value.doubles();
      d.globalTargets.insert(d.globalTargets.end(), g.begin(), g.end());
    }
    if (d.nAtomicTargets > 0) {
      auto t = dp["atomictargets"].value.doubles();
      d.atomicTargets.insert(d.atomicTargets.end(), t.begin(), t.end());
    }
    if (d.nExtFeatures > 0) {
      auto e = dp["extfeatures"].value.doubles();
      d.extFeatures.insert(d.extFeatures.end(), e.begin(), e.end());
    }
    d.atomOffsets.push_back(d.atomOffsets.back() + n);
  }
  return d;
}

Netstat readNetstat(const std::string &path) {
  auto root = h5::read(path);
  const h5::Node &ns = (*root)["netstat"];
  Netstat out;
  if (ns.has("mapping")) {
    const h5::Node &mp = ns["mapping"];
    const int nf = (int)mp.attr("nfunctions").as_int();
    for (int i = 1; i <= nf; i++) {
      const h5::Node &f = mp["function" + std::to_string(i)];
      fnetg_gfunc g{};
      const std::string type = lower(f.attr("type").str());
      if (type.size() != 2 || type[0] != 'g' || type[1] < '1' || type[1] > '5')
        throw Error(FNETG_E_INVALID, "unknown G-function type '" + type + "'");
      g.type = type[1] - '0';
      auto num = [&](const char *name, double dflt) {
        return f.has_attr(name) ? f.attr(name).as_double() : dflt;
      };
      g.rcut = num("cutoff", 0.0);
      g.kappa = num("kappa", 0.0);
      g.rs = num("rs", 0.0);
      g.eta = num("eta", 0.0);
      g.lambda = num("lambda", 0.0);
      g.xi = num("xi", 0.0);
      g.atomid = f.has_attr("atomid") ? (int32_t)f.attr("atomid").as_int() : 0;
      if (f.has_attr("atomicnumbers")) {
        auto zz = f.attr("atomicnumbers").integers();
        g.z1 = zz.size() > 0 ? (int32_t)zz[0] : 0;
        g.z2 = zz.size() > 1 ? (int32_t)zz[1] : 0;
      }
      out.gFunctions.push_back(g);
    }
    if (mp.has("preconditioning")) {
      auto m = mp["preconditioning/means"].value.doubles();
      auto v = mp["preconditioning/variances"].value.doubles();
      out.zPrec = m;
      out.zPrec.insert(out.zPrec.end(), v.begin(), v.end());
    }
  }
  if (ns.has("external"))
    for (auto k : ns["external/indices"].value.integers()) out.extIndices.push_back((int32_t)k);
  const h5::Node &bp = ns["bpnn"];
  for (auto z : bp["atomicnumbers"].value.integers()) out.atomicNumbers.push_back((int32_t)z);
  out.nGlobalTargets = (int)bp.attr("nglobaltargets").as_int();
  out.nAtomicTargets = (int)bp.attr("natomictargets").as_int();
  for (size_t s = 0; s < out.atomicNumbers.size(); s++) {
    std::string sym = lower(elementSymbol(out.atomicNumbers[s]));
    const h5::Node &sub = bp[sym + "-subnetwork"];
    std::vector<int32_t> dims;
    for (auto x : sub["topology"].value.integers()) dims.push_back((int32_t)x);
    const int32_t act = activationCode(sub.attr("activation").str());
    if (s == 0) {
      out.dims = dims;
      out.activation = act;
    } else if (dims != out.dims || act != out.activation) {
      throw Error(FNETG_E_UNSUPPORTED, "sub-networks with different topologies");
    }
    // serialised order: every ww column-major (layer by layer, the output layer's ww too),
    // then every bb (network.F90:397-427); the file holds ww(l) transposed
    const int L = (int)dims.size();
    std::vector<int64_t> woff(L), boff(L);
    int64_t ind = 0;
    for (int l = 0; l < L; l++) {
      woff[l] = ind;
      ind += (int64_t)dims[l] * (l < L - 1 ? dims[l + 1] : 1);
    }
    for (int l = 0; l < L; l++) {
      boff[l] = ind;
      ind += dims[l];
    }
    std::vector<double> p((size_t)ind, 0.0);
    for (int l = 0; l + 1 < L; l++) {
      const h5::Node &lay = sub["layer" + std::to_string(l + 1)];
      auto w = lay["weights"].value.doubles();
      auto b = lay["bias"].value.doubles();
      if ((int64_t)w.size() != (int64_t)dims[l] * dims[l + 1] || (int)b.size() != dims[l + 1])
        throw Error(FNETG_E_SHAPE, "layer size does not match the topology");
      std::copy(w.begin(), w.end(), p.begin() + woff[l]);
      std::copy(b.begin(), b.end(), p.begin() + boff[l + 1]);
    }
    out.params.insert(out.params.end(), p.begin(), p.end());
  }
  return out;
}

// ---------------------------------------------------------------- context

Context::Context(int32_t precision, int32_t device) {
  check(fnetg_create(&ctx_, precision, device));
}

Context::~Context() {
  if (ctx_) fnetg_destroy(ctx_);
}

void Context::check(int rc) const {
  if (rc != 0) throw Error(rc, ctx_ ? fnetg_last_error(ctx_) : "fnetg_create failed");
}

void Context::upload(const Dataset &d) {
  check(fnetg_upload_structures(ctx_, d.nDatapoints(), d.atomOffsets.data(),
                                d.localAtToAtNum.data(), d.coords.data(), d.periodic.data(),
                                d.latVecs.data(),
                                d.nExtFeatures > 0 ? d.extFeatures.data() : nullptr,
                                d.nExtFeatures));
  check(fnetg_set_species(ctx_, d.localAtToGlobalSp.data()));
  data_ = &d;
}

// ---------------------------------------------------------------- TAcsf

void TAcsf::calculate(Context &ctx, bool tZscore) {
  if (!ctx.data()) throw Error(FNETG_E_INVALID, "TAcsf::calculate: no dataset uploaded");
  ctx.check(fnetg_set_gfunctions(ctx.get(), (int32_t)gFunctions.size(), gFunctions.data()));
  ctx.check(fnetg_set_external_inputs(ctx.get(), (int32_t)extIndices.size(), extIndices.data()));
  ctx.check(fnetg_acsf(ctx.get(), nullptr));
  if (!zPrec.empty()) {
    ctx.check(fnetg_acsf_zscore(ctx.get(), nullptr, zPrec.data(), 0));
  } else if (tZscore) {
    zPrec.assign(2 * gFunctions.size(), 0.0);
    ctx.check(fnetg_acsf_zscore(ctx.get(), ctx.data()->weights.data(), zPrec.data(), 1));
  }
}

std::vector<double> TAcsf::vals(Context &ctx) const {
  int32_t nf = 0;
  ctx.check(fnetg_get_features(ctx.get(), nullptr, &nf));
  std::vector<double> out((size_t)ctx.data()->nTotalAtoms() * nf);
  ctx.check(fnetg_get_features(ctx.get(), out.data(), &nf));
  return out;
}

// ---------------------------------------------------------------- TBpnn

TBpnn::TBpnn(std::vector<int32_t> d, std::vector<int32_t> z, int32_t act)
    : dims(std::move(d)), atomicNumbers(std::move(z)), activation(act) {
  params_.assign((size_t)atomicNumbers.size() * nParams(dims), 0.0);
}

TBpnn TBpnn::fromNetstat(const Netstat &ns) {
  TBpnn b(ns.dims, ns.atomicNumbers, ns.activation);
  if (ns.params.size() != b.params_.size())
    throw Error(FNETG_E_SHAPE, "netstat parameters do not match the topology");
  b.params_ = ns.params;
  return b;
}

void TBpnn::initRandom(int32_t seed) {
  void *rng = fnetg_rng_create(seed);
  if (!rng) throw Error(FNETG_E_INVALID, "RANLUX initialisation");
  const int rc = fnetg_rng_init_params(rng, (int32_t)atomicNumbers.size(), (int32_t)dims.size(),
                                       dims.data(), params_.data());
  fnetg_rng_destroy(rng);
  if (rc != 0) throw Error(rc, "normalXavier initialisation");
}

void TBpnn::load(Context &ctx) const {
  ctx.check(fnetg_set_network(ctx.get(), (int32_t)atomicNumbers.size(), (int32_t)dims.size(),
                              dims.data(), activation, params_.data()));
}

Predicts TBpnn::predictBatch(Context &ctx) const {
  const Dataset &d = *ctx.data();
  Predicts p;
  p.atomic.assign((size_t)d.nTotalAtoms() * dims.back(), 0.0);
  p.global.assign((size_t)d.nDatapoints() * dims.back(), 0.0);
  ctx.check(fnetg_predict(ctx.get(), p.atomic.data(), p.global.data()));
  return p;
}

std::vector<double> TBpnn::nJacobian(Context &ctx) const {
  std::vector<double> jac((size_t)ctx.data()->nTotalAtoms() * dims.back() * dims.front());
  ctx.check(fnetg_jacobian(ctx.get(), jac.data()));
  return jac;
}

TrainingLog TBpnn::nTrain(Context &ctx, const TrainingSettings &st) {
  const Dataset &d = *ctx.data();
  ctx.check(fnetg_set_targets(ctx.get(), d.nGlobalTargets, d.nAtomicTargets,
                              d.nGlobalTargets > 0 ? d.globalTargets.data() : nullptr,
                              d.nAtomicTargets > 0 ? d.atomicTargets.data() : nullptr,
                              d.atomicWeights.data(), d.weights.data()));
  ctx.check(fnetg_optimizer_init(ctx.get(), st.optimizer, st.threshold, st.minDisplacement,
                                 st.maxDisplacement, st.learningRate, st.memory,
                                 st.lineMin ? 1 : 0, st.maxForQNDisplacement ? 1 : 0));
  TrainingLog log;
  for (int it = 0; it < st.nIterations; it++) {
    double loss = 0.0, grad = 0.0;
    int32_t conv = 0;
    ctx.check(fnetg_train_iteration(ctx.get(), st.loss, st.reguStrength, st.reguAlpha, nullptr,
                                    &loss, &grad, &conv));
    log.loss.push_back(loss);
    log.gradients.push_back(grad);
    if (conv) {
      log.converged = true;
      break;
    }
  }
  ctx.check(fnetg_get_params(ctx.get(), params_.data()));
  return log;
}

// ---------------------------------------------------------------- force analyses

std::vector<double> forceAnalysisAnalytical(Context &ctx, const TBpnn &bpnn) {
  std::vector<double> f((size_t)ctx.data()->nTotalAtoms() * bpnn.dims.back() * 3, 0.0);
  ctx.check(fnetg_forces(ctx.get(), f.data()));
  return f;
}

std::vector<double> forceAnalysisFiniteDiff(Context &ctx, const TBpnn &bpnn, double delta) {
  std::vector<double> f((size_t)ctx.data()->nTotalAtoms() * bpnn.dims.back() * 3, 0.0);
  ctx.check(fnetg_forces_fd(ctx.get(), delta, f.data()));
  return f;
}

// ---------------------------------------------------------------- writers

void writeNetstat(const std::string &path, const Netstat &ns) {
  h5w::File f;
  f.group("netstat");
  const int ng = (int)ns.gFunctions.size();
  if (ng > 0) {
    f.attr_str("netstat/mapping", "type", "acsf");
    f.attr_i32("netstat/mapping", "nfunctions", {ng});
    for (int i = 0; i < ng; i++) {
      const fnetg_gfunc &g = ns.gFunctions[i];
      if (g.type < 1 || g.type > 5) throw Error(FNETG_E_INVALID, "unknown G-function type");
      const std::string fp = "netstat/mapping/function" + std::to_string(i + 1);
      const bool ang = g.type >= 4;
      f.attr_str(fp, "type", "g" + std::to_string(g.type));
      f.attr_i32(fp, "atomid", {g.atomid});
      f.attr_f64(fp, "cutoff", {g.rcut});
      f.attr_i32(fp, "atomicnumbers", {g.z1, g.z2});
      f.attr_i32(fp, "tradial", {ang ? 0 : 1});
      f.attr_i32(fp, "tangular", {ang ? 1 : 0});
      if (g.type == 2) {
        f.attr_f64(fp, "eta", {g.eta});
        f.attr_f64(fp, "rs", {g.rs});
      } else if (g.type == 3) {
        f.attr_f64(fp, "kappa", {g.kappa});
      } else if (ang) {
        f.attr_f64(fp, "xi", {g.xi});
        f.attr_f64(fp, "lambda", {g.lambda});
        f.attr_f64(fp, "eta", {g.eta});
      }
    }
    if (!ns.zPrec.empty()) {
      if ((int)ns.zPrec.size() != 2 * ng) throw Error(FNETG_E_SHAPE, "z-score statistics size");
      f.attr_str("netstat/mapping/preconditioning", "type", "zscore");
      f.dataset_f64("netstat/mapping/preconditioning/means", {(uint64_t)ng},
                    std::vector<double>(ns.zPrec.begin(), ns.zPrec.begin() + ng));
      f.dataset_f64("netstat/mapping/preconditioning/variances", {(uint64_t)ng},
                    std::vector<double>(ns.zPrec.begin() + ng, ns.zPrec.end()));
    }
  }
  if (!ns.extIndices.empty()) {
    f.attr_i32("netstat/external", "nextfeatures", {(int32_t)ns.extIndices.size()});
    f.dataset_i32("netstat/external/indices", {ns.extIndices.size()}, ns.extIndices);
  }
  const int nsp = (int)ns.atomicNumbers.size();
  const int L = (int)ns.dims.size();
  f.attr_i32("netstat/bpnn", "nglobaltargets", {ns.nGlobalTargets});
  f.attr_i32("netstat/bpnn", "natomictargets", {ns.nAtomicTargets});
  f.dataset_i32("netstat/bpnn/atomicnumbers", {(uint64_t)nsp}, ns.atomicNumbers);
  static const char *act_names[] = {"tanh", "sigmoid", "relu", "lrelu", "softplus",
                                    "bent", "atan", "gaussian", "heaviside", "linear"};
  if (ns.activation < 0 || ns.activation > 9) throw Error(FNETG_E_INVALID, "activation code");
  const int64_t np = fnetg_nparams(L, ns.dims.data());
  if ((int64_t)ns.params.size() != np * nsp) throw Error(FNETG_E_SHAPE, "parameter count");
  // serialised order (network.F90:397-427): every ww column-major, then every bb
  std::vector<int64_t> woff(L), boff(L);
  int64_t ind = 0;
  for (int l = 0; l < L; l++) {
    woff[l] = ind;
    ind += (int64_t)ns.dims[l] * (l < L - 1 ? ns.dims[l + 1] : 1);
  }
  for (int l = 0; l < L; l++) {
    boff[l] = ind;
    ind += ns.dims[l];
  }
  for (int s = 0; s < nsp; s++) {
    const std::string sp = "netstat/bpnn/" + lower(elementSymbol(ns.atomicNumbers[s])) + "-subnetwork";
    f.attr_i32(sp, "element", {ns.atomicNumbers[s]});
    f.attr_i32(sp, "nlayer", {L});
    f.attr_str(sp, "activation", act_names[ns.activation]);
    f.dataset_i32(sp + "/topology", {(uint64_t)L}, ns.dims);
    const double *p = ns.params.data() + (size_t)s * np;
    for (int l = 0; l + 1 < L; l++) {
      const std::string lp = sp + "/layer" + std::to_string(l + 1);
      // ww(l) of shape (dims[l], dims[l+1]) in Fortran order: the file lists (dims[l+1], dims[l])
      f.dataset_f64(lp + "/weights", {(uint64_t)ns.dims[l + 1], (uint64_t)ns.dims[l]},
                    std::vector<double>(p + woff[l], p + woff[l] + (int64_t)ns.dims[l] * ns.dims[l + 1]));
      f.dataset_f64(lp + "/bias", {(uint64_t)ns.dims[l + 1]},
                    std::vector<double>(p + boff[l + 1], p + boff[l + 1] + ns.dims[l + 1]));
    }
  }
  f.write(path);
}

void writeHdfDataset(const std::string &path, const Dataset &d) {
  h5w::File f;
  const int S = d.nDatapoints();
  const std::string ds = "fnetdata/dataset";
  f.attr_i32(ds, "ndatapoints", {S});
  f.attr_i32(ds, "nextfeatures", {d.nExtFeatures});
  f.attr_i32(ds, "withstructures", {1});
  f.attr_i32(ds, "ntotatoms", {(int32_t)d.nTotalAtoms()});
  f.dataset_i32(ds + "/atomicnumbers", {d.atomicNumbers.size()}, d.atomicNumbers);
  f.attr_i32(ds + "/training", "nglobaltargets", {d.nGlobalTargets});
  f.attr_i32(ds + "/training", "natomictargets", {d.nAtomicTargets});
  for (int s = 0; s < S; s++) {
    const int64_t a0 = d.atomOffsets[s], a1 = d.atomOffsets[s + 1];
    const uint64_t n = (uint64_t)(a1 - a0);
    const std::string dp = ds + "/datapoint" + std::to_string(s + 1);
    f.attr_i32(dp, "weight", {d.weights.empty() ? 1 : d.weights[s]});
    f.dataset_f64(dp + "/atomicweights", {n},
                  d.atomicWeights.empty() ? std::vector<double>(n, 1.0)
                                          : std::vector<double>(d.atomicWeights.begin() + a0,
                                                                d.atomicWeights.begin() + a1));
    const std::string geo = dp + "/geometry";
    f.attr_i32(geo, "fractional", {0});
    f.attr_i32(geo, "periodic", {d.periodic[s] ? 1 : 0});
    f.dataset_f64(geo + "/coordinates", {n, 3},
                  std::vector<double>(d.coords.begin() + 3 * a0, d.coords.begin() + 3 * a1));
    if (d.periodic[s])
      f.dataset_f64(geo + "/basis", {3, 3},
                    std::vector<double>(d.latVecs.begin() + 9 * s, d.latVecs.begin() + 9 * (s + 1)));
    f.dataset_i32(geo + "/localattoatnum", {n},
                  std::vector<int32_t>(d.localAtToAtNum.begin() + a0, d.localAtToAtNum.begin() + a1));
    std::vector<int32_t> sp(d.localAtToGlobalSp.begin() + a0, d.localAtToGlobalSp.begin() + a1);
    for (int32_t &x : sp) x += 1;
    f.dataset_i32(geo + "/localattoglobalsp", {n}, sp);
    if (d.nGlobalTargets > 0)
      f.dataset_f64(dp + "/globaltargets", {(uint64_t)d.nGlobalTargets},
                    std::vector<double>(d.globalTargets.begin() + (int64_t)s * d.nGlobalTargets,
                                        d.globalTargets.begin() + (int64_t)(s + 1) * d.nGlobalTargets));
    if (d.nAtomicTargets > 0)
      f.dataset_f64(dp + "/atomictargets", {n, (uint64_t)d.nAtomicTargets},
                    std::vector<double>(d.atomicTargets.begin() + a0 * d.nAtomicTargets,
                                        d.atomicTargets.begin() + a1 * d.nAtomicTargets));
    if (d.nExtFeatures > 0)
      f.dataset_f64(dp + "/extfeatures", {n, (uint64_t)d.nExtFeatures},
                    std::vector<double>(d.extFeatures.begin() + a0 * d.nExtFeatures,
                                        d.extFeatures.begin() + a1 * d.nExtFeatures));
  }
  f.write(path);
}

void writeFnetout(const std::string &path, const std::string &mode, int nGlobalTargets,
                  int nAtomicTargets, const std::vector<FnetoutDatapoint> &points) {
  if (mode != "validate" && mode != "predict")
    throw Error(FNETG_E_INVALID, "Invalid program running mode selected.");
  const int nTargets = nGlobalTargets + nAtomicTargets;
  if (mode == "validate" && nTargets == 0)
    throw Error(FNETG_E_INVALID, "Validation mode only valid in combination with target data.");
  const bool tForces = !points.empty() && !points[0].forces.empty();
  h5w::File f;
  f.attr_str("fnetout", "mode", mode);
  f.attr_i32("fnetout/output", "ndatapoints", {(int32_t)points.size()});
  f.attr_i32("fnetout/output", "tforces", {tForces ? 1 : 0});
  f.attr_i32("fnetout/output", "nglobaltargets", {nGlobalTargets});
  f.attr_i32("fnetout/output", "natomictargets", {nAtomicTargets});
  for (size_t k = 0; k < points.size(); k++) {
    const FnetoutDatapoint &d = points[k];
    const std::string dp = "fnetout/output/datapoint" + std::to_string(k + 1);
    if (nTargets <= 0) throw Error(FNETG_E_SHAPE, "no outputs");
    const uint64_t nAtom = d.rawPredictions.size() / (uint64_t)nTargets;
    if (nAtom * (uint64_t)nTargets != d.rawPredictions.size())
      throw Error(FNETG_E_SHAPE, "raw predictions size");
    f.group(dp);
    if (nGlobalTargets > 0) {
      std::vector<double> g(nGlobalTargets, 0.0);
      for (uint64_t a = 0; a < nAtom; a++)
        for (int o = 0; o < nGlobalTargets; o++) g[o] += d.rawPredictions[a * nTargets + o];
      f.dataset_f64(dp + "/globalpredictions", {(uint64_t)nGlobalTargets}, g);
      if (mode == "validate")
        f.dataset_f64(dp + "/globaltargets", {d.globalTargets.size()}, d.globalTargets);
    }
    f.dataset_f64(dp + "/rawpredictions", {nAtom, (uint64_t)nTargets}, d.rawPredictions);
    if (mode == "validate" && nAtomicTargets > 0)
      f.dataset_f64(dp + "/atomictargets", {nAtom, (uint64_t)nAtomicTargets}, d.atomicTargets);
    if (tForces) f.dataset_f64(dp + "/forces", {nAtom, 3 * (uint64_t)nTargets}, d.forces);
  }
  f.write(path);
}

}  // namespace fnet
