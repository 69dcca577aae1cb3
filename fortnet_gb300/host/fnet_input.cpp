// fortnet_in.hsd -> run settings (see fnet_input.hpp).
#include "fnet_input.hpp"

#include <cmath>
#include <sstream>

namespace fnet {

namespace {

constexpr double kAA__Bohr = 1.0 / 0.529177249;  // lib_dftbp/constants.F90:18-21

[[noreturn]] void fail(const std::string &msg) { throw Error(FNETG_E_INVALID, msg); }

std::string unquoted_lower(const std::string &s) { return hsd::lower(s); }

int32_t activation_of(const std::string &name) { return activationCode(name); }

fnetg_gfunc make(int type, double rcut, int atomid) {
  fnetg_gfunc g{};
  g.type = type;
  g.rcut = rcut;
  g.atomid = atomid;
  return g;
}

void read_functions(const hsd::Node &acsf, InputSettings &in) {
  const auto fns = acsf.all("Function");
  if (fns.empty()) fail("No ACSF functions specified.");
  std::vector<fnetg_gfunc> autos;
  for (const hsd::Node *f : fns) {
    if (f->type.empty()) fail("Function needs a type (Auto, G1 .. G5)");
    const std::string type = hsd::lower(f->type);
    const double rcut = f->real("RCut");
    if (rcut <= 0.0) fail("Specified cutoff less or equal zero.");
    const double rc = rcut * kAA__Bohr;
    const int atomid = (int)f->integer("AtomID", 0);
    if (atomid < 0) fail("Specified AtomID below zero.");
    if (type == "auto") {
      const int nr = (int)f->integer("NRadial"), na = (int)f->integer("NAngular");
      if (nr < 0) fail("Specified number of radial functions below zero.");
      if (na < 0) fail("Specified number of angular functions below zero.");
      const auto a = autoFunctions(rc, nr, na, atomid);
      autos.insert(autos.end(), a.begin(), a.end());
    } else if (type == "g1") {
      in.baseFunctions.push_back(make(1, rc, atomid));
    } else if (type == "g2") {
      fnetg_gfunc g = make(2, rc, atomid);
      g.eta = f->real("eta");
      g.rs = f->real("rs");
      in.baseFunctions.push_back(g);
    } else if (type == "g3") {
      fnetg_gfunc g = make(3, rc, atomid);
      g.kappa = f->real("kappa");
      in.baseFunctions.push_back(g);
    } else if (type == "g4" || type == "g5") {
      fnetg_gfunc g = make(type == "g4" ? 4 : 5, rc, atomid);
      g.xi = f->real("xi");
      g.eta = f->real("eta");
      g.lambda = f->real("lambda");
      if (g.lambda > 1.0 || g.lambda < -1.0)
        fail("Specified lambda parameter leaves interval [-1, 1].");
      in.baseFunctions.push_back(g);
    } else {
      fail("Invalid mapping type.");
    }
  }
  in.baseFunctions.insert(in.baseFunctions.end(), autos.begin(), autos.end());
}

void read_training(const hsd::Node &t, InputSettings &in) {
  TrainingSettings &s = in.training;
  const std::string kind = hsd::lower(t.type);
  if (kind == "sd") {
    s.optimizer = FNETG_OPT_SD;
    s.learningRate = t.real("LearningRate", 0.01);
  } else if (kind == "cg") {
    s.optimizer = FNETG_OPT_CG;
  } else if (kind == "lbfgs") {
    s.optimizer = FNETG_OPT_LBFGS;
    s.maxForQNDisplacement = t.logical("MaxForQNDisplacement", false);
    s.lineMin = t.logical("Linemin", true);
    s.memory = (int32_t)t.integer("Memory", 1000);
  } else if (kind == "fire") {
    s.optimizer = FNETG_OPT_FIRE;
  } else {
    fail("Invalid training algorithm");
  }
  s.minDisplacement = t.real("MinDisplacement", 1e-6);
  s.maxDisplacement = t.real("MaxDisplacement", 1e4);
  const long long nit = t.integer("NIterations", 2147483647LL);
  s.nIterations = (int)std::min<long long>(nit, 2147483647LL);
  s.threshold = t.real("Threshold", 2.2250738585072014e-308);
  in.nPrintout = t.integer("NPrintout", 10);
  in.nSaveNet = t.integer("NSaveNet", 100);
  const std::string loss = hsd::lower(t.str("Loss", "mse"));
  if (loss == "mse") s.loss = FNETG_LOSS_MSE;
  else if (loss == "rms") s.loss = FNETG_LOSS_RMS;
  else if (loss == "mae") s.loss = FNETG_LOSS_MAE;
  else if (loss == "mape") s.loss = FNETG_LOSS_MAPE;
  else fail("Invalid loss function '" + loss + "'");
  in.shuffle = t.logical("Shuffle", false);
  if (const hsd::Node *r = t.find("Regularization")) {
    const std::string rt = hsd::lower(r->type);
    double strength = 0.0, alpha = 0.0;
    if (rt == "lasso") {
      alpha = 1.0;
      strength = r->real("Strength");
    } else if (rt == "ridge") {
      alpha = 0.0;
      strength = r->real("Strength");
    } else if (rt == "elasticnet") {
      strength = r->real("Strength");
      alpha = r->real("Alpha");
      if (alpha < 0.0 || alpha > 1.0) fail("Elastic net regularization alpha out of bounds [0, 1].");
    } else {
      fail("Invalid regularization type.");
    }
    if (strength < 0.0) fail("Regularzation strength must be zero or positive.");
    if (strength == 0.0) alpha = 0.0;
    s.reguStrength = strength;
    s.reguAlpha = alpha;
  }
}

}  // namespace

std::vector<fnetg_gfunc> autoFunctions(double rcut, int nRadial, int nAngular, int atomId) {
  const double rsStep = rcut / (double)(nRadial - 1);
  const double g2eta = 5.0 * std::log(10.0) / ((2.0 * rsStep) * (2.0 * rsStep));
  const double g5eta = 2.0 * std::log(10.0) / (rcut * rcut);
  std::vector<fnetg_gfunc> out;
  for (int ii = 0; ii < nRadial; ii++) {
    fnetg_gfunc g = make(2, rcut, atomId);
    g.rs = ii == 0 ? 0.0 : ii * rsStep;
    g.eta = g2eta;
    out.push_back(g);
  }
  std::vector<double> lam, xis;
  int ind = 1;
  const int last = (int)std::ceil(nAngular / 2.0 - 1.0);
  bool stop = false;
  for (int ii = 0; ii <= last && !stop; ii++) {
    const double xi = nAngular <= 2 ? 1.0 : 1.0 + ii * 30.0 / (nAngular - 2.0);
    for (int jj : {1, -1}) {
      lam.push_back((double)jj);
      xis.push_back(xi);
      if (ind >= nAngular) {
        stop = true;
        break;
      }
      ind++;
    }
  }
  for (int ii = 0; ii < nAngular; ii++) {
    fnetg_gfunc g = make(5, rcut, atomId);
    g.xi = xis[ii];
    g.eta = g5eta;
    g.lambda = lam[ii];
    out.push_back(g);
  }
  return out;
}

std::vector<fnetg_gfunc> expandFunctions(const std::vector<fnetg_gfunc> &base,
                                         const std::vector<int32_t> &z, bool reduce) {
  if (reduce || z.size() <= 1) return base;
  std::vector<std::pair<int32_t, int32_t>> comb;
  for (size_t a = 0; a < z.size(); a++)
    for (size_t b = a; b < z.size(); b++) comb.emplace_back(z[a], z[b]);
  std::vector<fnetg_gfunc> out;
  for (const fnetg_gfunc &f : base) {
    if (f.type <= 3) {
      for (int32_t zz : z) {
        fnetg_gfunc g = f;
        g.z1 = zz;
        g.z2 = 0;
        out.push_back(g);
      }
    } else {
      for (const auto &c : comb) {
        fnetg_gfunc g = f;
        g.z1 = c.first;
        g.z2 = c.second;
        out.push_back(g);
      }
    }
  }
  return out;
}

std::vector<int32_t> rangeToInt(const std::string &spec, int n) {
  std::vector<int32_t> out;
  std::stringstream ss(spec);
  std::string tok;
  auto conv = [&](const std::string &s) {
    const long v = std::stol(s);
    return (int32_t)(v < 0 ? n + v + 1 : v);
  };
  while (ss >> tok) {
    const size_t c = tok.find(':');
    if (c == std::string::npos) {
      out.push_back(conv(tok));
    } else {
      const int32_t a = conv(tok.substr(0, c)), b = conv(tok.substr(c + 1));
      for (int32_t k = a; k <= b; k++) out.push_back(k);
    }
  }
  for (int32_t k : out)
    if (k < 1 || k > n) fail("external feature index " + std::to_string(k) + " out of range");
  return out;
}

InputSettings readInput(const hsd::Node &root) {
  InputSettings in;
  // Options
  const hsd::Node *opt = root.find("Options");
  if (!opt) fail("missing Options block");
  in.readNetStats = opt->logical("ReadNetStats", false);
  in.writeIterTraj = opt->logical("WriteIterationTrajectory", false);
  in.mode = unquoted_lower(opt->str("Mode"));
  if (in.mode != "train" && in.mode != "validate" && in.mode != "predict")
    fail("Invalid program running mode selected.");
  if (in.mode != "train") {
    in.writeIterTraj = false;
    in.readNetStats = true;
  }
  if (opt->find("RandomSeed")) {
    in.seed = opt->integer("RandomSeed");
    in.seedGiven = true;
    if (in.seed < 0) fail("Random seed must be greater or equal zero.");
  }
  // Data
  const hsd::Node *data = root.find("Data");
  if (!data) fail("missing Data block");
  in.netstatFile = data->str("NetstatFile", "fortnet.hdf5");
  in.dataset = data->str("Dataset");
  if (in.mode == "train") {
    const std::string v = data->str("Validset", "");
    in.validset = v == "none" ? "" : v;
  }
  // Network
  if (const hsd::Node *net = root.find("Network")) {
    if (hsd::lower(net->type) != "bpnn") fail("Invalid network type.");
    in.hasNetwork = true;
    for (long long h : net->integers("Hidden")) in.hidden.push_back((int32_t)h);
    in.activation = activation_of(net->str("Activation"));
  }
  // Features
  if (const hsd::Node *feat = root.find("Features")) {
    if (const hsd::Node *ext = feat->find("External")) {
      if (ext->find("Indices")) {
        if (hsd::lower(ext->type) != "fromdataset") fail("Invalid external feature type.");
        in.hasExternal = true;
        in.extIndexSpec = ext->str("Indices");
      }
    }
    if (const hsd::Node *map = feat->find("Mapping")) {
      if (hsd::lower(map->type) != "acsf") fail("Invalid mapping type");
      in.standardize = map->logical("Standardization", false);
      in.reduce = map->logical("Reduce", false);
      in.hasMapping = true;
      read_functions(*map, in);
    }
    if (!in.hasMapping && !in.hasExternal) fail("Neither mappings nor features provided.");
  }
  // Training
  if (in.mode == "train" && !in.socket) {
    if (const hsd::Node *t = root.find("Training")) {
      in.hasTraining = true;
      read_training(*t, in);
    }
  }
  // Analysis
  if (const hsd::Node *an = root.find("Analysis")) {
    if (const hsd::Node *f = an->find("Forces")) {
      in.forces = hsd::lower(f->type.empty() ? (f->tokens.empty() ? "" : f->tokens[0]) : f->type);
      if (in.forces == "finitedifferences") {
        in.fdDelta = f->real("Delta", 1e-2);
        if (in.fdDelta <= 0.0)
          fail("Invalid delta parameter of finite differences, must be greater than zero.");
      } else if (in.forces != "analytical") {
        fail("Invalid method specified to calculate atomic forces.");
      }
    }
  }
  // Driver = Socket
  if (const hsd::Node *drv = root.find("Driver")) {
    const std::string kind = hsd::lower(drv->type.empty() ? (drv->tokens.empty() ? "" : drv->tokens[0]) : drv->type);
    if (kind == "socket") {
      in.socket = true;
      if (in.forces.empty()) in.forces = "analytical";
      const hsd::Node *file = drv->find("File"), *host = drv->find("Host");
      if ((file == nullptr) == (host == nullptr))
        fail("Either Host or File (but not both) must be set for socket communication.");
      SocketDriverSettings &st = in.socketSettings;
      if (file) {
        st.socket.host = drv->str("Prefix", "/tmp/ipi_") + drv->str("File");
        st.socket.port = 0;
      } else {
        st.socket.host = drv->str("Host");
        st.socket.port = (int)drv->integer("Port");
        if (st.socket.port <= 0) fail("Invalid port number");
      }
      const hsd::Node *proto = drv->find("Protocol");
      if (proto && hsd::lower(proto->type) != "i-pi") fail("Invalid protocol '" + proto->type + "'");
      if (proto) {
        st.periodic = proto->logical("Periodic", false);
        const hsd::Node *an = proto->find("AtomicNumbers");
        if (!an) fail("missing AtomicNumbers of the socket protocol");
        std::string spec;
        for (const auto &t : an->tokens) spec += t + " ";
        // AtomicNumbers accept ranges like convRangeToInt over 1..118
        for (int32_t z : rangeToInt(spec, 118)) st.atomicNumbers.push_back(z);
      }
      st.socket.verbosity = (int)drv->integer("Verbosity", 0);
      const long long maxRun = drv->integer("MaxSteps", 200);
      st.nGeoSteps = maxRun == -1 ? (int64_t(1) << 62) : maxRun;
    } else if (!kind.empty() && kind != "none") {
      fail("Invalid driver '" + kind + "'");
    }
  }
  if (in.mode == "train" && !in.readNetStats && !in.hasNetwork)
    fail("training without ReadNetStats needs a Network block");
  return in;
}

}  // namespace fnet
