// C++ host side of the GPU hot path, mirroring the reference's Fortran interface for it:
// TDataset ingestion (lib_io/fnetdata.F90:994-1216), netstat reading (TAcsf_fromFile,
// lib_descriptors/acsf.F90:1908-2135; TBpnn_fromFile, lib_nn/bpnn.F90:1141-1288), TAcsf
// (acsf.F90:91-138), TBpnn (bpnn.F90:46-90) and the force analyses (lib_analysis/forces.F90).
// Every device operation goes through the C-ABI of include/fnetg.h.  Where the reference
// calls error() and stops, these classes throw fnet::Error with the library's code and
// message.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "fnetg.h"

namespace fnet {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// TDataset in flat form: structures back to back, cartesian coordinates in Bohr.
struct Dataset {
  std::vector<int64_t> atomOffsets;       // [S + 1]
  std::vector<double> coords;             // [3 N]
  std::vector<int32_t> localAtToAtNum;    // [N]
  std::vector<int32_t> localAtToGlobalSp; // [N], 0-based index into atomicNumbers
  std::vector<int32_t> periodic;          // [S]
  std::vector<double> latVecs;            // [9 S], latVecs(i, k) at i + 3 k
  std::vector<int32_t> atomicNumbers;     // global species
  std::vector<int32_t> weights;           // [S]
  std::vector<double> atomicWeights;      // [N]
  int nGlobalTargets = 0, nAtomicTargets = 0, nExtFeatures = 0;
  std::vector<double> globalTargets;      // [S nGlobalTargets]
  std::vector<double> atomicTargets;      // [N nAtomicTargets]
  std::vector<double> extFeatures;        // [N nExtFeatures]

  int nDatapoints() const { return (int)atomOffsets.size() - 1; }
  int64_t nTotalAtoms() const { return atomOffsets.empty() ? 0 : atomOffsets.back(); }
};

// readHdfDataset (fnetdata.F90:994-1216): geometry, targets, weights, external features.
Dataset readHdfDataset(const std::string &path);
// The dataset file layout readHdfDataset reads (cartesian coordinates), for converting data
// into the fnet format.
void writeHdfDataset(const std::string &path, const Dataset &d);

// A netstat file: ACSF configuration, z-score statistics and the trained sub-networks.
struct Netstat {
  std::vector<fnetg_gfunc> gFunctions;
  std::vector<double> zPrec;              // [2 nG]: means, deviations (empty: none)
  std::vector<int32_t> extIndices;        // 1-based external-feature columns (may be empty)
  std::vector<int32_t> atomicNumbers;     // sub-network order
  std::vector<int32_t> dims;
  int32_t activation = FNETG_ACT_TANH;
  int nGlobalTargets = 0, nAtomicTargets = 0;
  std::vector<double> params;             // [nSpecies][nParams], serialised reference order
};

Netstat readNetstat(const std::string &path);
int32_t activationCode(const std::string &name);
// The netstat file of a model: createNetstat + writeBpnnHeader (lib_io/netstat.F90:37-60,
// 312-402), writeExtFeaturesConfig (406-453), TAcsf_toFile (acsf.F90:1759-1906) and the
// layer parameters of TBpnn_toFile (bpnn.F90:1062-1140).
void writeNetstat(const std::string &path, const Netstat &ns);

// One structure's results for writeFnetout.
struct FnetoutDatapoint {
  std::vector<double> rawPredictions;   // [nAtom][nOut]
  std::vector<double> forces;           // [nAtom][nOut][3] or empty
  std::vector<double> globalTargets;    // validate mode: [nGlobalTargets]
  std::vector<double> atomicTargets;    // validate mode: [nAtom][nAtomicTargets]
};
// writeFnetout (lib_io/fnetout.F90:33-158); mode "predict" or "validate".  Global predictions
// are the per-structure sums of the first nGlobalTargets outputs.
void writeFnetout(const std::string &path, const std::string &mode, int nGlobalTargets,
                  int nAtomicTargets, const std::vector<FnetoutDatapoint> &points);

// One GPU context holding a dataset (the program state of fortnet.F90:110-215).
class Context {
 public:
  explicit Context(int32_t precision = FNETG_FP64, int32_t device = 0);
  ~Context();
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  fnetg_ctx *get() const { return ctx_; }
  // geometry and species of every atom (species index = localAtToGlobalSp)
  void upload(const Dataset &data);
  void check(int rc) const;  // throws Error for a non-zero return code
  const Dataset *data() const { return data_; }

 private:
  fnetg_ctx *ctx_ = nullptr;
  const Dataset *data_ = nullptr;
};

// TAcsf: ACSF featurisation with z-score standardisation.
class TAcsf {
 public:
  std::vector<fnetg_gfunc> gFunctions;
  std::vector<double> zPrec;       // statistics used for standardisation (empty: none)
  std::vector<int32_t> extIndices; // external atomic features appended to every row

  // TAcsf_calculate (acsf.F90:540-639): featurise the context's dataset; with tZscore and
  // no statistics yet, compute them weighted by the datapoint weights (getMeansAndVariances).
  void calculate(Context &ctx, bool tZscore);
  // standardised network inputs of every atom, [N][nF]
  std::vector<double> vals(Context &ctx) const;
};

struct Predicts {
  std::vector<double> atomic;  // [N][nOut]
  std::vector<double> global;  // [S][nOut], per-structure sums
};

struct TrainingSettings {
  int32_t optimizer = FNETG_OPT_LBFGS;
  double threshold = 2.2250738585072014e-308, minDisplacement = 1e-6, maxDisplacement = 1e4;
  double learningRate = 0.01;
  int32_t memory = 1000;
  bool lineMin = true, maxForQNDisplacement = false;
  int nIterations = 1;
  int32_t loss = FNETG_LOSS_MSE;
  double reguStrength = 0.0, reguAlpha = 0.0;
};

struct TrainingLog {
  std::vector<double> loss, gradients;  // per iteration (tmpLoss, tmpGradients)
  bool converged = false;
};

// TBpnn: one sub-network per global species.
class TBpnn {
 public:
  TBpnn(std::vector<int32_t> dims, std::vector<int32_t> atomicNumbers, int32_t activation);
  static TBpnn fromNetstat(const Netstat &ns);

  // TBpnn_init with the reference's RANLUX lux-3 normalXavier draw (bpnn.F90:96-143)
  void initRandom(int32_t seed);
  void load(Context &ctx) const;                  // weights onto the device
  Predicts predictBatch(Context &ctx) const;      // TBpnn_predictBatch (bpnn.F90:1001-1058)
  std::vector<double> nJacobian(Context &ctx) const;  // [N][nOut][nF] (bpnn.F90:937-997)
  // TBpnn_nTrain (bpnn.F90:293-363): gradient, update, optimiser, nIterations times
  TrainingLog nTrain(Context &ctx, const TrainingSettings &settings);
  const std::vector<double> &serializedWeightsAndBiases() const { return params_; }

  std::vector<int32_t> dims;
  std::vector<int32_t> atomicNumbers;
  int32_t activation;

 private:
  std::vector<double> params_;  // [nSpecies][nParams]
};

// forceAnalysis_analytical (forces.F90:317-425) with the network loaded on ctx: [N][nOut][3]
std::vector<double> forceAnalysisAnalytical(Context &ctx, const TBpnn &bpnn);
// forceAnalysis_finiteDiff (forces.F90:182-306): [N][nOut][3]
std::vector<double> forceAnalysisFiniteDiff(Context &ctx, const TBpnn &bpnn, double delta);

}  // namespace fnet
