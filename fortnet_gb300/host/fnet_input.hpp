// The fnet program's input (fortnet_in.hsd) turned into run settings, mirroring
// TProgramVariables_init and its block readers (lib_fortnet/initprogram.F90): Options
// (readOptionBlock 720-765), Data (readDataBlock 825-905), Network (readNetworkBlock 940-975),
// Features (readFeaturesBlock 1280-1420 with TGFunctions_fromAutoScheme,
// lib_descriptors/acsf.F90:276-363, and the species expansion of processAcsfFunctions
// 1453-1527), Training (readTrainingBlock 985-1083), Analysis (readAnalysisBlock 775-800) and
// Driver (606-690).  Defaults are the reference's.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fnet_host.hpp"
#include "hsd.hpp"
#include "ipi.hpp"

namespace fnet {

struct InputSettings {
  // Options
  std::string mode = "train";  // train | validate | predict
  bool readNetStats = false;
  bool writeIterTraj = false;
  int64_t seed = 0;
  bool seedGiven = false;
  // Data
  std::string dataset, validset, netstatFile = "fortnet.hdf5";
  // Network = BPNN
  bool hasNetwork = false;
  std::vector<int32_t> hidden;
  int32_t activation = FNETG_ACT_TANH;
  // Features
  bool hasMapping = false, reduce = false, standardize = false;
  std::vector<fnetg_gfunc> baseFunctions;  // explicit functions in input order, then Auto ones
  bool hasExternal = false;
  std::string extIndexSpec;                // FromDataset { Indices = ... }
  // Training
  bool hasTraining = false;
  TrainingSettings training;
  int64_t nPrintout = 10, nSaveNet = 100;
  bool shuffle = false;
  // Analysis
  std::string forces;  // "", "analytical", "finitedifferences"
  double fdDelta = 1e-2;
  // Driver = Socket
  bool socket = false;
  SocketDriverSettings socketSettings;
};

InputSettings readInput(const hsd::Node &root);

// TGFunctions_fromAutoScheme (acsf.F90:276-363); rcut in Bohr
std::vector<fnetg_gfunc> autoFunctions(double rcut, int nRadial, int nAngular, int atomId);
// processAcsfFunctions (initprogram.F90:1453-1527): radial functions once per species,
// angular ones once per combination with replacement (intmanip.F90:84-142), in input order;
// unchanged when reduce is set or there is one species
std::vector<fnetg_gfunc> expandFunctions(const std::vector<fnetg_gfunc> &base,
                                         const std::vector<int32_t> &atomicNumbers, bool reduce);
// convRangeToInt: "a b", "a:b"; negative numbers count from the end (n + v + 1)
std::vector<int32_t> rangeToInt(const std::string &spec, int n);

}  // namespace fnet
