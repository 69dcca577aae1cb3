// Test driver for the HDF5 writers of the host layer.
//
//   h5_writers netstat MODEL.bin OUT.hdf5
//       MODEL.bin (little-endian): int32 nsp, int32 atomicnumbers[nsp], int32 ng,
//       fnetg_gfunc g[ng], int32 has_zprec, double zprec[2 ng] if has_zprec, int32 nlayer,
//       int32 dims[nlayer], int32 activation, int32 nglobal, int32 natomic,
//       double params[nsp * nparams], int32 next, int32 ext_indices[next]; writes the
//       netstat file.
//   h5_writers dataset DATA.bin OUT.hdf5
//       writes a dataset file (layout below) through writeHdfDataset.
//   h5_writers fnetout REFERENCE_FNETOUT OUT.hdf5
//       rewrites an fnetout file from the contents of another (mode, targets, predictions,
//       forces) through writeFnetout.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "fnet_host.hpp"
#include "hdf5lite.hpp"

namespace {

template <typename T> T get(std::ifstream &in) {
  T v{};
  in.read(reinterpret_cast<char *>(&v), sizeof v);
  if (!in) throw fnet::Error(FNETG_E_INVALID, "model file truncated");
  return v;
}
template <typename T> std::vector<T> get_n(std::ifstream &in, size_t n) {
  std::vector<T> v(n);
  in.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(sizeof(T) * n));
  if (!in) throw fnet::Error(FNETG_E_INVALID, "model file truncated");
  return v;
}

int netstat(const char *model, const char *out) {
  std::ifstream in(model, std::ios::binary);
  fnet::Netstat ns;
  const int nsp = get<int32_t>(in);
  ns.atomicNumbers = get_n<int32_t>(in, nsp);
  const int ng = get<int32_t>(in);
  ns.gFunctions = get_n<fnetg_gfunc>(in, ng);
  if (get<int32_t>(in)) ns.zPrec = get_n<double>(in, 2 * (size_t)ng);
  const int L = get<int32_t>(in);
  ns.dims = get_n<int32_t>(in, L);
  ns.activation = get<int32_t>(in);
  ns.nGlobalTargets = get<int32_t>(in);
  ns.nAtomicTargets = get<int32_t>(in);
  ns.params = get_n<double>(in, (size_t)nsp * fnetg_nparams(L, ns.dims.data()));
  const int next = get<int32_t>(in);
  ns.extIndices = get_n<int32_t>(in, next);
  fnet::writeNetstat(out, ns);
  return 0;
}

// DATA.bin (little-endian): int32 S, int64 offsets[S+1], double coords[3N], int32 atnum[N],
// int32 species[N] (0-based), int32 periodic[S], double latvecs[9S], int32 nz,
// int32 atomicnumbers[nz], int32 weights[S], double atomicweights[N], int32 ngt, int32 nat,
// double gt[S ngt], double at[N nat], int32 next, double ext[N next]
int dataset(const char *bin, const char *out) {
  std::ifstream in(bin, std::ios::binary);
  fnet::Dataset d;
  const int S = get<int32_t>(in);
  d.atomOffsets = get_n<int64_t>(in, S + 1);
  const size_t N = (size_t)d.atomOffsets.back();
  d.coords = get_n<double>(in, 3 * N);
  d.localAtToAtNum = get_n<int32_t>(in, N);
  d.localAtToGlobalSp = get_n<int32_t>(in, N);
  d.periodic = get_n<int32_t>(in, S);
  d.latVecs = get_n<double>(in, 9 * (size_t)S);
  const int nz = get<int32_t>(in);
  d.atomicNumbers = get_n<int32_t>(in, nz);
  d.weights = get_n<int32_t>(in, S);
  d.atomicWeights = get_n<double>(in, N);
  d.nGlobalTargets = get<int32_t>(in);
  d.nAtomicTargets = get<int32_t>(in);
  d.globalTargets = get_n<double>(in, (size_t)S * d.nGlobalTargets);
  d.atomicTargets = get_n<double>(in, N * d.nAtomicTargets);
  d.nExtFeatures = get<int32_t>(in);
  d.extFeatures = get_n<double>(in, N * d.nExtFeatures);
  fnet::writeHdfDataset(out, d);
  return 0;
}

int fnetout(const char *ref, const char *out) {
  auto root = fnet::h5::read(ref);
  const fnet::h5::Node &fo = (*root)["fnetout"];
  const std::string mode = fo.attr("mode").str();
  const fnet::h5::Node &op = fo["output"];
  const int n = (int)op.attr("ndatapoints").as_int();
  const int ng = (int)op.attr("nglobaltargets").as_int();
  const int na = (int)op.attr("natomictargets").as_int();
  const bool tf = op.attr("tforces").as_int() != 0;
  std::vector<fnet::FnetoutDatapoint> pts(n);
  for (int k = 0; k < n; k++) {
    const fnet::h5::Node &dp = op["datapoint" + std::to_string(k + 1)];
    pts[k].rawPredictions = dp["rawpredictions"].value.doubles();
    if (tf) pts[k].forces = dp["forces"].value.doubles();
    if (mode == "validate" && ng > 0) pts[k].globalTargets = dp["globaltargets"].value.doubles();
    if (mode == "validate" && na > 0) pts[k].atomicTargets = dp["atomictargets"].value.doubles();
  }
  fnet::writeFnetout(out, mode, ng, na, pts);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    if (argc == 4 && !std::strcmp(argv[1], "netstat")) return netstat(argv[2], argv[3]);
    if (argc == 4 && !std::strcmp(argv[1], "fnetout")) return fnetout(argv[2], argv[3]);
    if (argc == 4 && !std::strcmp(argv[1], "dataset")) return dataset(argv[2], argv[3]);
    std::fprintf(stderr, "usage: h5_writers (netstat MODEL.bin | dataset DATA.bin | fnetout REF) OUT.hdf5\n");
    return 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "h5_writers: %s\n", e.what());
    return 1;
  }
}
