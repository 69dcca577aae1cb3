// Test driver for the HDF5 writers of the host layer.
//
//   h5_writers netstat MODEL.bin OUT.hdf5
//       MODEL.bin (little-endian): int32 nsp, int32 atomicnumbers[nsp], int32 ng,
//       fnetg_gfunc g[ng], double zprec[2 ng] (ng = 0 entries allowed), int32 nlayer,
//       int32 dims[nlayer], int32 activation, int32 nglobal, int32 natomic,
//       double params[nsp * nparams]; writes the netstat file.
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
  if (ng > 0) ns.zPrec = get_n<double>(in, 2 * (size_t)ng);
  const int L = get<int32_t>(in);
  ns.dims = get_n<int32_t>(in, L);
  ns.activation = get<int32_t>(in);
  ns.nGlobalTargets = get<int32_t>(in);
  ns.nAtomicTargets = get<int32_t>(in);
  ns.params = get_n<double>(in, (size_t)nsp * fnetg_nparams(L, ns.dims.data()));
  fnet::writeNetstat(out, ns);
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
    std::fprintf(stderr, "usage: h5_writers (netstat MODEL.bin | fnetout REF) OUT.hdf5\n");
    return 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "h5_writers: %s\n", e.what());
    return 1;
  }
}
