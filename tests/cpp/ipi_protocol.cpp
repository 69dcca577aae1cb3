// The i-PI client (fnet::IpiSocketComm) against a server, with a toy model computed on the
// host: E = sum |r_a|^2 over the atoms, F_a = -2 r_a, and the virial set to the trace of the
// received cell.  Runs until the server sends EXIT; prints the number of geometries served.
//
//   ipi_protocol (--host H --port P | --unix PATH) NATOM
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ipi.hpp"

int main(int argc, char **argv) {
  fnet::IpiSocketCommInp inp;
  for (int k = 1; k + 1 < argc; k++) {
    if (!std::strcmp(argv[k], "--host")) inp.host = argv[++k];
    else if (!std::strcmp(argv[k], "--port")) inp.port = std::atoi(argv[++k]);
    else if (!std::strcmp(argv[k], "--unix")) { inp.host = argv[++k]; inp.port = 0; }
  }
  inp.nAtom = std::atoi(argv[argc - 1]);
  try {
    fnet::IpiSocketComm socket(inp);
    std::vector<double> coords, forces(3 * (size_t)inp.nAtom);
    double cell[9];
    int served = 0;
    while (socket.receive(coords, cell)) {
      double e = 0.0;
      for (int q = 0; q < 3 * inp.nAtom; q++) {
        e += coords[q] * coords[q];
        forces[q] = -2.0 * coords[q];
      }
      double virial[9];
      for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) virial[3 * i + k] = cell[i + 3 * k];  // echo latVecs(i, k)
      socket.send(e, forces, virial);
      served++;
    }
    std::printf("%d\n", served);
    return 0;
  } catch (const fnet::Error &err) {
    std::fprintf(stderr, "ipi_protocol: %s\n", err.what());
    return 1;
  }
}
