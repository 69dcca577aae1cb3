// fnetg_ipi: the socket-driven mode of the fnet program (prg_fnet/fortnet.F90:126-169) — an
// i-PI client that predicts energies and forces of every geometry the server sends, with the
// model of a netstat file, on the GPU prediction service.  The options are the entries of the
// input's Driver = Socket {...} block (lib_fortnet/initprogram.F90:606-690):
//
//   fnetg_ipi NETSTAT --atomic-numbers Z1,Z2,... [--periodic]
//             (--file NAME [--prefix /tmp/ipi_] | --host HOST --port PORT)
//             [--max-steps N (default 200, -1: no limit)] [--verbosity V] [--fp32]
//
// Prints the number of geometries served on exit.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <string>

#include "ipi.hpp"

int main(int argc, char **argv) {
  try {
    if (argc < 2) throw fnet::Error(FNETG_E_INVALID, "usage: fnetg_ipi NETSTAT --atomic-numbers ...");
    fnet::SocketDriverSettings st;
    std::string file, host, prefix = "/tmp/ipi_";
    int port = 0;
    int64_t maxSteps = 200;
    for (int k = 2; k < argc; k++) {
      const std::string a = argv[k];
      auto next = [&]() -> std::string {
        if (k + 1 >= argc) throw fnet::Error(FNETG_E_INVALID, a + " needs a value");
        return argv[++k];
      };
      if (a == "--atomic-numbers") {
        std::stringstream ss(next());
        std::string item;
        while (std::getline(ss, item, ',')) st.atomicNumbers.push_back(std::stoi(item));
      } else if (a == "--periodic") {
        st.periodic = true;
      } else if (a == "--file") {
        file = next();
      } else if (a == "--prefix") {
        prefix = next();
      } else if (a == "--host") {
        host = next();
      } else if (a == "--port") {
        port = std::stoi(next());
      } else if (a == "--max-steps") {
        maxSteps = std::stoll(next());
      } else if (a == "--verbosity") {
        st.socket.verbosity = std::stoi(next());
      } else if (a == "--fp32") {
        st.precision = FNETG_FP32;
      } else {
        throw fnet::Error(FNETG_E_INVALID, "unknown option " + a);
      }
    }
    if (file.empty() == host.empty())
      throw fnet::Error(FNETG_E_INVALID, "Either Host or File (but not both) must be set for socket communication.");
    if (!file.empty()) {
      st.socket.host = prefix + file;
      st.socket.port = 0;
    } else {
      if (port <= 0) throw fnet::Error(FNETG_E_INVALID, "Invalid port number");
      st.socket.host = host;
      st.socket.port = port;
    }
    st.nGeoSteps = maxSteps == -1 ? std::numeric_limits<int64_t>::max() : maxSteps;
    const fnet::Netstat ns = fnet::readNetstat(argv[1]);
    const int64_t served = fnet::runSocketDriver(ns, st);
    std::printf("%lld\n", (long long)served);
    return 0;
  } catch (const fnet::Error &e) {
    std::fprintf(stderr, "fnetg_ipi: error %d: %s\n", e.code, e.what());
    return 1;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "fnetg_ipi: %s\n", e.what());
    return 1;
  }
}
