// i-PI socket client and the socket-driven prediction loop of the fnet program, on the GPU
// prediction service (include/fnetg_serve.h).
//
// IpiSocketComm follows lib_io/ipisocket.F90 (receive 200-282, send 289-359, shutdown 363-371)
// over the POSIX socket layer of external/fsockets/sockets.c (connect_inet_socket 48,
// connect_unix_socket 101, writebuffer 146, readbuffer 165, close 192): 12-byte space-padded
// message headers, FP64 cell / inverse cell / positions in, FP64 energy / forces / virial out,
// 32-bit atom counts.  Where the reference calls error() and stops, these throw fnet::Error.
// runSocketDriver is the loop of prg_fnet/fortnet.F90:126-169 with predictForSocketComm
// (503-609): every received geometry goes through the service and its energy and forces are
// sent back.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fnet_host.hpp"

namespace fnet {

// IpiSocketCommInp (ipisocket.F90:30-50).  port < 1: a UNIX socket at the path `host`.
struct IpiSocketCommInp {
  int nAtom = 0;
  std::string host;
  int verbosity = 0;
  int protocol = 1;  // IPI_PROTOCOLS%IPI_1
  int port = 0;
};

class IpiSocketComm {
 public:
  explicit IpiSocketComm(const IpiSocketCommInp &input);  // IpiSocketComm_init
  ~IpiSocketComm();
  IpiSocketComm(const IpiSocketComm &) = delete;
  IpiSocketComm &operator=(const IpiSocketComm &) = delete;

  // Answers STATUS with READY until POSDATA (returns true, coordinates [3 nAtom] in Bohr and
  // lattice vectors latVecs(i, k) at cell[i + 3k]) or EXIT (returns false).
  bool receive(std::vector<double> &coords, double cell[9]);
  // Answers STATUS with HAVEDATA until GETFORCE, then FORCEREADY, energy, atom count,
  // forces [3 nAtom], virial [9] and an empty extra string.
  void send(double energy, const std::vector<double> &forces, const double stress[9]);
  void shutdown();

 private:
  void readAll(void *buf, size_t n);
  void writeAll(const void *buf, size_t n);
  std::string readHeader();
  void writeHeader(const char *msg);
  void log(int level, const std::string &msg) const;

  int fd_ = -1;
  int nAtom_ = 0;
  int verbosity_ = 0;
};

// Driver = Socket {...} of the fnet input (initprogram.F90:606-690).
struct SocketDriverSettings {
  IpiSocketCommInp socket;              // host (with the prefix already applied) or port
  std::vector<int32_t> atomicNumbers;   // per atom of the driven structure
  bool periodic = false;
  int64_t nGeoSteps = 200;              // MaxSteps; -1 in the input means no limit
  int32_t precision = FNETG_FP64;
  int32_t lanes = 1;
};

// The socket loop: returns the number of geometries served.
int64_t runSocketDriver(const Netstat &ns, const SocketDriverSettings &settings);

}  // namespace fnet
