// i-PI socket client (lib_io/ipisocket.F90 over external/fsockets/sockets.c) and the
// socket-driven prediction loop (prg_fnet/fortnet.F90:126-169) on the prediction service.
#include "ipi.hpp"

#include <netdb.h>
#include <sys/socket.h>
#include <sys/types.h>
#include <sys/un.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "fnetg_serve.h"

namespace fnet {

namespace {

constexpr size_t kMsgLen = 12;  // IPI_MSGLEN (ipisocket.F90:103)

[[noreturn]] void fail(const std::string &msg) { throw Error(FNETG_E_INVALID, msg); }

int connect_inet(const std::string &host, int port) {
  addrinfo hints{}, *res = nullptr;
  hints.ai_socktype = SOCK_STREAM;
  hints.ai_family = AF_UNSPEC;
  const std::string service = std::to_string(port);
  const int err = getaddrinfo(host.c_str(), service.c_str(), &hints, &res);
  if (err != 0) fail("ipisocket: cannot resolve host '" + host + "': " + gai_strerror(err));
  int fd = -1;
  for (addrinfo *p = res; p; p = p->ai_next) {
    fd = socket(p->ai_family, p->ai_socktype, p->ai_protocol);
    if (fd < 0) continue;
    if (connect(fd, p->ai_addr, p->ai_addrlen) == 0) break;
    close(fd);
    fd = -1;
  }
  freeaddrinfo(res);
  if (fd < 0) fail("ipisocket: cannot connect to " + host + ":" + service);
  return fd;
}

int connect_unix(const std::string &path) {
  sockaddr_un addr{};
  addr.sun_family = AF_UNIX;
  if (path.size() >= sizeof(addr.sun_path)) fail("ipisocket: UNIX socket path too long");
  std::memcpy(addr.sun_path, path.c_str(), path.size() + 1);
  const int fd = socket(AF_UNIX, SOCK_STREAM, 0);
  if (fd < 0) fail("ipisocket: cannot create a UNIX socket");
  if (connect(fd, reinterpret_cast<sockaddr *>(&addr), sizeof(addr)) != 0) {
    close(fd);
    fail("ipisocket: cannot connect to UNIX socket " + path);
  }
  return fd;
}

}  // namespace

IpiSocketComm::IpiSocketComm(const IpiSocketCommInp &input)
    : nAtom_(input.nAtom), verbosity_(input.verbosity) {
  if (input.nAtom <= 0) fail("ipisocket: number of atoms must be positive");
  if (input.protocol != 1) fail("ipisocket: unknown message protocol " + std::to_string(input.protocol));
  fd_ = input.port < 1 ? connect_unix(input.host) : connect_inet(input.host, input.port);
  log(1, "socketCreate: ...Done");
}

IpiSocketComm::~IpiSocketComm() { shutdown(); }

void IpiSocketComm::shutdown() {
  if (fd_ >= 0) close(fd_);
  fd_ = -1;
}

void IpiSocketComm::log(int level, const std::string &msg) const {
  if (verbosity_ >= level) std::fprintf(stderr, "%s\n", msg.c_str());
}

void IpiSocketComm::readAll(void *buf, size_t n) {
  char *p = static_cast<char *>(buf);
  while (n > 0) {
    const ssize_t got = read(fd_, p, n);
    if (got < 0 && errno == EINTR) continue;
    if (got <= 0) fail("ipisocket: connection closed while reading");
    p += got;
    n -= (size_t)got;
  }
}

void IpiSocketComm::writeAll(const void *buf, size_t n) {
  const char *p = static_cast<const char *>(buf);
  while (n > 0) {
    const ssize_t put = write(fd_, p, n);
    if (put < 0 && errno == EINTR) continue;
    if (put <= 0) fail("ipisocket: connection closed while writing");
    p += put;
    n -= (size_t)put;
  }
}

std::string IpiSocketComm::readHeader() {
  char h[kMsgLen];
  readAll(h, kMsgLen);
  std::string s(h, kMsgLen);
  while (!s.empty() && (s.back() == ' ' || s.back() == '\0')) s.pop_back();
  return s;
}

void IpiSocketComm::writeHeader(const char *msg) {
  char h[kMsgLen];
  std::memset(h, ' ', kMsgLen);
  std::memcpy(h, msg, std::min(kMsgLen, std::strlen(msg)));
  writeAll(h, kMsgLen);
}

bool IpiSocketComm::receive(std::vector<double> &coords, double cell[9]) {
  std::string header;
  for (;;) {
    header = readHeader();
    log(3, "ipisocket%receive: read from socket: " + header);
    if (header != "STATUS") break;
    writeHeader("READY");
  }
  if (header == "EXIT") {
    log(1, "ipisocket%receive: EXIT");
    return false;
  }
  if (header != "POSDATA")
    fail("ipisocket%receive: Unexpected message from server, received '" + header + "'");
  double buf[9], inv[9];
  readAll(buf, sizeof buf);
  // cell = transpose(reshape(buffer, [3, 3])): cell(i, k) = buffer(k + 3 i)
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) cell[i + 3 * k] = buf[k + 3 * i];
  readAll(inv, sizeof inv);  // inverse cell, not used
  int32_t natom = 0;
  readAll(&natom, sizeof natom);
  if (natom != nAtom_)
    fail("Mismatch in number of atoms received " + std::to_string(natom) + " " +
         std::to_string(nAtom_));
  coords.resize(3 * (size_t)natom);
  readAll(coords.data(), sizeof(double) * coords.size());
  return true;
}

void IpiSocketComm::send(double energy, const std::vector<double> &forces, const double stress[9]) {
  if (forces.size() != 3 * (size_t)nAtom_) fail("Mismatch in number of atoms in socketSend");
  std::string header;
  for (;;) {
    header = readHeader();
    log(3, "ipisocket%send: read from socket: " + header);
    if (header != "STATUS") break;
    writeHeader("HAVEDATA");
  }
  if (header != "GETFORCE")
    fail("ipisocket%send: Error in socket communication! (expected 'GETFORCE', received '" +
         header + "')");
  writeHeader("FORCEREADY");
  writeAll(&energy, sizeof energy);
  const int32_t natom = nAtom_;
  writeAll(&natom, sizeof natom);
  writeAll(forces.data(), sizeof(double) * forces.size());
  writeAll(stress, sizeof(double) * 9);
  const int32_t nextra = 0;
  writeAll(&nextra, sizeof nextra);
}

int64_t runSocketDriver(const Netstat &ns, const SocketDriverSettings &st) {
  const int nAtom = (int)st.atomicNumbers.size();
  if (nAtom == 0) fail("socket driver: no atoms");
  // predictForSocketComm (fortnet.F90:560-565) and handleInitialisationForSocketComm (443)
  if (ns.nAtomicTargets != 0 || ns.nGlobalTargets != 1)
    fail("Socket driven operation only working for exactly one global target.");
  if (!ns.extIndices.empty())
    fail("Socket operation does not support additional external input features.");
  for (int32_t z : st.atomicNumbers) {
    bool found = false;
    for (int32_t w : ns.atomicNumbers) found = found || w == z;
    if (!found) fail("BPNN does not contain sub-network of atomic number " + std::to_string(z) + ".");
  }
  if (ns.gFunctions.empty()) fail("socket driver: the netstat holds no ACSF mapping");
  // without stored statistics the features enter unstandardised: mean 0, deviation 1
  std::vector<double> zprec = ns.zPrec;
  if (zprec.empty()) {
    zprec.assign(2 * ns.gFunctions.size(), 0.0);
    std::fill(zprec.begin() + ns.gFunctions.size(), zprec.end(), 1.0);
  }
  if (zprec.size() != 2 * ns.gFunctions.size()) fail("socket driver: z-score statistics size");
  fnetg_server_config cfg{};
  cfg.precision = st.precision;
  cfg.lanes = st.lanes;
  cfg.max_batch_atoms = std::max<int64_t>(65536, nAtom);
  fnetg_server *srv = nullptr;
  int rc = fnetg_server_create(&srv, &cfg, (int32_t)ns.atomicNumbers.size(),
                               ns.atomicNumbers.data(), (int32_t)ns.gFunctions.size(),
                               ns.gFunctions.data(), zprec.data(), (int32_t)ns.dims.size(),
                               ns.dims.data(), ns.activation, ns.params.data());
  if (rc) throw Error(rc, "fnetg_server_create failed");
  IpiSocketCommInp inp = st.socket;
  inp.nAtom = nAtom;
  int64_t served = 0;
  try {
    IpiSocketComm socket(inp);
    std::vector<double> coords, forces(3 * (size_t)nAtom);
    double cell[9];
    const int nout = ns.dims.back();
    std::vector<double> energy(nout), f((size_t)nAtom * nout * 3);
    for (int64_t step = 0; step < st.nGeoSteps; step++) {
      if (!socket.receive(coords, cell)) break;
      double cellVol = 0.0;
      if (st.periodic) {
        const double *a = cell;  // determinant33 of latVecs
        cellVol = std::fabs(a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) +
                            a[6] * (a[1] * a[5] - a[4] * a[2]));
      }
      int64_t ticket = 0;
      rc = fnetg_server_submit(srv, nAtom, st.atomicNumbers.data(), coords.data(),
                               st.periodic ? 1 : 0, cell, 0, &ticket);
      if (!rc) rc = fnetg_server_wait(srv, ticket, -1.0, energy.data(), f.data(), nullptr);
      if (rc) throw Error(rc, fnetg_server_last_error(srv));
      for (int a = 0; a < nAtom; a++)
        for (int c = 0; c < 3; c++) forces[3 * a + c] = f[((size_t)a * nout + 0) * 3 + c];
      // the reference sends stress(:,:) = 1 times the cell volume as the virial
      // (fortnet.F90:127-128, 220-254)
      double virial[9];
      for (double &v : virial) v = cellVol;
      socket.send(energy[0], forces, virial);
      served++;
    }
    socket.shutdown();
  } catch (...) {
    fnetg_server_destroy(srv);
    throw;
  }
  fnetg_server_destroy(srv);
  return served;
}

}  // namespace fnet
