// Energy/force prediction service (include/fnetg_serve.h): a request queue served by
// continuous batching over a fixed set of lanes.  Each lane is one library context (its own
// CUDA stream) driven by its own host thread; a free lane takes every queued request that
// fits its admission budget and runs the plain device pipeline on the batch.  Host code only:
// the device work is the library's kernels, reached through its C-ABI.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fnetg_batch.h"
#include "fnetg_serve.h"
#include "internal.cuh"

namespace {

int64_t clock_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Request {
  int64_t ticket = 0;
  int32_t natoms = 0;
  int32_t periodic = 0;
  std::vector<int32_t> atnum, species;
  std::vector<double> coords, lat;
  int64_t arrival_ns = 0, done_ns = 0;
  int status = 1;  // 1 pending; FNETG_OK done; < 0 failed
  std::vector<double> energy, forces;
};
using RequestPtr = std::shared_ptr<Request>;

struct Lane {
  fnetg_ctx *ctx = nullptr;
  fnetg::PoolAlloc alloc{};  // the server's pool on this lane's stream
  std::thread th;
  std::atomic<int64_t> dev_bytes{0};  // device memory held by the lane's context
  int64_t peak_atoms = 0;   // largest batch served
  // host staging of one batch, reused
  std::vector<int64_t> off;
  std::vector<int32_t> atnum, species, periodic;
  std::vector<double> coords, lat, global, forces;
};

constexpr double kDefaultBytesPerAtom = 16384.0;

}  // namespace

struct fnetg_server {
  fnetg_server_config cfg{};
  int32_t nspecies = 0, nout = 1;
  std::vector<int32_t> atomic_numbers, dims;
  std::vector<fnetg_gfunc> g;
  std::vector<double> zprec, params;
  int32_t activation = FNETG_ACT_TANH;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<RequestPtr> queue;
  std::unordered_map<int64_t, RequestPtr> live;
  int64_t next_ticket = 1;
  bool stop = false;
  std::vector<std::unique_ptr<Lane>> lanes;
  cudaMemPool_t pool = nullptr;
  std::string err;
  fnetg_server_stats st{};
  int32_t in_flight = 0;
  double bytes_per_atom = kDefaultBytesPerAtom;
  bool measured = false;

  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
  // atoms a batch may hold: max_batch_atoms, and the lane's share of the memory budget
  int64_t batch_cap() const {
    const double share = (double)cfg.hbm_budget_bytes / std::max(1, cfg.lanes);
    const int64_t by_mem = (int64_t)(share / std::max(bytes_per_atom, 1.0));
    return std::max<int64_t>(1, std::min<int64_t>(cfg.max_batch_atoms, by_mem));
  }
};

namespace {

// one batch through the device pipeline; results into the requests
int run_batch(fnetg_server *s, Lane &ln, std::vector<RequestPtr> &batch) {
  fnetg_ctx *ctx = ln.ctx;
  const int S = (int)batch.size();
  ln.off.assign(1, 0);
  ln.atnum.clear();
  ln.species.clear();
  ln.coords.clear();
  ln.periodic.assign(S, 0);
  ln.lat.assign((size_t)9 * S, 0.0);
  for (int k = 0; k < S; k++) {
    const Request &r = *batch[k];
    ln.off.push_back(ln.off.back() + r.natoms);
    ln.atnum.insert(ln.atnum.end(), r.atnum.begin(), r.atnum.end());
    ln.species.insert(ln.species.end(), r.species.begin(), r.species.end());
    ln.coords.insert(ln.coords.end(), r.coords.begin(), r.coords.end());
    ln.periodic[k] = r.periodic;
    if (r.periodic) std::copy(r.lat.begin(), r.lat.end(), ln.lat.begin() + 9 * k);
  }
  const int64_t N = ln.off.back();
  const int nout = s->nout;
  int rc = fnetg_upload_structures(ctx, S, ln.off.data(), ln.atnum.data(), ln.coords.data(),
                                   ln.periodic.data(), ln.lat.data(), nullptr, 0);
  if (!rc) rc = fnetg_set_species(ctx, ln.species.data());
  if (!rc) rc = fnetg_acsf(ctx, nullptr);
  if (!rc) rc = fnetg_acsf_zscore(ctx, nullptr, s->zprec.data(), 0);
  ln.global.resize((size_t)S * nout);
  ln.forces.resize((size_t)N * nout * 3);
  if (s->cfg.tensor_cores) {
    // the batch as one mini-batch of species tiles; forward and Jacobian on the tensor cores
    if (!rc) rc = fnetg_batch_setup(ctx, S);
    if (!rc) rc = fnetg_batch_forces(ctx, ln.global.data(), ln.forces.data());
  } else {
    if (!rc) rc = fnetg_predict(ctx, nullptr, ln.global.data());
    if (!rc) rc = fnetg_forces(ctx, ln.forces.data());
  }
  if (rc) return rc;
  for (int k = 0; k < S; k++) {
    Request &r = *batch[k];
    r.energy.assign(ln.global.begin() + (size_t)k * nout, ln.global.begin() + (size_t)(k + 1) * nout);
    r.forces.assign(ln.forces.begin() + ln.off[k] * nout * 3,
                    ln.forces.begin() + ln.off[k + 1] * nout * 3);
  }
  return FNETG_OK;
}

void lane_loop(fnetg_server *s, Lane *ln) {
  cudaSetDevice(s->cfg.device);
  fnetg::DBuf::account = &ln->dev_bytes;
  fnetg::DBuf::pool = &ln->alloc;
  std::vector<RequestPtr> batch;
  for (;;) {
    int64_t atoms = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
      if (s->stop) break;
      const int64_t cap = s->batch_cap();
      while (!s->queue.empty()) {
        const RequestPtr &r = s->queue.front();
        if (!batch.empty() && atoms + r->natoms > cap) break;
        atoms += r->natoms;
        batch.push_back(r);
        s->queue.pop_front();
      }
      s->in_flight++;
      s->st.max_in_flight = std::max(s->st.max_in_flight, s->in_flight);
    }
    // requests left behind are for the next free lane
    s->cv_work.notify_one();
    const int64_t t0 = clock_ns();
    const int rc = run_batch(s, *ln, batch);
    const int64_t t1 = clock_ns();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->in_flight--;
      ln->peak_atoms = std::max(ln->peak_atoms, atoms);
      // device bytes per atom, measured on batches large enough to hide the fixed tables
      if (!rc && ln->peak_atoms >= 256) {
        const double bpa = (double)ln->dev_bytes.load() / (double)ln->peak_atoms;
        s->bytes_per_atom = s->measured ? std::max(s->bytes_per_atom, bpa) : bpa;
        s->measured = true;
      }
      if (rc) s->err = fnetg_last_error(ln->ctx);
      for (auto &r : batch) {
        r->status = rc;
        r->done_ns = t1;
        if (!rc) {
          s->st.requests++;
          s->st.atoms += r->natoms;
        }
      }
      s->st.batches++;
      s->st.max_batch_atoms = std::max(s->st.max_batch_atoms, atoms);
      s->st.max_batch_requests = std::max<int64_t>(s->st.max_batch_requests, (int64_t)batch.size());
      s->st.busy_s += 1e-9 * (double)(t1 - t0);
      s->st.max_batch_s = std::max(s->st.max_batch_s, 1e-9 * (double)(t1 - t0));
    }
    s->cv_done.notify_all();
    batch.clear();
  }
  fnetg::DBuf::account = nullptr;
  fnetg::DBuf::pool = nullptr;
}

// Frees the lanes' contexts and the pool (after their stream-ordered frees have run).
void teardown(fnetg_server *s) {
  for (auto &ln : s->lanes)
    if (ln->ctx) fnetg_destroy(ln->ctx);
  s->lanes.clear();
  if (s->pool) {
    cudaDeviceSynchronize();
    cudaMemPoolDestroy(s->pool);
    s->pool = nullptr;
  }
}

}  // namespace

extern "C" {

int64_t fnetg_server_clock_ns(void) { return clock_ns(); }

const char *fnetg_server_last_error(const fnetg_server *srv) {
  return srv ? srv->err.c_str() : "null server";
}

int fnetg_server_create(fnetg_server **out, const fnetg_server_config *cfg, int32_t nspecies,
                        const int32_t *atomic_numbers, int32_t ng, const fnetg_gfunc *g,
                        const double *zprec, int32_t nlayer, const int32_t *dims,
                        int32_t activation, const double *params) {
  if (!out || !cfg || !atomic_numbers || !g || !zprec || !dims || !params) return FNETG_E_INVALID;
  *out = nullptr;
  if (nspecies < 1 || ng < 1 || nlayer < 2 || dims[0] != ng) return FNETG_E_SHAPE;
  if (cfg->lanes < 0 || cfg->lanes > 16 || cfg->max_batch_atoms < 0 || cfg->hbm_budget_bytes < 0)
    return FNETG_E_INVALID;
  if (cfg->tensor_cores &&
      (cfg->precision != FNETG_FP32 || nlayer != 4 || dims[3] != 1 ||
       activation != FNETG_ACT_TANH || std::max(dims[1], dims[2]) > 64 || dims[0] > 239))
    return FNETG_E_UNSUPPORTED;
  std::unique_ptr<fnetg_server> s(new fnetg_server());
  s->cfg = *cfg;
  if (s->cfg.lanes == 0) s->cfg.lanes = 3;
  if (s->cfg.max_batch_atoms == 0) s->cfg.max_batch_atoms = 65536;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return FNETG_E_CUDA;
  if (s->cfg.hbm_budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return FNETG_E_CUDA;
    s->cfg.hbm_budget_bytes = (int64_t)(0.8 * (double)free_b);
  }
  s->nspecies = nspecies;
  s->atomic_numbers.assign(atomic_numbers, atomic_numbers + nspecies);
  s->g.assign(g, g + ng);
  s->zprec.assign(zprec, zprec + 2 * ng);
  s->dims.assign(dims, dims + nlayer);
  s->nout = dims[nlayer - 1];
  s->activation = activation;
  const int64_t np = fnetg_nparams(nlayer, dims);
  s->params.assign(params, params + (size_t)nspecies * np);
  // one pool for every lane's buffers, keeping what it reserves
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = cfg->device;
  if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) return FNETG_E_CUDA;
  uint64_t keep = ~uint64_t(0);
  if (cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
    teardown(s.get());
    return FNETG_E_CUDA;
  }
  const int64_t reserve = std::min<int64_t>(
      s->cfg.hbm_budget_bytes,
      s->cfg.reserve_bytes > 0 ? s->cfg.reserve_bytes : (int64_t)s->cfg.lanes << 29);
  for (int l = 0; l < s->cfg.lanes; l++) {
    std::unique_ptr<Lane> ln(new Lane());
    int rc = fnetg_create(&ln->ctx, s->cfg.precision, s->cfg.device);
    void *stream = nullptr;
    if (!rc) rc = fnetg_get_stream(ln->ctx, &stream);
    ln->alloc = fnetg::PoolAlloc{s->pool, static_cast<cudaStream_t>(stream)};
    if (!rc && l == 0 && reserve > 0) {
      // reserve the pool's memory once: allocate and free it in stream order
      void *p = nullptr;
      if (cudaMallocFromPoolAsync(&p, (size_t)reserve, s->pool, ln->alloc.stream) != cudaSuccess ||
          cudaFreeAsync(p, ln->alloc.stream) != cudaSuccess ||
          cudaStreamSynchronize(ln->alloc.stream) != cudaSuccess)
        rc = FNETG_E_NOMEM;
    }
    fnetg::DBuf::account = &ln->dev_bytes;
    fnetg::DBuf::pool = &ln->alloc;
    if (!rc) rc = fnetg_set_gfunctions(ln->ctx, ng, g);
    if (!rc) rc = fnetg_set_network(ln->ctx, nspecies, nlayer, dims, activation, params);
    fnetg::DBuf::account = nullptr;
    fnetg::DBuf::pool = nullptr;
    s->lanes.push_back(std::move(ln));
    if (rc) {
      teardown(s.get());
      return rc;
    }
  }
  for (auto &ln : s->lanes) ln->th = std::thread(lane_loop, s.get(), ln.get());
  *out = s.release();
  return FNETG_OK;
}

int fnetg_server_destroy(fnetg_server *srv) {
  if (!srv) return FNETG_E_INVALID;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
    for (auto &r : srv->queue) {
      r->status = FNETG_E_INVALID;
      r->done_ns = clock_ns();
    }
    srv->queue.clear();
  }
  srv->cv_work.notify_all();
  srv->cv_done.notify_all();
  for (auto &ln : srv->lanes)
    if (ln->th.joinable()) ln->th.join();
  teardown(srv);
  delete srv;
  return FNETG_OK;
}

int fnetg_server_submit(fnetg_server *srv, int32_t natoms, const int32_t *atnum,
                        const double *coords, int32_t periodic, const double *latvecs,
                        int64_t arrival_ns, int64_t *ticket) {
  if (!srv || !ticket || natoms < 1 || !atnum || !coords || (periodic && !latvecs))
    return FNETG_E_INVALID;
  *ticket = 0;
  auto r = std::make_shared<Request>();
  r->arrival_ns = arrival_ns > 0 ? arrival_ns : clock_ns();
  r->natoms = natoms;
  r->periodic = periodic ? 1 : 0;
  r->atnum.assign(atnum, atnum + natoms);
  r->species.resize(natoms);
  for (int32_t a = 0; a < natoms; a++) {
    int sp = -1;
    for (int k = 0; k < srv->nspecies; k++)
      if (srv->atomic_numbers[k] == atnum[a]) sp = k;
    if (sp < 0) {
      std::lock_guard<std::mutex> lk(srv->mu);
      return srv->fail(FNETG_E_INVALID, "atomic number " + std::to_string(atnum[a]) +
                                            " has no sub-network");
    }
    r->species[a] = sp;
  }
  r->coords.assign(coords, coords + 3 * (size_t)natoms);
  for (double c : r->coords)
    if (!std::isfinite(c)) {
      std::lock_guard<std::mutex> lk(srv->mu);
      return srv->fail(FNETG_E_GEOMETRY, "non-finite coordinate");
    }
  if (periodic) r->lat.assign(latvecs, latvecs + 9);
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stop) return srv->fail(FNETG_E_INVALID, "server stopped");
    if (natoms > srv->cfg.max_batch_atoms)
      return srv->fail(FNETG_E_NOMEM, "request of " + std::to_string(natoms) +
                                          " atoms exceeds the admission limit");
    r->ticket = srv->next_ticket++;
    srv->live[r->ticket] = r;
    srv->queue.push_back(r);
    *ticket = r->ticket;
  }
  srv->cv_work.notify_one();
  return FNETG_OK;
}

int fnetg_server_wait(fnetg_server *srv, int64_t ticket, double timeout_s, double *energy,
                      double *forces, double *latency_ms) {
  if (!srv) return FNETG_E_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->live.find(ticket);
  if (it == srv->live.end()) return srv->fail(FNETG_E_INVALID, "unknown ticket");
  RequestPtr r = it->second;
  auto done = [&] { return r->status != 1; };
  if (timeout_s < 0) {
    srv->cv_done.wait(lk, done);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return FNETG_E_TIMEOUT;
  }
  srv->live.erase(ticket);
  if (r->status != FNETG_OK) return r->status;
  if (energy) std::memcpy(energy, r->energy.data(), sizeof(double) * r->energy.size());
  if (forces) std::memcpy(forces, r->forces.data(), sizeof(double) * r->forces.size());
  if (latency_ms) *latency_ms = 1e-6 * (double)(r->done_ns - r->arrival_ns);
  return FNETG_OK;
}

int fnetg_server_stats_get(fnetg_server *srv, fnetg_server_stats *out) {
  if (!srv || !out) return FNETG_E_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  *out = srv->st;
  out->lanes = srv->cfg.lanes;
  out->batch_cap_atoms = srv->batch_cap();
  int64_t b = 0;
  for (auto &ln : srv->lanes) b += ln->dev_bytes.load();
  out->device_bytes = b;
  return FNETG_OK;
}

}  // extern "C"
