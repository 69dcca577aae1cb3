/* fnetg_serve.h — energy/force prediction service on one GPU (C-ABI, part of libfnetg).
 *
 * Replaces the reference's online path: the socket-driven loop of the fnet program
 * (prog/fortnet/prg_fnet/fortnet.F90:126-169 with predictForSocketComm 503-609;
 * lib_io/ipisocket.F90:175-359), which featurises and predicts one structure per request,
 * serially.  Here requests of any size
 * are queued by any number of host threads and served by continuous batching: a fixed set
 * of lanes (each one library context with its own CUDA stream and host thread) takes, as
 * soon as it is free, every queued request that fits its admission budget, runs the device
 * pipeline of the plain form on that batch (neighbour search, ACSF, z-score, network
 * forward, analytical forces) and hands each request its energies and forces.  Requests that
 * arrive while other batches are on the device are admitted by the next free lane, so the
 * lanes' batches overlap on the device.
 *
 * Device memory of the lanes comes from one stream-ordered memory pool that keeps what it
 * has reserved: after the first batches no allocation synchronises the device or maps new
 * memory (both of which stall every lane and, on a coherent CPU-GPU node, the host process).
 *
 * Admission is by device memory: every lane may hold at most hbm_budget_bytes / lanes of
 * device memory, and a batch takes queued requests in arrival order while its atoms times
 * the measured device bytes per atom stay inside that share (and inside max_batch_atoms).
 * A single request larger than max_batch_atoms is refused at submission (FNETG_E_NOMEM).
 *
 * The result of a request does not depend on the batch it was served in, up to the order of
 * the FP64 force accumulation (relative differences of order 1e-15).
 *
 * Return codes are the FNETG_* codes of fnetg.h.  Every entry point is thread-safe.
 */
#ifndef FNETG_SERVE_H
#define FNETG_SERVE_H

#include <stdint.h>

#include "fnetg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fnetg_server fnetg_server;

typedef struct {
  int32_t precision;        /* FNETG_FP32 or FNETG_FP64: arithmetic of ACSF, network, forces */
  int32_t device;           /* CUDA device ordinal */
  int32_t lanes;            /* batches in flight at once; 0 -> 3 */
  int32_t tensor_cores;     /* 1: the network passes (forward and input Jacobian) in BF16 on the
                               tensor cores (fnetg_batch_forces); FP32 precision and networks of
                               two tanh hidden layers of at most 64 units, one output, at most
                               239 inputs.  0: the plain kernels */
  int64_t max_batch_atoms;  /* atoms per batch (and per request) at most; 0 -> 65536 */
  int64_t hbm_budget_bytes; /* device memory all lanes may hold; 0 -> 80% of free memory */
  int64_t reserve_bytes;    /* device memory reserved up front in the lanes' memory pool;
                               0 -> 512 MiB per lane (capped by the budget) */
} fnetg_server_config;

/* The model: G-functions g[ng] with their z-score statistics zprec[2*ng] (means, then
 * standard deviations, as fnetg_acsf_zscore returns them), and nspecies sub-networks of
 * topology dims[nlayer] with parameters params[nspecies * nparams] in the order of
 * fnetg_set_network.  Sub-network s serves the atoms of atomic number atomic_numbers[s]. */
int fnetg_server_create(fnetg_server **srv, const fnetg_server_config *cfg, int32_t nspecies,
                        const int32_t *atomic_numbers, int32_t ng, const fnetg_gfunc *g,
                        const double *zprec, int32_t nlayer, const int32_t *dims,
                        int32_t activation, const double *params);
/* Stops the lanes after the batches in flight; requests still queued complete with
 * FNETG_E_INVALID.  Waiting on a ticket after destroy is not allowed. */
int fnetg_server_destroy(fnetg_server *srv);
const char *fnetg_server_last_error(const fnetg_server *srv);

/* Monotonic clock of the service, in nanoseconds (the time base of arrival_ns). */
int64_t fnetg_server_clock_ns(void);

/* Queue one structure: natoms atoms with atomic numbers atnum[natoms] and cartesian
 * coordinates coords[3*natoms] (Bohr); periodic != 0 with lattice vectors latvecs[9]
 * (latvecs[3k + i] = component i of vector k).  arrival_ns is the request's arrival time
 * on fnetg_server_clock_ns (0: now); latencies are measured from it.  The arrays are
 * copied before return.  *ticket identifies the request. */
int fnetg_server_submit(fnetg_server *srv, int32_t natoms, const int32_t *atnum,
                        const double *coords, int32_t periodic, const double *latvecs,
                        int64_t arrival_ns, int64_t *ticket);

/* Wait up to timeout_s seconds (< 0: no limit) for a request.  On success energy[nout]
 * receives the structure's summed outputs, forces[natoms*nout*3] (may be NULL) the forces
 * in the layout of fnetg_forces, latency_ms (may be NULL) the time from arrival to
 * completion, and the ticket is released.  FNETG_E_TIMEOUT leaves the request pending;
 * a failed request returns its batch's error code (and releases the ticket). */
int fnetg_server_wait(fnetg_server *srv, int64_t ticket, double timeout_s, double *energy,
                      double *forces, double *latency_ms);

typedef struct {
  int64_t requests;          /* completed */
  int64_t batches;
  int64_t atoms;             /* atoms in completed requests */
  int64_t max_batch_atoms;   /* largest batch served */
  int64_t max_batch_requests;
  int64_t device_bytes;      /* device memory held by the lanes' contexts */
  int64_t batch_cap_atoms;   /* current admission cap per batch */
  int32_t lanes;
  int32_t max_in_flight;     /* most batches on the device at once */
  double busy_s;             /* summed batch service time of all lanes */
  double max_batch_s;        /* longest batch service time */
} fnetg_server_stats;

int fnetg_server_stats_get(fnetg_server *srv, fnetg_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* FNETG_SERVE_H */
