/*
 * ORACLE — test infrastructure only.  FP64 CPU restatement of Fortnet's hot path
 * (ACSF featurisation, per-species BPNN forward/backward, forces, optimisers).
 * It exists so that the GPU library can be checked against the reference's
 * arithmetic; it is never linked into, loaded by or called from the product.
 * Each function cites the reference file:line it restates (paths relative to the
 * Fortnet source tree).
 */
#ifndef FNET_ORACLE_H
#define FNET_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* G-function description, mirrors TGFunction (prog/fortnet/lib_descriptors/acsf.F90:40-75). */
typedef struct {
  int32_t type;        /* 1..5 = G1..G5 */
  int32_t atomid;      /* 0 = none, else 1-based row of the external features */
  int32_t z1, z2;      /* atomicNumbers(1:2); both 0 = species unresolved */
  double rcut, kappa, rs, eta, lambda, xi;
} orc_gfunc;

/* A batch of structures in flat CSR form (Fortran arrays of TGeometry flattened). */
typedef struct {
  int32_t nstruct;
  const int64_t *atom_offsets; /* [nstruct+1] */
  const double *coords;        /* [ntot*3] cartesian, Bohr, atom-major (Fortran coords(3,nAtom)) */
  const int32_t *atnum;        /* [ntot] atomic number of every atom (localAtToAtNum) */
  const int32_t *periodic;     /* [nstruct] 0/1 */
  const double *latvecs;       /* [nstruct*9] Fortran latVecs(3,3), column k = lattice vector k */
  const double *ext;           /* [ntot*next] external features, atom-major, or NULL */
  int32_t next;
} orc_batch;

/* Network topology, mirrors TNetwork (prog/fortnet/lib_nn/network.F90). */
typedef struct {
  int32_t nlayer;        /* size(dims) */
  const int32_t *dims;   /* [nlayer] */
  int32_t activation;    /* ORC_ACT_* */
} orc_net;

enum {
  ORC_ACT_TANH = 0, ORC_ACT_SIGMOID = 1, ORC_ACT_RELU = 2, ORC_ACT_LRELU = 3,
  ORC_ACT_SOFTPLUS = 4, ORC_ACT_BENT = 5, ORC_ACT_ATAN = 6, ORC_ACT_GAUSSIAN = 7,
  ORC_ACT_HEAVISIDE = 8, ORC_ACT_LINEAR = 9
};

enum { ORC_LOSS_MSE = 0, ORC_LOSS_RMS = 1, ORC_LOSS_MAE = 2, ORC_LOSS_MAPE = 3, ORC_LOSS_MSL = 4 };

/* ---- RANLUX (prog/fortnet/lib_dftbp/ranlux.F90) ---- */
void *orc_ranlux_new(int32_t luxlev, int32_t seed);
void orc_ranlux_get(void *h, double *out, int64_t n);
void orc_ranlux_free(void *h);
/* TBpnn_init draw order (bpnn.F90:96-143 -> network.F90:95-122 -> layer.F90:58-86). */
void orc_init_bpnn_params(void *h, const orc_net *net, int32_t nspecies, double *params);
/* knuthShuffle (lib_common/random.F90:33-55); arr holds 1-based indices. */
void orc_knuth_shuffle(void *h, int32_t *arr, int32_t n);

/* ---- geometry helpers ---- */
/* recVecs2p of fnetdata.F90:1141-1148 (determinant33/invert33 of simplealgebra.F90, transposed). */
int orc_recvecs2p(const double *latvecs, double *recvecs2p);

/* ---- neighbour search (dynneighlist.F90:182-320, latpointiter.F90:62-253) ---- */
/* Full (species-unrestricted) neighbour list of every atom, in the iterator's order.
 * counts[a] receives the number of neighbours; if out_* are non-NULL they are filled at
 * offsets[a] (exclusive scan of counts supplied by the caller). shifts are integer lattice
 * translations (n1,n2,n3) of the neighbour image; d2 is the squared distance. */
int orc_neighbours(const orc_batch *b, double rcut, int64_t *counts, const int64_t *offsets,
                   int32_t *out_j, int32_t *out_shift, double *out_d2, int32_t nthreads);

/* ---- ACSF values (acsf.F90:540-639, 797-866, 1287-1492) ----
 * vals[a*ng + g]; mode 0 rebuilds the neighbour list per (atom, G-function) exactly like
 * buildGFunctionNeighborlists; mode 1 builds one list per atom and filters it per function
 * (same lists, same order).  nthreads > 1 splits structures in contiguous blocks like
 * getStartAndEndIndex (lib_common/parallel.F90:23-56). */
int orc_acsf(const orc_batch *b, const orc_gfunc *g, int32_t ng, int32_t mode, double *vals,
             int32_t nthreads);

/* ---- ACSF derivatives of one structure (acsf.F90:643-717, 870-939, 1496-1697) ----
 * prime in Fortran order (3, ng, N, N): prime[c + 3*(g + ng*(i + N*j))] = dG_g(i)/dr_j[c],
 * with the reference's vector-subscript assignment semantics. */
int orc_acsf_prime(const orc_batch *b, int32_t s, const orc_gfunc *g, int32_t ng, double *prime);
/* physical = 1: every periodic image adds its own derivative (the exact dG/dR); it equals the
 * reference's array whenever no atom has two images of one atom inside the cutoff. */
int orc_acsf_prime_ex(const orc_batch *b, int32_t s, const orc_gfunc *g, int32_t ng,
                      int32_t physical, double *prime);

/* ---- z-score (acsf.F90:445-536) ---- */
void orc_zscore_stats(const double *vals, int64_t ntot, int32_t ng, const int64_t *atom_offsets,
                      int32_t nstruct, const int32_t *weights, double *zprec /* [2*ng]: means, std */);
void orc_zscore_apply(double *vals, int64_t ntot, int32_t ng, const double *zprec);

/* ---- network (network.F90:95-459) ---- */
int64_t orc_nparams(const orc_net *net);
/* iPredict for every atom; species[a] is the 0-based sub-network index; out[a*nout + o]. */
void orc_predict(const orc_net *net, const double *params, int32_t nf, const double *feats,
                 int64_t ntot, const int32_t *species, double *out);
/* fdevi Jacobian [nout, nf] (Fortran order) per atom: jac[a*nout*nf + o + nout*f]. */
void orc_jacobian(const orc_net *net, const double *params, int32_t nf, const double *feats,
                  int64_t ntot, const int32_t *species, double *jac);

/* ---- training gradient (bpnn.F90:394-481, 610-704) ----
 * Accumulates the raw (not yet normalised) gradients dd[nparams*nspecies] over the
 * structures in order[] (1-based shuffle indices) and writes every atom's predictions
 * predicts[a*nout + o].  targets: gt[s*ngt + t], at[a*nat + t]. */
int orc_train_gradients(const orc_net *net, const double *params, int32_t nspecies, int32_t nf,
                        const double *feats, const int32_t *species, int32_t nstruct,
                        const int64_t *atom_offsets, int32_t ngt, int32_t nat,
                        const double *gt, const double *at, const double *atomic_w,
                        const int32_t *weights, const int32_t *order, int32_t loss,
                        double *dd, double *predicts);

/* TBpnn_update preamble (bpnn.F90:708-778): elastic-net term, serialisation, 1/sum(w).
 * grad[nparams*nspecies] is normalised in place; returns norm2 of the whole matrix. */
double orc_update_prepare(const orc_net *net, const double *params, int32_t nspecies, double *grad,
                          double regu_strength, double regu_alpha, double sum_weights);

/* ---- forces (forces.F90:317-425) ---- forces[a*3*nout + c + 3*o] */
int orc_forces(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
               int32_t nout, const double *jac, double *forces);
int orc_forces_ex(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
                  int32_t nout, const double *jac, int32_t physical, double *forces);
/* the same with structures split over nthreads host threads (contiguous blocks) */
int orc_forces_mt(const orc_batch *b, const orc_gfunc *g, int32_t ng, const double *zprec,
                  int32_t nout, const double *jac, int32_t physical, double *forces,
                  int32_t nthreads);

/* ---- optimisers ---- */
/* steepest descent (lib_dftbp/steepdesc.F90:104-204) */
void *orc_sd_new(int32_t n, double tol, double maxdisp, double lr, const double *x0);
int orc_sd_next(void *h, const double *grad, double *xnew);
/* L-BFGS with TLineMin (lib_dftbp/lbfgs.F90:214-488, linemin.F90:112-391) */
void *orc_lbfgs_new(int32_t n, double tol, double mindisp, double maxdisp, int32_t mem,
                    int32_t linesearch, int32_t qndisp, const double *x0);
int orc_lbfgs_next(void *h, double fx, const double *grad, double *xnew);
void *orc_cg_new(int32_t n, double tol, double maxdisp, const double *x0);
int orc_cg_next(void *h, double fx, const double *grad, double *xnew);
void *orc_fire_new(int32_t n, double tol, double maxstep, const double *x0);
int orc_fire_next(void *h, const double *grad, double *xnew);
void orc_opt_free(void *h);

#ifdef __cplusplus
}
#endif
#endif
