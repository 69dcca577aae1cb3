/*
 * fnetg — GB300 (sm_103a) implementation of Fortnet's data-parallel hot path:
 * ACSF featurisation (G1..G5 values and their derivatives) and the per-species
 * Behler-Parrinello network forward/backward used in training and prediction.
 *
 * Plain C ABI: every entry point takes plain pointers and sizes, returns 0 on success or
 * a negative FNETG_E_* code, never aborts the process, and records a message retrievable
 * with fnetg_last_error().  All host arrays are owned by the caller and copied at the call
 * boundary; device buffers are owned by the context and persist across calls.
 *
 * Array conventions (0-based, C order):
 *   atom_offsets[S+1]      CSR structure -> atom ranges (Ntot = atom_offsets[S])
 *   coords[Ntot*3]         cartesian coordinates in Bohr (Fortran coords(3, nAtom))
 *   latvecs[S*9]           Fortran latVecs(3,3) per structure: latvecs[9s + i + 3k] = L(i,k)
 *   per-atom feature rows  feats[a*nf + f]
 *   network parameters     params[s*nparams + q] in the reference's serialised order
 *                          (prog/fortnet/lib_nn/network.F90:397-427): all layers' weight
 *                          matrices column-major (the output layer's ww(d_L,1) included),
 *                          then all layers' bias vectors (the input layer's included).
 *
 * References to the interface each function replaces are given as file:line of the
 * Fortnet source tree (prog/fortnet/...).
 */
#ifndef FNETG_H
#define FNETG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FNETG_ABI_VERSION 1

/* error codes */
#define FNETG_OK 0
#define FNETG_E_INVALID (-1)   /* invalid argument or call order */
#define FNETG_E_SHAPE (-2)     /* inconsistent sizes */
#define FNETG_E_NOMEM (-3)     /* device allocation failed / over the HBM budget */
#define FNETG_E_CUDA (-4)      /* CUDA runtime error */
#define FNETG_E_TIMEOUT (-5)   /* a bounded device wait gave up */
#define FNETG_E_GEOMETRY (-6)  /* dependent lattice vectors, non-finite coordinates */
#define FNETG_E_UNSUPPORTED (-7)

/* arithmetic of the featurisation / network kernels */
#define FNETG_FP32 32
#define FNETG_FP64 64

/* activations, as the reference's transfer functions (lib_nn/transfer.F90:53-342) */
#define FNETG_ACT_TANH 0
#define FNETG_ACT_SIGMOID 1
#define FNETG_ACT_RELU 2
#define FNETG_ACT_LRELU 3
#define FNETG_ACT_SOFTPLUS 4
#define FNETG_ACT_BENT 5
#define FNETG_ACT_ATAN 6
#define FNETG_ACT_GAUSSIAN 7
#define FNETG_ACT_HEAVISIDE 8
#define FNETG_ACT_LINEAR 9

/* losses (lib_common/loss.F90:217-721) */
#define FNETG_LOSS_MSE 0
#define FNETG_LOSS_RMS 1
#define FNETG_LOSS_MAE 2
#define FNETG_LOSS_MAPE 3

/* optimisers (lib_optimizers/optimizers.F90) */
#define FNETG_OPT_SD 0
#define FNETG_OPT_LBFGS 1
#define FNETG_OPT_CG 2     /* conjgrad.F90 with linemin.F90 */
#define FNETG_OPT_FIRE 3   /* fire.F90 */

typedef struct fnetg_ctx fnetg_ctx;

/* One G-function; mirrors TGFunction (lib_descriptors/acsf.F90:40-75).
 * type 1..5 = G1..G5; z1 = z2 = 0 means species unresolved; rcut in Bohr. */
typedef struct {
  int32_t type;
  int32_t atomid; /* 0 = none, else 1-based column of the external features */
  int32_t z1, z2;
  double rcut, kappa, rs, eta, lambda, xi;
} fnetg_gfunc;

/* ---------------------------------------------------------------- context */
/* Replaces the program-level state of fortnet.F90:110-215 (one context per host thread). */
int fnetg_create(fnetg_ctx **ctx, int32_t precision, int32_t device);
int fnetg_destroy(fnetg_ctx *ctx);
const char *fnetg_last_error(const fnetg_ctx *ctx);
int fnetg_abi_version(void);

/* ---------------------------------------------------------------- structures */
/* Geometry ingestion of readHdfDataset (lib_io/fnetdata.F90:1094-1148): cartesian
 * coordinates, lattice vectors, localAtToAtNum; recVecs2p is derived on the device side
 * exactly as fnetdata.F90:1141-1148.  ext may be NULL (next = 0). */
int fnetg_upload_structures(fnetg_ctx *ctx, int32_t nstruct, const int64_t *atom_offsets,
                            const int32_t *atnum, const double *coords,
                            const int32_t *periodic, const double *latvecs,
                            const double *ext, int32_t next);
/* Replace only the coordinates (same structures, same order) — the per-request path. */
int fnetg_update_coords(fnetg_ctx *ctx, const double *coords);
/* localAtToGlobalSp (fnetdata.F90:1115-1117): 0-based sub-network index of every atom. */
int fnetg_set_species(fnetg_ctx *ctx, const int32_t *species);

/* ---------------------------------------------------------------- ACSF */
/* TAcsf_init / TGFunctions (acsf.F90:148-167, 40-88). */
int fnetg_set_gfunctions(fnetg_ctx *ctx, int32_t ng, const fnetg_gfunc *g);

/* Neighbour search replacing buildNeighborlist + TNeighIterator (acsf.F90:1070-1138,
 * lib_dftbp/dynneighlist.F90:233-320): every (i, j, image) with |r_i - r_j - L n|^2 <= rc^2
 * in FP64 with the reference's operation order, in the reference iterator's order per atom.
 * rcut <= 0 uses the largest cutoff of the G-functions. */
int fnetg_neighbors(fnetg_ctx *ctx, double rcut, int64_t *npairs);
/* Download the pair list: pair_offsets[Ntot+1], j (structure-local atom index),
 * shift[3*P] integer lattice translation of the image, d2[P] squared distance. */
int fnetg_get_neighbors(fnetg_ctx *ctx, int64_t *pair_offsets, int32_t *j, int32_t *shift,
                        double *d2);

/* TAcsf_calculate without standardisation (acsf.F90:540-624 -> iGeoAcsf 797-866):
 * raw G-values of every atom; vals may be NULL to keep them on the device only. */
int fnetg_acsf(fnetg_ctx *ctx, double *vals);
/* TAcsf_getMeansAndVariances + applyZscore (acsf.F90:445-511, 626-631): compute = 1
 * computes zprec[2*ng] (means, population standard deviations, weighted by the integer
 * datapoint weights or 1 if weights is NULL) and returns it; compute = 0 uses the given
 * zprec.  Standardises the device-resident features in place. */
int fnetg_acsf_zscore(fnetg_ctx *ctx, const int32_t *weights, double *zprec, int32_t compute);
/* No counterpart in the reference.  The statistics half of fnetg_acsf_zscore(..., compute = 1)
 * (weighted means and population standard deviations of the ACSF columns of the current,
 * unstandardised features) for callers that must keep the library from allocating: a host
 * program that owns a fixed device-memory budget, or a training/serving loop that cannot
 * afford the device-wide synchronisation of cudaMalloc/cudaFree.  On success the call
 * allocates no device or host memory: partial sums use a fixed 1 MiB device array inside the
 * library, weights are read from device memory (d_weights: int32 [nstruct], or NULL for unit
 * weights) and the result goes to d_zprec (device, double [2 * nG]: means, then deviations).
 * Asynchronous on the context's stream; the features are not modified.  Limits: 1 <= nG <=
 * 4095 (FNETG_E_UNSUPPORTED beyond).  Features already standardised by fnetg_acsf_zscore are
 * refused (FNETG_E_INVALID).  The weights are not checked on the host: a zero weight total
 * gives non-finite statistics (0/0), and negative weights give meaningless ones.
 * The first call on a device looks up the scratch array's
 * address (make it before any stream capture).  The scratch array is shared per device:
 * calls that overlap in time (other streams or contexts on the same device) race, so
 * serialise them. */
int fnetg_acsf_zscore_stats_noalloc(fnetg_ctx *ctx, const int32_t *d_weights, double *d_zprec);
/* TFeatures_collect (lib_types/features.F90:200-265): network inputs are
 * [ACSF ; external features ext[:, indices-1]].  n = 0 removes external inputs. */
int fnetg_set_external_inputs(fnetg_ctx *ctx, int32_t n, const int32_t *indices);
/* Download the assembled network inputs feats[Ntot*nf]. */
int fnetg_get_features(fnetg_ctx *ctx, double *feats, int32_t *nf);
/* Upload network inputs directly (skips ACSF); feats[Ntot*nf]. */
int fnetg_set_features(fnetg_ctx *ctx, int32_t nf, const double *feats);

/* ---------------------------------------------------------------- network */
/* TBpnn_init / TBpnn_fromFile (lib_nn/bpnn.F90:96-143, 1141-1288): nspecies equal
 * sub-networks of topology dims[nlayer] (dims[0] = nf) with the given activation (output
 * layer linear).  params[nspecies*nparams] in the serialised order described above. */
int fnetg_set_network(fnetg_ctx *ctx, int32_t nspecies, int32_t nlayer, const int32_t *dims,
                      int32_t activation, const double *params);
int fnetg_get_params(fnetg_ctx *ctx, double *params);
int64_t fnetg_nparams(int32_t nlayer, const int32_t *dims);

/* TBpnn_predictBatch / iPredict (bpnn.F90:1001-1058, 867-900): atomic outputs
 * atomic_out[Ntot*nout]; global_out[S*nout] = per-structure sums in atom order.  Either may be
 * NULL; with atomic_out NULL the sums are formed on the device (the same operations in the same
 * order) and only they are copied.  Pinned host buffers copy at full link bandwidth. */
int fnetg_predict(fnetg_ctx *ctx, double *atomic_out, double *global_out);
/* TBpnn_nJacobian / fdevi (bpnn.F90:937-997, network.F90:183-244):
 * jac[a*nout*nf + o*nf + f] = d out_o / d feature_f of atom a. */
int fnetg_jacobian(fnetg_ctx *ctx, double *jac);
/* forceAnalysis_analytical (lib_analysis/forces.F90:317-425) with calculatePrime
 * (acsf.F90:643-717): forces[a*nout*3 + o*3 + c] = -d(sum_i out_o(i)) / d r_a[c], using the
 * z-score of the last fnetg_acsf_zscore call.  Uses the physical derivative (every periodic
 * image contributes); it equals the reference's whenever no atom sees two images of the
 * same atom within the cutoff. */
int fnetg_forces(fnetg_ctx *ctx, double *forces);
/* forceAnalysis_finiteDiff (lib_analysis/forces.F90:85-117, 182-306): central differences
 * forces[a*nout*3 + o*3 + c] = (P_o(r_ac - delta) - P_o(r_ac + delta)) / (2 delta) of the
 * structure's summed outputs, every displaced copy featurised with the z-score of the last
 * fnetg_acsf_zscore call.  Runs the copies through the device pipeline in batches. */
int fnetg_forces_fd(fnetg_ctx *ctx, double delta, double *forces);

/* Matrix-free dG/dR: the derivative of every atom's standardised network inputs (z-score of
 * the last fnetg_acsf_zscore call) along per-atom vectors w[Ntot*3],
 *   u[a*nf + g] = sum_b sum_c d x_a[g] / d r_b[c] * w[3b + c],
 * i.e. TAcsf_calculatePrime's dense [3, nF, N, N] derivative (acsf.F90:643-717, gFuncGrad
 * 1496-1670) contracted with w, without storing it (physical derivative: every periodic image
 * contributes).  Columns of external features are 0.  G1, G2, G3 and G5 without atom ids;
 * at most 256 neighbours per atom (FNETG_E_UNSUPPORTED otherwise). */
int fnetg_features_jvp(fnetg_ctx *ctx, const double *w, double *u);

/* ---------------------------------------------------------------- training */
/* Targets and weights of TDataset (fnetdata.F90:58-130). gt[S*ngt], at[Ntot*nat],
 * atomic_w[Ntot] (NULL = 1), weights[S] (NULL = 1). */
int fnetg_set_targets(fnetg_ctx *ctx, int32_t ngt, int32_t nat, const double *gt,
                      const double *at, const double *atomic_w, const int32_t *weights);
/* TBpnn_updateGradients / sysTrain (bpnn.F90:394-481, 610-704): raw accumulated
 * gradients grad[nspecies*nparams] (FP64, not yet divided by sum(weights)), the dataset loss
 * (loss.F90:512-721) and the atomic predictions.  order[S] (1-based, NULL = identity) only
 * changes the accumulation order, as the reference's shuffle does.  Outputs may be NULL. */
int fnetg_train_gradients(fnetg_ctx *ctx, int32_t loss, const int32_t *order, double *grad,
                          double *loss_out, double *atomic_out);
/* No counterpart in the reference (it trains on energies only): adds a force term to the
 * training loss, L = L_E + weight / (3 Ntot) sum_a |F_a - F*_a|^2, with F the analytical forces
 * of fnetg_forces and F*[Ntot*3] the target forces.  fnetg_train_gradients and
 * fnetg_train_iteration then return the gradient of L (the energy part in the reference's raw
 * convention, the force part multiplied by the summed datapoint weights, so that the update's
 * normalisation leaves exactly dL_F/dtheta) and L as the loss.  Needs the neighbour list,
 * z-scored features and tanh networks with one output.  weight = 0 switches the term off. */
int fnetg_set_force_targets(fnetg_ctx *ctx, double weight, const double *forces);
/* The energy and force parts of the last loss evaluated with a force term (loss_forces = 0
 * without one). */
int fnetg_last_losses(fnetg_ctx *ctx, double *loss_energy, double *loss_forces);
/* TBpnn_update preamble (bpnn.F90:751-766): elastic-net term, 1/sum(weights) and norm2 of
 * a gradient matrix grad[nspecies*nparams] in place (host buffer, FP64 on the device). */
int fnetg_update_prepare(fnetg_ctx *ctx, double *grad, double regu_strength, double regu_alpha,
                         double *grad_norm);
/* TTraining_initOptimizer (lib_fortnet/initprogram.F90:1102-1191): one optimiser per
 * sub-network, started from the current parameters, state kept in FP64 on the device. */
int fnetg_optimizer_init(fnetg_ctx *ctx, int32_t kind, double threshold, double min_disp,
                         double max_disp, double learning_rate, int32_t memory,
                         int32_t linemin, int32_t qn_max_disp);
/* One iteration of TBpnn_nTrain's loop (bpnn.F90:293-363): update (regularise, normalise,
 * optimiser step per sub-network, bpnn.F90:708-778) with the current gradients, then new
 * gradients and loss at the new parameters (updateGradients).  The first call after
 * fnetg_optimizer_init evaluates the starting gradients first.  Outputs may be NULL. */
int fnetg_train_iteration(fnetg_ctx *ctx, int32_t loss, double regu_strength,
                          double regu_alpha, const int32_t *order, double *loss_out,
                          double *grad_norm_out, int32_t *converged);

/* ---------------------------------------------------------------- initialisation RNG */
/* RANLUX luxury level 3 (lib_dftbp/ranlux.F90, initialised as lib_fortnet/initprogram.F90:392
 * with Options{RandomSeed}); host-side, independent of any context. */
void *fnetg_rng_create(int32_t seed);
void fnetg_rng_destroy(void *rng);
int fnetg_rng_uniform(void *rng, double *out, int64_t n);
/* Initial parameters of TBpnn_init (lib_nn/bpnn.F90:96-143 -> layer.F90:72-86): normalXavier
 * draws (lib_common/random.F90:122-181) per sub-network and layer, zero biases, zero output
 * weights ww(d_L,1); params[nspecies*nparams] in the serialised order. */
int fnetg_rng_init_params(void *rng, int32_t nspecies, int32_t nlayer, const int32_t *dims,
                          double *params);
/* knuthShuffle (lib_common/random.F90:33-55) of arr[n] in place. */
int fnetg_rng_shuffle(void *rng, int32_t *arr, int32_t n);

/* ---------------------------------------------------------------- timing / plumbing */
/* The context's CUDA stream (cudaStream_t) — every kernel of the context runs on it. */
int fnetg_get_stream(fnetg_ctx *ctx, void **stream);
/* Per-kernel CUDA-event timing on the context's stream (0 = off). */
int fnetg_profile_enable(fnetg_ctx *ctx, int32_t enable);
/* Accumulated device time and launch count of one kernel family by name
 * ("neighbors", "acsf_radial", "acsf_angular", "zscore", "mlp_forward", "mlp_backward",
 * "forces", "reduce", "optimizer", "segsum"); -1 if unknown. */
int fnetg_profile_read(fnetg_ctx *ctx, const char *name, double *ms, int64_t *launches);
int fnetg_profile_reset(fnetg_ctx *ctx);
/* Total kernel launches of the context since creation (or the last reset). */
int64_t fnetg_launch_count(fnetg_ctx *ctx);
int fnetg_synchronize(fnetg_ctx *ctx);
/* Bounds-checked build only (the library compiled with -DFNETG_CHECKS): after synchronising
 * the context's stream, *site receives the first failed index check since the last call
 * (file code x 100000 + source line; the access it guarded was skipped) and the record is
 * cleared; 0 = every check passed.  The default build has no checks and always gives 0.  No
 * counterpart in the reference beyond its debug builds' -fbounds-check (sys/gnu.cmake:33). */
int fnetg_check_status(fnetg_ctx *ctx, int32_t *site);
/* Sustained issue rates of the device, measured on the context's stream with CUDA events:
 * FP32 fused multiply-adds (TFLOP/s, two FLOPs each), the special-function unit's ex2
 * (10^12 operations/s) and FP64 fused multiply-adds (TFLOP/s).  Self-written loops of
 * independent dependency chains over every SM, about two seconds in total.  The
 * compute-roofline denominators of the featurisation, force and optimiser kernels; no
 * counterpart in the reference.  Any output pointer may be NULL. */
int fnetg_probe_peaks(fnetg_ctx *ctx, double *fp32_tflops, double *ex2_tops,
                      double *fp64_tflops);

#ifdef __cplusplus
}
#endif
#endif /* FNETG_H */
