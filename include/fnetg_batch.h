/*
 * fnetg batched mixed-precision form — training epochs and predictions of Fortnet's per-species
 * networks over mini-batches of structures, with the layer GEMMs on Blackwell tensor cores
 * (tcgen05, BF16 operands, FP32 accumulation) and FP64 gradient sums, master parameters and
 * optimiser step.
 *
 * The call sequence is that of the plain form (include/fnetg.h): structures, species,
 * G-functions, fnetg_acsf + fnetg_acsf_zscore (features computed once per run, as the reference
 * does at prog/fortnet/prg_fnet/fortnet.F90:840-921), fnetg_set_network, fnetg_set_targets;
 * then fnetg_batch_setup once, and fnetg_batch_epoch / fnetg_batch_predict as often as needed.
 * The parameters live in the context's FP64 master copy (fnetg_get_params reads them).
 *
 * Networks: [nf, H1, H2, 1], tanh hidden layers of at most 64 units, linear output, nf <= 239,
 * one global target (energy).  Other shapes give FNETG_E_UNSUPPORTED.
 */
#ifndef FNETG_BATCH_H
#define FNETG_BATCH_H

#include <stdint.h>

#include "fnetg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Mini-batches of batch_structures consecutive structures (the last may be smaller).  Packs the
 * current (z-scored) features of every mini-batch into species tiles of 128 atoms as BF16, and
 * the current parameters as BF16 weight images.  Targets are needed by the training calls
 * below, not by the setup.  The mini-batch loop replaces the full-batch
 * loop of TBpnn_nTrain (prog/fortnet/lib_nn/bpnn.F90:293-363). */
int fnetg_batch_setup(fnetg_ctx *ctx, int32_t batch_structures);
/* Mini-batch count, tile count and the CTA counts the autotuner chose (0 before the first
 * epoch or prediction). */
int fnetg_batch_info(fnetg_ctx *ctx, int32_t *nbatch, int64_t *ntiles, int32_t *ctas_forward,
                     int32_t *ctas_train);
/* The raw accumulated gradient of mini-batch `batch` at the current parameters (the quantity of
 * TBpnn_updateGradients, bpnn.F90:394-481, over that mini-batch's structures only, not yet
 * divided by their summed weights): grad[nspecies*nparams] in the reference order, and the
 * atomic outputs of the mini-batch's atoms (atom order).  Either output may be NULL. */
int fnetg_batch_gradients(fnetg_ctx *ctx, int32_t batch, int32_t loss, double *grad,
                          double *atomic_out);
/* One epoch: for every mini-batch in order, forward, loss gradients (lib_common/loss.F90:
 * 512-721), reverse pass, FP64 gradient, and the reference's steepest-descent step
 * (lib_dftbp/steepdesc.F90:126-204 after the normalisation of TBpnn_update, bpnn.F90:751-766)
 * with that mini-batch's gradient.  The epoch runs as one captured CUDA graph (captured on the
 * first call and whenever loss, learning rate or maximal displacement change).  loss_out
 * (may be NULL) receives the dataset loss accumulated from each mini-batch's loss before its
 * update. */
int fnetg_batch_epoch(fnetg_ctx *ctx, int32_t loss, double learning_rate, double max_disp,
                      double *loss_out);
/* TBpnn_predictBatch (bpnn.F90:1001-1058) in one tensor-core launch over every tile: atomic
 * outputs atomic_out[Ntot] and per-structure sums global_out[S] (atom order).  Either may be
 * NULL (results stay on the device). */
int fnetg_batch_predict(fnetg_ctx *ctx, double *atomic_out, double *global_out);
/* Energies and analytical forces of every structure with the network passes on the tensor
 * cores: one launch computes every atom's output and input Jacobian (BF16 operands, FP32
 * accumulation; TNetwork_fdevi, network.F90:183-244, in reverse mode), and the FP32 force
 * kernel contracts it with dG/dR (forceAnalysis_analytical, lib_analysis/forces.F90:317-425).
 * FP32 context with z-scored features, after fnetg_batch_setup for the current structures
 * (targets are not needed).  global_out[S] (may be NULL) receives the per-structure sums in
 * atom order, forces_out[N*3] (may be NULL) the forces in the layout of fnetg_forces. */
int fnetg_batch_forces(fnetg_ctx *ctx, double *global_out, double *forces_out);
/* on != 0: fnetg_train_gradients and fnetg_train_iteration (the full-batch L-BFGS / SD loop of
 * TBpnn_nTrain, bpnn.F90:293-363) take their gradients from the tensor-core kernels over every
 * tile of the mini-batch plan: forward, reverse pass and weight gradients in BF16 with FP32
 * accumulation, FP64 sums, parameters and optimiser state.  With a force term
 * (fnetg_set_force_targets) the input Jacobian also comes from the tensor cores, while the
 * analytical forces and the dG/dR contraction stay FP32 (FP32 context required).  This is
 * the precision form; on = 0 returns to the plain kernels. */
int fnetg_batch_train_bf16(fnetg_ctx *ctx, int32_t on);
/* After epochs: refresh the plain form's compute copy of the parameters (and the BF16 images)
 * from the FP64 master, so fnetg_predict / fnetg_forces use the trained parameters. */
int fnetg_batch_sync_params(fnetg_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* FNETG_BATCH_H */
