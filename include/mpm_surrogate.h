/* Learned return map for the von Mises hardening material: C ABI.
 *
 * A small network (13 inputs: stress[6], isotropic back stress R, strain
 * increment[6]; 3 hidden layers of 128 with ReLU; 7 outputs: stress
 * increment[6], dR) that stands in for
 * ConstitutiveRelation::calculateIncrement_VonMisesHardening
 * (ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp:4-92)
 * away from the yield surface.  The reference has no such component; the
 * network is trained here on samples of the exact return map (computed in
 * FP64 by the engine's own kernel), by the library's own CUDA forward,
 * backward and Adam kernels, and runs as a BF16 tensor-core (tcgen05)
 * inference kernel with FP32 accumulation.  The network's stress outputs are
 * the plastic correction dsigma - D de; the kernels add the elastic
 * predictor D de (exact, FP32), so elastic trial states come out exact.
 *
 * In an engine (mpm_attach_surrogate), pass 2 keeps the exact map for
 * particles whose trial yield function lies within `band` x k0 of the
 * surface (k0 = yield/sqrt 3) and for elastic trial states, queues the
 * clearly plastic ones for the network, and re-checks a random fraction of
 * the queued particles against the exact map (in FP64) every step: the judge
 * of the network's error, recorded in mpm_surrogate_stats.  A guard then
 * checks every network result: its inputs must lie in the box of inputs the
 * network was trained on, and the result must be the radial return of its
 * trial state (the new stress on the yield surface k0 + R/sqrt 2, the
 * correction dsigma - D de deviatoric, and each stress component and dR
 * equal to the FP32 radial return, all to MPM_OPT_SURROGATE_GUARD x k0,
 * default 0.001); a result that fails takes the exact map in FP64 instead
 * (counted as rejected).
 *
 * All functions return MPM_OK (0) or a negative MPM_ERR_* code.  Samples
 * are rows of floats in physical units: inputs n x 13, outputs n x 7.
 */
#ifndef MPM_SURROGATE_H
#define MPM_SURROGATE_H

#include <stdint.h>

#include "mpm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_net mpm_net;

typedef struct mpm_net_config {
    double E, nu, yield, C0, C1; /* the material (Material_BC fields, as mpm_material) */
    int64_t n_samples;           /* training set size */
    int32_t batch, epochs;       /* Adam minibatch size and passes over the set */
    double lr;                   /* Adam step size (decayed by a cosine over the run) */
    double stress_range;         /* prior stress components uniform in +-stress_range x yield */
    double epbar_max;            /* equivalent plastic strain uniform in [0, epbar_max] -> R */
    double deps_sigma;           /* strain increment components N(0, deps_sigma) */
    uint64_t seed;
    int32_t sampling;            /* 0: prior stress as above; 1: near the yield surface (sqrt J2 in
                                    [0.85, 1] x (k0 + R/sqrt 2), hydrostatic part U(+-yield)), like states
                                    a step after a return */
    int32_t pad;
} mpm_net_config;

typedef struct mpm_net_report {
    double loss_first, loss_last;   /* mean training loss (normalised units) of the first and last epoch */
    double val_rms_dsig;            /* held-out RMS error of dstress / yield (all samples) */
    double val_rms_dsig_outside;    /* the same over samples outside the fallback band */
    double val_max_dsig;            /* held-out max |error| of dstress / yield outside the band */
    double val_rms_dR;              /* held-out RMS error of dR / yield */
    double seconds_generate, seconds_train;
    int64_t steps, n_val;
    double out_scale[8];            /* output normalisation (physical = normalised x scale + shift) */
    double out_shift[8];
} mpm_net_report;

int mpm_net_create(const mpm_net_config* cfg, mpm_net** out);
void mpm_net_destroy(mpm_net* net);
/* Generate the training set with the exact FP64 return map and train. */
int mpm_net_train(mpm_net* net, mpm_net_report* report);
/* Train on given input rows (device, n x 13 physical, e.g. harvested from a
 * run of the plain method with mpm_harvest_begin), labelled by the exact FP64
 * map; the last n/20 rows (at most 65536) are held out for validation. */
int mpm_net_train_rows(mpm_net* net, const float* d_rows, int64_t n, mpm_net_report* report);
/* Parameters (FP32 master copy), packed W1[128][16], b1[128], W2[128][128],
 * b2, W3[128][128], b3, W4[8][128], b4[8]; n must be mpm_net_param_count(). */
int64_t mpm_net_param_count(void);
int mpm_net_get_params(mpm_net* net, float* host, int64_t n);
int mpm_net_set_params(mpm_net* net, const float* host, int64_t n);
/* Loss and gradient of the current parameters on n normalised samples
 * (host rows x[n][16], t[n][8]) by the training kernels (gradient check). */
int mpm_net_loss_grad(mpm_net* net, const float* x, const float* t, int64_t n, float* grad, double* loss);
/* Inference on device rows (inputs n x 13, outputs n x 7, physical units).
 * kernel: 0 = BF16 tcgen05, 1 = FP32 CUDA cores (reference), 2 = the exact
 * FP32 return map (the method without the network), 3 = the exact return map
 * in FP64 on the float inputs, outputs rounded once to float (the FP32 form's
 * fallback path and the judge of the network, MPM_OPT_FP64_FALLBACK). */
int mpm_net_infer(mpm_net* net, const float* d_in, float* d_out, int64_t n, int kernel, void* stream);
/* Normalisation in use: physical input = normalised x in_scale; physical
 * output = normalised x out_scale + out_shift (+ D de for the stress). */
int mpm_net_scales(mpm_net* net, double in_scale[13], double out_scale[7], double out_shift[7]);

typedef struct mpm_surrogate_stats {
    int64_t queued;          /* particles whose return map the network computed */
    int64_t band;            /* particles kept on the exact map by the fallback band */
    int64_t rechecked;       /* queued particles re-checked against the exact map */
    double recheck_rms;      /* RMS of |dsigma_net - dsigma_exact| / yield over the rechecks */
    double recheck_max;      /* max of the same */
    int64_t rejected;        /* queued particles whose network result the guard replaced by the exact FP64 map */
} mpm_surrogate_stats;

/* Use the network in the engine's FP32 form for von Mises hardening
 * particles (NULL detaches).  band: fallback half-width as a fraction of k0
 * (0.02); recheck: fraction of queued particles re-checked per step (0.01). */
int mpm_attach_surrogate(mpm_ctx* ctx, mpm_net* net, double band, double recheck);
int mpm_surrogate_stats_read(mpm_ctx* ctx, mpm_surrogate_stats* out, int reset);

/* Harvest return-map inputs from an engine run (either form): while on, each
 * step appends (stress[6], R, strain increment[6]) of every particle whose
 * material bit is set in mat_mask and whose trial yield function is at least
 * band x k0, to the device rows d_rows (up to cap rows); the engine's own
 * results are unchanged.  mpm_harvest_end stops and reports the rows written
 * (rows beyond cap are counted, not written). */
int mpm_harvest_begin(mpm_ctx* ctx, float* d_rows, int64_t cap, uint32_t mat_mask, double band);
int mpm_harvest_end(mpm_ctx* ctx, int64_t* rows);

#ifdef __cplusplus
}
#endif

#endif
