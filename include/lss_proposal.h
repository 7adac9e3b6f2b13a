/*
 * lss_proposal.h -- C ABI of the learned proposal gate: a small channel-local 1-D convolution
 * network that marks which (channel neighbourhood, 32-sample window) cells of a batch may hold a
 * spike, so that the matching loop (src/SpikeSorter/OnlineSpikesV2.cu:903-1001, Kilosort
 * template_matching.py:141-202) considers template t at sample s only where the cell of t's peak
 * channel and s is open.  The reference has no such stage; the plain matcher stays the default
 * and is the source of the network's training labels.
 *
 * Network: x [16][L] (the whitened samples of 16 consecutive channels, channel-major) ->
 * conv(16->64) ReLU -> conv(64->64) ReLU -> conv(64->64) ReLU -> conv(64->1): one logit per
 * sample; every conv has 7 taps with 'same' zero padding,
 *     out[o][l] = b[o] + sum_i sum_k w[o][i][k] * in[i][l + k - 3].
 * Parameters are one float vector of LSS_PROP_N_PARAMS values, layer by layer, each layer's
 * weights [out][in][7] followed by its biases [out].
 * Windows: 32-sample windows tile a batch window's interior [nt, W - nt) (the last one may be
 * shorter); a window's logit is the largest logit of its samples.
 * Neighbourhoods: 16 channels starting every 8 channels, the last one ending at channel C - 1
 * (one neighbourhood, zero-padded, when C <= 16).  A channel belongs to the neighbourhood whose
 * centre (start + 7.5) is nearest (the lower one on ties); a template to the neighbourhood of its
 * peak channel (largest sum_k Wall3[t][k][c]^2).
 * Status codes are those of lss_gb300.h.
 */
#ifndef LSS_PROPOSAL_H
#define LSS_PROPOSAL_H

#include <stdint.h>

#include "lss_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LSS_PROP_CHANNELS 16
#define LSS_PROP_HIDDEN 64
#define LSS_PROP_TAPS 7
#define LSS_PROP_WINDOW 32
#define LSS_PROP_N_PARAMS 65153

/* Neighbourhood starts of an n_chan-channel probe (host only).  *n_nbhd receives the count;
 * starts (may be NULL) receives min(count, cap) starts. */
int lss_prop_neighbourhoods(int32_t n_chan, int32_t* n_nbhd, int32_t* starts, int32_t cap);

/* owner[t] = neighbourhood of template t's peak channel, from Wall3 [T][K][C] (host only). */
int lss_prop_template_owner(const float* wall3, int32_t T, int32_t K, int32_t C, int32_t* owner);

/* ---- training on the device ------------------------------------------------------------ */

typedef struct lss_prop_train_params {
    int32_t device;        /* CUDA ordinal */
    int32_t max_examples;  /* largest number of examples per call */
    int32_t W;             /* samples per example (a batch window: NT + 2 nt) */
    int32_t nt;            /* template length: the interior is [nt, W - nt) */
    float lr, beta1, beta2, eps;   /* Adam; 0 selects 1e-3, 0.9, 0.999, 1e-8 */
} lss_prop_train_params;

typedef struct lss_prop_trainer lss_prop_trainer;

/* init_params: LSS_PROP_N_PARAMS host floats (the trainer keeps an FP32 master copy). */
int lss_prop_trainer_open(const lss_prop_train_params* p, const float* init_params, lss_prop_trainer** out);
int lss_prop_trainer_close(lss_prop_trainer* tr);
const char* lss_prop_trainer_last_error(const lss_prop_trainer* tr);

/* Every call below reads its examples from z_dev, DEVICE memory holding n_windows whitened batch
 * windows [n_windows][W][C] (time-major, FP32; the caller has finished writing it): example e is
 * window pairs[2e] restricted to the 16 channels from pairs[2e + 1] (host int32 pairs).
 * labels: host uint8 [E][n_win] with n_win = ceil((W - 2 nt) / 32).  Each call returns when its
 * work on the device is done. */

/* One Adam step on the mean binary cross-entropy of the window logits; *loss = the loss before
 * the step. */
int lss_prop_train_step(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C,
                        const int32_t* pairs, const uint8_t* labels, int32_t E, float* loss);

/* Loss and its gradient (LSS_PROP_N_PARAMS host floats) at the current parameters; no update. */
int lss_prop_loss_grad(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C,
                       const int32_t* pairs, const uint8_t* labels, int32_t E, float* loss, float* grad);

/* Per-sample logits (host [E][W]) and window logits (host [E][n_win]; either may be NULL). */
int lss_prop_forward(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C,
                     const int32_t* pairs, int32_t E, float* logits, float* window_logits);

int lss_prop_get_params(lss_prop_trainer* tr, float* params);
/* Replaces the parameters and restarts Adam (moments zeroed, step count 0). */
int lss_prop_set_params(lss_prop_trainer* tr, const float* params);

/* ---- gating a sorter --------------------------------------------------------------------- */

/* Enable the gate on a sorter handle (params: LSS_PROP_N_PARAMS host floats, stored on the
 * device with BF16 weights and FP32 biases; NULL disables it).  Each group of windows then runs
 * the network on its whitened windows before the matching loop; a cell is open when its window
 * logit is above logit_threshold, and `dilate` more windows either side of every open cell are
 * opened too.  Scores of closed cells are set to -1e30 so the loop never accepts them.
 * Takes effect for the next group launched. */
int lss_set_proposal(lss_handle* h, const float* params, float logit_threshold, int32_t dilate);

/* Cells gated since the gate was last set: *cells = (window, neighbourhood, 32-sample window)
 * cells evaluated, *open = those left open after dilation.  Waits for the handle's launched
 * groups to finish. */
int lss_proposal_stats(lss_handle* h, int64_t* cells, int64_t* open);

#ifdef __cplusplus
}
#endif

#endif
