/* gpet_surrogate.h - learned detector response: C ABI.
 *
 * No counterpart in the reference, which always transports each photon
 * through the panel crystals (photonde, gPET_kernals.cu:839-1233). An MLP
 * (16 inputs -> 4 x 256 SiLU -> 204 outputs, BF16 weights, FP32
 * accumulation on the tcgen05 tensor cores) maps a photon entering a panel to
 * its detector response; photons outside the domain it was validated on are
 * transported by the plain Monte Carlo. */
#ifndef GPET_SURROGATE_H
#define GPET_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gpet_ctx gpet_ctx;
typedef struct gpet_surrogate gpet_surrogate;

/* A photon entering a panel and its detector response after the adder and
 * readout: the surrogate's training record (40 bytes). Option
 * record_entries=1 on a context keeps one per photon that reaches a panel
 * (photons the surrogate handled are not recorded). */
typedef struct {
    int32_t panel;        /* panel index */
    float y, z;           /* entry point in the panel's local frame (cm) */
    float ux, uy, uz;     /* direction in the panel's local frame */
    float E;              /* energy at entry (eV) */
    int32_t crystal;      /* crystal of the photon's first pulse, -1: no pulse */
    float depth;          /* depth of that pulse below the entry face (cm) */
    float Edep;           /* its energy (eV) */
} gpet_entry;

int gpet_get_entries(gpet_ctx* ctx, gpet_entry* buf, int64_t cap, int64_t* n);

/* A surrogate for the detector of `ctx` (its panel geometry, materials and
 * readout, which must give at most one pulse per photon: one module per
 * panel, readout depth <= 2), with seeded random initial weights, on ctx's
 * device. Up to 64 crystals per panel, each energy class's crystal set is one
 * softmax over the crystals; a grid of up to 32 x 32 crystals (the
 * whole-body ring's 16 x 16) is factorised: the set's first 32 columns are
 * row logits, its last 32 column logits, the crystal row + crystalNy x
 * column. */
int gpet_surrogate_create(gpet_ctx* ctx, uint64_t seed, gpet_surrogate** out);
void gpet_surrogate_destroy(gpet_surrogate* s);
const char* gpet_surrogate_last_error(gpet_surrogate* s);
/* Parameters, fp32, in this order: for each layer l = 0..4 its weights
 * [out][in] then biases [out] (in: 16, 256, 256, 256, 256; out: 256, 256,
 * 256, 256, 208; output rows 204-207 are padding
 * and stay zero), then the panel embedding [npanels][6]. */
int64_t gpet_surrogate_param_count(gpet_surrogate* s);
int gpet_surrogate_get_params(gpet_surrogate* s, float* out, int64_t n);
int gpet_surrogate_set_params(gpet_surrogate* s, const float* in, int64_t n);
/* Validated domain: photons entering with energy in [e_lo, e_hi] eV, at
 * least `margin` cm inside the panel's y and z edges, on a panel flagged in
 * panel_ok (NULL: all) take the surrogate; the others the Monte Carlo. */
int gpet_surrogate_set_domain(gpet_surrogate* s, float e_lo, float e_hi, float margin, const uint8_t* panel_ok,
                              int32_t npanels);
/* Mean loss of n records and its gradient (param_count floats, NULL: none)
 * at the current parameters; no update. */
int gpet_surrogate_grad(gpet_surrogate* s, const gpet_entry* rec, int64_t n, float* loss, float* grad);
/* Raw head outputs [n][208] of n records (for checks): crystal logits of the
 * partial-deposit class [0, 64) and of the near-full class [64, 128) (energy
 * bin >= 40 of 64; factorised: rows then columns in each), mixture weights [128, 132), means [132, 136), log sigmas
 * [136, 140), energy-fraction logits [140, 204). */
int gpet_surrogate_forward(gpet_surrogate* s, const gpet_entry* rec, int64_t n, float* out208);
/* Adam (beta 0.9, 0.999) over `epochs` shuffled passes in batches of
 * `batch`, the learning rate falling from lr to lr / 50 along a cosine over
 * the call's steps; epoch_loss[epochs] (may be NULL) receives each pass's
 * mean loss. */
int gpet_surrogate_train(gpet_surrogate* s, const gpet_entry* rec, int64_t n, int32_t epochs, int32_t batch,
                         float lr, uint64_t seed, float* epoch_loss);
/* Calibration on the records of the surrogate's current domain: `iters`
 * passes each move the biases of the crystal logits of each energy class
 * (factorised head: the cell weights of each (class, row, column)) and of the
 * energy-bin logits by log(observed / expected) of that (class, crystal) or
 * energy-bin count over the records, so that the model's expected
 * counts match the Monte Carlo ones (iterative proportional fitting; the
 * other parameters stay). *max_adjust (may be NULL) receives the last pass's
 * largest |log ratio|. Call after gpet_surrogate_set_domain. */
int gpet_surrogate_calibrate(gpet_surrogate* s, const gpet_entry* rec, int64_t n, int32_t iters, float* max_adjust);
/* Factorised head only: the weight of each (energy class, row, column) cell
 * on the product of the row and column probabilities, float[2][32][32]
 * (class, row, column; n = 2048), 1 after create, fitted by
 * gpet_surrogate_calibrate so that the model's expected (class, crystal)
 * counts match the records'. Saved and restored beside the parameters. */
int gpet_surrogate_get_cell_weights(gpet_surrogate* s, float* out, int64_t n);
int gpet_surrogate_set_cell_weights(gpet_surrogate* s, const float* in, int64_t n);
/* Use (s) or stop using (NULL) the surrogate in this context's runs; s must
 * outlive its use. Its photons produce pulses but no hits. */
int gpet_set_surrogate(gpet_ctx* ctx, gpet_surrogate* s);

/* Tensor-core self-test: D[128 x N] = A[128 x K] * B[N x K]^T with A, B
 * row-major bf16 (raw 16-bit patterns) and D row-major f32, one tile on
 * `device`. K, N multiples of 16 in [16, 256]. */
int gpet_umma_selftest(int device, const uint16_t* a_bf16, const uint16_t* b_bf16, int32_t K, int32_t N,
                       float* d_out);

#ifdef __cplusplus
}
#endif
#endif
