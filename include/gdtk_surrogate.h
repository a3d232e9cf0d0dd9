/* gdtk_surrogate.h -- learned surrogate of the chemistry update, with FP64 fallback.
 *
 * No counterpart in the reference.  A multilayer perceptron maps a cell's state and update
 * interval to its increment:
 *   inputs  (nin = nsp + 3):  ln T, ln p, the nsp mass fractions, ln dt
 *   outputs (nout = nsp + 1): the nsp mass-fraction increments and the temperature increment
 * `depth` hidden layers of `width` units with GELU (tanh form).  Weights and activations are
 * BF16, products accumulate in FP32 on the tensor cores, and training keeps FP32 master weights
 * updated by AdamW.  Inputs and outputs are standardised by per-feature shift and scale fitted on
 * the training samples; nin and nout are padded with zero features to multiples of 8
 * (nin_pad, nout_pad).  All array arguments are device pointers unless marked "host".
 *
 * chem_surrogate_update_cells is the chemistry update of chem_reactor_update_cells with the
 * network in front.  Each cell's predicted increment is checked in FP64, in the kernel that
 * applies it:
 *   domain          every raw input lies within the training samples' [min, max];
 *   elements        the predicted increment changes no element's mass fraction by more than
 *                   elem_tol, and is then projected onto exact element conservation;
 *   non-negativity  no mass fraction falls below -neg_tol (small negatives are clipped to 0, the
 *                   element balance is restored by a second projection that moves only the
 *                   species present, and the mass fractions are renormalised);
 *   energy          T from (rho, u, Y_new) by the reference's Newton iteration
 *                   (therm_perf_gas_mix.d:426-468) converges and agrees with T + the predicted
 *                   dT within T_tol (relative);
 *   magnitude       no predicted |dY| exceeds max_dY (when max_dY > 0);
 *   predicted error when an error model is attached and its gate set: the error network's
 *                   estimate of log10 of the prediction's error (the larger of its largest |dY|
 *                   error and 0.1 times its relative error in dT; trained as a quantile) does
 *                   not exceed log10(tol).
 * Accepted cells take Y_new, that T and p = rho R T; their dt_chem is left as it was.  A cell
 * that fails any check is integrated by the plain FP64 update from its original state, exactly
 * as chem_reactor_update_cells would.  Cells at or below T_frozen and cells of invalid density
 * are flagged as the plain update flags them.
 */
#ifndef GDTK_SURROGATE_H
#define GDTK_SURROGATE_H

#ifdef __cplusplus
extern "C" {
#endif

/* per-cell gate codes */
#define GDTK_GATE_ACCEPTED 0
#define GDTK_GATE_FROZEN 1
#define GDTK_GATE_BAD_INPUT 2
#define GDTK_GATE_DOMAIN 3
#define GDTK_GATE_ELEMENTS 4
#define GDTK_GATE_NEGATIVE 5
#define GDTK_GATE_ENERGY 6
#define GDTK_GATE_NEWTON 7
#define GDTK_GATE_MAGNITUDE 8
#define GDTK_GATE_PREDICTED_ERROR 9
#define GDTK_GATE_COUNT 10

/* A network for reactor cr_i's gas model (its species and, for the element check, the species'
 * atomic constituents), parameters drawn from U(-1/sqrt(fan_in), 1/sqrt(fan_in)) with a
 * seeded generator.  Returns a handle, or -1. */
int chem_surrogate_new(int cr_i, int width, int depth, unsigned long long seed);
int chem_surrogate_free(int sg);
/* host dims[8]: nin, nin_pad, nout, nout_pad, width, depth, n_params, n_elements */
int chem_surrogate_dims(int sg, int* dims);
/* FP32 master parameters, host arrays of n_params floats, flat: W_0 .. W_depth (W_l row-major
 * [fan_out][fan_in]), then b_0 .. b_depth.  Setting them also resets the AdamW state. */
int chem_surrogate_get_params(int sg, float* params);
int chem_surrogate_set_params(int sg, const float* params);
/* Standardisation and training domain, host arrays: x_shift, x_scale, x_min, x_max (nin_pad),
 * y_shift, y_scale (nout_pad). */
int chem_surrogate_get_normalisation(int sg, float* x_shift, float* x_scale, float* y_shift, float* y_scale,
                                     double* x_min, double* x_max);
int chem_surrogate_set_normalisation(int sg, const float* x_shift, const float* x_scale, const float* y_shift,
                                     const float* y_scale, const double* x_min, const double* x_max);
/* Fits the standardisation (mean, standard deviation) and the domain (min, max) to the raw
 * samples rows[0..nrows) of X [.][nin_pad] and Y [.][nout_pad] (rows NULL: 0..nrows-1). */
int chem_surrogate_fit_normalisation(int sg, int nrows, const float* X, const float* Y, const int* rows,
                                     void* stream);
/* Loss weight of each raw output (host, nout floats; default 1). */
int chem_surrogate_set_loss_weights(int sg, const float* w);
/* Training samples from a batch that the FP64 update advanced by dt: raw features X[c] and
 * increments Y[c] for every cell (zeros where status[c] is not OK), valid[c] = 1 where it is. */
int chem_surrogate_make_samples(int sg, int ncell, const double* T0, const double* p0, const double* massf0,
                                double dt, const double* T1, const double* massf1, const int* status, float* X,
                                float* Y, int* valid, void* stream);
/* One AdamW step (beta 0.9, 0.999, eps 1e-8) on the mean weighted squared error of the
 * standardised outputs over rows[0..batch) of raw X, Y.  loss_sum (may be NULL) += the summed
 * weighted squared error of the batch. */
int chem_surrogate_train_step(int sg, int batch, const float* X, const float* Y, const int* rows, float lr,
                              float weight_decay, float* loss_sum, void* stream);
/* The gradient of that loss with respect to the parameters (grad: n_params floats, layout as
 * chem_surrogate_get_params), without an update. */
int chem_surrogate_gradients(int sg, int batch, const float* X, const float* Y, const int* rows, float* grad,
                             float* loss_sum, void* stream);
/* Raw predicted increments out[n][nout_pad] of raw features X[n][nin_pad]. */
int chem_surrogate_predict(int sg, int n, const float* X, float* out, void* stream);
/* Gate tolerances (defaults 1e-4, 1e-5, 1e-3, 5e-4). */
int chem_surrogate_set_gate(int sg, double elem_tol, double neg_tol, double T_tol, double max_dY);
/* The surrogate update with FP64 fallback.  Arguments as chem_reactor_update_cells; gate (may be
 * NULL) receives each cell's GDTK_GATE_* code; counts (host, may be NULL) receives
 * GDTK_GATE_COUNT + 2 values: cells per gate code, then the cells integrated by the fallback and
 * how many of those failed.  monitor_stride > 0 also integrates every accepted cell whose index
 * is a multiple of monitor_stride with the FP64 update and writes to monitor (host, 4 doubles):
 * cells judged, the largest |dY| of the surrogate against the FP64 update, the largest relative
 * dT, and the mean of the per-cell largest |dY|.  Synchronises the stream (the number of
 * rejected cells is read back to size the fallback). */
int chem_surrogate_update_cells(int sg, int ncell, const double* rho, const double* u, double* T, double* p,
                                double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                                int flags, void* stream, int* gate, long long* counts, int monitor_stride,
                                double* monitor);
/* Error model: a second network (same BF16 kernels) attached to the surrogate.  Its input is the
 * surrogate's standardised input and standardised output (nin_pad + nout_pad values), its output
 * an estimate of log10 of that output's error: the larger of its largest |dY| error and 0.1 times
 * its relative error in the temperature increment (so that 1e-3 in T weighs as 1e-4 in Y).  It is
 * trained on samples with a
 * pinball (quantile) loss, so with quantile 0.9 its estimate lies above the actual error for about
 * 90% of the samples it was trained on. */
int chem_surrogate_error_model_new(int sg, int width, int depth, unsigned long long seed);
/* host dims[5]: nin, nout_pad, width, depth, n_params */
int chem_surrogate_error_dims(int sg, int* dims);
int chem_surrogate_error_get_params(int sg, float* params);
int chem_surrogate_error_set_params(int sg, const float* params);
/* One AdamW step of the error network on rows[0..batch) of raw X, Y (the surrogate's own
 * parameters are not changed); loss_sum (may be NULL) += the summed pinball loss. */
int chem_surrogate_error_train_step(int sg, int batch, const float* X, const float* Y, const int* rows, float lr,
                                    float weight_decay, float quantile, float* loss_sum, void* stream);
/* The gradient of the error network's mean pinball loss (grad: its n_params floats), no update. */
int chem_surrogate_error_gradients(int sg, int batch, const float* X, const float* Y, const int* rows, float quantile,
                                   float* grad, float* loss_sum, void* stream);
/* The error network's estimate (log10 of the error defined above) for raw features X[n][nin_pad]. */
int chem_surrogate_predict_error(int sg, int n, const float* X, float* out, void* stream);
/* Reject cells whose estimated error exceeds tol (mass-fraction units); tol <= 0 turns it off. */
int chem_surrogate_set_error_gate(int sg, double tol);
/* The network's BF16 GEMM, exposed for testing: D[M][N] = op(A)[M][K] op(B)[K][N] (+ bias[N]),
 * act 0 none, 1 GELU (pre receives the pre-activation when not NULL); A, B are bf16 arrays;
 * D (fp32) and Dh (bf16) may each be NULL; splits > 1 splits K (no bias or act then). */
int gdtk_mlp_gemm(int M, int N, int K, const void* A, int lda, int trans_a, const void* B, int ldb, int trans_b,
                  const float* bias, int act, float* pre, float* D, void* Dh, int ldd, int splits, void* stream);
/* The tcgen05 form of that GEMM (the network's forward shapes: A [M][K] and B stored [N][K], K and N
 * multiples of 16 up to 256, no split): enable 1 uses it where it applies, 0 uses the mma.sync kernel
 * everywhere, -1 leaves the setting (initially off only with GDTK_MLP_TCGEN05=0 in the environment).
 * Returns the previous setting; *launches (if not NULL) receives the tcgen05 launches so far and *error
 * (if not NULL, synchronising) the kernel's error flag, then cleared: 0, or 1 / 2 when a wait for its
 * loads / its MMAs gave up. */
int gdtk_mlp_tcgen05(int enable, unsigned long long* launches, int* error);

#ifdef __cplusplus
}
#endif
#endif /* GDTK_SURROGATE_H */
