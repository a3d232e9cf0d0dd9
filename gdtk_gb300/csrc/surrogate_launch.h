// surrogate_launch.h -- host launchers of the surrogate's per-cell FP64 kernels (surrogate_kernels.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gdtk {

constexpr int SURR_MAX_ELEMENTS = 8;

enum GateCode {
    GATE_ACCEPTED = 0,
    GATE_FROZEN = 1,
    GATE_BAD_INPUT = 2,
    GATE_DOMAIN = 3,
    GATE_ELEMENTS = 4,
    GATE_NEGATIVE = 5,
    GATE_ENERGY = 6,
    GATE_NEWTON = 7,
    GATE_MAGNITUDE = 8,
    GATE_PREDICTED_ERROR = 9,
    GATE_COUNT = 10
};

// Raw features of a cell: ln T, ln p, Y[0..nsp), ln dt, zero padding to nin_pad.
// Raw targets: dY[0..nsp), dT, zero padding to nout_pad.
struct SampleArgs {
    int ncell, nsp, nin_pad, nout_pad;
    double dt;
    const double *T0, *p0, *massf0, *T1, *massf1;
    const int* status;
    float *X, *Y;
    int* valid;
};
cudaError_t launch_make_samples(const SampleArgs& a, cudaStream_t s);

// Per-column mean / standard deviation / min / max over rows (double accumulation, fixed order).
cudaError_t launch_column_stats(int nrows, int ncol, const float* X, const int* rows, double* partial, int npartial,
                                double* out /* [4][ncol]: mean, std, min, max */, cudaStream_t s);

// Standardised bf16 features of cells [first, first + n) and their domain/frozen/bad-input codes.
struct FeatureArgs {
    int n, first, ncell, nsp, nin_pad;
    double dt, T_frozen;
    const double *rho, *T, *p, *massf;
    const float *x_shift, *x_scale;
    const double *x_min, *x_max;
    __nv_bfloat16* Xh;   // [n][nin_pad]
    int* gate;           // [ncell]
};
cudaError_t launch_features(const FeatureArgs& a, cudaStream_t s);

// The FP64 gate of the predicted increments of cells [first, first + n).
struct GateArgs {
    int n, first, ncell, nsp, nout_pad, ne;
    int update_thermo;
    const int* mech_i;
    const double* mech_d;
    const double* elem;      // [ne][nsp]: atoms of element e in species s per kg of species (1 / M_s units)
    const double* elem_M;    // [ne] element molar masses
    const float *y_shift, *y_scale;
    const float* out;        // [n][nout_pad] standardised network outputs
    double elem_tol, neg_tol, T_tol, max_dY;
    const double *rho, *u;
    double *T, *p, *massf;
    int* status;
    int* gate;               // [ncell], in: feature codes, out: final codes
    int* reject;             // [ncell] list of rejected cell indices
    int* counters;           // [0] rejected, [1] monitored
    unsigned long long* code_counts;   // [GATE_COUNT]
    int monitor_stride, monitor_cap;
    int* mon_idx;            // [monitor_cap]
    double* mon_state;       // [(5 + nsp) * monitor_cap]: rho, u, T, p, dt_chem, Y (original)
    const double* dt_chem;
    const float* pred_err;   // [n][pred_err_ld] error network output (log10 |dY| error) or null
    int pred_err_ld;
    double err_log10_tol;
};
cudaError_t launch_gate(const GateArgs& a, cudaStream_t s);

// Rejected cells <-> compact SoA buffers [rho, u, T, p, dt_chem, massf(nsp)] of n cells.
cudaError_t launch_gather_cells(int n, const int* idx, int ncell, int nsp, const double* rho, const double* u,
                                const double* T, const double* p, const double* dt_chem, const double* massf,
                                double* compact, cudaStream_t s);
cudaError_t launch_scatter_cells(int n, const int* idx, int ncell, int nsp, const double* compact,
                                 const int* cstatus, double* T, double* p, double* dt_chem, double* massf,
                                 int* status, int* fail_count, cudaStream_t s);
// Surrogate results of monitored cells against their FP64 update (compact buffer, status):
// res[0] = cells compared, res[1] = max |dY| (bits), res[2] = max relative dT (bits), res[3] = sum of max|dY| (bits of a double, atomically added)
cudaError_t launch_monitor_compare(int n, const int* idx, int ncell, int nsp, const double* compact,
                                   const int* cstatus, const double* T, const double* massf,
                                   unsigned long long* res, double* sum, cudaStream_t s);

cudaError_t launch_repack(int n, int cap, int nk, const double* src, double* dst, cudaStream_t s);

}  // namespace gdtk
