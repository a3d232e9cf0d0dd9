// chem_launch.h -- kernel argument blocks and launchers (internal to the library).
#pragma once
#include <cuda_runtime.h>

namespace gdtk {

enum { CHEM_FLAG_UPDATE_THERMO = 1, CHEM_FLAG_RETRY = 2, CHEM_FLAG_REFERENCE_ORDER = 4 };

// All pointers are device pointers.  Mass fractions are species-major: massf[isp * ncell + cell].
struct ChemUpdateArgs {
    const int* mech_i;
    const double* mech_d;
    int n_mech_i, n_mech_d;
    int ncell;
    const double* rho;
    const double* u;
    double* T;
    double* p;
    double* massf;
    double* dt_chem;
    int* status;              // may be null
    double t_interval;
    double T_frozen;
    int flags;
    unsigned* counter;        // work counter, zero at launch
    int* cell_counters;       // optional [6][ncell]: step attempts, rhs, rate-constant evals, Newton
                              // iterations, rejected attempts, initial step-size estimates
    unsigned long long* totals;   // optional [6], same quantities summed
};

struct GasServiceArgs {
    const int* mech_i;
    const double* mech_d;
    int n_mech_i, n_mech_d;
    int nsp_hint, nr_hint, neff_hint;
    int ncell;
    int mode;
    int clip;
    double* rho;
    double* u;
    double* T;
    double* p;
    const double* massf;
    double* out1;
    double* out2;
    int* status;
    double* gscratch;   // set by the launcher when a thread's vectors do not fit in shared memory
};

struct LaunchInfo {
    int grid, block, smem, blocks_per_sm;
};

int chem_scratch_doubles(int nsp, int nr, int neff, int method);
cudaError_t launch_chem_update(const ChemUpdateArgs& a, int method, int scratch_doubles, int sm_count,
                               cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_gas_service(const GasServiceArgs& a, int sm_count, cudaStream_t stream);
// One warp per cell (mechanisms too large for the thread-per-cell kernels): the reference-order update with
// species and reactions over the lanes.  csr_*: each species' (reaction, net coefficient) entries in
// reaction order; warp_doubles = chem_warp_doubles(...), the shared-memory doubles of one warp.
int chem_warp_doubles(int nsp, int nr, int neff, int method);
cudaError_t launch_chem_update_warp(const ChemUpdateArgs& a, int method, const int* csr_start, const int* csr_rx,
                                    const int* csr_nu, int warp_doubles, int sm_count, cudaStream_t stream,
                                    LaunchInfo* info);
// Cost buckets of the longest-first ordering: launch_bucket_order's hist scratch holds this many ints.
constexpr int ORDER_BUCKETS = 256;

// Counting sort of n cells by cost key (descending) into order[n]; hist is ORDER_BUCKETS ints of scratch.
cudaError_t launch_bucket_order(const float* key, int n, int* order, int* hist, int sm_count, cudaStream_t stream);

}  // namespace gdtk
