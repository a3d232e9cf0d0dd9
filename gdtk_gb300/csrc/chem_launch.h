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
// species and reactions over the lanes.  Its tables (built by the host from the packed mechanism):
//   ints [0, n_smem_ints), staged in shared memory by every block:
//     [off_tstart + ir]  first concentration term of reaction ir (nr + 1 entries)
//     [off_tmid + ir]    first product term of reaction ir
//     [off_terms + k]    term k: species | coeff << 8; reactants, then products, each in the reaction's order
//     [off_rxeff + ir]   efficiency list of reaction ir's third body, or -1
//     [off_slot + j]     scaled tick-rate slot j: reaction | |nu| << 16, for each (reaction, |nu| >= 2) pair
//     [off_lane + l]     first gather entry of lane l (33 entries)
//     [off_ent + k]      gather entry: species | index << 8 | (1 for L) << 21, adding element `index` of
//                        the warp's w_f[nr], w_b[nr], |nu| w_f[nslot], |nu| w_b[nslot] (end to end) to q or
//                        L of the species.  The tasks (one species' q, or its L) are dealt whole to the
//                        lanes, longest first; a task's entries are in ascending reaction order
//   ints [off_efflen, ...) and doubles, read from global memory:
//     [off_efflen + s]            length of efficiency list s
//     [off_effidx + k*neff + s]   species of the k-th entry of list s (transposed: lanes read one list each)
//     eff_val[k*neff + s]         its efficiency
struct WarpTables {
    const int* gi;
    const double* eff_val;
    int n_smem_ints, nslot;
    int off_tstart, off_tmid, off_terms, off_rxeff, off_slot, off_lane, off_ent, off_efflen, off_effidx;
};
// Shared-memory doubles of one warp's vectors.
int chem_warp_doubles(int nsp, int nr, int neff, int method, int nslot);
cudaError_t launch_chem_update_warp(const ChemUpdateArgs& a, int method, const WarpTables& t, int warp_doubles,
                                    int sm_count, cudaStream_t stream, LaunchInfo* info);
// Cost buckets of the longest-first ordering: launch_bucket_order's hist scratch holds this many ints.
constexpr int ORDER_BUCKETS = 256;

// Counting sort of n cells by cost key (descending) into order[n]; hist is ORDER_BUCKETS ints of scratch.
cudaError_t launch_bucket_order(const float* key, int n, int* order, int* hist, int sm_count, cudaStream_t stream);

}  // namespace gdtk
