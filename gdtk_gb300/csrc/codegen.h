// codegen.h -- mechanism-specialised kernels: source generation, NVRTC compilation, launch.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "mechanism.h"

namespace gdtk {

// Host mirrors of gdtk_fast::CellBlock / FastArgs (chem_fast.cuh); the layouts must agree.
enum { FAST_MAX_BLOCKS = 128 };

struct CellBlock {
    int ncell;
    int first;
    double t_interval;
    const double* rho;
    const double* u;
    double* T;
    double* p;
    double* massf;
    double* dt_chem;
    int* status;
};

struct FastArgs {
    const double* thermo;
    const double* exp_table;
    int nblocks;
    int total;
    int flags;
    int refill_chunk;   // visit positions a warp reserves per atomic (<= 1: exactly the lanes that need a cell)
    double T_frozen;
    unsigned* counter;
    int* cell_counters;
    unsigned long long* totals;
    const int* order;
    unsigned long long* lane_stats;
    CellBlock blocks[FAST_MAX_BLOCKS];
};

struct FastKernel {
    void* module = nullptr;     // CUmodule
    void* function = nullptr;   // CUfunction
    void* cost_function = nullptr;   // CUfunction of the cost pre-pass
    int block = 0;              // threads per block the kernel was compiled for
    int min_blocks = 1;
    int per_thread_doubles = 0;
    int table_doubles = 0;
    int blocks_per_sm = 0;      // occupancy at full block size
    double* d_thermo = nullptr;
    double* d_exp = nullptr;
    std::string log;            // NVRTC/ptxas log
    std::string source;
    ~FastKernel();
};

// Thermo table of chem_fast.cuh (120 doubles per species).
std::vector<double> fast_thermo_table(const GasModelHost& gm);
// CUDA source of the generated prologue + kernel for one mechanism.
std::string generate_fast_source(const GasModelHost& gm, const MechanismHost& mh, int block, int min_blocks);
// Compiles the generated source for compute capability major.minor without loading it
// (no GPU needed); returns the NVRTC/ptxas log, throws on a compilation error.
std::string compile_fast_check(const GasModelHost& gm, const MechanismHost& mh, int major, int minor);
// Compiles (or fetches from the in-process / on-disk cache) and loads the fast kernel.
// block/min_blocks <= 0: chosen from the shared-memory budget.
FastKernel* build_fast_kernel(const GasModelHost& gm, const MechanismHost& mh, int block = 0, int min_blocks = 0);
// Launches it; `info` receives the launch shape.
cudaError_t launch_fast(FastKernel& k, FastArgs& a, int sm_count, cudaStream_t stream, int* grid_out, int* block_out,
                        int* smem_out);
// Longest-first visit order: cost pre-pass into key[total], then a bucket sort into order[total]
// (hist: 257 ints of scratch).  All on `stream`.
cudaError_t launch_order(FastKernel& k, FastArgs& a, int sm_count, float* key, int* order, int* hist,
                         cudaStream_t stream);

}  // namespace gdtk
