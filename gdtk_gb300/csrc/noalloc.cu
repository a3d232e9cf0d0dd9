// noalloc.cu -- the chemistry update for callers that cannot allocate device memory.
//
// chem_reactor_update_cells sizes its per-call scratch (the persistent kernel's work counter
// and the longest-first ordering buffers: one cost key and one visit-order slot per cell) on
// first use with cudaMalloc.  Some callers cannot do that where they run the chemistry:
// code recorded into a CUDA graph (cudaMalloc is not allowed during stream capture), solvers
// that run with a fixed, pre-reserved device-memory budget, and host threads that must not
// take cudaMalloc's device-wide synchronisation in the middle of a time step.  This entry
// point runs the same kernels with that scratch taken from one static device array instead.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/gdtk_chem.h"
#include "chem_launch.h"

namespace gdtk {
int update_cells_with_scratch(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p,
                              double* massf, double* dt_chem, int* status, double t_interval, double T_frozen,
                              int flags, void* stream, unsigned* counter, float* key, int* order, int* hist);
void report_error(const std::string& msg);
}  // namespace gdtk

namespace {

constexpr int kMaxCells = 1 << 20;                 // cells per call
constexpr size_t kCounterBytes = 256;              // work counter (padded to the alignment)
constexpr size_t kHistBytes = gdtk::ORDER_BUCKETS * sizeof(int);   // ordering histogram
static_assert(kHistBytes % 16 == 0, "the key array after the histogram stays 16-byte aligned");
constexpr size_t kScratchBytes = kCounterBytes + kHistBytes + (size_t)kMaxCells * (sizeof(float) + sizeof(int));

// About 8 MiB, held by every GPU on which this library's device code is loaded, until exit.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device (the host-side symbol is not a device address).
std::mutex g_mu;
constexpr int kMaxDevices = 128;
void* g_addr[kMaxDevices] = {};

}  // namespace

extern "C" int chem_reactor_update_cells_noalloc(int cr_i, int ncell, const double* rho, const double* u, double* T,
                                                 double* p, double* massf, double* dt_chem, int* status,
                                                 double t_interval, double T_frozen, int flags, void* stream) {
    if (ncell > kMaxCells) {
        gdtk::report_error("chem_reactor_update_cells_noalloc: " + std::to_string(ncell) +
                           " cells exceed its static scratch of " + std::to_string(kMaxCells) +
                           " cells; split the batch or use chem_reactor_update_cells");
        return -1;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        gdtk::report_error(std::string("chem_reactor_update_cells_noalloc: no usable CUDA device (") +
                           cudaGetErrorString(e) + ")");
        return -1;
    }
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {   // once per device, with that device current
            e = cudaGetSymbolAddress(&g_addr[dev], g_scratch);
            if (e != cudaSuccess) {
                g_addr[dev] = nullptr;
                gdtk::report_error(std::string("chem_reactor_update_cells_noalloc: cudaGetSymbolAddress failed: ") +
                                   cudaGetErrorString(e));
                return -1;
            }
        }
        base = g_addr[dev];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    unsigned* counter = reinterpret_cast<unsigned*>(b);
    int* hist = reinterpret_cast<int*>(b + kCounterBytes);
    float* key = reinterpret_cast<float*>(b + kCounterBytes + kHistBytes);
    int* order = reinterpret_cast<int*>(b + kCounterBytes + kHistBytes + (size_t)kMaxCells * sizeof(float));
    return gdtk::update_cells_with_scratch(cr_i, ncell, rho, u, T, p, massf, dt_chem, status, t_interval, T_frozen,
                                           flags, stream, counter, key, order, hist);
}
