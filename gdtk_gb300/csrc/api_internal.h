// api_internal.h -- what chem_api.cpp shares with the other translation units of the library
// (the allocation-free entry point and the surrogate).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "mechanism.h"

namespace gdtk {

void report_error(const std::string& msg);

struct ReactorInternals {
    int nsp = 0;
    const int* mech_i = nullptr;      // packed mechanism on the device (chem_types.h)
    const double* mech_d = nullptr;
    const GasModelHost* gm = nullptr;
    int sm_count = 0;
};
// Throws std::runtime_error for an invalid handle or without a GPU.
ReactorInternals reactor_internals(int cr_i);

// The plain FP64 update of chem_reactor_update_cells on device arrays (throws on error).
void reactor_update(int cr_i, int ncell, const double* rho, const double* u, double* T, double* p, double* massf,
                    double* dt_chem, int* status, double t_interval, double T_frozen, int flags, cudaStream_t s);

}  // namespace gdtk
