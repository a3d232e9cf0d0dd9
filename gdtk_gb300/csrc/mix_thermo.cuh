// mix_thermo.cuh -- mixture thermo of the thermally perfect gas on packed species records
// (chem_types.h), shared by the reference-order kernels and the surrogate gate.
//
//   therm_perf_gas_mix.d:406-413  internal energy      therm_perf_gas_mix.d:416-423  Cv
//   gas_model.d:410-418           mixture gas constant therm_perf_gas_mix.d:426-468  T from (rho, u)
#pragma once
#include "cea_thermo.h"
#include "chem_types.h"

namespace gdtk {
namespace {

// Per-thread vector in shared memory: element k of this thread lives at b[k * s].
struct Vec {
    double* b;
    int s;
    __device__ __forceinline__ double& operator[](int k) const { return b[k * s]; }
    __device__ __forceinline__ Vec operator+(int k) const { return Vec{b + k * s, s}; }
};

// therm_perf_gas_mix.d:406-413
__device__ double internal_energy(const MechView& m, Vec mf, double T, double logT, int& err) {
    double u = 0.0;
    for (int i = 0; i < m.nsp; ++i) u += mf[i] * (cea_h(m, i, T, logT, err) - m.sp(i)[SP_R] * T);
    return u;
}

// therm_perf_gas_mix.d:416-423
__device__ double cv_mix(const MechView& m, Vec mf, double T, int& err) {
    double c = 0.0;
    for (int i = 0; i < m.nsp; ++i) c += mf[i] * (cea_Cp(m, i, T, err) - m.sp(i)[SP_R]);
    return c;
}

__device__ double gas_constant(const MechView& m, Vec mf) {   // mass_average(Q, mR), gas_model.d:410-418
    double r = 0.0;
    for (int i = 0; i < m.nsp; ++i) r += mf[i] * m.sp(i)[SP_R];
    return r;
}

// therm_perf_gas_mix.d:426-468.  Returns T; sets err on failure.  *iters counts Newton iterations.
__device__ double T_from_u(const MechView& m, Vec mf, double u_tgt, double T_guess, int& err, int& iters) {
    const double TOL = 1e-10;
    double T = T_guess;
    double f = internal_energy(m, mf, T, log(T), err) - u_tgt;
    double dT = 0.0;
    for (int iter = 0; iter < 10; ++iter) {
        ++iters;
        double cv = cv_mix(m, mf, T, err);
        dT = -f / cv;
        T += dT;
        if (fabs(dT) / T < TOL) return T;
        f = internal_energy(m, mf, T, log(T), err) - u_tgt;
    }
    if (fabs(dT) > 1e-3) err = CELL_NEWTON_FAIL;
    return T;
}

}  // namespace
}  // namespace gdtk
