// twotemp.h -- the two-temperature reactor's tables and launch arguments (internal to the library).
//
// The gas is two_temperature_gas.d's: translation and rotation at T with fully excited heat capacities,
// vibration and electronic excitation at T_ve taken as the NASA-9 enthalpy at T_ve less the
// translational-rotational part; electrons carry their translation in the T_ve mode.  The reactor is
// multi_temperature_thermochemical_reactor.d's (RKF on concentrations and u_ve).  Energy exchange is
// energy_exchange_system.d's two-temperature form: Landau-Teller vibration-translation exchange with
// Millikan-White relaxation times (optionally with Park's high-temperature corrections), and Marrone-
// Treanor chemistry-vibration coupling with impartial dissociation.
#pragma once
#include <cuda_runtime.h>

namespace gdtk {

enum { EEM_LANDAU_TELLER = 0, EEM_MARRONE_TREANOR = 1 };
enum { RT_MILLIKAN_WHITE = 0, RT_PARK_HTC = 1, RT_PARK_HTC2 = 2 };
enum { CPL_IMPARTIAL = 0, CPL_MARRONE_TREANOR = 1, CPL_MODIFIED_MARRONE_TREANOR = 2 };

// One energy-exchange mechanism (energy_exchange_mechanism.d).
struct Eem2T {
    int kind;        // EEM_*
    int p;           // relaxing (or dissociating) species
    int q;           // colliding species (Landau-Teller)
    int rt;          // RT_* (Landau-Teller)
    int reaction;    // reaction index (Marrone-Treanor)
    int coupling;    // CPL_* (Marrone-Treanor)
    double a, b;     // Millikan-White constants (relaxation_time.d:27-60)
    double sigma;    // Park high-temperature cross section [m^2]
    double mu;       // reduced mass of the p-q pair [kg]
    double D, Thetav;   // dissociation energy [J/mol] (T_D [K] for the modified form), vibrational temperature
    double U;           // Marrone-Treanor U [K] (exchange_chemistry_coupling.d:133-175)
    double aU, Ustar, nb;   // modified Marrone-Treanor (:181-227)
};

// Per-species two-temperature constants (two_temperature_gas.d:45-80).
struct Species2T {
    double cp_tr;   // translation-rotation Cp [J/kg/K]: 5/2 R atoms, 7/2 R linear, 4 R non-linear, 0 electrons
    double h_f;     // CEA enthalpy at T_REF = 298.15 K [J/kg]
};

struct TwoTArgs {
    const int* mech_i;
    const double* mech_d;
    int n_mech_i, n_mech_d;
    const Species2T* species;
    const Eem2T* eem;
    int neem;
    int electron;   // index of e-, or -1
    double tol;     // RKF errTol (atol = rtol)
    int max_subcycles, max_attempts;
    int ncell;
    int pad;
    const double* rho;
    double* T;
    double* Tve;
    double* p;
    double* massf;     // [nsp][ncell]
    double* u;         // out (may be null): translation-rotation energy
    double* u_ve;      // out (may be null): vibration-electronic energy
    double* dt_chem;
    int* status;       // may be null
    double t_interval;
    unsigned long long* steps;   // optional: total RKF step attempts
    unsigned* counter;           // work counter of the persistent launch (zeroed by the launcher)
};

// p, T, T_ve, Y -> rho, u, u_ve (two_temperature_gas.d:84-92).
struct Thermo2TArgs {
    const int* mech_i;
    const double* mech_d;
    int n_mech_i, n_mech_d;
    const Species2T* species;
    int electron;
    int ncell;
    const double* p;
    const double* T;
    const double* Tve;
    const double* massf;
    double* rho;
    double* u;
    double* u_ve;
};

cudaError_t launch_two_temperature_update(const TwoTArgs& a, int sm_count, cudaStream_t s);
cudaError_t launch_two_temperature_thermo_pT(const Thermo2TArgs& a, int sm_count, cudaStream_t s);

}  // namespace gdtk
