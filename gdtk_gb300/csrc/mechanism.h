// mechanism.h -- host-side gas model and reaction mechanism, read from prep-gas / prep-chem files
// and packed into the device layout of chem_types.h.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "chem_types.h"
#include "chem_types.h"
#include "lua_table.h"

namespace gdtk {

struct CeaCurveHost {
    int nseg = 0;
    std::vector<double> breaks, blends, coeffs;   // coeffs: nseg * 9
};

// The thermally-perfect gas model (gas/composite_gas.d:37-120 with physical_model
// 'thermally-perfect-gas', or the legacy 'ThermallyPerfectGas' file format).
struct GasModelHost {
    std::string type_str;
    std::vector<std::string> names;
    std::vector<double> M;
    std::vector<CeaCurveHost> curves;
    std::vector<std::string> elements;                    // in order of first appearance
    std::vector<std::map<std::string, int>> composition;  // per species: element -> atoms
    // two-temperature gas (gas/thermo/two_temperature_gas.d): particle kind per species
    bool two_temperature = false;
    std::vector<int> particle;   // PARTICLE_ATOM, PARTICLE_LINEAR, PARTICLE_NONLINEAR or PARTICLE_ELECTRON
    int n_species() const { return (int)names.size(); }
};

enum { PARTICLE_ATOM = 0, PARTICLE_LINEAR = 1, PARTICLE_NONLINEAR = 2, PARTICLE_ELECTRON = 3 };

struct RateConstHost {
    int model = 0;   // RATE_* (chem_types.h)
    double A = 0, n = 0, C = 0;            // Arrhenius; k_inf for the pressure-dependent models;
                                           // logA, B, C for Arrhenius2 (k = exp(logA + B T - C/T))
    double A0 = 0, n0 = 0, C0 = 0;         // k_0 of the pressure-dependent models
    double Fcent = 0, a = 0, T1 = 0, T2 = 0, T3 = 0;   // Troe (a, T1, T2 hold a, b, c for Yungster-Rabinowitz)
    int troe_flags = 0;                    // TROE_FCENT | TROE_T1 | TROE_T2: parameters given
    double s = 0;                          // Park: exponent of T in the rate-controlling temperature
    int base = 0;                          // (modified) Marrone-Treanor: model of the underlying rate in A, n, C, s
    double TD = 0, U = 0, theta = 0, aU = 0, Ustar = 0, nb = 1;   // their parameters (nb: non-Boltzmann factor)
    bool pressure_dependent() const { return model == RATE_LH || model == RATE_TROE || model == RATE_YR; }
    bool simple() const { return model == RATE_ARRHENIUS || model == RATE_ARRHENIUS2; }   // no third body
};

struct ReactionHost {
    bool collider = false;
    RateConstHost frc, brc;
    std::vector<std::pair<int, int>> reac, prod;
    std::vector<std::pair<int, double>> eff;   // in Lua traversal order (ascending species index)
    std::string equation;
};

struct MechanismHost {
    std::vector<ReactionHost> reactions;
    // config table (kinetics/prep_chem.lua:49-91 defaults, chemistry_update.d:75-135 consumer)
    double T_lower = 300.0, T_upper = 50000.0;
    int method = 0;
    double errTol = 1e-3, eps1 = 1e-3, eps2 = 5e-4, delta = 1e-10;
    int maxIters = 10;
    bool tight = false;
    int maxSubcycles = 10000, maxAttempts = 4;
};

struct PackedMech {
    std::vector<int> I;
    std::vector<double> D;
    int nsp = 0, nr = 0, neff = 0, method = 0;
};

// A thermally perfect gas; with allow_two_temperature also a two-temperature gas (two_temperature = true).
GasModelHost load_gas_model(const std::string& path, bool allow_two_temperature = false);
// reads `reaction` (and `config` when with_config) of a prep-chem file; checks species order.
MechanismHost load_mechanism(const std::string& path, const GasModelHost& gm, bool with_config);
PackedMech pack(const GasModelHost& gm, const MechanismHost* mech);
// Reference-algorithm FP64 operation counts (see chem_reactor_flop_model in gdtk_chem.h).
void flop_model(const GasModelHost& gm, const MechanismHost& mh, double out[5]);

}  // namespace gdtk
