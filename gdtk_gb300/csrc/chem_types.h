// chem_types.h -- packed, device-resident description of a gas model + reaction mechanism.
//
// The host (mechanism.cpp) flattens the prep-gas / prep-chem files into two arrays, one of
// ints and one of doubles, with the layout below.  Kernels copy both into shared memory once
// per block and read them through MechView.  All offsets depend only on nsp, nr and neff.
//
// int array
//   [0..HI)            header: nsp, nr, neff, method, maxIters, tight, maxSubcycles, maxAttempts
//   [HI + isp]         nseg of species isp                                 (nsp ints)
//   [RX + 40*ir + k]   reaction ir: collider, frc_model, brc_model, eff_set, nreac, nprod, npart, frc_base,
//                      reac_idx[4], reac_coeff[4], prod_idx[4], prod_coeff[4], part[8], part_nu[8]
//   [EF + (1+nsp)*s]   efficiency set s: n, idx[nsp]
// double array
//   [0..HD)            header: T_lower, T_upper, errTol, eps1, eps2, delta, -, -
//   [SP + 56*isp + k]  species isp: M, R, T_low, T_high, Cp_low, Cp_high, h_low, h_high, s_low, s_high,
//                      breaks[5], blends[4], -, coeffs[4][9]
//   [RD + 16*ir]       reaction ir: fA, fn, fC, bA, bn, bC (kInf in fA..fC for the pressure-dependent
//                      models; logA, B, C for Arrhenius2), k0 A, n, C, Troe F_cent, a, T1, T2, T3 (or
//                      Yungster-Rabinowitz a, b, c in
//                      the a, T1, T2 slots), Troe flags (1 F_cent given, 2 T1 given, 4 T2 given), Park s;
//                      a (modified) Marrone-Treanor forward rate keeps its underlying Arrhenius or Park
//                      rate (model in frc_base) in A, n, C and s, and T_D, U (aU), theta, U*, the
//                      non-Boltzmann factor in the k_0 / Troe slots
//   [ED + nsp*s]       efficiency set s: values[nsp]
#pragma once

#define GDTK_MAX_SPECIES 32        // thread-per-cell kernels (fast, reference-order, surrogate, 2-T)
#define GDTK_MAX_REACTIONS 128
#define GDTK_MAX_SPECIES_ANY 128   // the reader; beyond GDTK_MAX_SPECIES / _REACTIONS the update runs one
#define GDTK_MAX_REACTIONS_ANY 1024   // warp per cell
#define GDTK_MAX_SEGMENTS 4
#define GDTK_MAX_EFFSETS 128
#define GDTK_MAX_TERMS 4
#define GDTK_MAX_PARTICIPANTS 8

#ifdef __CUDACC__
#define GDTK_HD __host__ __device__ __forceinline__
#else
#define GDTK_HD inline
#endif

namespace gdtk {

enum { HI = 8, RXI = 40, HD = 8, SPD = 56, RXD = 16 };

// species double-record fields
enum { SP_M = 0, SP_R, SP_TLOW, SP_THIGH, SP_CPLOW, SP_CPHIGH, SP_HLOW, SP_HHIGH, SP_SLOW, SP_SHIGH,
       SP_BREAKS = 10, SP_BLENDS = 15, SP_COEFFS = 20 };
// reaction int-record fields
enum { RX_COLLIDER = 0, RX_FRC, RX_BRC, RX_EFFSET, RX_NREAC, RX_NPROD, RX_NPART, RX_BASE,
       RX_REAC_IDX = 8, RX_REAC_COEFF = 12, RX_PROD_IDX = 16, RX_PROD_COEFF = 20, RX_PART = 24, RX_PART_NU = 32 };
// rate-constant models (kinetics/rate_constant.d): Arrhenius 52-80, from K_c, the pressure-dependent
// Lindemann-Hinshelwood 123-160, Troe 162-290, Yungster-Rabinowitz 292-355 (third-body concentration of
// the reaction's efficiency list, 114-121), and Arrhenius2 / Arrhenius-logA 82-121,
// k = exp(logA + B T - C/T), whose (logA, B, C) take the places of (A, n, C)
enum { RATE_ARRHENIUS = 0, RATE_FROM_EQ = 1, RATE_LH = 2, RATE_TROE = 3, RATE_YR = 4, RATE_ARRHENIUS2 = 5,
       RATE_PARK = 6,   // Park 2-T (rate_constant.d:364-393): A, n, C with T_eff = T^s T_ve^(1-s), s in RD_S
       RATE_MT = 7,     // Marrone-Treanor (rate_constant.d:395-452) over an Arrhenius or Park rate
       RATE_MMT = 8 };  // modified Marrone-Treanor (rate_constant.d:454-566)
// reaction double-record fields beyond the six Arrhenius parameters
enum { RD_K0A = 6, RD_K0N, RD_K0C, RD_FCENT, RD_TA, RD_T1, RD_T2, RD_T3, RD_TFLAGS, RD_S };
enum { RD_MT_TD = 6, RD_MT_U, RD_MT_THETA, RD_MT_USTAR, RD_MT_NB };   // U holds aU for the modified form
enum { TROE_FCENT = 1, TROE_T1 = 2, TROE_T2 = 4 };
enum { METHOD_RKF = 0, METHOD_ALPHA_QSS = 1 };

GDTK_HD int mech_n_ints(int nsp, int nr, int neff) { return HI + nsp + RXI * nr + (1 + nsp) * neff; }
GDTK_HD int mech_n_doubles(int nsp, int nr, int neff) { return HD + SPD * nsp + RXD * nr + nsp * neff; }

struct MechView {
    const int* I;
    const double* D;
    int nsp, nr, neff;
    GDTK_HD void bind(const int* i, const double* d) {
        I = i; D = d; nsp = i[0]; nr = i[1]; neff = i[2];
    }
    GDTK_HD int method() const { return I[3]; }
    GDTK_HD int max_iters() const { return I[4]; }
    GDTK_HD bool tight() const { return I[5] != 0; }
    GDTK_HD int max_subcycles() const { return I[6]; }
    GDTK_HD int max_attempts() const { return I[7]; }
    GDTK_HD double T_lower() const { return D[0]; }
    GDTK_HD double T_upper() const { return D[1]; }
    GDTK_HD double err_tol() const { return D[2]; }
    GDTK_HD double eps1() const { return D[3]; }
    GDTK_HD double eps2() const { return D[4]; }
    GDTK_HD double delta() const { return D[5]; }
    GDTK_HD int nseg(int isp) const { return I[HI + isp]; }
    GDTK_HD const double* sp(int isp) const { return D + HD + SPD * isp; }
    GDTK_HD const int* rx(int ir) const { return I + HI + nsp + RXI * ir; }
    GDTK_HD const double* rxd(int ir) const { return D + HD + SPD * nsp + RXD * ir; }
    GDTK_HD const int* eff_i(int s) const { return I + HI + nsp + RXI * nr + (1 + nsp) * s; }
    GDTK_HD const double* eff_d(int s) const { return D + HD + SPD * nsp + RXD * nr + nsp * s; }
};

// Per-cell status codes (shared with include/gdtk_chem.h).
enum CellStatus {
    CELL_OK = 0,
    CELL_H_MIN = 1,          // "Hit the minimum allowable timestep" (chemistry_update.d:233-238)
    CELL_MAX_ATTEMPTS = 2,   // chemistry_update.d:241-247
    CELL_MAX_SUBCYCLES = 3,  // chemistry_update.d:281-289
    CELL_NEWTON_FAIL = 4,    // therm_perf_gas_mix.d:458-466
    CELL_BAD_INPUT = 5,      // gas_model.d:246-248 (invalid density)
    CELL_FROZEN = 6,         // T <= T_frozen: skipped (fluidfvcell.d:887)
    CELL_CEA_RANGE = 7       // cea_thermo_curves.d:178-181
};

}  // namespace gdtk
