// chem_oracle.cpp -- CPU restatement of Eilmer's operator-split chemistry update.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA product path is
// checked against, and the CPU baseline that bench.py times beside it.  Nothing in the
// product (gdtk_gb300/) links, loads or calls it.
//
// It restates, operation for operation and in the reference's evaluation order, the D code
// of gdtk (paths relative to the gdtk source tree):
//   src/kinetics/chemistry_update.d      ChemistryUpdate.opCall 139-326, RKFStep 404-478,
//                                        AlphaQssStep 533-655, constants 23-31
//   src/kinetics/reaction_mechanism.d    eval_rate_constants 49-63, eval_split_rates 82-96,
//                                        estimateStepSize 161-203, Gibbs at P_atm 204-218
//   src/kinetics/reaction.d              compute_equilibrium_constant 26-52,
//                                        Reaction.eval_rate_constants 94-143,
//                                        Elementary 267-311, AnonymousCollider 393-456
//   src/kinetics/rate_constant.d         ArrheniusRateConstant.eval 72-75
//   src/gas/thermo/cea_thermo_curves.d   eval_Cp/eval_h/eval_s 55-137, determineCoefficients 149-182
//   src/gas/thermo/therm_perf_gas_mix.d  GibbsFreeEnergies 354-364, update_pressure 379-383,
//                                        update_density 386-390, internal_energy 406-413,
//                                        constant_volume_specific_heat 416-423,
//                                        update_temperature_from_energy 426-468
//   src/kinetics/rate_constant.d        Arrhenius 72-75, third-body concentration 114-121,
//                                        Lindemann-Hinshelwood 155-160, Troe 258-287,
//                                        Yungster-Rabinowitz 338-350
//   src/gas/gas_model.d                  massf2conc 237-253, conc2massf 255-271, mass_average 410-418
//   src/gas/physical_constants.d         R_universal, P_atm 13-16
//   src/lmr/fluidfvcell.d                thermochemical_increment 883-997 (caller contract:
//                                        T_frozen skip, one retry with dt_chem = -1, rhou update)
//
// Arithmetic differences from the reference that cannot be removed on this machine:
//   * exp/log/pow/sqrt are the C library's (the D runtime's are of the same accuracy class);
//   * integer powers pow(c, k) use double-precision binary exponentiation, whereas the D
//     runtime accumulates them in 80-bit `real` on x86;
//   * sum(Q.massf) follows Phobos' pairwise summation order (std.algorithm.sum).
// These are ulp-level effects; parity with the reference is asserted to tolerance.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <array>
#include <atomic>
#ifdef _OPENMP
#include <omp.h>
#endif


// Work-array sizes: the reader takes mechanisms up to these.
constexpr int ORACLE_MAX_SPECIES = 128;
constexpr int ORACLE_MAX_REACTIONS = 1024;
namespace {

constexpr double R_universal = 8.31451;      // physical_constants.d:13
constexpr double P_atm = 101.325e3;          // physical_constants.d:16
constexpr double MIN_MOLES = 1.0e-30;        // gas_model.d:43
constexpr double MIN_MASS_FRACTION = 1.0e-30;// gas_model.d:42
// chemistry_update.d:23-31
constexpr double DT_INCREASE_PERCENT = 10.0;
constexpr double DT_REDUCTION_FACTOR = 10.0;
constexpr double H_MIN = 1.0e-15;
constexpr double ALLOWABLE_MASSF_ERROR = 1.0e-3;

enum Status : int {
    ST_OK = 0, ST_H_MIN = 1, ST_MAX_ATTEMPTS = 2, ST_MAX_SUBCYCLES = 3,
    ST_NEWTON_FAIL = 4, ST_BAD_INPUT = 5, ST_FROZEN = 6, ST_CEA_RANGE = 7
};

struct Failure { int code; };

struct CEACurve {
    double R = 0;
    std::vector<double> breaks, blends;
    std::vector<std::array<double, 9>> coeffs;
    double T_low, T_high, Cp_low, Cp_high, h_low, h_high, s_low, s_high;

    // cea_thermo_curves.d:150-182
    void determine(double T, double a[9]) const {
        size_t nb = breaks.size();
        if (T < (breaks[1] - 0.5 * blends[0])) { std::memcpy(a, coeffs[0].data(), 9 * sizeof(double)); return; }
        if (T > (breaks[nb - 2] + 0.5 * blends[blends.size() - 1])) {
            std::memcpy(a, coeffs.back().data(), 9 * sizeof(double)); return;
        }
        for (size_t i = 1; i < nb - 1; ++i) {
            double T_blend_low = breaks[i] - 0.5 * blends[i - 1];
            double T_blend_high = breaks[i] + 0.5 * blends[i - 1];
            if (T >= T_blend_low && T <= T_blend_high) {
                double wB = (1. / blends[i - 1]) * (T - T_blend_low);
                double wA = 1.0 - wB;
                for (int j = 0; j < 9; ++j) a[j] = wA * coeffs[i - 1][j] + wB * coeffs[i][j];
                return;
            }
            // The reference reads _T_blends[i] here; for the last interior break that index is
            // past the end, but T cannot reach this test there (caught by the extremity test).
            if (T > T_blend_high && i < blends.size() && T < (breaks[i + 1] - 0.5 * blends[i])) {
                std::memcpy(a, coeffs[i].data(), 9 * sizeof(double)); return;
            }
        }
        throw Failure{ST_CEA_RANGE};
    }
    // cea_thermo_curves.d:56-73
    double eval_Cp(double T) const {
        if (T < T_low) return Cp_low;
        if (T > T_high) return Cp_high;
        double a[9]; determine(T, a);
        double Cp_on_R = a[0] / (T * T) + a[1] / T + a[2] + a[3] * T;
        Cp_on_R += a[4] * T * T + a[5] * T * T * T + a[6] * T * T * T * T;
        return R * Cp_on_R;
    }
    // cea_thermo_curves.d:81-108
    double eval_h(double T, double logT) const {
        if (T < T_low) return h_low - Cp_low * (T_low - T);
        if (T > T_high) return h_high + Cp_high * (T - T_high);
        double a[9]; determine(T, a);
        double h_on_RT = -a[0] / T + a[1] * logT + a[2] * T + a[3] * T * T / 2.0;
        h_on_RT += a[4] * T * T * T / 3.0 + a[5] * T * T * T * T / 4.0 + a[6] * T * T * T * T * T / 5.0 + a[7];
        return R * h_on_RT;
    }
    // cea_thermo_curves.d:116-137
    double eval_s(double T, double logT) const {
        if (T < T_low) return s_low - Cp_low * std::log(T_low / T);
        if (T > T_high) return s_high + Cp_high * std::log(T / T_high);
        double a[9]; determine(T, a);
        double s_on_R = -a[0] / (2.0 * T * T) - a[1] / T + a[2] * logT + a[3] * T;
        s_on_R += a[4] * T * T / 2.0 + a[5] * T * T * T / 3.0 + a[6] * T * T * T * T / 4.0 + a[8];
        return R * s_on_R;
    }
    // cea_thermo_curves.d:46-53
    void finish() {
        T_low = breaks.front(); T_high = breaks.back();
        Cp_low = eval_Cp(T_low); Cp_high = eval_Cp(T_high);
        h_low = eval_h(T_low, std::log(T_low)); h_high = eval_h(T_high, std::log(T_high));
        s_low = eval_s(T_low, std::log(T_low)); s_high = eval_s(T_high, std::log(T_high));
    }
};

// model 0 Arrhenius, 1 fromEqConst, the pressure-dependent 2 Lindemann-Hinshelwood, 3 Troe,
// 4 Yungster-Rabinowitz (A, n, C are then k_inf; yr a, b, c are held in a, T1, T2), and
// 5 Arrhenius2 / Arrhenius-logA (A, n, C hold logA, B, C)
struct RateConst {
    int model = 0;
    double A = 0, n = 0, C = 0;
    double A0 = 0, n0 = 0, C0 = 0, Fcent = 0, a = 0, T1 = 0, T2 = 0, T3 = 0;
    int flags = 0;   // Troe: 1 F_cent given, 2 T1 given, 4 T2 given
};

// D's pow(double, int): binary exponentiation (std.math.exponential), here in double.
inline double ipow(double x, int n) {
    if (n < 0) {
        if (n == -1) return 1 / x;
        unsigned m = (unsigned)(-n); double p = 1.0, v = p / x;
        while (true) { if (m & 1) p *= v; m >>= 1; if (!m) break; v *= v; }
        return p;
    }
    switch (n) { case 0: return 1.0; case 1: return x; case 2: return x * x; default: break; }
    unsigned m = (unsigned)n; double p = 1.0, v = x;
    while (true) { if (m & 1) p *= v; m >>= 1; if (!m) break; v *= v; }
    return p;
}

// rate_constant.d:72-75
inline double arrhenius(const RateConst& rc, double T) { return rc.A * std::pow(T, rc.n) * std::exp(-rc.C / T); }
inline double arrhenius0(const RateConst& rc, double T) { return rc.A0 * std::pow(T, rc.n0) * std::exp(-rc.C0 / T); }
// rate_constant.d:112-115 (ArrheniusRateConstant2.eval)
inline double arrhenius2(const RateConst& rc, double T) { return std::exp(rc.A + rc.n * T - rc.C / T); }
inline double simple_rate(const RateConst& rc, double T) { return rc.model == 5 ? arrhenius2(rc, T) : arrhenius(rc, T); }
inline bool pressure_dependent_model(int model) { return model >= 2 && model <= 4; }

// Pressure-dependent rate constants with third-body concentration M (rate_constant.d:114-121 forms
// M = sum eff * massf * rho / M_i): Lindemann-Hinshelwood 155-160, Troe 258-287, Yungster-Rabinowitz 338-350.
inline double pressure_dependent(const RateConst& rc, double T, double M) {
    double kInf = arrhenius(rc, T);
    double k0 = arrhenius0(rc, T);
    if (rc.model == 2) return k0 * kInf * M / (k0 * M + kInf);
    const double essentially_zero = 1.0e-30;
    if (rc.model == 3) {
        double p_r = k0 * M / kInf;
        double log_p_r = std::log10(std::fmax(p_r, essentially_zero));
        double Fcent = rc.Fcent;
        if (!(rc.flags & 1)) {
            Fcent = (1.0 - rc.a) * std::exp(-T / rc.T3);
            if (rc.flags & 2) Fcent += rc.a * std::exp(-T / rc.T1);
            if (rc.flags & 4) Fcent += std::exp(-rc.T2 / T);
        }
        double log_F_cent = std::log10(std::fmax(Fcent, essentially_zero));
        double c = -0.4 - 0.67 * log_F_cent;
        double n = 0.75 - 1.27 * log_F_cent;
        double d = 0.14;
        double numer = log_p_r + c;
        double denom = n - d * numer;
        double frac = numer / denom;
        double log_F = log_F_cent / (1.0 + frac * frac);
        double F = std::pow(10.0, log_F);
        return F * k0 * kInf * M / (k0 * M + kInf);
    }
    double p_r = k0 * M / kInf;
    double log_p_r = std::log(p_r);
    double Fc = rc.a * std::exp(-rc.T1 / T) + (1.0 - rc.a) * std::exp(-rc.T2 / T);
    double xt = 1.0 / (1.0 + log_p_r * log_p_r);
    return kInf * (p_r / (1.0 + p_r)) * Fc * xt;
}

struct Reaction {
    bool collider = false;
    RateConst frc, brc;
    std::vector<std::pair<int, int>> reactants, products;
    std::vector<int> participants;   // sorted (reaction.d:220-221)
    std::vector<int> nu;             // per species
    std::vector<std::pair<int, double>> eff;
};

struct Model {
    int nsp = 0;
    std::vector<double> M, R;
    std::vector<CEACurve> curves;
    std::vector<Reaction> reactions;
    double T_lower = 300.0, T_upper = 50000.0;
    int method = 0;  // 0 rkf, 1 alpha-qss
    double errTol = 1e-3, eps1 = 1e-3, eps2 = 5e-4, delta = 1e-10;
    int maxIters = 10;
    bool tight = false;
    int maxSubcycles = 10000, maxAttempts = 4;
};

// Phobos std.algorithm.iteration.sumPairwise for a random-access range of doubles.
double sum_pairwise(const double* d, int n) {
    if (n == 0) return 0.0;
    double store[64];   // pairwise-summation stack (depth ~log2 n)
    size_t idx = 0;
    auto collapse = [&](size_t k) {
        size_t lastToKeep = idx - (size_t)__builtin_ctzll((unsigned long long)(k + 1));
        while (idx > lastToKeep) { store[idx - 1] += store[idx]; --idx; }
    };
    int pos = 0;
    for (size_t k = 0; k < (size_t)n / 16; ++k) {
        const double* x = d + pos;
        double s = (((x[0] + x[1]) + (x[2] + x[3])) + ((x[4] + x[5]) + (x[6] + x[7])))
                 + (((x[8] + x[9]) + (x[10] + x[11])) + ((x[12] + x[13]) + (x[14] + x[15])));
        store[idx] = s; pos += 16;
        collapse(k); ++idx;
    }
    size_t i = 0;
    for (; pos < n; ++pos) { store[idx] = d[pos]; collapse(i); ++idx; ++i; }
    double s = store[idx - 1];
    for (size_t j = idx - 1; j-- > 0;) s += store[j];
    return 0.0 + s;
}

struct Counters { long steps = 0, rhs = 0, kc = 0, newton = 0, rejects = 0; };

struct Cell {   // the reference GasState fields used on this path
    double rho, u, T, p;
    double massf[ORACLE_MAX_SPECIES];
};

struct Work {
    const Model& m;
    Counters cnt;
    double g[ORACLE_MAX_SPECIES], kf[ORACLE_MAX_REACTIONS], kb[ORACLE_MAX_REACTIONS], wf[ORACLE_MAX_REACTIONS], wb[ORACLE_MAX_REACTIONS];
    explicit Work(const Model& mm) : m(mm) {}

    // therm_perf_gas_mix.d:354-364 with Q.p = P_atm (reaction_mechanism.d:205-218)
    void gibbs(double T) {
        double logT = std::log(T);
        double logp = std::log(P_atm / P_atm);
        for (int i = 0; i < m.nsp; ++i) {
            double h = m.curves[i].eval_h(T, logT);
            double s = m.curves[i].eval_s(T, logT) - m.R[i] * logp;
            g[i] = h - T * s;
        }
    }
    // reaction.d:26-52
    double Kc(const Reaction& r, double T) const {
        double dG = 0.0, nuSum = 0.0;
        for (int isp : r.participants) {
            dG += r.nu[isp] * g[isp] * m.M[isp];
            nuSum += r.nu[isp];
        }
        double K_p = std::exp(-dG / (R_universal * T));
        double nsi = nuSum;
        double base = P_atm / (R_universal * T);
        double pw = (nsi == std::floor(nsi) && std::fabs(nsi) < 32768.0) ? ipow(base, (int)nsi) : std::pow(base, nsi);
        return K_p * pw;
    }
    // reaction_mechanism.d:49-63 and reaction.d:94-143 (single-temperature gas: n_modes == 0).
    // tbc[i] = Q.massf[i] * Q.rho / M_i, the third-body terms of pressure-dependent rates.
    void rate_constants(double Tq, const double* tbc) {
        cnt.kc++;
        double T = Tq;
        if (T < m.T_lower) T = m.T_lower;
        if (T > m.T_upper) T = m.T_upper;
        gibbs(T);
        for (size_t ir = 0; ir < m.reactions.size(); ++ir) {
            const Reaction& r = m.reactions[ir];
            if (r.frc.model != 1) {
                if (!pressure_dependent_model(r.frc.model)) {
                    kf[ir] = simple_rate(r.frc, T);
                } else {
                    double M = 0.0;
                    for (auto& e : r.eff) M += e.second * tbc[e.first];
                    kf[ir] = pressure_dependent(r.frc, T, M);
                }
                if (r.brc.model == 1) kb[ir] = kf[ir] / Kc(r, T);
                else kb[ir] = simple_rate(r.brc, T);
            } else {
                kb[ir] = simple_rate(r.brc, T);
                kf[ir] = kb[ir] * Kc(r, T);
            }
        }
    }
    // reaction.d:145-149, 290-311, 416-456
    void tick_rates(const double* c) {
        for (size_t ir = 0; ir < m.reactions.size(); ++ir) {
            const Reaction& r = m.reactions[ir];
            double term = 1.0;
            if (r.collider) {
                term = 0.0;
                for (auto& e : r.eff) term += e.second * c[e.first];
            }
            double vf = r.collider ? kf[ir] * term : kf[ir];
            for (auto& rc : r.reactants) vf *= ipow(c[rc.first], rc.second);
            double vb = r.collider ? kb[ir] * term : kb[ir];
            for (auto& pc : r.products) vb *= ipow(c[pc.first], pc.second);
            wf[ir] = vf; wb[ir] = vb;
        }
    }
    // reaction_mechanism.d:82-96 with production/loss of reaction.d:267-287
    void split_rates(const double* c, double* q, double* L) {
        cnt.rhs++;
        tick_rates(c);
        for (int i = 0; i < m.nsp; ++i) { q[i] = 0.0; L[i] = 0.0; }
        for (size_t ir = 0; ir < m.reactions.size(); ++ir) {
            const Reaction& r = m.reactions[ir];
            for (int isp : r.participants) {
                int nu = r.nu[isp];
                double prod = nu > 0 ? nu * wf[ir] : (nu < 0 ? -nu * wb[ir] : 0.0);
                double loss = nu > 0 ? nu * wb[ir] : (nu < 0 ? -nu * wf[ir] : 0.0);
                q[isp] += prod;
                L[isp] += loss;
            }
        }
    }
    void rates(const double* c, double* out) {   // reaction_mechanism.d:75-81
        double q[ORACLE_MAX_SPECIES], L[ORACLE_MAX_SPECIES];
        split_rates(c, q, L);
        for (int i = 0; i < m.nsp; ++i) out[i] = q[i] - L[i];
    }
    // reaction_mechanism.d:161-203
    double estimate_step(const double* c) {
        const double MUCH_LARGER_FACTOR = 10000.0, ZERO_EPS = 1.0e-50, ZERO_TOL = 1.0e-30, EPS1 = 1.0e-3;
        double q[ORACLE_MAX_SPECIES], L[ORACLE_MAX_SPECIES];
        double min_dt = 1.0e6, dt;
        split_rates(c, q, L);
        for (int i = 0; i < m.nsp; ++i) {
            if (c[i] > 0.0 && (std::fabs(q[i] - L[i]) > ZERO_TOL)) {
                if (q[i] > MUCH_LARGER_FACTOR * L[i]) dt = c[i] / (L[i] + ZERO_EPS);
                else dt = std::fabs(c[i] / (q[i] - L[i]));
                min_dt = std::min(min_dt, dt);
            }
        }
        double dt_chem = EPS1 * min_dt;
        dt_chem = std::min(dt_chem, 1.0e-10);
        dt_chem = std::max(dt_chem, 1.0e-15);
        return dt_chem;
    }
    // chemistry_update.d:404-478
    bool rkf_step(const double* y0, double h, double* yOut, double& hSuggest) {
        const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10., a43 = 6. / 5.,
            a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27.,
            a61 = 1631. / 55296., a62 = 175. / 512., a63 = 575. / 13824., a64 = 44275. / 110592., a65 = 253. / 4096.;
        const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771.,
            b41 = 2825. / 27648., b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336., b46 = 1.0 / 4.0;
        const int n = m.nsp;
        double k1[ORACLE_MAX_SPECIES], k2[ORACLE_MAX_SPECIES], k3[ORACLE_MAX_SPECIES], k4[ORACLE_MAX_SPECIES], k5[ORACLE_MAX_SPECIES], k6[ORACLE_MAX_SPECIES], yT[ORACLE_MAX_SPECIES], yErr[ORACLE_MAX_SPECIES];
        rates(y0, k1);
        for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a21 * k1[i]);
        rates(yT, k2);
        for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a31 * k1[i] + a32 * k2[i]);
        rates(yT, k3);
        for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
        rates(yT, k4);
        for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
        rates(yT, k5);
        for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
        rates(yT, k6);
        for (int i = 0; i < n; ++i) yOut[i] = y0[i] + h * (b51 * k1[i] + b53 * k3[i] + b54 * k4[i] + b56 * k6[i]);
        for (int i = 0; i < n; ++i)
            yErr[i] = yOut[i] - (y0[i] + h * (b41 * k1[i] + b43 * k3[i] + b44 * k4[i] + b45 * k5[i] + b46 * k6[i]));
        double err = 0.0, sk;
        const double atol = m.errTol, rtol = m.errTol;
        for (int i = 0; i < n; ++i) {
            sk = atol + rtol * std::max(std::fabs(y0[i]), std::fabs(yOut[i]));
            err += (yErr[i] / sk) * (yErr[i] / sk);
        }
        err = std::sqrt(err / n);
        const double maxscale = 10.0, minscale = 0.2, safe = 0.9, alpha = 0.2;
        double scale;
        if (err <= 1.0) {
            if (err == 0.0) scale = maxscale;
            else {
                scale = safe * std::pow(err, -alpha);
                if (scale < minscale) scale = minscale;
                if (scale > maxscale) scale = maxscale;
            }
            hSuggest = scale * h;
            return true;
        }
        scale = std::max(safe * std::pow(err, -alpha), minscale);
        hSuggest = scale * h;
        return false;
    }
    // chemistry_update.d:533-655
    bool aqss_step(const double* y0, double h, double* yOut, double& hSuggest) {
        const double ZERO_EPS = 1.0e-50;
        const int n = m.nsp;
        double q0[ORACLE_MAX_SPECIES], L0[ORACLE_MAX_SPECIES], p0[ORACLE_MAX_SPECIES], alpha[ORACLE_MAX_SPECIES], yp[ORACLE_MAX_SPECIES], yp0[ORACLE_MAX_SPECIES], qp[ORACLE_MAX_SPECIES], Lp[ORACLE_MAX_SPECIES], pp[ORACLE_MAX_SPECIES], ab[ORACLE_MAX_SPECIES], qt[ORACLE_MAX_SPECIES], pb[ORACLE_MAX_SPECIES], yc[ORACLE_MAX_SPECIES];
        auto p_on_y = [&](const double* L, const double* y, double* p) {
            for (int i = 0; i < n; ++i) p[i] = L[i] / (y[i] + ZERO_EPS);
        };
        auto alpha_compute = [&](const double* p, double* a) {
            for (int i = 0; i < n; ++i) {
                double r = 1.0 / (p[i] * h + ZERO_EPS);
                a[i] = (180.0 * r * r * r + 60.0 * r * r + 11.0 * r + 1.0) / (360.0 * r * r * r + 60.0 * r * r + 12.0 * r + 1.0);
            }
        };
        auto update_conc = [&](double* yT, const double* q, const double* p, const double* a) {
            for (int i = 0; i < n; ++i) yT[i] = y0[i] + (h * (q[i] - p[i] * y0[i])) / (1.0 + a[i] * h * p[i]);
        };
        auto converged = [&](const double* c, const double* pr) {
            for (int i = 0; i < n; ++i) {
                if (c[i] < ZERO_EPS) continue;
                double test = std::fabs(c[i] - pr[i]);
                if (test >= (m.eps1 * (c[i] + m.delta))) return false;
            }
            return true;
        };
        auto step_suggest = [&](const double* c, const double* pr) {
            double sigma = 0.0;
            for (int i = 0; i < n; ++i) {
                if (c[i] < ZERO_EPS) continue;
                double test = std::fabs(c[i] - pr[i]) / (m.eps2 * (c[i] + m.delta));
                if (test > sigma) sigma = test;
            }
            if (sigma <= 0.0) return 10.0 * h;
            double x = sigma;
            x = x - 0.5 * (x * x - sigma) / x;
            x = x - 0.5 * (x * x - sigma) / x;
            x = x - 0.5 * (x * x - sigma) / x;
            return h * ((1.0 / x) + 0.005);
        };
        split_rates(y0, q0, L0);
        p_on_y(L0, y0, p0);
        alpha_compute(p0, alpha);
        update_conc(yp, q0, p0, alpha);
        for (int i = 0; i < n; ++i) yp0[i] = yp[i];
        for (int corr = 0; corr < m.maxIters; ++corr) {
            split_rates(yp, qp, Lp);
            p_on_y(Lp, yp, pp);
            alpha_compute(pp, ab);
            for (int i = 0; i < n; ++i) {
                qt[i] = ab[i] * qp[i] + (1 - ab[i]) * q0[i];
                pb[i] = 0.5 * (p0[i] + pp[i]);
            }
            update_conc(yc, qt, pb, ab);
            if (converged(yc, yp0)) {
                for (int i = 0; i < n; ++i) yOut[i] = yc[i];
                hSuggest = step_suggest(yc, yp0);
                return true;
            }
            for (int i = 0; i < n; ++i) yp[i] = yc[i];
        }
        hSuggest = step_suggest(yc, yp0);
        return false;
    }
    bool ode_step(const double* y0, double h, double* yOut, double& hs) {
        cnt.steps++;
        return m.method == 0 ? rkf_step(y0, h, yOut, hs) : aqss_step(y0, h, yOut, hs);
    }

    // gas_model.d:237-253
    double tb[ORACLE_MAX_SPECIES];
    const double* third_body_terms(const Cell& Q) {   // rate_constant.d:117-119
        for (int i = 0; i < m.nsp; ++i) tb[i] = Q.massf[i] * Q.rho / m.M[i];
        return tb;
    }
    void massf2conc(const Cell& Q, double* c) const {
        if (std::isnan(Q.rho) || Q.rho <= 0.0) throw Failure{ST_BAD_INPUT};
        for (int i = 0; i < m.nsp; ++i) {
            c[i] = Q.massf[i] * Q.rho / m.M[i];
            if (c[i] < MIN_MOLES) c[i] = 0.0;
        }
    }
    // gas_model.d:255-271
    void conc2massf(const double* c, Cell& Q) const {
        if (std::isnan(Q.rho) || Q.rho <= 0.0) throw Failure{ST_BAD_INPUT};
        for (int i = 0; i < m.nsp; ++i) {
            Q.massf[i] = c[i] * m.M[i] / Q.rho;
            if (Q.massf[i] < MIN_MASS_FRACTION) Q.massf[i] = 0.0;
        }
    }
    double mass_average(const Cell& Q, const double* phi) const {   // gas_model.d:410-418
        double r = 0.0;
        for (int i = 0; i < m.nsp; ++i) r += Q.massf[i] * phi[i];
        return r;
    }
    // therm_perf_gas_mix.d:406-413
    double internal_energy(const double* mf, double T, double logT) const {
        double u = 0.0;
        for (int i = 0; i < m.nsp; ++i) u += mf[i] * (m.curves[i].eval_h(T, logT) - m.R[i] * T);
        return u;
    }
    // therm_perf_gas_mix.d:416-423
    double Cv(const double* mf, double T) const {
        double c = 0.0;
        for (int i = 0; i < m.nsp; ++i) c += mf[i] * (m.curves[i].eval_Cp(T) - m.R[i]);
        return c;
    }
    // therm_perf_gas_mix.d:426-468
    double T_from_u(const Cell& Q) {
        const double TOL = 1e-10;
        const double u_tgt = Q.u;
        double T = Q.T;
        double f = internal_energy(Q.massf, T, std::log(T)) - u_tgt;
        double dT = 0.0;
        for (int iter = 0; iter < 10; ++iter) {
            cnt.newton++;
            double cv = Cv(Q.massf, T);
            dT = -f / cv;
            T += dT;
            if (std::fabs(dT) / T < TOL) return T;
            f = internal_energy(Q.massf, T, std::log(T)) - u_tgt;
        }
        if (std::fabs(dT) > 1e-3) throw Failure{ST_NEWTON_FAIL};
        return T;
    }
    // therm_perf_gas_mix.d:63-67 and 379-383
    void update_from_rhou(Cell& Q) {
        Q.T = T_from_u(Q);
        Q.p = Q.rho * mass_average(Q, m.R.data()) * Q.T;
    }
    // therm_perf_gas_mix.d:57-61, 386-403
    void update_from_pT(Cell& Q) const {
        Q.rho = Q.p / (mass_average(Q, m.R.data()) * Q.T);
        double logT = std::log(Q.T);
        double vals[ORACLE_MAX_SPECIES];
        for (int i = 0; i < m.nsp; ++i) vals[i] = m.curves[i].eval_h(Q.T, logT) - m.R[i] * Q.T;
        Q.u = mass_average(Q, vals);
    }

    // chemistry_update.d:140-326
    void opCall(Cell& Q, double tInterval, double& dtSuggest) {
        Cell Qinit = Q;
        double conc0[ORACLE_MAX_SPECIES], concOut[ORACLE_MAX_SPECIES];
        try {
            massf2conc(Q, conc0);
            rate_constants(Q.T, third_body_terms(Q));
            double t = 0.0, h, dtSave = dtSuggest;
            if (dtSuggest > tInterval) h = tInterval;
            else if (dtSuggest <= 0.0) h = estimate_step(conc0);
            else h = dtSuggest;
            int cycle = 0, attempt = 0;
            for (; cycle < m.maxSubcycles; ++cycle) {
                dtSave = dtSuggest;
                h = std::min(h, tInterval - t);
                attempt = 0;
                for (; attempt < m.maxAttempts; ++attempt) {
                    bool ok = ode_step(conc0, h, concOut, dtSuggest);
                    bool massOK = true;
                    if (ok) {
                        conc2massf(concOut, Q);
                        double tot = sum_pairwise(Q.massf, m.nsp);
                        if (std::fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) massOK = false;
                    }
                    if (ok && massOK) {
                        t += h;
                        for (int i = 0; i < m.nsp; ++i) conc0[i] = concOut[i];
                        double hMax = h * (1.0 + DT_INCREASE_PERCENT / 100.0);
                        if (dtSuggest > h) h = std::min(dtSuggest, hMax);
                        break;
                    } else {
                        cnt.rejects++;
                        h /= DT_REDUCTION_FACTOR;
                        if (h < H_MIN) throw Failure{ST_H_MIN};
                    }
                }
                if (attempt == m.maxAttempts) throw Failure{ST_MAX_ATTEMPTS};
                if (m.tight) {
                    conc2massf(conc0, Q);
                    update_from_rhou(Q);
                    rate_constants(Q.T, third_body_terms(Q));
                }
                if (t >= tInterval) {
                    if (cycle == 0) dtSave = dtSuggest;
                    break;
                }
            }
            if (cycle == m.maxSubcycles) throw Failure{ST_MAX_SUBCYCLES};
            conc2massf(concOut, Q);
            double tot = sum_pairwise(Q.massf, m.nsp);
            for (int i = 0; i < m.nsp; ++i) Q.massf[i] /= tot;
            dtSuggest = dtSave;
        } catch (Failure& f) {
            Q = Qinit;
            throw;
        }
    }

    // fluidfvcell.d:883-997 minus the gas-dynamics bookkeeping.
    int increment(Cell& Q, double dt, double& dt_chem, double T_frozen, int flags) {
        if (Q.T <= T_frozen) return ST_FROZEN;
        try {
            opCall(Q, dt, dt_chem);
        } catch (Failure& f) {
            if (!(flags & 2) || (f.code != ST_H_MIN && f.code != ST_MAX_ATTEMPTS && f.code != ST_MAX_SUBCYCLES))
                return f.code;
            dt_chem = -1.0;
            try { opCall(Q, dt, dt_chem); } catch (Failure& f2) { return f2.code; }
        }
        if (flags & 1) {
            try { update_from_rhou(Q); } catch (Failure& f) { return f.code; }
        }
        return ST_OK;
    }
};

}  // namespace

// ------------------------------------------------------------------------------------------
// C ABI used by tests/ and bench.py (ctypes).  Handles are heap pointers.
extern "C" {

void* oracle_model_new(int nsp) {
    if (nsp < 1 || nsp > ORACLE_MAX_SPECIES) return nullptr;
    Model* m = new Model(); m->nsp = nsp; m->M.resize(nsp); m->R.resize(nsp); m->curves.resize(nsp); return m; }
void oracle_model_free(void* h) { delete (Model*)h; }

// Per species: molar mass and its CEA curve (ThermPerfGasMixture ctor, therm_perf_gas_mix.d:30-47).
int oracle_set_species(void* h, int isp, double M, int nseg, const double* breaks, const double* blends,
                       const double* coeffs /* nseg*9 */) {
    Model* m = (Model*)h;
    if (isp < 0 || isp >= m->nsp || nseg < 1) return -1;
    m->M[isp] = M;
    m->R[isp] = R_universal / M;
    CEACurve& c = m->curves[isp];
    c.R = m->R[isp];
    c.breaks.assign(breaks, breaks + nseg + 1);
    c.blends.assign(blends, blends + std::max(nseg - 1, 0));
    c.coeffs.resize(nseg);
    for (int s = 0; s < nseg; ++s) for (int j = 0; j < 9; ++j) c.coeffs[s][j] = coeffs[s * 9 + j];
    try { c.finish(); } catch (Failure&) { return -1; }
    return 0;
}

// One reaction (reaction.d:478-535).  frc_model/brc_model: 0 Arrhenius, 1 fromEqConst; frc_model
// 2-4 pressure-dependent (see RateConst; completed by oracle_set_pressure_dependent).
int oracle_add_reaction(void* h, int collider, int frc_model, double fA, double fn, double fC,
                        int brc_model, double bA, double bn, double bC,
                        int nreac, const int* reac_idx, const int* reac_coeff,
                        int nprod, const int* prod_idx, const int* prod_coeff,
                        int neff, const int* eff_idx, const double* eff_val) {
    if ((int)((Model*)h)->reactions.size() >= ORACLE_MAX_REACTIONS) return -1;
    Model* m = (Model*)h;
    Reaction r;
    r.collider = collider != 0;
    r.frc.model = frc_model; r.frc.A = fA; r.frc.n = fn; r.frc.C = fC;
    r.brc.model = brc_model; r.brc.A = bA; r.brc.n = bn; r.brc.C = bC;
    std::vector<int> part;
    for (int i = 0; i < nreac; ++i) { r.reactants.push_back({reac_idx[i], reac_coeff[i]}); part.push_back(reac_idx[i]); }
    for (int i = 0; i < nprod; ++i) { r.products.push_back({prod_idx[i], prod_coeff[i]}); part.push_back(prod_idx[i]); }
    std::sort(part.begin(), part.end());
    part.erase(std::unique(part.begin(), part.end()), part.end());
    r.participants = part;
    r.nu.assign(m->nsp, 0);
    for (int isp = 0; isp < m->nsp; ++isp) {   // reaction.d:222-238 (first match on each side)
        int nu1 = 0, nu2 = 0;
        for (auto& x : r.reactants) if (x.first == isp) { nu1 = x.second; break; }
        for (auto& x : r.products) if (x.first == isp) { nu2 = x.second; break; }
        r.nu[isp] = nu2 - nu1;
    }
    for (int i = 0; i < neff; ++i) r.eff.push_back({eff_idx[i], eff_val[i]});
    m->reactions.push_back(r);
    return (int)m->reactions.size() - 1;
}

// k_0 and the Troe / Yungster-Rabinowitz parameters of reaction ir's forward rate constant
// (its model and k_inf were given to oracle_add_reaction).
int oracle_set_pressure_dependent(void* h, int ir, double A0, double n0, double C0, double Fcent, double a, double T1,
                                  double T2, double T3, int flags) {
    Model* m = (Model*)h;
    if (ir < 0 || ir >= (int)m->reactions.size()) return -1;
    RateConst& rc = m->reactions[ir].frc;
    rc.A0 = A0; rc.n0 = n0; rc.C0 = C0; rc.Fcent = Fcent; rc.a = a; rc.T1 = T1; rc.T2 = T2; rc.T3 = T3;
    rc.flags = flags;
    return 0;
}

int oracle_set_config(void* h, double T_lower, double T_upper, int method, double errTol, double eps1, double eps2,
                      double delta, int maxIters, int tight, int maxSubcycles, int maxAttempts) {
    Model* m = (Model*)h;
    m->T_lower = T_lower; m->T_upper = T_upper; m->method = method; m->errTol = errTol;
    m->eps1 = eps1; m->eps2 = eps2; m->delta = delta; m->maxIters = maxIters; m->tight = tight != 0;
    m->maxSubcycles = maxSubcycles; m->maxAttempts = maxAttempts;
    return 0;
}

int oracle_n_reactions(void* h) { return (int)((Model*)h)->reactions.size(); }

// Species enthalpy at T given ln T, and Cp at T (per species, J/kg); nonzero on a CEA range failure.
int oracle_species_h(void* h, int isp, double T, double logT, double* out) {
    Model* m = (Model*)h;
    try { *out = m->curves[isp].eval_h(T, logT); } catch (Failure& f) { return f.code; }
    return 0;
}

int oracle_species_cp(void* h, int isp, double T, double* out) {
    Model* m = (Model*)h;
    try { *out = m->curves[isp].eval_Cp(T); } catch (Failure& f) { return f.code; }
    return 0;
}

// Species thermo (per species, J/kg): Cp, h, s at T (s at p = P_atm).
int oracle_species_thermo(void* h, int isp, double T, double* Cp, double* hh, double* s) {
    Model* m = (Model*)h;
    try {
        *Cp = m->curves[isp].eval_Cp(T);
        *hh = m->curves[isp].eval_h(T, std::log(T));
        *s = m->curves[isp].eval_s(T, std::log(T));
    } catch (Failure& f) { return f.code; }
    return 0;
}

// kf, kb at T (clamped to the mechanism's limits), as ReactionMechanism.eval_rate_constants.
// conc (may be NULL without pressure-dependent reactions) gives their third-body concentrations.
int oracle_rate_constants(void* h, double T, const double* conc, double* kf, double* kb) {
    Model* m = (Model*)h;
    Work w(*m);
    // without concentrations the third bodies of pressure-dependent rates are zero
    std::vector<double> zero(m->nsp, 0.0);
    try { w.rate_constants(T, conc ? conc : zero.data()); } catch (Failure& f) { return f.code; }
    for (size_t i = 0; i < m->reactions.size(); ++i) { kf[i] = w.kf[i]; kb[i] = w.kb[i]; }
    return 0;
}

// q, L (mol/m^3/s) and the per-reaction tick rates at given concentrations and T.
int oracle_split_rates(void* h, double T, const double* conc, double* q, double* L, double* wf, double* wb) {
    Model* m = (Model*)h;
    Work w(*m);
    try { w.rate_constants(T, conc); } catch (Failure& f) { return f.code; }
    w.split_rates(conc, q, L);
    if (wf) for (size_t i = 0; i < m->reactions.size(); ++i) wf[i] = w.wf[i];
    if (wb) for (size_t i = 0; i < m->reactions.size(); ++i) wb[i] = w.wb[i];
    return 0;
}

double oracle_estimate_step(void* h, double T, const double* conc) {
    Model* m = (Model*)h;
    Work w(*m);
    w.rate_constants(T, conc);
    return w.estimate_step(conc);
}

// One bare ODE step (the unit-test driver numericalEstimate, chemistry_update.d:664-678).
// method: 0 rkf, 1 alpha-qss (uses the model's tolerances).  Returns 1 on success.
int oracle_ode_step(void* h, int method, double T, const double* y0, double dt, double* yOut, double* hSuggest) {
    Model* m = (Model*)h;
    Model mm = *m; mm.method = method;
    Work w(mm);
    w.rate_constants(T, y0);
    return w.ode_step(y0, dt, yOut, *hSuggest) ? 1 : 0;
}

// Fixed-step integration with one ODE method over [0, tMax] (numericalEstimate,
// chemistry_update.d:664-678): `while ((tMax - t) > 1.0e-9) { dt = min(dt, tMax - t); step; t += dt; }`.
int oracle_integrate_fixed(void* h, int method, double T, double* y, double dt, double tMax) {
    Model* m = (Model*)h;
    Model mm = *m; mm.method = method;
    Work w(mm);
    w.rate_constants(T, y);
    double t = 0.0, dummy, y1[ORACLE_MAX_SPECIES];
    int count = 0;
    while ((tMax - t) > 1.0e-9) {
        dt = std::min(dt, tMax - t);
        w.ode_step(y, dt, y1, dummy);
        t += dt;
        for (int i = 0; i < m->nsp; ++i) y[i] = y1[i];
        count++;
    }
    return count;
}

// Batched gas-state services.  massf is cell-major: massf[cell*nsp + isp].
int oracle_update_thermo_from_pT(void* h, int n, const double* p, const double* T, const double* massf,
                                 double* rho, double* u) {
    Model* m = (Model*)h;
    Work w(*m);
    for (int c = 0; c < n; ++c) {
        Cell Q; Q.p = p[c]; Q.T = T[c];
        for (int i = 0; i < m->nsp; ++i) Q.massf[i] = massf[(size_t)c * m->nsp + i];
        try { w.update_from_pT(Q); } catch (Failure& f) { return f.code; }
        rho[c] = Q.rho; u[c] = Q.u;
    }
    return 0;
}

int oracle_update_thermo_from_rhou(void* h, int n, const double* rho, const double* u, const double* massf,
                                   double* T, double* p, int* status) {
    Model* m = (Model*)h;
    Work w(*m);
    for (int c = 0; c < n; ++c) {
        Cell Q; Q.rho = rho[c]; Q.u = u[c]; Q.T = T[c]; Q.p = p[c];
        for (int i = 0; i < m->nsp; ++i) Q.massf[i] = massf[(size_t)c * m->nsp + i];
        int st = 0;
        try { w.update_from_rhou(Q); } catch (Failure& f) { st = f.code; }
        if (!st) { T[c] = Q.T; p[c] = Q.p; }
        if (status) status[c] = st;
    }
    return 0;
}

// The chemistry update over a batch of independent cells (one thermochemical_increment each).
// flags: bit0 = follow with update_thermo_from_rhou (fluidfvcell.d:956);
//        bit1 = retry once with dt_chem = -1 on a ThermochemicalReactorUpdateException (:924-941).
// counters (may be NULL): per cell [steps, rhs evaluations, rate-constant evaluations, Newton iterations, rejects].
// nthreads <= 0 uses all OpenMP threads.  Returns the number of cells with a failure status.
int oracle_chem_update(void* h, int n, const double* rho, const double* u, double* T, double* p, double* massf,
                       double* dt_chem, int* status, double t_interval, double T_frozen, int flags, int nthreads,
                       long* counters) {
    Model* m = (Model*)h;
    std::atomic<int> nfail{0};
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
    {
        Work w(*m);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int c = 0; c < n; ++c) {
            w.cnt = Counters();
            Cell Q; Q.rho = rho[c]; Q.u = u[c]; Q.T = T[c]; Q.p = p[c];
            for (int i = 0; i < m->nsp; ++i) Q.massf[i] = massf[(size_t)c * m->nsp + i];
            double dtc = dt_chem[c];
            int st = w.increment(Q, t_interval, dtc, T_frozen, flags);
            if (st == ST_OK) {
                T[c] = Q.T; p[c] = Q.p; dt_chem[c] = dtc;
                for (int i = 0; i < m->nsp; ++i) massf[(size_t)c * m->nsp + i] = Q.massf[i];
            } else if (st != ST_FROZEN) {
                nfail++;
            }
            if (status) status[c] = st;
            if (counters) {
                long* k = counters + (size_t)c * 5;
                k[0] = w.cnt.steps; k[1] = w.cnt.rhs; k[2] = w.cnt.kc; k[3] = w.cnt.newton; k[4] = w.cnt.rejects;
            }
        }
    }
    return nfail.load();
}

int oracle_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
