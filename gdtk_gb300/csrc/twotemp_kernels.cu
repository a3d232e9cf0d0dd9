// twotemp_kernels.cu -- the multi-temperature thermochemical reactor for a two-temperature gas, one
// thread per cell, compiled with FMA contraction, with the rate constants and equilibrium constants in
// log form (one exp where the reference takes pows and an exp) and the rate, relaxation and coupling
// exponentials by Tang's table method: results differ from the reference's evaluation order in rounding
// only (tested to 1e-8 in Y, 1e-7 relative in T, T_ve and p).
//
// kinetics/multi_temperature_thermochemical_reactor.d:137-294 (opCall) and :334-431 (Cash-Karp RKF
// on the concentrations and u_ve), with
//   * rate constants once per subcycle at the clamped T (reaction_mechanism.d:49-63): Gibbs energies
//     at p = P_atm and T_ve = T (:204-218, two_temperature_gas.d:469-482), forward Arrhenius or Park
//     (rate_constant.d:72-75, 364-393: T_eff = T^s T_ve^(1-s)) or (modified) Marrone-Treanor over either
//     (rate_constant.d:395-566), backward k_f(T, T_ve = T) / K_c(T)
//     (reaction.d:94-143, 26-52);
//   * tick rates and q - L (reaction.d:290-311, 416-440; reaction_mechanism.d:74-96);
//   * energy exchange (energy_exchange_system.d:93-104): Landau-Teller (energy_exchange_mechanism.d:
//     83-101) with Millikan-White / Park high-temperature relaxation times (relaxation_time.d:27-175),
//     evaluated once per subcycle on the subcycle's gas state, and Marrone-Treanor coupling with
//     impartial, Marrone-Treanor or modified Marrone-Treanor dissociation (energy_exchange_mechanism.d:
//     228-241, exchange_chemistry_coupling.d:41-227; G_appear and G_vanish on the subcycle's state) on
//     the current stage's tick rates;
//   * T from u by direct inversion and T_ve by Newton iteration (two_temperature_gas.d:95-117, 656-700).
// A cell that fails keeps its input state and gets the reference's failure as its status.
#include <cuda_runtime.h>

#include <cmath>

#include "cea_thermo.h"
#include "chem_types.h"
#include "fast_exp.h"
#include "twotemp.h"

namespace gdtk {
namespace {

constexpr double R_universal = 8.31451;       // gas/physical_constants.d:13
constexpr double P_atm = 101.325e3;           // gas/physical_constants.d:16
constexpr double Boltzmann = 1.380658e-23;    // gas/physical_constants.d:18
constexpr double Avogadro = 6.02214e23;       // gas/physical_constants.d:19
constexpr double PI_D = 3.141592653589793;
constexpr double T_REF = 298.15;              // two_temperature_gas.d:26
constexpr double SMALL_MOLE_FRACTION = 1.0e-15;   // gas_model.d:42
constexpr double IGAMMA_SWITCH = 1.0e-7;      // exchange_chemistry_coupling.d:24
constexpr double IGAMMA_OVERFLOW = 0.001;     // exchange_chemistry_coupling.d:25
constexpr double H_MIN = 1.0e-15;             // multi_temperature_thermochemical_reactor.d:31
constexpr double LN_PATM_R = 0x1.2d0f0af013269p+3;   // ln(P_atm / R_universal) = 9.408086270233257
constexpr double ALLOWABLE_MASSF_ERROR = 1.0e-3;
constexpr int NV = GDTK_MAX_SPECIES + 1;
constexpr int MAX_EEM = 64;

// exp by Tang's table method (fast_exp.h, within 1.3 ulp): 9 FP64 operations where the library's takes
// about 20 FMA slots on this GPU.  The update kernel stages the table in shared memory once per block.
__device__ const double kExp2Table[GDTK_EXP2_TABLE_SIZE] = GDTK_EXP2_TABLE_INIT;
__shared__ double s_exp2[GDTK_EXP2_TABLE_SIZE];
__device__ __forceinline__ double ex(double x) { return gdtk_exp(x, s_exp2); }

// NASA-9 Cp, h and s of cea_thermo_curves.d:55-137 (cea_thermo.h's segment choice and blending,
// cea_coeffs) in Horner form with the reciprocal temperature rT = 1 / T: the reference's divisions by T,
// T^2 and the small integers become multiplications.
__device__ double cea_Cp_r(const MechView& m, int isp, double T, double rT, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_CPLOW];
    if (T > s[SP_THIGH]) return s[SP_CPHIGH];
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    // Cp/R = a0/T^2 + a1/T + a2 + a3 T + a4 T^2 + a5 T^3 + a6 T^4
    const double c = fma(rT, fma(a[0], rT, a[1]), a[2]) + T * fma(T, fma(T, fma(T, a[6], a[5]), a[4]), a[3]);
    return s[SP_R] * c;
}
__device__ double cea_h_r(const MechView& m, int isp, double T, double rT, double logT, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_HLOW] - s[SP_CPLOW] * (s[SP_TLOW] - T);
    if (T > s[SP_THIGH]) return s[SP_HHIGH] + s[SP_CPHIGH] * (T - s[SP_THIGH]);
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    // h/R = -a0/T + a1 ln T + a2 T + a3 T^2/2 + a4 T^3/3 + a5 T^4/4 + a6 T^5/5 + a7
    const double poly = fma(T, fma(T, fma(T, a[6] * 0.2, a[5] * 0.25), a[4] * (1.0 / 3.0)), a[3] * 0.5);
    const double h = fma(-a[0], rT, fma(a[1], logT, a[7])) + T * fma(T, poly, a[2]);
    return s[SP_R] * h;
}
__device__ double cea_s_r(const MechView& m, int isp, double T, double rT, double logT, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_SLOW] - s[SP_CPLOW] * log(s[SP_TLOW] / T);
    if (T > s[SP_THIGH]) return s[SP_SHIGH] + s[SP_CPHIGH] * log(T / s[SP_THIGH]);
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    // s/R = -a0/(2 T^2) - a1/T + a2 ln T + a3 T + a4 T^2/2 + a5 T^3/3 + a6 T^4/4 + a8
    const double poly = fma(T, fma(T, a[6] * 0.25, a[5] * (1.0 / 3.0)), a[4] * 0.5);
    const double v = fma(rT, fma(-0.5 * a[0], rT, -a[1]), fma(a[2], logT, a[8])) + T * fma(T, poly, a[3]);
    return s[SP_R] * v;
}

struct Gas2T {
    MechView m;
    const Species2T* sp;
    int electron;
    __device__ double R(int i) const { return m.sp(i)[SP_R]; }
    // two_temperature_gas.d:427-445, 538-545, 558-590
    // rTve = 1 / T_ve, logTve = ln T_ve
    __device__ double e_ve(int i, double Tve, double rTve, double logTve, int& err) const {
        if (i == electron) return 1.5 * R(i) * Tve;
        return cea_h_r(m, i, Tve, rTve, logTve, err) - sp[i].cp_tr * (Tve - T_REF) - sp[i].h_f;
    }
    __device__ double cv_ve(int i, double Tve, double rTve, int& err) const {
        if (i == electron) return 1.5 * R(i);
        return cea_Cp_r(m, i, Tve, rTve, err) - sp[i].cp_tr;
    }
    __device__ double e_tr(int i, double T) const {
        if (i == electron) return 0.0;
        return sp[i].cp_tr * (T - T_REF) + sp[i].h_f - R(i) * T;
    }
    __device__ double e_ve_mix(const double* Y, double Tve, int& err) const { return e_ve_mix(Y, Tve, log(Tve), err); }
    __device__ double e_ve_mix(const double* Y, double Tve, double lt, int& err) const {
        return e_ve_mix(Y, Tve, 1.0 / Tve, lt, err);
    }
    __device__ double e_ve_mix(const double* Y, double Tve, double r, double lt, int& err) const {   // r = 1 / Tve
        double e = 0.0;
        for (int i = 0; i < m.nsp; ++i) e += Y[i] * e_ve(i, Tve, r, lt, err);
        return e;
    }
    __device__ double e_tr_mix(const double* Y, double T) const {
        double e = 0.0;
        for (int i = 0; i < m.nsp; ++i)
            if (i != electron) e += Y[i] * e_tr(i, T);
        return e;
    }
    __device__ double cv_ve_mix(const double* Y, double Tve, int& err) const { return cv_ve_mix(Y, Tve, 1.0 / Tve, err); }
    __device__ double cv_ve_mix(const double* Y, double Tve, double r, int& err) const {   // r = 1 / Tve
        double c = 0.0;
        for (int i = 0; i < m.nsp; ++i) c += Y[i] * cv_ve(i, Tve, r, err);
        return c;
    }
    __device__ double pressure(double rho, const double* Y, double T, double Tve) const {
        double p = 0.0;
        for (int i = 0; i < m.nsp; ++i) p += rho * Y[i] * R(i) * (i == electron ? Tve : T);
        return p;
    }
    // updateFromRhoU: T directly, T_ve by Newton from the guess in Tve (40 iterations, |dT| < 1e-9 K,
    // or the guess itself when its energy is within 1e-5 J/kg); false when the iteration fails.
    __device__ bool from_rhou(double rho, double u, double u_ve, const double* Y, double& T, double& Tve,
                              double& p) const {
        double sumA = 0.0, sumB = 0.0;
        for (int i = 0; i < m.nsp; ++i) {
            if (i == electron) continue;
            sumA += Y[i] * (sp[i].cp_tr * T_REF - sp[i].h_f);
            sumB += Y[i] * (sp[i].cp_tr - R(i));
        }
        T = (u + sumA) / sumB;
        int err = 0;
        double Tg = Tve, lg = log(Tve), rg = 1.0 / Tve;   // T_ve's iterate, its log and reciprocal
        double f = e_ve_mix(Y, Tg, rg, lg, err) - u_ve;
        if (fabs(f) >= 1e-5) {
            int count = 0;
            double dT = 0.0;
            for (int it = 0; it < 40; ++it) {
                const double Cv = cv_ve_mix(Y, Tg, rg, err);
                dT = -f / Cv;
                // ln(Tg + dT) = ln Tg + log1p(x), x = dT / Tg: the Taylor series to x^6 when |x| < 2^-10 (its
                // truncation is below 2^-60 |x|), else a fresh log
                const double x = dT * rg;
                Tg += dT;
                if (fabs(dT) < 1.0e-9) break;
                lg = (fabs(x) < 0x1p-10)
                         ? lg + x * fma(x, fma(x, fma(x, fma(x, fma(x, -1.0 / 6.0, 0.2), -0.25), 1.0 / 3.0), -0.5), 1.0)
                         : log(Tg);
                rg = 1.0 / Tg;
                f = e_ve_mix(Y, Tg, rg, lg, err) - u_ve;
                ++count;
            }
            if (count == 40 && fabs(dT) > 1e-3) return false;
        }
        if (err) return false;
        Tve = Tg;
        p = pressure(rho, Y, T, Tve);
        return true;
    }
};

__device__ __forceinline__ double pow_int(double x, int n) {   // small positive coefficients
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

// An Arrhenius (at T) or Park (at T_e = T^s T_ve^(1-s)) rate constant from the record's A, n, C, s, in log
// form: A exp(n ln T_e - C / T_e) with ln T_e = s ln T + (1 - s) ln T_ve from the logs of the subcycle
// (rate_constant.d:72-75, 364-393 evaluate the same expression with three pow calls and an exp).
// Temperatures enter as reciprocals (rT = 1 / T), formed once per subcycle where the reference divides.
__device__ double base_rc(int model, const double* d, double rT, double lnT, double lnTve) {
    if (model == RATE_PARK) {
        const double lnTe = d[RD_S] * lnT + (1.0 - d[RD_S]) * lnTve;
        return d[0] * ex(d[1] * lnTe - d[2] * ex(-lnTe));
    }
    return d[0] * ex(d[1] * lnT - d[2] * rT);
}

// rate_constant.d:397-404 at the temperature whose reciprocal is rT
__device__ __forceinline__ double Q_mt(double rT, double D, double theta) {
    const double num = 1 - ex(-D * rT);
    const double den = 1 - ex(-theta * rT);
    return num / den;
}

// Forward rate constant of reaction ir at (T, T_ve): Arrhenius, Park, or the (modified) Marrone-Treanor
// non-equilibrium factor times the underlying one (rate_constant.d:438-447, 541-554).
__device__ double forward_rc(const int* r, const double* d, double rT, double rTve, double lnT, double lnTve) {
    const int model = r[RX_FRC];
    if (model != RATE_MT && model != RATE_MMT) return base_rc(model, d, rT, lnT, lnTve);
    const double kEQ = base_rc(r[RX_BASE], d, rT, lnT, lnTve);
    const double TD = d[RD_MT_TD], th = d[RD_MT_THETA];
    if (model == RATE_MT) {
        const double rU = 1. / d[RD_MT_U];
        const double rGamma = rTve - rT - rU;   // 1 / Gamma
        const double Q_T = Q_mt(rT, TD, th), Q_Gamma = Q_mt(rGamma, TD, th), Q_Tv = Q_mt(rTve, TD, th),
                     Q_U = Q_mt(-rU, TD, th);
        return kEQ * Q_T * Q_Gamma / (Q_Tv * Q_U);
    }
    const double Uinv = d[RD_MT_U] * rT + 1. / d[RD_MT_USTAR];
    const double rTF = rTve - rT - Uinv;   // 1 / T_F
    const double Q_T = Q_mt(rT, TD, th), Q_TF = Q_mt(rTF, TD, th), Q_Tv = Q_mt(rTve, TD, th),
                 Q_U = Q_mt(-Uinv, TD, th);
    return d[RD_MT_NB] * kEQ * Q_T * Q_TF / (Q_Tv * Q_U);
}

struct Reactor2T {
    Gas2T g;
    const Eem2T* eem;
    int neem;
    double tol;
    int max_subcycles, max_attempts;

    // reaction.d:94-143 (multi-temperature branch) at the clamped T; gs: Gibbs scratch [nsp]
    // logTq, logTve: ln Tq and ln T_ve (Tq unclamped), which the caller needs as well.
    __device__ void rate_constants(double Tq, double Tve, double logTq, double logTve, double* kf, double* kb,
                                   double* gs, int& err) const {
        const MechView& m = g.m;
        double T = Tq, logT = logTq;
        if (T < m.T_lower()) { T = m.T_lower(); logT = log(T); }
        if (T > m.T_upper()) { T = m.T_upper(); logT = log(T); }
        const double lnPRT = LN_PATM_R - logT;   // ln(P_atm / R T)
        const double rT = 1.0 / T, rTve = 1.0 / Tve;
        for (int i = 0; i < m.nsp; ++i) gs[i] = cea_h_r(m, i, T, rT, logT, err) - T * cea_s_r(m, i, T, rT, logT, err);
        for (int ir = 0; ir < m.nr; ++ir) {
            const int* r = m.rx(ir);
            const double* d = m.rxd(ir);
            double lnKc = 0.0;
            if (r[RX_FRC] == RATE_FROM_EQ || r[RX_BRC] == RATE_FROM_EQ) {
                double dG = 0.0, nuSum = 0.0;
                for (int k = 0; k < r[RX_NPART]; ++k) {
                    const int isp = r[RX_PART + k], nu = r[RX_PART_NU + k];
                    dG += nu * gs[isp] * m.sp(isp)[SP_M];
                    nuSum += nu;
                }
                // ln of K_p (P_atm / R T)^sum(nu) (reaction.d:26-52)
                lnKc = fma(nuSum, lnPRT, -dG * (rT * (1.0 / R_universal)));
            }
            if (r[RX_FRC] != RATE_FROM_EQ) {
                kf[ir] = forward_rc(r, d, rT, rTve, logT, logTve);
                kb[ir] = (r[RX_BRC] == RATE_FROM_EQ) ? forward_rc(r, d, rT, rT, logT, logT) * ex(-lnKc)
                                                     : d[3] * ex(d[4] * logT - d[5] * rT);
            } else {
                kb[ir] = d[3] * ex(d[4] * logT - d[5] * rT);
                kf[ir] = kb[ir] * ex(lnKc);   // the backward rate constant at the state itself (reaction.d:131)
            }
        }
    }

    // Tick rates at conc into wf, wb, and q, L (reaction_mechanism.d:82-95).
    __device__ void split_rates(const double* c, const double* kf, const double* kb, double* wf, double* wb,
                                double* q, double* L) const {
        const MechView& m = g.m;
        for (int i = 0; i < m.nsp; ++i) { q[i] = 0.0; L[i] = 0.0; }
        for (int ir = 0; ir < m.nr; ++ir) {
            const int* r = m.rx(ir);
            double mc = 1.0;
            if (r[RX_COLLIDER]) {
                const int* ei = m.eff_i(r[RX_EFFSET]);
                const double* ev = m.eff_d(r[RX_EFFSET]);
                mc = 0.0;
                for (int k = 0; k < ei[0]; ++k) mc += ev[ei[1 + k]] * c[ei[1 + k]];
            }
            double f = kf[ir] * mc, b = kb[ir] * mc;
            for (int k = 0; k < r[RX_NREAC]; ++k) f *= pow_int(c[r[RX_REAC_IDX + k]], r[RX_REAC_COEFF + k]);
            for (int k = 0; k < r[RX_NPROD]; ++k) b *= pow_int(c[r[RX_PROD_IDX + k]], r[RX_PROD_COEFF + k]);
            wf[ir] = f;
            wb[ir] = b;
            for (int k = 0; k < r[RX_NPART]; ++k) {
                const int isp = r[RX_PART + k], nu = r[RX_PART_NU + k];
                if (nu > 0) { q[isp] += nu * f; L[isp] += nu * b; }
                else if (nu < 0) { q[isp] += -nu * b; L[isp] += -nu * f; }
            }
        }
    }

    __device__ double nu_of(int ir, int isp) const {
        const int* r = g.m.rx(ir);
        for (int k = 0; k < r[RX_NPART]; ++k)
            if (r[RX_PART + k] == isp) return (double)r[RX_PART_NU + k];
        return 0.0;
    }

    // Relaxation time of a Landau-Teller mechanism (relaxation_time.d:27-175); -1 for a rare collider.
    // T13 = T^(-1/3), formed once per subcycle.
    __device__ double tau(const Eem2T& e, double T, double T13, double p, const double* molef,
                          const double* numden) const {
        if (molef[e.q] <= SMALL_MOLE_FRACTION) return -1.0;
        const double pBath = molef[e.q] * p / P_atm;
        const double t_mw = (1.0 / pBath) * ex(e.a * (T13 - e.b) - 18.42);
        if (e.rt == RT_MILLIKAN_WHITE) return t_mw;
        const double sigma = (e.rt == RT_PARK_HTC) ? e.sigma : e.sigma * (50e3 / T) * (50e3 / T);
        const double cs = sqrt(8.0 * Boltzmann * T / PI_D / e.mu);
        return t_mw + 1.0 / (sigma * cs * numden[e.q]);
    }

    // Knab's equation (39) and its small-iG and overflow forms (exchange_chemistry_coupling.d:41-69).
    __device__ static double L_knab(double iG, double D, double Th) {
        if (fabs(iG) < IGAMMA_SWITCH)
            return 0.5 * (D - Th * R_universal) + iG * (Th * Th * R_universal * R_universal - D * D) / 12.0 / R_universal;
        if (iG > IGAMMA_OVERFLOW)
            return R_universal * Th / (ex(Th * iG) - 1.0) - D * ex(-D / R_universal * iG);
        return R_universal * Th / (ex(Th * iG) - 1.0) - D / (ex(D / R_universal * iG) - 1.0);
    }

    // Energy brought in (ga) and removed (gv) per dissociation at (T, T_ve), J/mol
    // (exchange_chemistry_coupling.d:94-126 impartial, 152-174 Marrone-Treanor, 204-220 modified).
    // rT = 1 / T, rTv = 1 / T_v
    __device__ static void coupling(const Eem2T& e, double rT, double rTv, double& ga, double& gv) {
        const double th = e.Thetav;
        if (e.coupling == CPL_IMPARTIAL) {
            ga = 0.5 * (e.D - th * R_universal);
            gv = L_knab(rTv - rT, e.D, th);   // (T - T_v) / (T T_v)
        } else if (e.coupling == CPL_MARRONE_TREANOR) {
            gv = L_knab(rTv - rT - 1. / e.U, e.D, th);
            const double T_F_inv = -1. / e.U;
            ga = R_universal * th / (ex(th * T_F_inv) - 1.) - e.D / (ex(e.D / R_universal * T_F_inv) - 1.);
        } else {
            const double TD = e.D;
            const double Uinv = e.aU * rT + 1 / e.Ustar;
            double T_F_inv = rTv - rT - Uinv;
            gv = R_universal * (th / (ex(th * T_F_inv) - 1.) - TD / (ex(TD * T_F_inv) - 1.)) + e.nb * R_universal * TD;
            T_F_inv = -e.aU * rT - 1 / e.Ustar;
            ga = R_universal * (th / (ex(th * T_F_inv) - 1.) - TD / (ex(TD * T_F_inv) - 1.));
        }
    }

    // dy/dt at y (species rates and the energy exchange into u_ve); lt[k]: the Landau-Teller term of
    // mechanism k on this subcycle's state (0 for others); ga[k], gv[k]: its Marrone-Treanor G_appear and
    // G_vanish on that state; rrho = 1 / rho.
    __device__ void rates(const double* y, const double* kf, const double* kb, const double* lt, const double* ga,
                          const double* gv, double rrho, double* wf, double* wb, double* q, double* L,
                          double* out) const {
        const int nsp = g.m.nsp;
        split_rates(y, kf, kb, wf, wb, q, L);
        for (int i = 0; i < nsp; ++i) out[i] = q[i] - L[i];
        double rate = 0.0;
        for (int k = 0; k < neem; ++k) {
            const Eem2T& e = eem[k];
            if (e.kind == EEM_LANDAU_TELLER) {
                rate += lt[k];
            } else {
                const double nu = nu_of(e.reaction, e.p);
                const double f = wf[e.reaction], b = wb[e.reaction];
                const double prod = nu > 0 ? nu * f : (nu < 0 ? -nu * b : 0.0);
                const double loss = nu > 0 ? nu * b : (nu < 0 ? -nu * f : 0.0);
                rate += (prod * ga[k] - loss * gv[k]) * rrho;
            }
        }
        out[nsp] = rate;
    }
};

// One thread per cell in a persistent grid.  All 32 lanes of a warp stay in the loop until the warp is out
// of work, and every loop iteration is one RKF attempt (preceded, where a lane starts a cell or a subcycle,
// by that work) for every lane that holds a cell; lanes whose cell is done take the next cells from a
// work counter, one atomic per warp.  Cells of uneven attempt counts then keep the lanes busy, where a
// fixed cell per thread would leave a warp's lanes idle until its slowest cell finishes.  The operations
// per cell are those of the subcycle and attempt loops of multi_temperature_thermochemical_reactor.d:137-294.
__global__ void __launch_bounds__(128) two_temperature_update_kernel(const TwoTArgs a) {
    for (int k = threadIdx.x; k < GDTK_EXP2_TABLE_SIZE; k += blockDim.x) s_exp2[k] = kExp2Table[k];
    __syncthreads();
    Reactor2T R;
    R.g.m.bind(a.mech_i, a.mech_d);
    R.g.sp = a.species;
    R.g.electron = a.electron;
    R.eem = a.eem;
    R.neem = a.neem;
    R.tol = a.tol;
    R.max_subcycles = a.max_subcycles;
    R.max_attempts = a.max_attempts;
    const MechView& m = R.g.m;
    const int nsp = m.nsp, nv = nsp + 1;
    const double tI = a.t_interval;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned long long my_steps = 0;
    double Y[GDTK_MAX_SPECIES], y0[NV], yOut[NV], yT[NV], K[6][NV], yErr[NV];
    double kf[GDTK_MAX_REACTIONS], kb[GDTK_MAX_REACTIONS], wf[GDTK_MAX_REACTIONS], wb[GDTK_MAX_REACTIONS];
    double q[GDTK_MAX_SPECIES], L[GDTK_MAX_SPECIES], gs[GDTK_MAX_SPECIES], lt[MAX_EEM], ga[MAX_EEM], gv[MAX_EEM];
    double molef[GDTK_MAX_SPECIES], numden[GDTK_MAX_SPECIES];
    int c = 0, phase = 0, cycle = 0, attempt = 0, fail = 0, err = 0;
    bool have = false, alive = true;
    double rho = 0.0, rrho = 0.0, T = 0.0, Tve = 0.0, p = 0.0, t = 0.0, h = 0.0, dt_suggest = 0.0, dtSave = 0.0;
    double u_total = 0.0, u = 0.0, u_ve = 0.0;
    while (true) {
        const unsigned need = __ballot_sync(FULL, alive && !have);
        if (need) {   // refill: one atomic per warp for all lanes that need a cell
            const int leader = __ffs(need) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (alive && !have) {
                const unsigned pos = base + __popc(need & ((1u << lane) - 1u));
                if (pos >= (unsigned)a.ncell) {
                    alive = false;
                } else {
                    c = (int)pos;
                    have = true;
                    phase = 0;
                }
            }
        }
        if (!__any_sync(FULL, alive || have)) break;
        if (have) {
            bool done = false;
            if (phase == 0) {   // the cell's state and first step size
                rho = a.rho[c];
                rrho = 1.0 / rho;
                T = a.T[c]; Tve = a.Tve[c]; p = a.p[c];
                for (int i = 0; i < nsp; ++i) Y[i] = a.massf[(size_t)i * a.ncell + c];
                fail = 0; err = 0;
                dt_suggest = a.dt_chem[c]; dtSave = dt_suggest; u = 0.0; u_ve = 0.0;
                if (isnan(rho) || rho <= 0.0) {
                    fail = CELL_BAD_INPUT;
                } else {
                    u_total = R.g.e_tr_mix(Y, T) + R.g.e_ve_mix(Y, Tve, err);
                    t = 0.0;
                    for (int i = 0; i < nsp; ++i) {
                        const double v = Y[i] * rho / m.sp(i)[SP_M];
                        y0[i] = v < 1.0e-30 ? 0.0 : v;   // gas_model.d:237-256
                    }
                    y0[nsp] = R.g.e_ve_mix(Y, Tve, err);
                    R.rate_constants(T, Tve, log(T), log(Tve), kf, kb, gs, err);
                    if (dt_suggest > tI) {
                        h = tI;
                    } else if (dt_suggest <= 0.0) {   // reaction_mechanism.d:161-203
                        R.split_rates(y0, kf, kb, wf, wb, q, L);
                        double min_dt = 1.0e6;
                        for (int i = 0; i < nsp; ++i) {
                            if (y0[i] > 0.0 && fabs(q[i] - L[i]) > 1.0e-30) {
                                const double dt = (q[i] > 10000.0 * L[i]) ? y0[i] / (L[i] + 1.0e-50)
                                                                          : fabs(y0[i] / (q[i] - L[i]));
                                min_dt = fmin(min_dt, dt);
                            }
                        }
                        h = fmax(fmin(1.0e-3 * min_dt, 1.0e-10), 1.0e-15);
                    } else {
                        h = dt_suggest;
                    }
                    cycle = 0;
                    phase = 1;
                    if (R.max_subcycles <= 0) fail = CELL_MAX_SUBCYCLES;
                }
            }
            if (!fail && phase == 1) {   // a subcycle's rate constants, relaxation times and exchange terms
                const double logT = log(T), logTve = log(Tve), T13 = ex(logT * (-1. / 3.));
                const double rT = 1.0 / T, rTve = 1.0 / Tve;
                R.rate_constants(T, Tve, logT, logTve, kf, kb, gs, err);
                double mol = 0.0;
                // 1 / M_i = R_i / R_universal
                for (int i = 0; i < nsp; ++i) mol += Y[i] * (m.sp(i)[SP_R] * (1.0 / R_universal));
                const double rmol = 1.0 / mol;
                for (int i = 0; i < nsp; ++i) {
                    const double n_i = Y[i] * (m.sp(i)[SP_R] * (1.0 / R_universal));
                    molef[i] = n_i * rmol;
                    numden[i] = Avogadro * rho * n_i;
                }
                unsigned have_de = 0;   // species whose e_ve(T) - e_ve(T_ve) is in q (free until the attempt)
                for (int k = 0; k < R.neem; ++k) {
                    const Eem2T& e = R.eem[k];
                    lt[k] = 0.0;
                    ga[k] = 0.0;
                    gv[k] = 0.0;
                    if (e.kind == EEM_LANDAU_TELLER) {
                        const double tk = R.tau(e, T, T13, p, molef, numden);
                        if (tk >= 0.0) {
                            if (!((have_de >> e.p) & 1u)) {
                                q[e.p] = R.g.e_ve(e.p, T, rT, logT, err) - R.g.e_ve(e.p, Tve, rTve, logTve, err);
                                have_de |= 1u << e.p;
                            }
                            lt[k] = Y[e.p] * q[e.p] / tk;
                        }
                    } else {
                        Reactor2T::coupling(e, rT, rTve, ga[k], gv[k]);
                    }
                }
                dtSave = dt_suggest;
                h = fmin(h, tI - t);
                attempt = 0;
                phase = 2;
                if (R.max_attempts <= 0) fail = CELL_MAX_ATTEMPTS;
            }
            if (!fail && phase == 2) {   // one Cash-Karp attempt (multi_temperature_thermochemical_reactor.d:334-431)
                const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10.,
                             a43 = 6. / 5., a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27.,
                             a61 = 1631. / 55296., a62 = 175. / 512., a63 = 575. / 13824.,
                             a64 = 44275. / 110592., a65 = 253. / 4096.;
                const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771.,
                             b41 = 2825. / 27648., b43 = 18575. / 48384., b44 = 13525. / 55296.,
                             b45 = 277. / 14336., b46 = 1.0 / 4.0;
                R.rates(y0, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[0]);
                for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * a21 * K[0][i];
                R.rates(yT, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[1]);
                for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * (a31 * K[0][i] + a32 * K[1][i]);
                R.rates(yT, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[2]);
                for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * (a41 * K[0][i] + a42 * K[1][i] + a43 * K[2][i]);
                R.rates(yT, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[3]);
                for (int i = 0; i < nv; ++i)
                    yT[i] = y0[i] + h * (a51 * K[0][i] + a52 * K[1][i] + a53 * K[2][i] + a54 * K[3][i]);
                R.rates(yT, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[4]);
                for (int i = 0; i < nv; ++i)
                    yT[i] = y0[i] + h * (a61 * K[0][i] + a62 * K[1][i] + a63 * K[2][i] + a64 * K[3][i] +
                                         a65 * K[4][i]);
                R.rates(yT, kf, kb, lt, ga, gv, rrho, wf, wb, q, L, K[5]);
                for (int i = 0; i < nv; ++i)
                    yOut[i] = y0[i] + h * (b51 * K[0][i] + b53 * K[2][i] + b54 * K[3][i] + b56 * K[5][i]);
                for (int i = 0; i < nv; ++i)
                    yErr[i] = yOut[i] - (y0[i] + h * (b41 * K[0][i] + b43 * K[2][i] + b44 * K[3][i] +
                                                      b45 * K[4][i] + b46 * K[5][i]));
                double e2 = 0.0;
                for (int i = 0; i < nv; ++i) {
                    const double sk = R.tol + R.tol * fmax(fabs(y0[i]), fabs(yOut[i]));
                    e2 += (yErr[i] / sk) * (yErr[i] / sk);
                }
                const double en = sqrt(e2 / nv);
                bool ok;
                if (en <= 1.0) {
                    double scale = (en == 0.0) ? 10.0 : 0.9 * pow(en, -0.2);
                    if (en != 0.0) scale = fmin(fmax(scale, 0.2), 10.0);
                    dt_suggest = scale * h;
                    ok = true;
                } else {
                    dt_suggest = fmax(0.9 * pow(en, -0.2), 0.2) * h;
                    ok = false;
                }
                ++my_steps;
                bool passed = true;
                if (ok) {
                    double tot = 0.0;
                    for (int i = 0; i < nsp; ++i) {
                        const double v = yOut[i] * m.sp(i)[SP_M] * rrho;
                        Y[i] = v < 1.0e-30 ? 0.0 : v;   // conc2massf (gas_model.d:258-271)
                        tot += Y[i];
                    }
                    if (fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) passed = false;
                }
                if (ok && passed) {   // the attempt ends the subcycle
                    t += h;
                    for (int i = 0; i < nv; ++i) y0[i] = yOut[i];
                    const double hMax = h * (1.0 + 10.0 / 100.0);
                    if (dt_suggest > h) h = fmin(dt_suggest, hMax);
                    u_ve = y0[nsp];
                    u = u_total - u_ve;
                    if (!R.g.from_rhou(rho, u, u_ve, Y, T, Tve, p)) {
                        fail = CELL_NEWTON_FAIL;
                    } else if (t >= tI) {
                        if (cycle == 0) dtSave = dt_suggest;
                        done = true;
                    } else if (++cycle == R.max_subcycles) {
                        fail = CELL_MAX_SUBCYCLES;
                    } else {
                        phase = 1;
                    }
                } else {
                    h /= 10.0;
                    if (h < H_MIN) fail = CELL_H_MIN;
                    else if (++attempt == R.max_attempts) fail = CELL_MAX_ATTEMPTS;
                }
            }
            if (done && err) { fail = CELL_CEA_RANGE; done = false; }
            if (fail) {
                if (a.status) a.status[c] = fail;
                have = false;
            } else if (done) {
                double tot = 0.0;
                for (int i = 0; i < nsp; ++i) tot += Y[i];
                for (int i = 0; i < nsp; ++i) a.massf[(size_t)i * a.ncell + c] = Y[i] / tot;
                a.T[c] = T;
                a.Tve[c] = Tve;
                a.p[c] = p;
                if (a.u) a.u[c] = u;
                if (a.u_ve) a.u_ve[c] = u_ve;
                a.dt_chem[c] = dtSave;
                if (a.status) a.status[c] = CELL_OK;
                have = false;
            }
        }
        __syncwarp(FULL);
    }
    if (a.steps && my_steps) atomicAdd(a.steps, my_steps);
}

__global__ void two_temperature_thermo_pT_kernel(const Thermo2TArgs a) {
    Gas2T g;
    g.m.bind(a.mech_i, a.mech_d);
    g.sp = a.species;
    g.electron = a.electron;
    const int nsp = g.m.nsp;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.ncell; c += gridDim.x * blockDim.x) {
        double Y[GDTK_MAX_SPECIES];
        for (int i = 0; i < nsp; ++i) Y[i] = a.massf[(size_t)i * a.ncell + c];
        const double T = a.T[c], Tve = a.Tve[c];
        double denom = 0.0;   // two_temperature_gas.d updateDensity
        for (int i = 0; i < nsp; ++i) denom += Y[i] * g.R(i) * (i == g.electron ? Tve : T);
        int err = 0;
        a.rho[c] = a.p[c] / denom;
        a.u[c] = g.e_tr_mix(Y, T);
        a.u_ve[c] = g.e_ve_mix(Y, Tve, err);
    }
}

int grid_for_cells(int n, int block, int sm_count) {
    long long g = ((long long)n + block - 1) / block;
    const long long cap = (long long)sm_count * 16;
    if (g > cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

}  // namespace

cudaError_t launch_two_temperature_update(const TwoTArgs& a, int sm_count, cudaStream_t s) {
    if (a.ncell <= 0) return cudaSuccess;
    if (a.neem > MAX_EEM || !a.counter) return cudaErrorInvalidValue;
    // a persistent grid: as many blocks as are resident at once, the cells taken from the work counter
    static int per_sm = 0;
    if (per_sm <= 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, two_temperature_update_kernel, 128, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    long long grid = (long long)sm_count * per_sm;
    const long long want = ((long long)a.ncell + 127) / 128;
    if (grid > want) grid = want;
    cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    two_temperature_update_kernel<<<(unsigned)(grid < 1 ? 1 : grid), 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_two_temperature_thermo_pT(const Thermo2TArgs& a, int sm_count, cudaStream_t s) {
    if (a.ncell <= 0) return cudaSuccess;
    two_temperature_thermo_pT_kernel<<<grid_for_cells(a.ncell, 128, sm_count), 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gdtk
