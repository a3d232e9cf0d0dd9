// chem_kernels.cu -- FP64 chemistry-update kernels for sm_103a (reference-order arithmetic).
//
// One thread integrates one cell.  A block stages the packed mechanism (chem_types.h) into
// shared memory once; each thread's working vectors (concentrations, rate constants, stage
// values) also live in shared memory, lane-interleaved so that the 32 lanes of a warp touch
// 32 consecutive 8-byte words (no bank conflicts).  The grid is persistent: threads pull
// cells from a device work counter, and a thread whose cell finishes takes the next one
// while its neighbours carry on, so cells of very different step counts share warps without
// idling them.  Each loop iteration of a thread is one ODE attempt, so all lanes of a warp
// run the same code (rate constants -> ODE step -> step control) in lock-step.
//
// The arithmetic restates the reference in its evaluation order (this file is compiled with
// --fmad=false so that a*b+c keeps two roundings, as the reference's x86-64 build does):
//   kinetics/chemistry_update.d        opCall 139-326, RKFStep 404-478, AlphaQssStep 533-655
//   kinetics/reaction_mechanism.d      eval_rate_constants 49-63, eval_split_rates 82-96,
//                                      estimateStepSize 161-203, eval_gibbs_free_energies 204-218
//   kinetics/reaction.d                compute_equilibrium_constant 26-52, eval_rate_constants 94-143,
//                                      tick rates and production/loss 145-149, 267-311, 393-456
//   kinetics/rate_constant.d           ArrheniusRateConstant.eval 72-75
//   gas/thermo/cea_thermo_curves.d     eval_Cp/eval_h/eval_s 55-137, determineCoefficients 149-182
//   gas/thermo/therm_perf_gas_mix.d    GibbsFreeEnergies 354-364, update_temperature_from_energy 426-468
//   gas/gas_model.d                    massf2conc 237-253, conc2massf 255-271, rates2source 273-279
//   lmr/fluidfvcell.d                  thermochemical_increment 883-997 (caller contract)
//
// The one-warp-per-cell update (the last section) is compiled separately, from chem_warp.cu with
// GDTK_WARP_TU = 1 and FMA contraction; this translation unit (GDTK_WARP_TU = 0) holds the rest.
#include <cuda_runtime.h>

#include "chem_types.h"
#include "chem_launch.h"
#include "cea_thermo.h"
#include "mix_thermo.cuh"

#ifndef GDTK_WARP_TU
#define GDTK_WARP_TU 0
#endif
#if GDTK_WARP_TU
#include "fast_exp.h"
#endif

namespace gdtk {
namespace {

constexpr double R_universal = 8.31451;   // gas/physical_constants.d:13
constexpr double P_atm = 101.325e3;       // gas/physical_constants.d:16
constexpr double MIN_MOLES = 1.0e-30;     // gas/gas_model.d:43
constexpr double MIN_MASS_FRACTION = 1.0e-30;
constexpr double DT_INCREASE_PERCENT = 10.0;   // chemistry_update.d:23-31
constexpr double DT_REDUCTION_FACTOR = 10.0;
constexpr double H_MIN = 1.0e-15;
constexpr double ALLOWABLE_MASSF_ERROR = 1.0e-3;
constexpr double ZERO_EPS = 1.0e-50;

// D's pow(double, int) (std.math, binary exponentiation), in double.
__device__ __forceinline__ double ipow(double x, int n) {
    if (n < 0) {
        if (n == -1) return 1.0 / x;
        unsigned m = (unsigned)(-n);
        double p = 1.0, v = p / x;
        while (true) { if (m & 1u) p *= v; m >>= 1; if (!m) break; v *= v; }
        return p;
    }
    if (n == 0) return 1.0;
    if (n == 1) return x;
    if (n == 2) return x * x;
    unsigned m = (unsigned)n;
    double p = 1.0, v = x;
    while (true) { if (m & 1u) p *= v; m >>= 1; if (!m) break; v *= v; }
    return p;
}

// ---------------------------------------------------------------- kinetics
__device__ __forceinline__ double arrhenius(double A, double n, double C, double T) {   // rate_constant.d:72-75
    return A * pow(T, n) * exp(-C / T);
}

// Arrhenius (rate_constant.d:72-75) or Arrhenius2 (112-115) from the record's three parameters.
__device__ __forceinline__ double simple_rate(int model, const double* p, double T) {
    if (model == RATE_ARRHENIUS2) return exp(p[0] + p[1] * T - p[2] / T);
    return p[0] * pow(T, p[1]) * exp(-p[2] / T);
}

// Forward rate constant of a pressure-dependent reaction: the third-body concentration of its
// efficiency list from the gas state's mass fractions (rate_constant.d:114-121), then
// Lindemann-Hinshelwood (155-160), Troe (258-287) or Yungster-Rabinowitz (338-350).
__device__ double pressure_dependent_kf(const MechView& m, const int* r, const double* d, double T, Vec mf,
                                        double rho) {
    const int* ei = m.eff_i(r[RX_EFFSET]);
    const double* ev = m.eff_d(r[RX_EFFSET]);
    double M = 0.0;
    for (int k = 0; k < ei[0]; ++k) {
        const int isp = ei[1 + k];
        M += ev[isp] * (mf[isp] * rho / m.sp(isp)[SP_M]);
    }
    const double kInf = arrhenius(d[0], d[1], d[2], T);
    const double k0 = arrhenius(d[RD_K0A], d[RD_K0N], d[RD_K0C], T);
    if (r[RX_FRC] == RATE_LH) return k0 * kInf * M / (k0 * M + kInf);
    const double essentially_zero = 1.0e-30;
    if (r[RX_FRC] == RATE_TROE) {
        const double p_r = k0 * M / kInf;
        const double log_p_r = log10(fmax(p_r, essentially_zero));
        const int fl = (int)d[RD_TFLAGS];
        double Fcent = d[RD_FCENT];
        if (!(fl & TROE_FCENT)) {
            Fcent = (1.0 - d[RD_TA]) * exp(-T / d[RD_T3]);
            if (fl & TROE_T1) Fcent += d[RD_TA] * exp(-T / d[RD_T1]);
            if (fl & TROE_T2) Fcent += exp(-d[RD_T2] / T);
        }
        const double log_F_cent = log10(fmax(Fcent, essentially_zero));
        const double c = -0.4 - 0.67 * log_F_cent;
        const double n = 0.75 - 1.27 * log_F_cent;
        const double dd = 0.14;
        const double numer = log_p_r + c;
        const double denom = n - dd * numer;
        const double frac = numer / denom;
        const double log_F = log_F_cent / (1.0 + frac * frac);
        const double F = pow(10.0, log_F);
        return F * k0 * kInf * M / (k0 * M + kInf);
    }
    const double p_r = k0 * M / kInf;   // Yungster-Rabinowitz
    const double log_p_r = log(p_r);
    const double Fc = d[RD_TA] * exp(-d[RD_T1] / T) + (1.0 - d[RD_TA]) * exp(-d[RD_T2] / T);
    const double xt = 1.0 / (1.0 + log_p_r * log_p_r);
    return kInf * (p_r / (1.0 + p_r)) * Fc * xt;
}

// reaction_mechanism.d:49-63 with Gibbs energies at P_atm (:204-218, therm_perf_gas_mix.d:354-364),
// reaction.d:26-52 and 94-143 for a single-temperature gas.  g is scratch of nsp doubles; mf and
// rho are the gas state's mass fractions and density (third bodies of pressure-dependent rates).
__device__ void rate_constants(const MechView& m, double Tq, Vec kf, Vec kb, Vec g, Vec mf, double rho, int& err) {
    double T = Tq;
    if (T < m.T_lower()) T = m.T_lower();
    if (T > m.T_upper()) T = m.T_upper();
    const double logT = log(T);
    // logp = log(P_atm/P_atm) = 0 and s - R*0 = s exactly, so the pressure term is omitted.
    for (int i = 0; i < m.nsp; ++i) {
        double h = cea_h(m, i, T, logT, err);
        double s = cea_s(m, i, T, logT, err);
        g[i] = h - T * s;
    }
    for (int ir = 0; ir < m.nr; ++ir) {
        const int* r = m.rx(ir);
        const double* d = m.rxd(ir);
        double Kc = 1.0;
        if (r[RX_FRC] == RATE_FROM_EQ || r[RX_BRC] == RATE_FROM_EQ) {
            double dG = 0.0, nuSum = 0.0;
            for (int k = 0; k < r[RX_NPART]; ++k) {
                int isp = r[RX_PART + k];
                int nu = r[RX_PART_NU + k];
                dG += nu * g[isp] * m.sp(isp)[SP_M];
                nuSum += nu;
            }
            double K_p = exp(-dG / (R_universal * T));
            Kc = K_p * ipow(P_atm / (R_universal * T), (int)nuSum);
        }
        if (r[RX_FRC] != RATE_FROM_EQ) {
            double f = (r[RX_FRC] == RATE_ARRHENIUS || r[RX_FRC] == RATE_ARRHENIUS2)
                           ? simple_rate(r[RX_FRC], d, T) : pressure_dependent_kf(m, r, d, T, mf, rho);
            kf[ir] = f;
            kb[ir] = (r[RX_BRC] == RATE_FROM_EQ) ? f / Kc : simple_rate(r[RX_BRC], d + 3, T);
        } else {
            double b = simple_rate(r[RX_BRC], d + 3, T);
            kb[ir] = b;
            kf[ir] = b * Kc;
        }
    }
}

// Third-body sums of the distinct efficiency lists (identical lists are summed once; the
// sum for each list is in the reference's order, reaction.d:450-456).
__device__ __forceinline__ void collider_terms(const MechView& m, Vec c, Vec meff) {
    for (int s = 0; s < m.neff; ++s) {
        const int* ei = m.eff_i(s);
        const double* ev = m.eff_d(s);
        double term = 0.0;
        for (int k = 0; k < ei[0]; ++k) {
            int isp = ei[1 + k];
            term += ev[isp] * c[isp];
        }
        meff[s] = term;
    }
}

// reaction_mechanism.d:82-96: per-reaction tick rates, then q/L accumulation in reaction order.
__device__ void split_rates(const MechView& m, Vec c, Vec q, Vec L, Vec kf, Vec kb, Vec meff) {
    collider_terms(m, c, meff);
    for (int i = 0; i < m.nsp; ++i) { q[i] = 0.0; L[i] = 0.0; }
    for (int ir = 0; ir < m.nr; ++ir) {
        const int* r = m.rx(ir);
        double wf = kf[ir], wb = kb[ir];
        if (r[RX_COLLIDER]) { double t = meff[r[RX_EFFSET]]; wf = wf * t; wb = wb * t; }
        for (int k = 0; k < r[RX_NREAC]; ++k) wf *= ipow(c[r[RX_REAC_IDX + k]], r[RX_REAC_COEFF + k]);
        for (int k = 0; k < r[RX_NPROD]; ++k) wb *= ipow(c[r[RX_PROD_IDX + k]], r[RX_PROD_COEFF + k]);
        for (int k = 0; k < r[RX_NPART]; ++k) {
            int isp = r[RX_PART + k];
            int nu = r[RX_PART_NU + k];
            if (nu > 0) { q[isp] += nu * wf; L[isp] += nu * wb; }
            else if (nu < 0) { q[isp] += -nu * wb; L[isp] += -nu * wf; }
        }
    }
}

// Tick rates only (reaction_mechanism.d:65-73).
__device__ void tick_rates(const MechView& m, Vec c, Vec kf, Vec kb, Vec meff, double* wf_out, double* wb_out,
                           int stride) {
    collider_terms(m, c, meff);
    for (int ir = 0; ir < m.nr; ++ir) {
        const int* r = m.rx(ir);
        double wf = kf[ir], wb = kb[ir];
        if (r[RX_COLLIDER]) { double t = meff[r[RX_EFFSET]]; wf = wf * t; wb = wb * t; }
        for (int k = 0; k < r[RX_NREAC]; ++k) wf *= ipow(c[r[RX_REAC_IDX + k]], r[RX_REAC_COEFF + k]);
        for (int k = 0; k < r[RX_NPROD]; ++k) wb *= ipow(c[r[RX_PROD_IDX + k]], r[RX_PROD_COEFF + k]);
        wf_out[(size_t)ir * stride] = wf;
        wb_out[(size_t)ir * stride] = wb;
    }
}

// Phobos std.algorithm.sum (pairwise) over n doubles of a per-thread vector.
__device__ double sum_pairwise(Vec d, int n) {
    double store[8];
    int idx = 0;
    int pos = 0;
    auto collapse = [&](unsigned k) {
        int lastToKeep = idx - (__ffs((int)(k + 1)) - 1);
        while (idx > lastToKeep) { store[idx - 1] += store[idx]; --idx; }
    };
    for (unsigned k = 0; k < (unsigned)n / 16; ++k) {
        Vec x = d + pos;
        double s = (((x[0] + x[1]) + (x[2] + x[3])) + ((x[4] + x[5]) + (x[6] + x[7])))
                 + (((x[8] + x[9]) + (x[10] + x[11])) + ((x[12] + x[13]) + (x[14] + x[15])));
        store[idx] = s;
        pos += 16;
        collapse(k);
        ++idx;
    }
    unsigned i = 0;
    for (; pos < n; ++pos) { store[idx] = d[pos]; collapse(i); ++idx; ++i; }
    double s = store[idx - 1];
    for (int j = idx - 1; j-- > 0;) s += store[j];
    return 0.0 + s;
}

// reaction_mechanism.d:161-203 given the split rates at c.
__device__ double estimate_from_rates(int nsp, Vec c, Vec q, Vec L) {
    const double MUCH_LARGER_FACTOR = 10000.0, ZERO_TOL = 1.0e-30, EPS1 = 1.0e-3;
    double min_dt = 1.0e6, dt;
    for (int i = 0; i < nsp; ++i) {
        double ci = c[i], qi = q[i], Li = L[i];
        if (ci > 0.0 && (fabs(qi - Li) > ZERO_TOL)) {
            if (qi > MUCH_LARGER_FACTOR * Li) dt = ci / (Li + ZERO_EPS);
            else dt = fabs(ci / (qi - Li));
            min_dt = fmin(min_dt, dt);
        }
    }
    double dt_chem = EPS1 * min_dt;
    dt_chem = fmin(dt_chem, 1.0e-10);
    dt_chem = fmax(dt_chem, 1.0e-15);
    return dt_chem;
}

// ---------------------------------------------------------------- per-thread workspace
// Offsets (in doubles) into a thread's shared-memory vectors.
struct Layout {
    int y0, yout, q, L, kf, kb, meff, ext, total;
    __device__ __host__ void make(int nsp, int nr, int neff, int method) {
        y0 = 0; yout = nsp; q = 2 * nsp; L = 3 * nsp; kf = 4 * nsp; kb = kf + nr; meff = kb + nr;
        ext = meff + (neff > 0 ? neff : 1);
        total = ext + (method == METHOD_RKF ? 7 * nsp : 4 * nsp);
    }
};

// chemistry_update.d:404-478.  ext holds k1..k6 and yTmp.
__device__ bool rkf_step(const MechView& m, Vec y0, double h, Vec yOut, double& hSuggest, Vec q, Vec L, Vec kf,
                         Vec kb, Vec meff, Vec ext, int& nrhs) {
    const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10., a43 = 6. / 5.,
        a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27., a61 = 1631. / 55296., a62 = 175. / 512.,
        a63 = 575. / 13824., a64 = 44275. / 110592., a65 = 253. / 4096.;
    const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771., b41 = 2825. / 27648.,
        b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336., b46 = 1.0 / 4.0;
    const int n = m.nsp;
    Vec k1 = ext, k2 = ext + n, k3 = ext + 2 * n, k4 = ext + 3 * n, k5 = ext + 4 * n, k6 = ext + 5 * n,
        yT = ext + 6 * n;
    auto rates = [&](Vec c, Vec out) {
        split_rates(m, c, q, L, kf, kb, meff);
        ++nrhs;
        for (int i = 0; i < n; ++i) out[i] = q[i] - L[i];
    };
    rates(y0, k1);
    for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a21 * k1[i]);
    rates(yT, k2);
    for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a31 * k1[i] + a32 * k2[i]);
    rates(yT, k3);
    for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
    rates(yT, k4);
    for (int i = 0; i < n; ++i) yT[i] = y0[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
    rates(yT, k5);
    for (int i = 0; i < n; ++i)
        yT[i] = y0[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
    rates(yT, k6);
    const double atol = m.err_tol(), rtol = m.err_tol();
    double err = 0.0;
    for (int i = 0; i < n; ++i) {
        double yo = y0[i] + h * (b51 * k1[i] + b53 * k3[i] + b54 * k4[i] + b56 * k6[i]);
        yOut[i] = yo;
        double ye = yo - (y0[i] + h * (b41 * k1[i] + b43 * k3[i] + b44 * k4[i] + b45 * k5[i] + b46 * k6[i]));
        double sk = atol + rtol * fmax(fabs(y0[i]), fabs(yo));
        err += (ye / sk) * (ye / sk);
    }
    err = sqrt(err / n);
    const double maxscale = 10.0, minscale = 0.2, safe = 0.9, alpha = 0.2;
    double scale;
    if (err <= 1.0) {
        if (err == 0.0) scale = maxscale;
        else {
            scale = safe * pow(err, -alpha);
            if (scale < minscale) scale = minscale;
            if (scale > maxscale) scale = maxscale;
        }
        hSuggest = scale * h;
        return true;
    }
    scale = fmax(safe * pow(err, -alpha), minscale);
    hSuggest = scale * h;
    return false;
}

__device__ __forceinline__ double alpha_of(double p, double h) {   // chemistry_update.d:599-604
    double r = 1.0 / (p * h + ZERO_EPS);
    return (180.0 * r * r * r + 60.0 * r * r + 11.0 * r + 1.0) / (360.0 * r * r * r + 60.0 * r * r + 12.0 * r + 1.0);
}

// chemistry_update.d:533-655.  ext holds q0, p0, yp0, yp (yp becomes yc in place).
__device__ bool aqss_step(const MechView& m, Vec y0, double h, Vec yOut, double& hSuggest, Vec q, Vec L, Vec kf,
                          Vec kb, Vec meff, Vec ext, int& nrhs) {
    const int n = m.nsp;
    const double eps1 = m.eps1(), eps2 = m.eps2(), delta = m.delta();
    Vec q0 = ext, p0 = ext + n, yp0 = ext + 2 * n, yp = ext + 3 * n;
    split_rates(m, y0, q, L, kf, kb, meff);
    ++nrhs;
    for (int i = 0; i < n; ++i) {
        double y = y0[i];
        double qi = q[i];
        double pi = L[i] / (y + ZERO_EPS);
        double a = alpha_of(pi, h);
        double v = y + (h * (qi - pi * y)) / (1.0 + a * h * pi);
        q0[i] = qi; p0[i] = pi; yp[i] = v; yp0[i] = v;
    }
    bool converged = false;
    for (int corr = 0; corr < m.max_iters(); ++corr) {
        split_rates(m, yp, q, L, kf, kb, meff);
        ++nrhs;
        converged = true;
        for (int i = 0; i < n; ++i) {
            double y = y0[i];
            double pp = L[i] / (yp[i] + ZERO_EPS);
            double ab = alpha_of(pp, h);
            double qt = ab * q[i] + (1 - ab) * q0[i];
            double pb = 0.5 * (p0[i] + pp);
            double yc = y + (h * (qt - pb * y)) / (1.0 + ab * h * pb);
            yp[i] = yc;
            if (!(yc < ZERO_EPS)) {
                double test = fabs(yc - yp0[i]);
                if (test >= (eps1 * (yc + delta))) converged = false;
            }
        }
        if (converged) break;
    }
    // step_suggest (chemistry_update.d:629-655) with yc = yp, yp = yp0
    double sigma = 0.0;
    for (int i = 0; i < n; ++i) {
        double yc = yp[i];
        if (yc < ZERO_EPS) continue;
        double test = fabs(yc - yp0[i]) / (eps2 * (yc + delta));
        if (test > sigma) sigma = test;
    }
    double h_new;
    if (sigma <= 0.0) h_new = 10.0 * h;
    else {
        double x = sigma;
        x = x - 0.5 * (x * x - sigma) / x;
        x = x - 0.5 * (x * x - sigma) / x;
        x = x - 0.5 * (x * x - sigma) / x;
        h_new = h * ((1.0 / x) + 0.005);
    }
    hSuggest = h_new;
    if (converged)
        for (int i = 0; i < n; ++i) yOut[i] = yp[i];
    return converged;
}

__device__ __forceinline__ unsigned fetch_cell(unsigned* counter) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    unsigned rank = __popc(mask & ((1u << lane) - 1u));
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + rank;
}

__device__ void stage_mechanism(const int* gi, const double* gd, int ni, int nd, int*& si, double*& sd,
                                double*& scratch) {
    extern __shared__ double smem_d[];
    sd = smem_d;
    si = reinterpret_cast<int*>(smem_d + nd);
    for (int k = threadIdx.x; k < nd; k += blockDim.x) sd[k] = gd[k];
    for (int k = threadIdx.x; k < ni; k += blockDim.x) si[k] = gi[k];
    scratch = smem_d + nd + (ni + 1) / 2;
    __syncthreads();
}

#if !GDTK_WARP_TU
// ---------------------------------------------------------------- the chemistry update
template <int METHOD>
__global__ void __launch_bounds__(256) chem_update_kernel(ChemUpdateArgs a) {
    int* si;
    double* sd;
    double* scratch;
    stage_mechanism(a.mech_i, a.mech_d, a.n_mech_i, a.n_mech_d, si, sd, scratch);
    MechView m;
    m.bind(si, sd);
    Layout lay;
    lay.make(m.nsp, m.nr, m.neff, METHOD);
    Vec S{scratch + threadIdx.x, (int)blockDim.x};
    Vec y0 = S + lay.y0, yout = S + lay.yout, q = S + lay.q, L = S + lay.L, kf = S + lay.kf, kb = S + lay.kb,
        meff = S + lay.meff, ext = S + lay.ext;
    const int nsp = m.nsp;
    const unsigned ncell = (unsigned)a.ncell;
    const double tI = a.t_interval;

    unsigned c = 0;
    bool have = false, retried = false, need_kc = false, kc_from_input = false;
    int phase = 0, cycle = 0, attempt = 0, err = 0;
    double rho = 0, u = 0, T = 0, T0 = 0, p = 0, p0 = 0, dtS = 0, dtS0 = 0, dtSave = 0, h = 0, t = 0;
    int n_steps = 0, n_rhs = 0, n_kc = 0, n_newton = 0, n_rej = 0, n_est = 0;

    while (true) {
        if (!have) {
            c = fetch_cell(a.counter);
            if (c >= ncell) break;
            rho = a.rho[c]; u = a.u[c]; T0 = a.T[c]; p0 = a.p[c]; dtS0 = a.dt_chem[c];
            if (T0 <= a.T_frozen) {
                if (a.status) a.status[c] = CELL_FROZEN;
                continue;
            }
            if (isnan(rho) || rho <= 0.0) {
                if (a.status) a.status[c] = CELL_BAD_INPUT;
                continue;
            }
            have = true;
            retried = false;
            n_steps = n_rhs = n_kc = n_newton = n_rej = n_est = 0;
            phase = -1;
        }
        if (phase == -1) {   // (re)start the update from the stored input state
            T = T0; p = p0; dtS = dtS0; t = 0.0; err = 0;
            for (int i = 0; i < nsp; ++i) {
                double v = a.massf[(size_t)i * ncell + c] * rho / m.sp(i)[SP_M];
                y0[i] = (v < MIN_MOLES) ? 0.0 : v;
            }
            need_kc = true;
            kc_from_input = true;
            phase = 0;
        }
        if (need_kc) {
            // Q.massf at this point: the input mass fractions, or conc2massf of the last step (in q)
            rate_constants(m, T, kf, kb, L, kc_from_input ? Vec{a.massf + c, (int)ncell} : q, rho, err);
            kc_from_input = false;
            ++n_kc;
            need_kc = false;
        }
        if (phase == 0) {
            if (dtS > tI) h = tI;
            else if (dtS <= 0.0) {
                split_rates(m, y0, q, L, kf, kb, meff);
                ++n_rhs;
                ++n_est;
                h = estimate_from_rates(nsp, y0, q, L);
            } else h = dtS;
            cycle = 0;
            phase = 1;
        }
        if (phase == 1) {   // start of a subcycle
            dtSave = dtS;
            h = fmin(h, tI - t);
            attempt = 0;
            phase = 2;
        }
        // ---- one attempt of the ODE step
        ++n_steps;
        bool ok = (METHOD == METHOD_RKF) ? rkf_step(m, y0, h, yout, dtS, q, L, kf, kb, meff, ext, n_rhs)
                                         : aqss_step(m, y0, h, yout, dtS, q, L, kf, kb, meff, ext, n_rhs);
        if (ok) {   // mass-fraction test on conc2massf(concOut)
            for (int i = 0; i < nsp; ++i) {
                double mfv = yout[i] * m.sp(i)[SP_M] / rho;
                L[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
            }
            double tot = sum_pairwise(L, nsp);
            if (fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) ok = false;
        }
        int fail = 0;
        bool done = false;
        if (ok) {
            t += h;
            for (int i = 0; i < nsp; ++i) y0[i] = yout[i];
            double hMax = h * (1.0 + DT_INCREASE_PERCENT / 100.0);
            if (dtS > h) h = fmin(dtS, hMax);
            if (m.tight()) {   // chemistry_update.d:265-269
                for (int i = 0; i < nsp; ++i) {
                    double mfv = y0[i] * m.sp(i)[SP_M] / rho;
                    q[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
                }
                T = T_from_u(m, q, u, T, err, n_newton);
                p = rho * gas_constant(m, q) * T;
                need_kc = true;
            }
            if (err) fail = err;
            else if (t >= tI) {
                if (cycle == 0) dtSave = dtS;
                done = true;
            } else {
                ++cycle;
                if (cycle == m.max_subcycles()) fail = CELL_MAX_SUBCYCLES;
                else phase = 1;
            }
        } else {
            ++n_rej;
            h /= DT_REDUCTION_FACTOR;
            if (err) fail = err;
            else if (h < H_MIN) fail = CELL_H_MIN;
            else if (++attempt == m.max_attempts()) fail = CELL_MAX_ATTEMPTS;
        }
        if (fail) {
            bool retryable = fail == CELL_H_MIN || fail == CELL_MAX_ATTEMPTS || fail == CELL_MAX_SUBCYCLES;
            if ((a.flags & CHEM_FLAG_RETRY) && retryable && !retried) {   // fluidfvcell.d:924-941
                retried = true;
                dtS0 = -1.0;
                phase = -1;
                continue;
            }
            if (a.status) a.status[c] = fail;
            done = false;
            have = false;
        }
        if (done) {   // chemistry_update.d:290-325, then fluidfvcell.d:956
            for (int i = 0; i < nsp; ++i) {
                double mfv = y0[i] * m.sp(i)[SP_M] / rho;
                q[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
            }
            double tot = sum_pairwise(q, nsp);
            for (int i = 0; i < nsp; ++i) q[i] = q[i] / tot;
            int st = 0;
            if (a.flags & CHEM_FLAG_UPDATE_THERMO) {
                T = T_from_u(m, q, u, T, st, n_newton);
                p = rho * gas_constant(m, q) * T;
            }
            if (st) {
                if (a.status) a.status[c] = st;
            } else {
                for (int i = 0; i < nsp; ++i) a.massf[(size_t)i * ncell + c] = q[i];
                a.T[c] = T;
                a.p[c] = p;
                a.dt_chem[c] = dtSave;
                if (a.status) a.status[c] = CELL_OK;
            }
            have = false;
        }
        if (!have) {
            if (a.cell_counters) {
                a.cell_counters[0 * (size_t)ncell + c] = n_steps;
                a.cell_counters[1 * (size_t)ncell + c] = n_rhs;
                a.cell_counters[2 * (size_t)ncell + c] = n_kc;
                a.cell_counters[3 * (size_t)ncell + c] = n_newton;
                a.cell_counters[4 * (size_t)ncell + c] = n_rej;
                a.cell_counters[5 * (size_t)ncell + c] = n_est;
            }
            if (a.totals) {
                atomicAdd(a.totals + 0, (unsigned long long)n_steps);
                atomicAdd(a.totals + 1, (unsigned long long)n_rhs);
                atomicAdd(a.totals + 2, (unsigned long long)n_kc);
                atomicAdd(a.totals + 3, (unsigned long long)n_newton);
                atomicAdd(a.totals + 4, (unsigned long long)n_rej);
                atomicAdd(a.totals + 5, (unsigned long long)n_est);
            }
        }
    }
}

// ---------------------------------------------------------------- gas-state services
// mode 0: update_thermo_from_pT  (p, T, massf -> rho, u)          therm_perf_gas_mix.d:57-61
// mode 1: update_thermo_from_rhou (rho, u, massf, T guess -> T, p) therm_perf_gas_mix.d:63-67
// mode 2: source terms (rho, T, massf -> source[nsp])              reaction_mechanism.d:98-105
// mode 3: tick rates (rho, T, massf -> forward[nr], backward[nr])  gas_cwrap.d:968-990
// mode 4: update_thermo_from_rhoT (rho, T, massf -> p, u)          therm_perf_gas_mix.d:69-73
// mode 5: mixture properties at (T, p): out1[k] = Cv, Cp, R, u, h, s, a, dp/drho at constant T
//         (therm_perf_gas_mix.d:230-300 and 335-343, gas_model.d:205)
// mode 6: per-species h, s, g at (T, p): out1[0..nsp), [nsp..2nsp), [2nsp..3nsp)
//         (therm_perf_gas_mix.d:322-326 and 345-349, gas_model.d:180-186)
// mode 7: update_thermo_from_rhop (rho, p, massf -> T, u)          therm_perf_gas_mix.d:75-79, 393-403
// A thread's vectors sit in shared memory after the staged mechanism, or (large mechanisms, gscratch
// set) in global memory beside the other threads' with the mechanism read from global memory.
__global__ void __launch_bounds__(128) gas_service_kernel(GasServiceArgs a) {
    MechView m;
    Vec S;
    if (a.gscratch) {
        m.bind(a.mech_i, a.mech_d);
        S = Vec{a.gscratch + blockIdx.x * blockDim.x + threadIdx.x, (int)(gridDim.x * blockDim.x)};
    } else {
        int* si;
        double* sd;
        double* scratch;
        stage_mechanism(a.mech_i, a.mech_d, a.n_mech_i, a.n_mech_d, si, sd, scratch);
        m.bind(si, sd);
        S = Vec{scratch + threadIdx.x, (int)blockDim.x};
    }
    const int nsp = m.nsp, nr = m.nr;
    Vec mf = S, c = S + nsp, q = S + 2 * nsp, L = S + 3 * nsp, kf = S + 4 * nsp, kb = kf + nr, meff = kb + nr;
    for (int cell = blockIdx.x * blockDim.x + threadIdx.x; cell < a.ncell; cell += gridDim.x * blockDim.x) {
        for (int i = 0; i < nsp; ++i) mf[i] = a.massf[(size_t)i * a.ncell + cell];
        int err = 0;
        if (a.mode == 0) {
            double T = a.T[cell], pr = a.p[cell];
            double rho = pr / (gas_constant(m, mf) * T);
            double logT = log(T);
            double uu = 0.0;
            for (int i = 0; i < nsp; ++i) uu += mf[i] * (cea_h(m, i, T, logT, err) - m.sp(i)[SP_R] * T);
            a.rho[cell] = rho;
            a.u[cell] = uu;
        } else if (a.mode == 4) {
            double T = a.T[cell], rho = a.rho[cell];
            double logT = log(T);
            double uu = 0.0;
            for (int i = 0; i < nsp; ++i) uu += mf[i] * (cea_h(m, i, T, logT, err) - m.sp(i)[SP_R] * T);
            a.u[cell] = uu;
            a.p[cell] = rho * gas_constant(m, mf) * T;
        } else if (a.mode == 5) {
            const double T = a.T[cell], logT = log(T), lp = log(a.p[cell] / P_atm);
            double cv = 0.0, cp = 0.0, R = 0.0, uu = 0.0, hh = 0.0, ss = 0.0;
            for (int i = 0; i < nsp; ++i) {
                const double Ri = m.sp(i)[SP_R], Cpi = cea_Cp(m, i, T, err), hi = cea_h(m, i, T, logT, err);
                cv += mf[i] * (Cpi - Ri);
                cp += mf[i] * Cpi;
                R += mf[i] * Ri;
                uu += mf[i] * (hi - Ri * T);
                hh += mf[i] * hi;
                ss += mf[i] * (cea_s(m, i, T, logT, err) - Ri * lp);
            }
            double* o = a.out1 + cell;
            const size_t st = (size_t)a.ncell;
            o[0] = cv; o[st] = cp; o[2 * st] = R; o[3 * st] = uu; o[4 * st] = hh; o[5 * st] = ss;
            o[6 * st] = sqrt((cp / cv) * (R * T));   // frozen sound speed, therm_perf_gas_mix.d:230-240
            o[7 * st] = R * T;
        } else if (a.mode == 6) {
            const double T = a.T[cell], logT = log(T), lp = log(a.p[cell] / P_atm);
            for (int i = 0; i < nsp; ++i) {
                const double hi = cea_h(m, i, T, logT, err);
                const double si = cea_s(m, i, T, logT, err) - m.sp(i)[SP_R] * lp;
                a.out1[(size_t)i * a.ncell + cell] = hi;
                a.out1[(size_t)(nsp + i) * a.ncell + cell] = si;
                a.out1[(size_t)(2 * nsp + i) * a.ncell + cell] = hi - T * si;
            }
        } else if (a.mode == 7) {
            const double T = a.p[cell] / (gas_constant(m, mf) * a.rho[cell]);
            const double logT = log(T);
            double uu = 0.0;
            for (int i = 0; i < nsp; ++i) uu += mf[i] * (cea_h(m, i, T, logT, err) - m.sp(i)[SP_R] * T);
            a.T[cell] = T;
            a.u[cell] = uu;
        } else if (a.mode == 1) {
            int it = 0;
            double T = T_from_u(m, mf, a.u[cell], a.T[cell], err, it);
            if (!err) {
                a.T[cell] = T;
                a.p[cell] = a.rho[cell] * gas_constant(m, mf) * T;
            }
        } else {
            double rho = a.rho[cell];
            if (isnan(rho) || rho <= 0.0) err = CELL_BAD_INPUT;
            else {
                for (int i = 0; i < nsp; ++i) {
                    double v = mf[i] * rho / m.sp(i)[SP_M];
                    c[i] = (a.clip && v < MIN_MOLES) ? 0.0 : v;
                }
                rate_constants(m, a.T[cell], kf, kb, L, mf, rho, err);
                if (a.mode == 2) {
                    split_rates(m, c, q, L, kf, kb, meff);
                    for (int i = 0; i < nsp; ++i)
                        a.out1[(size_t)i * a.ncell + cell] = (q[i] - L[i]) * m.sp(i)[SP_M];
                } else {
                    tick_rates(m, c, kf, kb, meff, a.out1 + cell, a.out2 + cell, a.ncell);
                }
            }
        }
        if (a.status) a.status[cell] = err;
    }
}

// ---------------------------------------------------------------- longest-first ordering
// Counting sort of cells into ORDER_BUCKETS cost buckets (bucket = key/8, descending), the visit
// order of the persistent chemistry kernel.  Order within a bucket is arbitrary; only scheduling
// depends on it, never a cell's result.

__device__ __forceinline__ int order_bucket(float key) {
    int b = (int)(key * 0.125f);
    b = b < 0 ? 0 : (b > ORDER_BUCKETS - 1 ? ORDER_BUCKETS - 1 : b);
    return ORDER_BUCKETS - 1 - b;   // expensive first
}

__global__ void order_histogram(const float* key, int n, int* hist) {
    __shared__ int h[ORDER_BUCKETS];
    for (int k = threadIdx.x; k < ORDER_BUCKETS; k += blockDim.x) h[k] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[order_bucket(key[i])], 1);
    __syncthreads();
    for (int k = threadIdx.x; k < ORDER_BUCKETS; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

__global__ void order_scan(int* hist) {   // one block of ORDER_BUCKETS threads: exclusive scan in place
    __shared__ int v[ORDER_BUCKETS];
    const int t = threadIdx.x;
    v[t] = hist[t];
    __syncthreads();
    for (int off = 1; off < ORDER_BUCKETS; off <<= 1) {
        int x = t >= off ? v[t - off] : 0;
        __syncthreads();
        v[t] += x;
        __syncthreads();
    }
    hist[t] = v[t] - hist[t];
}

__global__ void order_scatter(const float* key, int n, int* hist, int* order) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        order[atomicAdd(&hist[order_bucket(key[i])], 1)] = i;
}
#endif   // !GDTK_WARP_TU


#if GDTK_WARP_TU
// ---------------------------------------------------------------- one warp per cell (large mechanisms)
// The reference-order update (chem_update_kernel above) with one warp integrating one cell: species
// and reactions are spread over the lanes, and the cell's vectors live in the warp's share of shared
// memory.  The right-hand side reads compact tables (WarpTables): each reaction's concentration terms
// from shared memory, the third-body efficiency lists transposed in global memory (one list per lane,
// consecutive words across lanes), and a species -> (reaction, coefficient) gather whose species are
// dealt to the lanes longest first, so that the lanes' loops are about equally long.  Rate constants
// and thermo read the packed mechanism from global memory (they need not fit in shared memory).
// Every sum the reference takes over species in order (energies, gas constant, mass-fraction total,
// RKF error norm) is taken by lane 0 in that order from per-species terms the lanes computed, and q, L
// gather each species' terms in reaction order, the reference-order kernel's summation order.  This
// translation unit is compiled with FMA contraction and its alpha-QSS step takes the two-division
// form (w_aqss_step), so values agree with the reference-order kernel to rounding, not bitwise.
// Minima and maxima (step estimate, sigma) are order-free.
constexpr unsigned FULL_MASK = 0xffffffffu;

struct WarpLayout {
    int y0, yout, q, L, mf, g, tmp, kf, kb, wf, wb, wsf, wsb, meff, ext, total;
    __device__ __host__ void make(int nsp, int nr, int neff, int method, int nslot) {
        y0 = 0; yout = nsp; q = 2 * nsp; L = 3 * nsp; mf = 4 * nsp; g = 5 * nsp; tmp = 6 * nsp;
        kf = 8 * nsp; kb = kf + nr; wf = kb + nr; wb = wf + nr; wsf = wb + nr; wsb = wsf + nslot;
        meff = wsb + nslot;
        ext = meff + (neff > 0 ? neff : 1);
        total = ext + (method == METHOD_RKF ? 7 * nsp : 4 * nsp);
    }
};

struct WarpCtx {
    MechView m;
    const int* tstart;      // shared: reaction ir's terms tstart[ir] .. tstart[ir + 1], products from tmid[ir]
    const int* tmid;
    const int* terms;       // shared: species | coeff << 8
    const int* rxeff;       // shared: third-body efficiency list of each reaction, or -1
    const int* slot;        // shared: reaction | |nu| << 16 of each scaled tick-rate slot
    int nslot;
    double* wsf;            // the warp's |nu| w_f and |nu| w_b of each slot
    double* wsb;
    int ent_lo, ent_hi;     // this lane's gather entries
    const int* ent;         // shared: species | index << 8 | L << 21 | source << 22
    const int* efflen;      // global: length of each efficiency list
    const int* effidx;      // global, [k][neff]: species of entry k of each list
    const double* effval;   // global, [k][neff]: its efficiency
    int lane;
};

__device__ __forceinline__ double bcast(double v) { return __shfl_sync(FULL_MASK, v, 0); }

// lane 0 sums v[0..n) in order; every lane gets the result
__device__ __forceinline__ double serial_sum(const WarpCtx& w, const double* v, int n) {
    double s = 0.0;
    if (w.lane == 0)
        for (int i = 0; i < n; ++i) s += v[i];
    return bcast(s);
}

__device__ __forceinline__ int warp_or(int e) { return __any_sync(FULL_MASK, e != 0) ? (e ? e : 1) : 0; }

__device__ void w_rate_constants(const WarpCtx& w, double Tq, double* kf, double* kb, double* g, const double* mf,
                                 double rho, int& err) {
    const MechView& m = w.m;
    double T = Tq;
    if (T < m.T_lower()) T = m.T_lower();
    if (T > m.T_upper()) T = m.T_upper();
    const double logT = log(T);
    int e = 0;
    for (int i = w.lane; i < m.nsp; i += 32) {
        double h = cea_h(m, i, T, logT, e);
        double sv = cea_s(m, i, T, logT, e);
        g[i] = h - T * sv;
    }
    __syncwarp();
    Vec mfv{const_cast<double*>(mf), 1};
    for (int ir = w.lane; ir < m.nr; ir += 32) {
        const int* r = m.rx(ir);
        const double* d = m.rxd(ir);
        double Kc = 1.0;
        if (r[RX_FRC] == RATE_FROM_EQ || r[RX_BRC] == RATE_FROM_EQ) {
            double dG = 0.0, nuSum = 0.0;
            for (int k = 0; k < r[RX_NPART]; ++k) {
                int isp = r[RX_PART + k];
                int nu = r[RX_PART_NU + k];
                dG += nu * g[isp] * m.sp(isp)[SP_M];
                nuSum += nu;
            }
            double K_p = exp(-dG / (R_universal * T));
            Kc = K_p * ipow(P_atm / (R_universal * T), (int)nuSum);
        }
        if (r[RX_FRC] != RATE_FROM_EQ) {
            double f = (r[RX_FRC] == RATE_ARRHENIUS || r[RX_FRC] == RATE_ARRHENIUS2)
                           ? simple_rate(r[RX_FRC], d, T) : pressure_dependent_kf(m, r, d, T, mfv, rho);
            kf[ir] = f;
            kb[ir] = (r[RX_BRC] == RATE_FROM_EQ) ? f / Kc : simple_rate(r[RX_BRC], d + 3, T);
        } else {
            double b = simple_rate(r[RX_BRC], d + 3, T);
            kb[ir] = b;
            kf[ir] = b * Kc;
        }
    }
    __syncwarp();
    const int any = warp_or(e);
    if (any) err = CELL_CEA_RANGE;
}

// tick rates, then q and L per species in reaction order (reaction_mechanism.d:82-96)
__device__ void w_split_rates(const WarpCtx& w, const double* c, double* q, double* L, const double* kf,
                              const double* kb, double* wf, double* wb, double* meff) {
    const MechView& m = w.m;
    const int neff = m.neff;
    for (int s = w.lane; s < neff; s += 32) {   // reaction.d:450-456, in the list's order
        const int len = w.efflen[s];
        double term = 0.0;
        for (int k = 0; k < len; ++k) term += w.effval[k * neff + s] * c[w.effidx[k * neff + s]];
        meff[s] = term;
    }
    for (int i = w.lane; i < m.nsp; i += 32) { q[i] = 0.0; L[i] = 0.0; }
    __syncwarp();
    for (int ir = w.lane; ir < m.nr; ir += 32) {
        double f = kf[ir], b = kb[ir];
        const int e = w.rxeff[ir];
        if (e >= 0) { const double t = meff[e]; f = f * t; b = b * t; }
        const int k0 = w.tstart[ir], km = w.tmid[ir], k1 = w.tstart[ir + 1];
        for (int k = k0; k < km; ++k) f *= ipow(c[w.terms[k] & 0xff], w.terms[k] >> 8);
        for (int k = km; k < k1; ++k) b *= ipow(c[w.terms[k] & 0xff], w.terms[k] >> 8);
        wf[ir] = f;
        wb[ir] = b;
    }
    __syncwarp();
    for (int j = w.lane; j < w.nslot; j += 32) {   // (double)nu * w, as the reference forms it
        const int sl = w.slot[j], ir = sl & 0xffff;
        const double nu = (double)(sl >> 16);
        w.wsf[j] = nu * wf[ir];
        w.wsb[j] = nu * wb[ir];
    }
    __syncwarp();
    // q, L: each of this lane's tasks adds its terms in reaction order from 0 (reaction_mechanism.d:82-96);
    // an entry's index runs over w_f, w_b and the slots' |nu| w_f, |nu| w_b, which lie end to end
    int cur = -1;
    double sum = 0.0;
    for (int k = w.ent_lo; k < w.ent_hi; ++k) {
        const int e = w.ent[k];
        const int key = e & 0x2000ff;   // species and the q / L bit
        if (key != cur) {
            if (cur >= 0) ((cur >> 21) ? L : q)[cur & 0xff] = sum;
            cur = key;
            sum = 0.0;
        }
        sum += wf[(e >> 8) & 0x1fff];
    }
    if (cur >= 0) ((cur >> 21) ? L : q)[cur & 0xff] = sum;
    __syncwarp();
}

__device__ double w_estimate(const WarpCtx& w, const double* c, const double* q, const double* L) {
    const double MUCH_LARGER_FACTOR = 10000.0, ZERO_TOL = 1.0e-30, EPS1 = 1.0e-3;
    double min_dt = 1.0e6;
    for (int i = w.lane; i < w.m.nsp; i += 32) {
        double ci = c[i], qi = q[i], Li = L[i], dt;
        if (ci > 0.0 && (fabs(qi - Li) > ZERO_TOL)) {
            if (qi > MUCH_LARGER_FACTOR * Li) dt = ci / (Li + ZERO_EPS);
            else dt = fabs(ci / (qi - Li));
            min_dt = fmin(min_dt, dt);
        }
    }
    for (int o = 16; o > 0; o >>= 1) min_dt = fmin(min_dt, __shfl_xor_sync(FULL_MASK, min_dt, o));
    double dt_chem = EPS1 * min_dt;
    dt_chem = fmin(dt_chem, 1.0e-10);
    dt_chem = fmax(dt_chem, 1.0e-15);
    return dt_chem;
}

// therm_perf_gas_mix.d:406-468 with the per-species terms in tmp[0..nsp) and tmp[nsp..2nsp)
__device__ double w_T_from_u(const WarpCtx& w, const double* mf, double u_tgt, double T_guess, int& err, int& iters,
                             double* tmp) {
    const MechView& m = w.m;
    const int n = m.nsp;
    const double TOL = 1e-10;
    auto energy = [&](double T) {
        const double logT = log(T);
        int e = 0;
        for (int i = w.lane; i < n; i += 32) tmp[i] = mf[i] * (cea_h(m, i, T, logT, e) - m.sp(i)[SP_R] * T);
        __syncwarp();
        if (warp_or(e)) err = CELL_CEA_RANGE;
        const double s = serial_sum(w, tmp, n);
        __syncwarp();
        return s;
    };
    auto cv = [&](double T) {
        int e = 0;
        for (int i = w.lane; i < n; i += 32) tmp[n + i] = mf[i] * (cea_Cp(m, i, T, e) - m.sp(i)[SP_R]);
        __syncwarp();
        if (warp_or(e)) err = CELL_CEA_RANGE;
        const double s = serial_sum(w, tmp + n, n);
        __syncwarp();
        return s;
    };
    double T = T_guess;
    double f = energy(T) - u_tgt;
    double dT = 0.0;
    for (int iter = 0; iter < 10; ++iter) {
        ++iters;
        double c = cv(T);
        dT = -f / c;
        T += dT;
        if (fabs(dT) / T < TOL) return T;
        f = energy(T) - u_tgt;
    }
    if (fabs(dT) > 1e-3) err = CELL_NEWTON_FAIL;
    return T;
}

__device__ double w_gas_constant(const WarpCtx& w, const double* mf, double* tmp) {
    for (int i = w.lane; i < w.m.nsp; i += 32) tmp[i] = mf[i] * w.m.sp(i)[SP_R];
    __syncwarp();
    const double r = serial_sum(w, tmp, w.m.nsp);
    __syncwarp();
    return r;
}

// lane 0: Phobos' pairwise sum of v[0..n), broadcast
__device__ double w_sum_pairwise(const WarpCtx& w, double* v, int n) {
    double s = 0.0;
    if (w.lane == 0) s = sum_pairwise(Vec{v, 1}, n);
    return bcast(s);
}

__device__ bool w_rkf_step(const WarpCtx& w, const double* y0, double h, double* yOut, double& hSuggest, double* q,
                           double* L, const double* kf, const double* kb, double* wf, double* wb, double* meff,
                           double* ext, double* tmp, int& nrhs) {
    const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10., a43 = 6. / 5.,
        a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27., a61 = 1631. / 55296., a62 = 175. / 512.,
        a63 = 575. / 13824., a64 = 44275. / 110592., a65 = 253. / 4096.;
    const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771., b41 = 2825. / 27648.,
        b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336., b46 = 1.0 / 4.0;
    const int n = w.m.nsp;
    double *k1 = ext, *k2 = ext + n, *k3 = ext + 2 * n, *k4 = ext + 3 * n, *k5 = ext + 4 * n, *k6 = ext + 5 * n,
           *yT = ext + 6 * n;
    auto rates = [&](const double* c, double* out) {
        w_split_rates(w, c, q, L, kf, kb, wf, wb, meff);
        ++nrhs;
        for (int i = w.lane; i < n; i += 32) out[i] = q[i] - L[i];
        __syncwarp();
    };
    rates(y0, k1);
    for (int i = w.lane; i < n; i += 32) yT[i] = y0[i] + h * (a21 * k1[i]);
    __syncwarp();
    rates(yT, k2);
    for (int i = w.lane; i < n; i += 32) yT[i] = y0[i] + h * (a31 * k1[i] + a32 * k2[i]);
    __syncwarp();
    rates(yT, k3);
    for (int i = w.lane; i < n; i += 32) yT[i] = y0[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
    __syncwarp();
    rates(yT, k4);
    for (int i = w.lane; i < n; i += 32) yT[i] = y0[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
    __syncwarp();
    rates(yT, k5);
    for (int i = w.lane; i < n; i += 32)
        yT[i] = y0[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
    __syncwarp();
    rates(yT, k6);
    const double atol = w.m.err_tol(), rtol = w.m.err_tol();
    for (int i = w.lane; i < n; i += 32) {
        double yo = y0[i] + h * (b51 * k1[i] + b53 * k3[i] + b54 * k4[i] + b56 * k6[i]);
        yOut[i] = yo;
        double ye = yo - (y0[i] + h * (b41 * k1[i] + b43 * k3[i] + b44 * k4[i] + b45 * k5[i] + b46 * k6[i]));
        double sk = atol + rtol * fmax(fabs(y0[i]), fabs(yo));
        tmp[i] = (ye / sk) * (ye / sk);
    }
    __syncwarp();
    double err = serial_sum(w, tmp, n);
    __syncwarp();
    err = sqrt(err / n);
    const double maxscale = 10.0, minscale = 0.2, safe = 0.9, alpha = 0.2;
    double scale;
    if (err <= 1.0) {
        if (err == 0.0) scale = maxscale;
        else {
            scale = safe * pow(err, -alpha);
            if (scale < minscale) scale = minscale;
            if (scale > maxscale) scale = maxscale;
        }
        hSuggest = scale * h;
        return true;
    }
    scale = fmax(safe * pow(err, -alpha), minscale);
    hSuggest = scale * h;
    return false;
}

// alpha = N(s) / D(s), s = p h: chemistry_update.d:599-604's rational function of r = 1 / (p h + eps) with
// numerator and denominator multiplied by s^3 (no division by s, so the reference's eps, which guards its
// 1 / (p h), changes nothing above s = 1e-34); s is capped at 1e50, where the ratio is 1 to double precision.
__device__ __forceinline__ void w_alpha_nd(double s, double& N, double& D) {
    s = fmin(s, 1.0e50);
    N = fma(s, fma(s, 11.0 + s, 60.0), 180.0);
    D = fma(s, s, N + 180.0);   // s^3 + 12 s^2 + 60 s + 360
}

// The alpha-QSS step of chemistry_update.d:533-655 with the predictor and corrector updates multiplied
// through by D (y + h (N (q - q0) + D (q0 - p_bar y)) / (N h p_bar + D)), so that a species costs two
// divisions instead of four, by the refined hardware reciprocal (fast_exp.h); sigma as the largest ratio
// found by cross products, one division per lane.  Mathematically the reference's step, in rounding only
// different.
__device__ bool w_aqss_step(const WarpCtx& w, const double* y0, double h, double* yOut, double& hSuggest, double* q,
                            double* L, const double* kf, const double* kb, double* wf, double* wb, double* meff,
                            double* ext, int& nrhs) {
    const MechView& m = w.m;
    const int n = m.nsp;
    const double eps1 = m.eps1(), eps2 = m.eps2(), delta = m.delta();
    double *q0 = ext, *p0 = ext + n, *yp0 = ext + 2 * n, *yp = ext + 3 * n;   // p0 holds p0 / 2
    w_split_rates(w, y0, q, L, kf, kb, wf, wb, meff);
    ++nrhs;
    for (int i = w.lane; i < n; i += 32) {
        const double y = y0[i];
        const double qi = q[i];
        const double pi = gdtk_div_nr(L[i], y + ZERO_EPS);
        double N, D;
        w_alpha_nd(pi * h, N, D);
        const double v = gdtk_add_div(y, h * (D * fma(-pi, y, qi)), fma(N, h * pi, D));
        q0[i] = qi; p0[i] = 0.5 * pi; yp[i] = v; yp0[i] = v;
    }
    __syncwarp();
    bool converged = false;
    for (int corr = 0; corr < m.max_iters(); ++corr) {
        w_split_rates(w, yp, q, L, kf, kb, wf, wb, meff);
        ++nrhs;
        bool conv = true;
        for (int i = w.lane; i < n; i += 32) {
            const double y = y0[i];
            const double pp = gdtk_div_nr(L[i], yp[i] + ZERO_EPS);
            double N, D;
            w_alpha_nd(pp * h, N, D);
            const double pb = fma(0.5, pp, p0[i]);
            const double yc = gdtk_add_div(y, h * fma(N, q[i] - q0[i], D * fma(-pb, y, q0[i])), fma(N, h * pb, D));
            yp[i] = yc;
            if (!(yc < ZERO_EPS)) {
                const double test = fabs(yc - yp0[i]);
                if (test >= fma(eps1, yc, eps1 * delta)) conv = false;
            }
        }
        __syncwarp();
        converged = __all_sync(FULL_MASK, conv);
        if (converged) break;
    }
    double snum = 0.0, sden = 1.0;   // this lane's largest |yc - yp0| / (eps2 (yc + delta))
    for (int i = w.lane; i < n; i += 32) {
        const double yc = yp[i];
        if (yc < ZERO_EPS) continue;
        const double num = fabs(yc - yp0[i]), den = fma(eps2, yc, eps2 * delta);
        if (num * sden > snum * den) { snum = num; sden = den; }
    }
    double sigma = snum / sden;
    for (int o = 16; o > 0; o >>= 1) {
        const double other = __shfl_xor_sync(FULL_MASK, sigma, o);
        if (other > sigma) sigma = other;
    }
    double h_new;
    if (sigma <= 0.0) h_new = 10.0 * h;
    else {
        double x = sigma;
        x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
        x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
        x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
        h_new = h * (gdtk_div_nr(1.0, x) + 0.005);
    }
    hSuggest = h_new;
    if (converged)
        for (int i = w.lane; i < n; i += 32) yOut[i] = yp[i];
    __syncwarp();
    return converged;
}

template <int METHOD>
__global__ void __launch_bounds__(512) chem_warp_kernel(ChemUpdateArgs a, WarpTables tb, int warp_doubles) {
    extern __shared__ double smem_w[];
    int* ti = reinterpret_cast<int*>(smem_w);
    for (int k = threadIdx.x; k < tb.n_smem_ints; k += blockDim.x) ti[k] = tb.gi[k];
    __syncthreads();
    WarpCtx w;
    w.m.bind(a.mech_i, a.mech_d);
    w.lane = threadIdx.x & 31;
    w.tstart = ti + tb.off_tstart;
    w.tmid = ti + tb.off_tmid;
    w.terms = ti + tb.off_terms;
    w.rxeff = ti + tb.off_rxeff;
    w.slot = ti + tb.off_slot;
    w.nslot = tb.nslot;
    w.ent = ti + tb.off_ent;
    w.ent_lo = ti[tb.off_lane + w.lane];
    w.ent_hi = ti[tb.off_lane + w.lane + 1];
    w.efflen = tb.gi + tb.off_efflen;
    w.effidx = tb.gi + tb.off_effidx;
    w.effval = tb.eff_val;
    const MechView& m = w.m;
    WarpLayout lay;
    lay.make(m.nsp, m.nr, m.neff, METHOD, tb.nslot);
    double* S = smem_w + (tb.n_smem_ints + 1) / 2 + (size_t)(threadIdx.x >> 5) * warp_doubles;
    w.wsf = S + lay.wsf;
    w.wsb = S + lay.wsb;
    double *y0 = S + lay.y0, *yout = S + lay.yout, *q = S + lay.q, *L = S + lay.L, *mf = S + lay.mf, *g = S + lay.g,
           *tmp = S + lay.tmp, *kf = S + lay.kf, *kb = S + lay.kb, *wf = S + lay.wf, *wb = S + lay.wb,
           *meff = S + lay.meff, *ext = S + lay.ext;
    const int nsp = m.nsp;
    const unsigned ncell = (unsigned)a.ncell;
    const double tI = a.t_interval;
    while (true) {
        unsigned c = 0;
        if (w.lane == 0) c = atomicAdd(a.counter, 1u);
        c = __shfl_sync(FULL_MASK, c, 0);
        if (c >= ncell) break;
        const double rho = a.rho[c], u = a.u[c], T0 = a.T[c], p0 = a.p[c];
        double dtS0 = a.dt_chem[c];
        if (T0 <= a.T_frozen) {
            if (w.lane == 0 && a.status) a.status[c] = CELL_FROZEN;
            continue;
        }
        if (isnan(rho) || rho <= 0.0) {
            if (w.lane == 0 && a.status) a.status[c] = CELL_BAD_INPUT;
            continue;
        }
        bool retried = false;
        int n_steps = 0, n_rhs = 0, n_kc = 0, n_newton = 0, n_rej = 0, n_est = 0;
        int final_status = 0;
        double T = 0, p = 0, dtS = 0, dtSave = 0, h = 0, t = 0;
        bool restart = true;
        while (restart) {   // one pass, or two after a retryable failure (fluidfvcell.d:924-941)
            restart = false;
            int err = 0;
            T = T0; p = p0; dtS = dtS0; t = 0.0;
            for (int i = w.lane; i < nsp; i += 32) {
                double v = a.massf[(size_t)i * ncell + c] * rho / m.sp(i)[SP_M];
                y0[i] = (v < MIN_MOLES) ? 0.0 : v;
                mf[i] = a.massf[(size_t)i * ncell + c];
            }
            __syncwarp();
            w_rate_constants(w, T, kf, kb, g, mf, rho, err);
            ++n_kc;
            if (dtS > tI) h = tI;
            else if (dtS <= 0.0) {
                w_split_rates(w, y0, q, L, kf, kb, wf, wb, meff);
                ++n_rhs;
                ++n_est;
                h = w_estimate(w, y0, q, L);
            } else h = dtS;
            int cycle = 0, fail = 0;
            bool done = false, need_kc = false;
            while (!fail && !done) {
                dtSave = dtS;   // start of a subcycle
                h = fmin(h, tI - t);
                int attempt = 0;
                while (true) {
                    if (need_kc) {   // rate constants at the state of the last step, before the next one
                        w_rate_constants(w, T, kf, kb, g, mf, rho, err);
                        ++n_kc;
                        need_kc = false;
                    }
                    ++n_steps;
                    bool ok = (METHOD == METHOD_RKF)
                                  ? w_rkf_step(w, y0, h, yout, dtS, q, L, kf, kb, wf, wb, meff, ext, tmp, n_rhs)
                                  : w_aqss_step(w, y0, h, yout, dtS, q, L, kf, kb, wf, wb, meff, ext, n_rhs);
                    if (ok) {   // mass-fraction test on conc2massf(concOut)
                        for (int i = w.lane; i < nsp; i += 32) {
                            double mfv = yout[i] * m.sp(i)[SP_M] / rho;
                            tmp[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
                        }
                        __syncwarp();
                        double tot = w_sum_pairwise(w, tmp, nsp);
                        __syncwarp();
                        if (fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) ok = false;
                    }
                    if (ok) {
                        t += h;
                        for (int i = w.lane; i < nsp; i += 32) y0[i] = yout[i];
                        __syncwarp();
                        double hMax = h * (1.0 + DT_INCREASE_PERCENT / 100.0);
                        if (dtS > h) h = fmin(dtS, hMax);
                        if (m.tight()) {   // chemistry_update.d:265-269
                            for (int i = w.lane; i < nsp; i += 32) {
                                double mfv = y0[i] * m.sp(i)[SP_M] / rho;
                                mf[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
                            }
                            __syncwarp();
                            T = w_T_from_u(w, mf, u, T, err, n_newton, tmp);
                            p = rho * w_gas_constant(w, mf, tmp) * T;
                            need_kc = true;
                        }
                        if (err) fail = err;
                        else if (t >= tI) {
                            if (cycle == 0) dtSave = dtS;
                            done = true;
                        } else {
                            ++cycle;
                            if (cycle == m.max_subcycles()) fail = CELL_MAX_SUBCYCLES;
                        }
                        break;
                    }
                    ++n_rej;
                    h /= DT_REDUCTION_FACTOR;
                    if (err) { fail = err; break; }
                    if (h < H_MIN) { fail = CELL_H_MIN; break; }
                    if (++attempt == m.max_attempts()) { fail = CELL_MAX_ATTEMPTS; break; }
                }
            }
            if (fail) {
                const bool retryable = fail == CELL_H_MIN || fail == CELL_MAX_ATTEMPTS || fail == CELL_MAX_SUBCYCLES;
                if ((a.flags & CHEM_FLAG_RETRY) && retryable && !retried) {
                    retried = true;
                    dtS0 = -1.0;
                    restart = true;
                    continue;
                }
                final_status = fail;
            }
        }
        if (final_status) {
            if (w.lane == 0 && a.status) a.status[c] = final_status;
        } else {   // chemistry_update.d:290-325, then fluidfvcell.d:956
            for (int i = w.lane; i < nsp; i += 32) {
                double mfv = y0[i] * m.sp(i)[SP_M] / rho;
                q[i] = (mfv < MIN_MASS_FRACTION) ? 0.0 : mfv;
            }
            __syncwarp();
            double tot = w_sum_pairwise(w, q, nsp);
            __syncwarp();
            for (int i = w.lane; i < nsp; i += 32) q[i] = q[i] / tot;
            __syncwarp();
            int st = 0;
            if (a.flags & CHEM_FLAG_UPDATE_THERMO) {
                T = w_T_from_u(w, q, u, T, st, n_newton, tmp);
                p = rho * w_gas_constant(w, q, tmp) * T;
            }
            if (st) {
                if (w.lane == 0 && a.status) a.status[c] = st;
            } else {
                for (int i = w.lane; i < nsp; i += 32) a.massf[(size_t)i * ncell + c] = q[i];
                if (w.lane == 0) {
                    a.T[c] = T;
                    a.p[c] = p;
                    a.dt_chem[c] = dtSave;
                    if (a.status) a.status[c] = CELL_OK;
                }
            }
        }
        if (w.lane == 0) {
            if (a.cell_counters) {
                a.cell_counters[0 * (size_t)ncell + c] = n_steps;
                a.cell_counters[1 * (size_t)ncell + c] = n_rhs;
                a.cell_counters[2 * (size_t)ncell + c] = n_kc;
                a.cell_counters[3 * (size_t)ncell + c] = n_newton;
                a.cell_counters[4 * (size_t)ncell + c] = n_rej;
                a.cell_counters[5 * (size_t)ncell + c] = n_est;
            }
            if (a.totals) {
                atomicAdd(a.totals + 0, (unsigned long long)n_steps);
                atomicAdd(a.totals + 1, (unsigned long long)n_rhs);
                atomicAdd(a.totals + 2, (unsigned long long)n_kc);
                atomicAdd(a.totals + 3, (unsigned long long)n_newton);
                atomicAdd(a.totals + 4, (unsigned long long)n_rej);
                atomicAdd(a.totals + 5, (unsigned long long)n_est);
            }
        }
        __syncwarp();
    }
}
#endif   // GDTK_WARP_TU

}  // namespace

#if !GDTK_WARP_TU
cudaError_t launch_bucket_order(const float* key, int n, int* order, int* hist, int sm_count, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(hist, 0, ORDER_BUCKETS * sizeof(int), stream);
    if (e != cudaSuccess) return e;
    int grid = (n + 255) / 256;
    if (grid > sm_count * 4) grid = sm_count * 4;
    order_histogram<<<grid, 256, 0, stream>>>(key, n, hist);
    order_scan<<<1, ORDER_BUCKETS, 0, stream>>>(hist);
    order_scatter<<<grid, 256, 0, stream>>>(key, n, hist, order);
    return cudaGetLastError();
}

#endif   // !GDTK_WARP_TU

// ---------------------------------------------------------------- host-side launchers

#if GDTK_WARP_TU
int chem_warp_doubles(int nsp, int nr, int neff, int method, int nslot) {
    WarpLayout l;
    l.make(nsp, nr, neff, method, nslot);
    return l.total;
}

cudaError_t launch_chem_update_warp(const ChemUpdateArgs& a, int method, const WarpTables& t, int warp_doubles,
                                    int sm_count, cudaStream_t stream, LaunchInfo* info) {
    if (a.ncell <= 0) return cudaSuccess;
    const size_t limit = 227 * 1024;
    const size_t tables = (size_t)((t.n_smem_ints + 1) / 2) * 8, per_warp = (size_t)warp_doubles * 8;
    if (tables + per_warp > limit) return cudaErrorInvalidConfiguration;
    const void* fn = (method == METHOD_RKF) ? (const void*)chem_warp_kernel<METHOD_RKF>
                                            : (const void*)chem_warp_kernel<METHOD_ALPHA_QSS>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    // the block size (warps each holding one cell's vectors beside the block's copy of the tables) that
    // keeps the most warps resident per SM; ties go to the larger block
    int warps = 0, per_sm = 0;
    for (int w : {16, 12, 8, 6, 4, 2, 1}) {
        if (tables + per_warp * w > limit) continue;
        int nb = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * w, tables + per_warp * w);
        if (e != cudaSuccess) return e;
        if (nb * w > per_sm * warps) { warps = w; per_sm = nb; }
    }
    if (warps < 1 || per_sm < 1) return cudaErrorInvalidConfiguration;
    const int block = 32 * warps;
    const size_t smem = tables + per_warp * warps;
    long long want = ((long long)a.ncell + warps - 1) / warps;
    long long grid = (long long)sm_count * per_sm;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    if (info) { info->grid = (int)grid; info->block = block; info->smem = (int)smem; info->blocks_per_sm = per_sm; }
    if (method == METHOD_RKF)
        chem_warp_kernel<METHOD_RKF><<<(unsigned)grid, block, smem, stream>>>(a, t, warp_doubles);
    else
        chem_warp_kernel<METHOD_ALPHA_QSS><<<(unsigned)grid, block, smem, stream>>>(a, t, warp_doubles);
    return cudaGetLastError();
}

#else
int chem_scratch_doubles(int nsp, int nr, int neff, int method) {
    Layout l;
    l.make(nsp, nr, neff, method);
    return l.total;
}

static size_t mech_smem_bytes(int ni, int nd) { return (size_t)nd * 8 + (size_t)((ni + 1) / 2) * 8; }

cudaError_t launch_chem_update(const ChemUpdateArgs& a, int method, int scratch_doubles, int sm_count,
                               cudaStream_t stream, LaunchInfo* info) {
    const size_t mech = mech_smem_bytes(a.n_mech_i, a.n_mech_d);
    const size_t limit = 227 * 1024;
    int block = 256;
    while (block > 32 && mech + (size_t)scratch_doubles * 8 * block > limit) block /= 2;
    // Small batches: narrower blocks so that the cells spread over every SM.
    while (block > 32 && ((long long)a.ncell + block - 1) / block < sm_count) block /= 2;
    size_t smem = mech + (size_t)scratch_doubles * 8 * block;
    if (smem > limit) return cudaErrorInvalidConfiguration;
    const void* fn = method == METHOD_RKF ? (const void*)chem_update_kernel<METHOD_RKF>
                                          : (const void*)chem_update_kernel<METHOD_ALPHA_QSS>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    long long want = ((long long)a.ncell + block - 1) / block;
    long long grid = (long long)sm_count * per_sm;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    if (info) { info->grid = (int)grid; info->block = block; info->smem = (int)smem; info->blocks_per_sm = per_sm; }
    if (method == METHOD_RKF)
        chem_update_kernel<METHOD_RKF><<<(unsigned)grid, block, smem, stream>>>(a);
    else
        chem_update_kernel<METHOD_ALPHA_QSS><<<(unsigned)grid, block, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gas_service(const GasServiceArgs& a, int sm_count, cudaStream_t stream) {
    if (a.ncell <= 0) return cudaSuccess;
    const size_t mech = mech_smem_bytes(a.n_mech_i, a.n_mech_d);
    const int nsp = a.nsp_hint, nr = a.nr_hint, neff = a.neff_hint > 0 ? a.neff_hint : 1;
    const size_t per_thread = (size_t)(4 * nsp + 2 * nr + neff) * 8;   // mf, c, q, L, kf, kb, meff
    int block = 128;
    while (block > 32 && mech + per_thread * block > 200 * 1024) block /= 2;
    size_t smem = mech + per_thread * block;
    if (smem <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)gas_service_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        long long grid = ((long long)a.ncell + block - 1) / block;
        if (grid > (long long)sm_count * 8) grid = (long long)sm_count * 8;
        if (grid < 1) grid = 1;
        gas_service_kernel<<<(unsigned)grid, block, smem, stream>>>(a);
        return cudaGetLastError();
    }
    // Global-memory vectors: at most two 64-thread blocks per SM, in a stream-ordered allocation.
    block = 64;
    long long grid = ((long long)a.ncell + block - 1) / block;
    if (grid > (long long)sm_count * 2) grid = (long long)sm_count * 2;
    GasServiceArgs g = a;
    void* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, per_thread * (size_t)(grid * block), stream);
    if (e != cudaSuccess) return e;
    g.gscratch = static_cast<double*>(buf);
    gas_service_kernel<<<(unsigned)grid, block, 0, stream>>>(g);
    e = cudaGetLastError();
    cudaError_t f = cudaFreeAsync(buf, stream);
    return e != cudaSuccess ? e : f;
}

#endif   // GDTK_WARP_TU

}  // namespace gdtk
