// chem_fast.cuh -- mechanism-specialised FP64 chemistry update for sm_103a.
//
// This file is compiled at run time by NVRTC, once per mechanism, after a generated prologue
// (codegen.cpp) that defines the mechanism as compile-time constants and two straight-line
// functions:
//   gen_kc(lnT, rT, g, K, ks, etab)   k_f, k_b of every reaction into K[r*ks], K[(NR + r)*ks]
//   gen_rhs(c, q, L, K, ks)           production q and loss L of every species at c
// so that per-species vectors live in registers and every index and coefficient is an
// immediate.  The algorithm is the reference's (kinetics/chemistry_update.d:139-326 and the
// calls below it), with the arithmetic rearranged to spend fewer FP64 operations, which are
// the binding resource on this GPU (FP64 issue is 1/64 of FP32):
//   * rate constants in log form, ln k = ln A + n ln T - C/T, and k_b = k_f / K_c as one
//     exponential of ln k_f + sum(nu G/RT) - sum(nu) ln(P_atm / RT)  (reaction.d:26-52,
//     rate_constant.d:72-75), with exp by Tang's table method (fast_exp.h);
//   * the NASA-9 enthalpy, heat capacity and G/RT in Horner form with coefficients scaled
//     once on the host (cea_thermo_curves.d:55-137);
//   * the alpha-QSS predictor/corrector with alpha = N(s)/D(s), s = p h + eps, folded into the
//     update so that each species needs two divisions instead of four (chemistry_update.d:592-610);
//   * the right-hand side at the start of a step is shared by the initial step-size estimate
//     and the first stage (reaction_mechanism.d:161-203 evaluates the same rates);
//   * RKF's step-size factor err^-0.2 as exp(-0.2 ln err).
// Results agree with the reference-order kernel and the oracle to rounding (tested to 1e-8
// absolute in Y and 1e-7 relative in T and p).

#ifndef GDTK_NSP
#error "chem_fast.cuh needs the generated mechanism prologue"
#endif

#define GDTK_TH_STRIDE 120
#define GDTK_TH_SEG0 24

namespace gdtk_fast {

using gdtk::gdtk_exp;

// must match the host's FastArgs (codegen.h)
struct FastArgs {
    const double* thermo;
    const double* exp_table;
    int ncell;
    int flags;
    const double* rho;
    const double* u;
    double* T;
    double* p;
    double* massf;
    double* dt_chem;
    int* status;
    double t_interval;
    double T_frozen;
    unsigned* counter;
    int* cell_counters;
    unsigned long long* totals;
};

enum { ST_OK = 0, ST_H_MIN = 1, ST_MAX_ATTEMPTS = 2, ST_MAX_SUBCYCLES = 3, ST_NEWTON = 4, ST_BAD = 5, ST_FROZEN = 6,
       ST_CEA = 7 };
enum { F_UPDATE_THERMO = 1, F_RETRY = 2 };

constexpr double MIN_MOLES = 1.0e-30;
constexpr double ZERO_EPS = 1.0e-50;
constexpr double H_MIN = 1.0e-15;
constexpr double ALLOWABLE_MASSF_ERROR = 1.0e-3;

// ---------------------------------------------------------------- species thermo
// Segment choice of cea_thermo_curves.d:150-182: coefficients sa blended towards sb by wb.
__device__ __forceinline__ bool seg_of(const double* th, double T, int& sa, int& sb, double& wb) {
    const int nseg = (int)th[10];
    const double* br = th + 11;
    const double* bl = th + 16;
    const double* rbl = th + 20;
    wb = 0.0;
    if (nseg == 1) { sa = sb = 0; return T == T; }
    if (T < (br[1] - 0.5 * bl[0])) { sa = sb = 0; return true; }
    if (T > (br[nseg - 1] + 0.5 * bl[nseg - 2])) { sa = sb = nseg - 1; return true; }
    for (int i = 1; i < nseg; ++i) {
        double lo = br[i] - 0.5 * bl[i - 1];
        double hi = br[i] + 0.5 * bl[i - 1];
        if (T >= lo && T <= hi) { wb = rbl[i - 1] * (T - lo); sa = i - 1; sb = i; return true; }
        if (T > hi && i < nseg - 1 && T < (br[i + 1] - 0.5 * bl[i])) { sa = sb = i; return true; }
    }
    sa = sb = 0;
    return false;
}

__device__ __forceinline__ double poly_H(const double* c, double T, double lnT, double rT) {   // H/R [K]
    return fma(T, fma(T, fma(T, fma(T, fma(T, c[6], c[5]), c[4]), c[3]), c[2]), fma(c[0], rT, fma(c[1], lnT, c[7])));
}
__device__ __forceinline__ double poly_Cp(const double* c, double T, double rT, double rT2) {   // Cp/R
    return fma(T, fma(T, fma(T, fma(T, c[6], c[5]), c[4]), c[3]), fma(c[0], rT2, fma(c[1], rT, c[2])));
}
__device__ __forceinline__ double poly_G(const double* c, double T, double rT, double rT2, double t1, double t2) {
    // G/RT = g0/T^2 + (g1 (ln T + 1) + g2)/T + g3 (1 - ln T) + g4 + T (g5 + T (g6 + T (g7 + T g8)))
    return fma(T, fma(T, fma(T, fma(T, c[8], c[7]), c[6]), c[5]),
               fma(fma(c[1], t1, c[2]), rT, fma(c[0], rT2, fma(c[3], t2, c[4]))));
}

// H/R and Cp/R of species i (extrapolated with constant Cp beyond the curve, as the reference).
__device__ __forceinline__ void sp_H_Cp(const double* TH, int i, double T, double lnT, double rT, double rT2, double& H,
                                        double& Cp, int& err) {
    const double* th = TH + i * GDTK_TH_STRIDE;
    if (T < th[0]) { H = th[2] - th[4] * (th[0] - T); Cp = th[4]; return; }
    if (T > th[1]) { H = th[3] + th[5] * (T - th[1]); Cp = th[5]; return; }
    int sa, sb;
    double wb;
    if (!seg_of(th, T, sa, sb, wb)) { err = ST_CEA; H = 0.0; Cp = 1.0; return; }
    const double* ca = th + GDTK_TH_SEG0 + 24 * sa;
    H = poly_H(ca, T, lnT, rT);
    Cp = poly_Cp(ca + 8, T, rT, rT2);
    if (wb != 0.0) {
        const double* cb = th + GDTK_TH_SEG0 + 24 * sb;
        H = fma(wb, poly_H(cb, T, lnT, rT) - H, H);
        Cp = fma(wb, poly_Cp(cb + 8, T, rT, rT2) - Cp, Cp);
    }
}

__device__ __forceinline__ double sp_G(const double* TH, int i, double T, double lnT, double rT, double rT2, double t1,
                                       double t2, int& err) {
    const double* th = TH + i * GDTK_TH_STRIDE;
    if (T < th[0]) {
        double H = th[2] - th[4] * (th[0] - T), S = th[6] - th[4] * (th[8] - lnT);
        return fma(H, rT, -S);
    }
    if (T > th[1]) {
        double H = th[3] + th[5] * (T - th[1]), S = th[7] + th[5] * (lnT - th[9]);
        return fma(H, rT, -S);
    }
    int sa, sb;
    double wb;
    if (!seg_of(th, T, sa, sb, wb)) { err = ST_CEA; return 0.0; }
    double g = poly_G(TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 24 * sa + 15, T, rT, rT2, t1, t2);
    if (wb != 0.0) g = fma(wb, poly_G(TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 24 * sb + 15, T, rT, rT2, t1, t2) - g, g);
    return g;
}

// T from (rho, u) at fixed composition, therm_perf_gas_mix.d:426-468 (same iteration, same
// stopping rules).  YR[i * ys] = Y_i R_i.  *iters counts iterations.
__device__ double T_from_u(const double* TH, const double* YR, int ys, double u_tgt, double T_guess, int& err,
                           int& iters) {
    const double TOL = 1e-10;
    double T = T_guess;
    double dT = 0.0;
    double lnT = log(T), rT = 1.0 / T;
    double f = 0.0, cv = 0.0;
    {
        double rT2 = rT * rT;
#pragma unroll
        for (int i = 0; i < GDTK_NSP; ++i) {
            double H, Cp;
            sp_H_Cp(TH, i, T, lnT, rT, rT2, H, Cp, err);
            const double yr = YR[i * ys];
            f = fma(yr, H - T, f);
            cv = fma(yr, Cp - 1.0, cv);
        }
        f -= u_tgt;
    }
    for (int iter = 0; iter < 10; ++iter) {
        ++iters;
        dT = -f / cv;
        T += dT;
        if (fabs(dT) / T < TOL) return T;
        lnT = log(T);
        rT = 1.0 / T;
        double rT2 = rT * rT;
        f = 0.0;
        cv = 0.0;
#pragma unroll
        for (int i = 0; i < GDTK_NSP; ++i) {
            double H, Cp;
            sp_H_Cp(TH, i, T, lnT, rT, rT2, H, Cp, err);
            const double yr = YR[i * ys];
            f = fma(yr, H - T, f);
            cv = fma(yr, Cp - 1.0, cv);
        }
        f -= u_tgt;
    }
    if (fabs(dT) > 1e-3) err = ST_NEWTON;
    return T;
}

// Phobos' pairwise summation order (std.algorithm.sum) for GDTK_NSP values d(i).
template <typename F>
__device__ __forceinline__ double sum_pairwise(F d) {
    double store[8];
    int idx = 0;
    int pos = 0;
#pragma unroll
    for (int k = 0; k < GDTK_NSP / 16; ++k) {
        double s = (((d(pos) + d(pos + 1)) + (d(pos + 2) + d(pos + 3))) + ((d(pos + 4) + d(pos + 5)) +
                   (d(pos + 6) + d(pos + 7)))) + (((d(pos + 8) + d(pos + 9)) + (d(pos + 10) + d(pos + 11))) +
                   ((d(pos + 12) + d(pos + 13)) + (d(pos + 14) + d(pos + 15))));
        store[idx] = s;
        pos += 16;
        int last = idx - (__ffs(k + 1) - 1);
        while (idx > last) { store[idx - 1] += store[idx]; --idx; }
        ++idx;
    }
#pragma unroll
    for (int i = 0; i < GDTK_NSP % 16; ++i) {
        store[idx] = d(pos + i);
        int last = idx - (__ffs(i + 1) - 1);
        while (idx > last) { store[idx - 1] += store[idx]; --idx; }
        ++idx;
    }
    double s = store[idx - 1];
    for (int j = idx - 1; j-- > 0;) s += store[j];
    return s;
}

// Rate constants at T (clamped to the mechanism's limits, reaction_mechanism.d:49-63).
__device__ __forceinline__ void rate_constants(const double* TH, double Tq, double* K, int ks, const double* etab,
                                               int& err) {
    double T = Tq;
    if (T < GDTK_T_LOWER) T = GDTK_T_LOWER;
    if (T > GDTK_T_UPPER) T = GDTK_T_UPPER;
    const double lnT = log(T), rT = 1.0 / T, rT2 = rT * rT, t1 = lnT + 1.0, t2 = 1.0 - lnT;
    double g[GDTK_NSP];
#pragma unroll
    for (int i = 0; i < GDTK_NSP; ++i) g[i] = sp_G(TH, i, T, lnT, rT, rT2, t1, t2, err);
    gen_kc(T, lnT, rT, g, K, ks, etab);
}

// reaction_mechanism.d:161-203 from the rates at c.
__device__ __forceinline__ double estimate_step(const double (&c)[GDTK_NSP], const double (&q)[GDTK_NSP],
                                                const double (&L)[GDTK_NSP]) {
    double min_dt = 1.0e6;
#pragma unroll
    for (int i = 0; i < GDTK_NSP; ++i) {
        if (c[i] > 0.0 && fabs(q[i] - L[i]) > 1.0e-30) {
            double dt = (q[i] > 10000.0 * L[i]) ? c[i] / (L[i] + ZERO_EPS) : fabs(c[i] / (q[i] - L[i]));
            min_dt = fmin(min_dt, dt);
        }
    }
    double dt_chem = 1.0e-3 * min_dt;
    dt_chem = fmin(dt_chem, 1.0e-10);
    return fmax(dt_chem, 1.0e-15);
}

// alpha = N/D (chemistry_update.d:599-604) as N(s)/D(s), s = p h + eps.
__device__ __forceinline__ void alpha_nd(double s, double& N, double& D) {
    if (s < 1.0e50) {
        N = fma(s, fma(s, 11.0 + s, 60.0), 180.0);
        D = fma(s, fma(s, 12.0 + s, 60.0), 360.0);
    } else {
        double r = 1.0 / s;
        N = fma(r, fma(r, fma(r, 180.0, 60.0), 11.0), 1.0);
        D = fma(r, fma(r, fma(r, 360.0, 60.0), 12.0), 1.0);
    }
}

// ---------------------------------------------------------------- the kernel
extern "C" __global__ void __launch_bounds__(GDTK_BLOCK, GDTK_MIN_BLOCKS) gdtk_chem_fast(FastArgs a) {
    extern __shared__ double smem[];
    double* TH = smem;                                   // thermo table, nsp * stride
    double* ETAB = smem + GDTK_NSP * GDTK_TH_STRIDE;     // exp table, 64
    double* S = ETAB + 64;                               // per-thread vectors
    for (int k = threadIdx.x; k < GDTK_NSP * GDTK_TH_STRIDE; k += blockDim.x) TH[k] = a.thermo[k];
    for (int k = threadIdx.x; k < 64; k += blockDim.x) ETAB[k] = a.exp_table[k];
    __syncthreads();
    const int ks = blockDim.x;
    double* K = S + threadIdx.x;                         // kf[NR], kb[NR]
    double* V = K + 2 * GDTK_NR * ks;                    // method vectors
    const unsigned ncell = (unsigned)a.ncell;
    const double tI = a.t_interval;

    unsigned c = 0;
    bool have = false, retried = false, need_kc = false;
    int phase = 0, cycle = 0, attempt = 0, err = 0;
    double rho = 0, rrho = 0, u = 0, T = 0, T0 = 0, p = 0, p0 = 0, dtS = 0, dtS0 = 0, dtSave = 0, h = 0, t = 0;
    double y0[GDTK_NSP];
    int n_steps = 0, n_rhs = 0, n_kc = 0, n_newton = 0, n_rej = 0, n_est = 0;

    while (true) {
        if (!have) {
            unsigned mask = __activemask();
            int lane = threadIdx.x & 31;
            int leader = __ffs(mask) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned)__popc(mask));
            base = __shfl_sync(mask, base, leader);
            c = base + __popc(mask & ((1u << lane) - 1u));
            if (c >= ncell) break;
            rho = a.rho[c]; u = a.u[c]; T0 = a.T[c]; p0 = a.p[c]; dtS0 = a.dt_chem[c];
            if (T0 <= a.T_frozen) { if (a.status) a.status[c] = ST_FROZEN; continue; }
            if (isnan(rho) || rho <= 0.0) { if (a.status) a.status[c] = ST_BAD; continue; }
            have = true;
            retried = false;
            rrho = 1.0 / rho;
            n_steps = n_rhs = n_kc = n_newton = n_rej = n_est = 0;
            phase = -1;
        }
        if (phase == -1) {
            T = T0; p = p0; dtS = dtS0; t = 0.0; err = 0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double v = a.massf[(size_t)i * ncell + c] * rho * GDTK_RM[i];
                y0[i] = (v < MIN_MOLES) ? 0.0 : v;
            }
            need_kc = true;
            phase = 0;
        }
        if (need_kc) {
            rate_constants(TH, T, K, ks, ETAB, err);
            ++n_kc;
            need_kc = false;
        }
        // rates at y0: shared by the step-size estimate and the first stage of the step
        double q[GDTK_NSP], L[GDTK_NSP];
        gen_rhs(y0, q, L, K, ks);
        ++n_rhs;
        if (phase == 0) {
            if (dtS > tI) h = tI;
            else if (dtS <= 0.0) {   // the reference evaluates these rates a second time; counted as it does
                h = estimate_step(y0, q, L);
                ++n_est;
                ++n_rhs;
            }
            else h = dtS;
            cycle = 0;
            phase = 1;
        }
        if (phase == 1) {
            dtSave = dtS;
            h = fmin(h, tI - t);
            attempt = 0;
            phase = 2;
        }
        ++n_steps;
        double yn[GDTK_NSP];   // stage input / predictor-corrector, then the step's result
        bool ok;
#if GDTK_METHOD == 0
        {   // Runge-Kutta-Fehlberg with Cash-Karp coefficients, chemistry_update.d:404-478
            const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10.,
                a43 = 6. / 5., a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27.,
                a61 = 1631. / 55296., a62 = 175. / 512., a63 = 575. / 13824., a64 = 44275. / 110592.,
                a65 = 253. / 4096.;
            const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771.,
                b41 = 2825. / 27648., b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336.,
                b46 = 1.0 / 4.0;
            double* k1 = V;
            double* k2 = V + GDTK_NSP * ks;
            double* k3 = V + 2 * GDTK_NSP * ks;
            double* k4 = V + 3 * GDTK_NSP * ks;
            double* k5 = V + 4 * GDTK_NSP * ks;
            double* yT = yn;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double k = q[i] - L[i];
                k1[i * ks] = k;
                yT[i] = fma(h, a21 * k, y0[i]);
            }
            gen_rhs(yT, q, L, K, ks);
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double k = q[i] - L[i];
                k2[i * ks] = k;
                yT[i] = fma(h, fma(a32, k, a31 * k1[i * ks]), y0[i]);
            }
            gen_rhs(yT, q, L, K, ks);
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double k = q[i] - L[i];
                k3[i * ks] = k;
                yT[i] = fma(h, fma(a43, k, fma(a42, k2[i * ks], a41 * k1[i * ks])), y0[i]);
            }
            gen_rhs(yT, q, L, K, ks);
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double k = q[i] - L[i];
                k4[i * ks] = k;
                yT[i] = fma(h, fma(a54, k, fma(a53, k3[i * ks], fma(a52, k2[i * ks], a51 * k1[i * ks]))), y0[i]);
            }
            gen_rhs(yT, q, L, K, ks);
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double k = q[i] - L[i];
                k5[i * ks] = k;
                yT[i] = fma(h, fma(a65, k, fma(a64, k4[i * ks], fma(a63, k3[i * ks], fma(a62, k2[i * ks],
                            a61 * k1[i * ks])))), y0[i]);
            }
            gen_rhs(yT, q, L, K, ks);
            n_rhs += 5;
            double err2 = 0.0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double K1 = k1[i * ks], K3 = k3[i * ks], K4 = k4[i * ks], K5 = k5[i * ks], K6 = q[i] - L[i];
                double o = fma(h, fma(b56, K6, fma(b54, K4, fma(b53, K3, b51 * K1))), y0[i]);
                double o4 = fma(h, fma(b46, K6, fma(b45, K5, fma(b44, K4, fma(b43, K3, b41 * K1)))), y0[i]);
                yT[i] = o;
                double sk = fma(GDTK_ERRTOL, fmax(fabs(y0[i]), fabs(o)), GDTK_ERRTOL);
                double e = (o - o4) / sk;
                err2 = fma(e, e, err2);
            }
            double errn = sqrt(err2 * (1.0 / GDTK_NSP));
            double scale;
            if (errn <= 1.0) {
                if (errn == 0.0) scale = 10.0;
                else scale = fmin(fmax(0.9 * gdtk_exp(-0.2 * log(errn), ETAB), 0.2), 10.0);
                ok = true;
            } else {
                scale = fmax(0.9 * gdtk_exp(-0.2 * log(errn), ETAB), 0.2);
                ok = false;
            }
            dtS = scale * h;
        }
#else
        {   // alpha-QSS, chemistry_update.d:533-655; V holds q0, p0, yp0
            double* Q0 = V;
            double* P0 = V + GDTK_NSP * ks;
            double* YP0 = V + 2 * GDTK_NSP * ks;
            double* yp = yn;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double y = y0[i];
                double pi = L[i] / (y + ZERO_EPS);
                double x = pi * h;
                double N, D;
                alpha_nd(x + ZERO_EPS, N, D);
                double v = y + (h * (q[i] - pi * y)) * D / fma(N, x, D);
                Q0[i * ks] = q[i];
                P0[i * ks] = pi;
                YP0[i * ks] = v;
                yp[i] = v;
            }
            bool conv = false;
            for (int corr = 0; corr < GDTK_MAX_ITERS; ++corr) {
                gen_rhs(yp, q, L, K, ks);
                ++n_rhs;
                conv = true;
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double y = y0[i];
                    double q0 = Q0[i * ks];
                    double pp = L[i] / (yp[i] + ZERO_EPS);
                    double x = pp * h;
                    double N, D;
                    alpha_nd(x + ZERO_EPS, N, D);
                    double pb = 0.5 * (P0[i * ks] + pp);
                    double num = h * (fma(N, q[i] - q0, D * q0) - D * (pb * y));
                    double yc = y + num / fma(N, h * pb, D);
                    yp[i] = yc;
                    if (!(yc < ZERO_EPS) && fabs(yc - YP0[i * ks]) >= GDTK_EPS1 * (yc + GDTK_DELTA)) conv = false;
                }
                if (conv) break;
            }
            double sigma = 0.0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double yc = yp[i];
                if (yc < ZERO_EPS) continue;
                double test = fabs(yc - YP0[i * ks]) / (GDTK_EPS2 * (yc + GDTK_DELTA));
                if (test > sigma) sigma = test;
            }
            if (sigma <= 0.0) dtS = 10.0 * h;
            else {
                double x = sigma;
                x = x - 0.5 * (x * x - sigma) / x;
                x = x - 0.5 * (x * x - sigma) / x;
                x = x - 0.5 * (x * x - sigma) / x;
                dtS = h * ((1.0 / x) + 0.005);
            }
            ok = conv;
        }
#endif
        if (ok) {   // mass-fraction test (chemistry_update.d:175-185)
            double tot = sum_pairwise([&](int i) {
                double v = yn[i] * GDTK_M[i] * rrho;
                return (v < 1.0e-30) ? 0.0 : v;
            });
            if (fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) ok = false;
        }
        int fail = 0;
        bool done = false;
        if (ok) {
            t += h;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) y0[i] = yn[i];
            double hMax = h * 1.1;
            if (dtS > h) h = fmin(dtS, hMax);
#if GDTK_TIGHT
            {   // chemistry_update.d:265-269; Y_i R_i go to the method vectors, free until the next step
                double Rm = 0.0;
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double v = y0[i] * GDTK_M[i] * rrho;
                    v = (v < 1.0e-30) ? 0.0 : v;
                    double yr = v * GDTK_R[i];
                    V[i * ks] = yr;
                    Rm += yr;
                }
                T = T_from_u(TH, V, ks, u, T, err, n_newton);
                p = rho * Rm * T;
                need_kc = true;
            }
#endif
            if (err) fail = err;
            else if (t >= tI) {
                if (cycle == 0) dtSave = dtS;
                done = true;
            } else {
                ++cycle;
                if (cycle == GDTK_MAX_SUBCYCLES) fail = ST_MAX_SUBCYCLES;
                else phase = 1;
            }
        } else {
            ++n_rej;
            h /= 10.0;
            if (err) fail = err;
            else if (h < H_MIN) fail = ST_H_MIN;
            else if (++attempt == GDTK_MAX_ATTEMPTS) fail = ST_MAX_ATTEMPTS;
        }
        if (fail) {
            bool retryable = fail == ST_H_MIN || fail == ST_MAX_ATTEMPTS || fail == ST_MAX_SUBCYCLES;
            if ((a.flags & F_RETRY) && retryable && !retried) {
                retried = true;
                dtS0 = -1.0;
                phase = -1;
                continue;
            }
            if (a.status) a.status[c] = fail;
            have = false;
        }
        if (done) {   // chemistry_update.d:290-325, then fluidfvcell.d:956
            auto mf_of = [&](int i) {
                double v = y0[i] * GDTK_M[i] * rrho;
                return (v < 1.0e-30) ? 0.0 : v;
            };
            double rtot = 1.0 / sum_pairwise(mf_of);
            double Rm = 0.0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double yr = mf_of(i) * rtot * GDTK_R[i];
                V[i * ks] = yr;
                Rm += yr;
            }
            int st = 0;
            if (a.flags & F_UPDATE_THERMO) {
                T = T_from_u(TH, V, ks, u, T, st, n_newton);
                p = rho * Rm * T;
            }
            if (st) {
                if (a.status) a.status[c] = st;
            } else {
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) a.massf[(size_t)i * ncell + c] = mf_of(i) * rtot;
                a.T[c] = T;
                a.p[c] = p;
                a.dt_chem[c] = dtSave;
                if (a.status) a.status[c] = ST_OK;
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

}  // namespace gdtk_fast
