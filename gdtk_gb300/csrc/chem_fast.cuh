// chem_fast.cuh -- mechanism-specialised FP64 chemistry update for sm_103a.
//
// This file is compiled at run time by NVRTC, once per mechanism, after a generated prologue
// (codegen.cpp) that defines the mechanism as compile-time constants and two functions:
//   gen_kc(T, lnT, rT, g, gs, K, ks, etab, Mv, ms)   k_f, k_b of every reaction into K[r*ks],
//                                    K[(NR + r)*ks]: a loop over a __constant__ table of the
//                                    Arrhenius reactions, pressure-dependent ones straight-line
//   gen_rhs(c, q, L, K, ks)          production q and loss L of every species at c, straight-line
// so that per-species vectors live in registers.  FP64 operations compile to several instructions
// each on sm_103a, so code size matters as much as operation count: loops over constant tables
// where they cost no extra FP64 work, straight-line code where registers must hold the vectors.
// The algorithm is the reference's (kinetics/chemistry_update.d:139-326 and the calls below it),
// with the arithmetic rearranged to spend fewer FP64 operations, which are the binding resource on
// this GPU (FP64 issue is 1/64 of FP32):
//   * rate constants in log form, ln k = ln A + n ln T - C/T (A T^n by multiplication when C = 0
//     and n is a small integer), and k_b = k_f / K_c = k_f (R T / P_atm)^sum(nu) prod E_i^nu_i with
//     E_i = exp(G_i / R T) formed once per species (reaction.d:26-52, rate_constant.d:72-75), or
//     as one exponential per reaction where those products could leave the double range; exp by
//     Tang's table method (fast_exp.h);
//   * ln T carried with each cell and updated by a log1p series in the Newton iteration, so that
//     the library log (as costly as about 36 FMAs) runs only at cell start and after large steps;
//   * divisions by Newton-Raphson refinement of the hardware reciprocal (fast_exp.h);
//   * compares of doubles on their bit patterns, on the integer pipe (each with the IEEE result), and
//     the curve-segment blend windows formed once on the host;
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
using gdtk::gdtk_div;
using gdtk::gdtk_div_nr;
using gdtk::gdtk_add_div;

// must match the host's CellBlock / FastArgs (codegen.h)
struct CellBlock {
    int ncell;
    int first;              // global index of the block's first cell
    double t_interval;
    const double* rho;
    const double* u;
    double* T;
    double* p;
    double* massf;          // [nsp][ncell]
    double* dt_chem;
    int* status;
};

#define GDTK_MAX_BLOCKS 128

// Passed by value (__grid_constant__): the block table travels in the launch parameters, so a
// launch needs no device-side table and a captured graph replays it exactly.
struct FastArgs {
    const double* thermo;
    const double* exp_table;
    int nblocks;
    int total;
    int flags;
    int refill_chunk;       // visit positions a warp reserves per atomic (<= 1: exactly the lanes that need one)
    double T_frozen;
    unsigned* counter;
    int* cell_counters;     // [6][total], global cell index
    unsigned long long* totals;
    const int* order;       // visit order of the global cell indices (null: index order)
    unsigned long long* lane_stats;   // optional [2 * 8]: per phase, warp executions and active lanes
    CellBlock blocks[GDTK_MAX_BLOCKS];
};

// Lane-occupancy instrumentation: for phase k, count warp executions and the lanes active in them.
// Generated with GDTK_PHASE_CLOCKS, each mark also adds the SM cycles since the warp's previous mark
// to that mark's phase (st[16 + phase]): a per-phase split of every warp's time.
#if GDTK_PHASE_CLOCKS
__shared__ long long gdtk_pc_t0[32];
__shared__ int gdtk_pc_ph[32];
#endif
__device__ __forceinline__ void lane_stat(unsigned long long* st, int k) {
    if (!st) return;
    const unsigned m = __activemask();
    if ((threadIdx.x & 31) == __ffs(m) - 1) {
        atomicAdd(st + 2 * k, 1ull);
        atomicAdd(st + 2 * k + 1, (unsigned long long)__popc(m));
#if GDTK_PHASE_CLOCKS
        const int w = threadIdx.x >> 5;
        const long long t = clock64();
        if (gdtk_pc_ph[w] >= 0) atomicAdd(st + 16 + gdtk_pc_ph[w], (unsigned long long)(t - gdtk_pc_t0[w]));
        gdtk_pc_t0[w] = t;
        gdtk_pc_ph[w] = k;
#endif
    }
}

enum { ST_OK = 0, ST_H_MIN = 1, ST_MAX_ATTEMPTS = 2, ST_MAX_SUBCYCLES = 3, ST_NEWTON = 4, ST_BAD = 5, ST_FROZEN = 6,
       ST_CEA = 7 };
enum { F_UPDATE_THERMO = 1, F_RETRY = 2 };

constexpr double MIN_MOLES = 1.0e-30;
constexpr double ZERO_EPS = 1.0e-50;
constexpr double H_MIN = 1.0e-15;
constexpr double ALLOWABLE_MASSF_ERROR = 1.0e-3;

// ---------------------------------------------------------------- compares on the integer pipe
// An FP64 compare (DSETP) takes an FP64 issue slot, as costly as an FMA on this GPU, while the
// bit patterns of doubles can be compared on the integer pipe: for doubles of the same sign the
// patterns order like the values.  Each helper below gives exactly the IEEE result, NaN included,
// for the operands its comment allows; the kernel's hot loops compare through them.
constexpr long long ABS_BITS = 0x7fffffffffffffffLL;
constexpr long long INF_BITS = 0x7ff0000000000000LL;
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
// x < c, any x, c > 0 finite
__device__ __forceinline__ bool lt_pos(double x, double c) {
    const long long b = dbits(x);
    return b < dbits(c) && (b >= 0 || (b & ABS_BITS) <= INF_BITS);
}
// x > c, any x, c >= 0 finite
__device__ __forceinline__ bool gt_pos(double x, double c) {
    const long long b = dbits(x);
    return b > dbits(c) && b <= INF_BITS;
}
// x >= c, any x, c > 0 finite
__device__ __forceinline__ bool ge_pos(double x, double c) {
    const long long b = dbits(x);
    return b >= dbits(c) && b <= INF_BITS;
}
// fmin(x, c), any x, c > 0 finite
__device__ __forceinline__ double min_pos(double x, double c) { return lt_pos(x, c) ? x : c; }
// a > b for a, b >= +0 or NaN of either sign (not -0.0)
__device__ __forceinline__ bool gt_nn(double a, double b) {
    const unsigned long long ua = (unsigned long long)dbits(a), ub = (unsigned long long)dbits(b);
    return ua > ub && ua <= (unsigned long long)INF_BITS && ub <= (unsigned long long)INF_BITS;
}
// a >= b for a, b >= +0 or NaN of either sign (not -0.0)
__device__ __forceinline__ bool ge_nn(double a, double b) {
    const unsigned long long ua = (unsigned long long)dbits(a), ub = (unsigned long long)dbits(b);
    return ua >= ub && ua <= (unsigned long long)INF_BITS && ub <= (unsigned long long)INF_BITS;
}
// x != 0.0 (either sign of zero), any x
__device__ __forceinline__ bool nonzero(double x) { return (dbits(x) & ABS_BITS) != 0; }
// |x| as a double with the sign bit cleared (an integer operation)
__device__ __forceinline__ double abs_bits(double x) { return __longlong_as_double(dbits(x) & ABS_BITS); }
#if GDTK_MIX_THERMO
// GDTK_MIX_TLO <= T <= GDTK_MIX_THI (both bounds positive), any T
__device__ __forceinline__ bool in_mix_range(double T) {
    const long long t = dbits(T);
    return t >= dbits(GDTK_MIX_TLO) && t <= dbits(GDTK_MIX_THI);
}
#endif

// ---------------------------------------------------------------- species thermo
// Segment choice of cea_thermo_curves.d:150-182: coefficients sa blended towards sb by wb.
// th[10] holds the segment count as integer bits; th[10 + i] and th[13 + i] the blend window
// [break_i - blend_{i-1}/2, break_i + blend_{i-1}/2] around break i (i = 1..nseg-1, formed on the
// host with the reference's arithmetic), th[16 + i] 1 / blend_{i-1}.  The bounds are positive, so
// for any T but NaN (rejected first) the compares are exact on the bit patterns.
__device__ __forceinline__ bool seg_of(const double* th, double T, int& sa, int& sb, double& wb) {
    const int nseg = (int)dbits(th[10]);
    const long long t = dbits(T);
    wb = 0.0;
    if ((t & ABS_BITS) > INF_BITS) return false;   // NaN
    if (nseg == 1) { sa = sb = 0; return true; }
    if (t < dbits(th[11])) { sa = sb = 0; return true; }
    if (t > dbits(th[12 + nseg])) { sa = sb = nseg - 1; return true; }
    for (int i = 1; i < nseg; ++i) {
        const long long lo = dbits(th[10 + i]), hi = dbits(th[13 + i]);
        if (t >= lo && t <= hi) { wb = th[16 + i] * (T - th[10 + i]); sa = i - 1; sb = i; return true; }
        if (t > hi && i < nseg - 1 && t < dbits(th[11 + i])) { sa = sb = i; return true; }
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
    if (lt_pos(T, th[0])) { H = th[2] - th[4] * (th[0] - T); Cp = th[4]; return; }
    if (gt_pos(T, th[1])) { H = th[3] + th[5] * (T - th[1]); Cp = th[5]; return; }
    int sa, sb;
    double wb;
    if (!seg_of(th, T, sa, sb, wb)) { err = ST_CEA; H = 0.0; Cp = 1.0; return; }
    const double* ca = th + GDTK_TH_SEG0 + 24 * sa;
    H = poly_H(ca, T, lnT, rT);
    Cp = poly_Cp(ca + 8, T, rT, rT2);
    if (nonzero(wb)) {
        const double* cb = th + GDTK_TH_SEG0 + 24 * sb;
        H = fma(wb, poly_H(cb, T, lnT, rT) - H, H);
        Cp = fma(wb, poly_Cp(cb + 8, T, rT, rT2) - Cp, Cp);
    }
}

__device__ __forceinline__ double sp_G(const double* TH, int i, double T, double lnT, double rT, double rT2, double t1,
                                       double t2, int& err) {
    const double* th = TH + i * GDTK_TH_STRIDE;
    if (lt_pos(T, th[0])) {
        double H = th[2] - th[4] * (th[0] - T), S = th[6] - th[4] * (th[8] - lnT);
        return fma(H, rT, -S);
    }
    if (gt_pos(T, th[1])) {
        double H = th[3] + th[5] * (T - th[1]), S = th[7] + th[5] * (lnT - th[9]);
        return fma(H, rT, -S);
    }
    int sa, sb;
    double wb;
    if (!seg_of(th, T, sa, sb, wb)) { err = ST_CEA; return 0.0; }
    double g = poly_G(TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 24 * sa + 15, T, rT, rT2, t1, t2);
    if (nonzero(wb)) g = fma(wb, poly_G(TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 24 * sb + 15, T, rT, rT2, t1, t2) - g, g);
    return g;
}

// T from (rho, u) at fixed composition, therm_perf_gas_mix.d:426-468 (same iteration, same
// stopping rules).  YR[i * ys] = Y_i R_i.  *iters counts iterations.  Out of line: it is
// called after accepted steps and at the end of a cell, and one copy of its code serves both.
//
// Where every species takes the same curve segment (GDTK_MIX_TLO <= T <= GDTK_MIX_THI, checked by
// the generator), the mixture's H/R is the same polynomial with coefficients sum_i Y_i R_i c_i,
// and its Cp/R the derivative of that polynomial: the 8 mixture coefficients are formed once per
// segment and solve (in the caller's scratch S, stride ys), and each iteration then costs one
// polynomial instead of one per species.  The sums are reassociated, so f and cv differ from the
// per-species sums in the last bits only.
#if GDTK_MIX_THERMO
// One pass over the species with the 8 sums in registers: each sum still adds the species in
// order 0..nsp-1, and the 8 chains are independent of one another.
__device__ __forceinline__ void mix_coeffs(const double* TH, const double* YR, int ys, int seg, double* m) {
    double acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0.0;
#pragma unroll 1
    for (int i = 0; i < GDTK_NSP; ++i) {
        const double yr = YR[i * ys];
        const double* c = TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 24 * seg;
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = fma(yr, c[k], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) m[k * ys] = acc[k];
    // the Cp/R = d(H/R)/dT coefficients k h_k of the polynomial part, once per segment
#pragma unroll
    for (int k = 3; k < 7; ++k) m[(5 + k) * ys] = (double)(k - 1) * acc[k];
}
// H/R and Cp/R = d(H/R)/dT of the mixture polynomial m (H/R = -a0/T + a1 lnT + a7 + a2 T + a3/2 T^2 + ...;
// m[8..11] = 2 h3, 3 h4, 4 h5, 5 h6)
__device__ __forceinline__ void mix_H_Cp(const double* m, int ys, double T, double lnT, double rT, double rT2,
                                         double& H, double& Cp) {
    const double h0 = m[0], h1 = m[ys], h2 = m[2 * ys], h3 = m[3 * ys], h4 = m[4 * ys], h5 = m[5 * ys],
                 h6 = m[6 * ys], h7 = m[7 * ys];
    H = fma(T, fma(T, fma(T, fma(T, fma(T, h6, h5), h4), h3), h2), fma(h0, rT, fma(h1, lnT, h7)));
    Cp = fma(T, fma(T, fma(T, fma(T, m[11 * ys], m[10 * ys]), m[9 * ys]), m[8 * ys]), fma(-h0, rT2, fma(h1, rT, h2)));
}
#endif

// ln(T (1 + x)) from ln T: ln T + log1p(x) by its Taylor series to x^6 when |x| < 2^-10 (the
// truncation is below 2^-60 |x|), else a fresh log.  The kernel carries ln T with each cell this way,
// because a library log costs as much FP64 issue as about 36 FMAs.
__device__ __forceinline__ double ln_step(double lnT, double x, double T) {
    if ((dbits(x) & ABS_BITS) < dbits(0x1p-10))
        return lnT + x * fma(x, fma(x, fma(x, fma(x, fma(x, -1.0 / 6.0, 0.2), -0.25), 1.0 / 3.0), -0.5), 1.0);
    return log(T);
}

// *lnT_io: ln T_guess on entry, ln of the returned T on exit.  ysum = sum_i Y_i R_i, added in species order.
// S: 24 doubles (stride ys) of scratch for the mixture coefficients.
__device__ __noinline__ double T_from_u(const double* TH, const double* YR, int ys, double* S, double u_tgt,
                                        double T_guess, double ysum, double* lnT_io, int* err, int* iters,
                                        unsigned long long* lst) {
    const double TOL = 1e-10;
    double T = T_guess, dT = 0.0, lnT = *lnT_io, rT = gdtk_div(1.0, T);
#if GDTK_MIX_THERMO
    double* ma = S;
    double* mb = S + 12 * ys;
    int seg_a = -1, seg_b = -1;
#else
    (void)S;
    (void)ysum;
#endif
    for (int it = 0; it <= 10; ++it) {
        lane_stat(lst, 4);
        if (it > 0) {
            const double x = dT * rT;   // dT / T of the previous iterate
            T += dT;
            lnT = ln_step(lnT, x, T);
            // |dT| / T < TOL (therm_perf_gas_mix.d:452) with the reciprocal the next iteration needs
            rT = gdtk_div(1.0, T);
            if (lt_pos(abs_bits(dT) * rT, TOL)) { *lnT_io = lnT; return T; }
            if (it == 10) break;
        }
        const double rT2 = rT * rT;
        double f = 0.0, cv = 0.0;
#if GDTK_MIX_THERMO
        int sa = 0, sb = 0;
        double wb = 0.0;
        if (in_mix_range(T) && seg_of(TH, T, sa, sb, wb)) {
            if (sa != seg_a) { mix_coeffs(TH, YR, ys, sa, ma); seg_a = sa; }
            double H, C;
            mix_H_Cp(ma, ys, T, lnT, rT, rT2, H, C);
            if (nonzero(wb)) {
                if (sb != seg_b) { mix_coeffs(TH, YR, ys, sb, mb); seg_b = sb; }
                double Hb, Cb;
                mix_H_Cp(mb, ys, T, lnT, rT, rT2, Hb, Cb);
                H = fma(wb, Hb - H, H);
                C = fma(wb, Cb - C, C);
            }
            f = fma(-ysum, T, H);
            cv = C - ysum;
        } else
#endif
        {
#pragma unroll 1
            for (int i = 0; i < GDTK_NSP; ++i) {
                double H, Cp;
                int e = 0;
                sp_H_Cp(TH, i, T, lnT, rT, rT2, H, Cp, e);
                if (e) *err = e;
                const double yr = YR[i * ys];
                f = fma(yr, H - T, f);
                cv = fma(yr, Cp - 1.0, cv);
            }
        }
        dT = -gdtk_div_nr(f - u_tgt, cv);
        ++*iters;
    }
    if (gt_pos(abs_bits(dT), 1e-3)) *err = ST_NEWTON;
    *lnT_io = lnT;
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

// Rate constants at T (clamped to the mechanism's limits, reaction_mechanism.d:49-63); the
// species G/RT go through the per-thread scratch vector G.
// G: scratch of GDTK_NSP slots (stride ks); the third-body concentrations of the pressure-dependent
// rate constants (gen_falloff_M) are read from the GDTK_NFALLOFF slots after it.
__device__ __noinline__ void rate_constants(const double* TH, double Tq, double lnTq, double* K, int ks,
                                            const double* etab, double* G, int* err) {
    double T = Tq, lnT = lnTq;   // lnTq = ln Tq
    if (lt_pos(T, GDTK_T_LOWER)) { T = GDTK_T_LOWER; lnT = GDTK_LN_T_LOWER; }
    if (gt_pos(T, GDTK_T_UPPER)) { T = GDTK_T_UPPER; lnT = GDTK_LN_T_UPPER; }
    const double rT = gdtk_div(1.0, T), rT2 = rT * rT, t1 = lnT + 1.0, t2 = 1.0 - lnT;
    int e = 0;
#if GDTK_MIX_THERMO
    // every species takes the same curve segment and blend here: choose them once
    int sa = 0, sb = 0;
    double wb = 0.0;
    if (in_mix_range(T) && seg_of(TH, T, sa, sb, wb)) {
        GDTK_G_UNROLL
        for (int i = 0; i < GDTK_NSP; ++i) {
            const double* c = TH + i * GDTK_TH_STRIDE + GDTK_TH_SEG0 + 15;
            double g = poly_G(c + 24 * sa, T, rT, rT2, t1, t2);
            if (nonzero(wb)) g = fma(wb, poly_G(c + 24 * sb, T, rT, rT2, t1, t2) - g, g);
            G[i * ks] = g;
        }
    } else
#endif
    {
        GDTK_G_UNROLL
        for (int i = 0; i < GDTK_NSP; ++i) G[i * ks] = sp_G(TH, i, T, lnT, rT, rT2, t1, t2, e);
    }
    if (e) *err = e;
    gen_kc(T, lnT, rT, G, ks, K, ks, etab, G + GDTK_NSP * ks, ks);
}

// reaction_mechanism.d:161-203 from the rates at c.
__device__ __forceinline__ double estimate_step(const double (&c)[GDTK_NSP], const double (&q)[GDTK_NSP],
                                                const double (&L)[GDTK_NSP]) {
    double min_dt = 1.0e6;
#pragma unroll
    for (int i = 0; i < GDTK_NSP; ++i) {
        if (c[i] > 0.0 && fabs(q[i] - L[i]) > 1.0e-30) {
            double dt = (q[i] > 10000.0 * L[i]) ? gdtk_div(c[i], L[i] + ZERO_EPS) : fabs(gdtk_div(c[i], q[i] - L[i]));
            min_dt = fmin(min_dt, dt);
        }
    }
    double dt_chem = 1.0e-3 * min_dt;
    dt_chem = fmin(dt_chem, 1.0e-10);
    return fmax(dt_chem, 1.0e-15);
}

// alpha = N/D (chemistry_update.d:599-604) as N(s)/D(s), s = p h, the reference's rational
// function of r = 1 / (p h + eps) with numerator and denominator multiplied by s^3.  The form has
// no division by s, so the reference's eps (1e-50, which guards its 1 / (p h)) changes nothing
// above s = 1e-34 and is left out.  For s >= 1e50 the ratio is 1 to double precision in either
// form, so s is capped there, which keeps N and D finite without a branch.
__device__ __forceinline__ void alpha_nd(double s, double& N, double& D) {
    s = min_pos(s, 1.0e50);
    N = fma(s, fma(s, 11.0 + s, 60.0), 180.0);
    D = fma(s, s, N + 180.0);   // s^3 + 12 s^2 + 60 s + 360 = N + s^2 + 180
}

// ---------------------------------------------------------------- the kernel
#if GDTK_METHOD == 0
// Cash-Karp stage coefficients a[s][j] (stage s + 1 from k_1..k_s), chemistry_update.d:409-412
__constant__ double RKF_A[5][5] = {
    {1. / 5., 0, 0, 0, 0},
    {3. / 40., 9. / 40., 0, 0, 0},
    {3. / 10., -9. / 10., 6. / 5., 0, 0},
    {-11. / 54., 5. / 2., -70. / 27., 35. / 27., 0},
    {1631. / 55296., 175. / 512., 575. / 13824., 44275. / 110592., 253. / 4096.}};
#endif
// GDTK_VEC (per-thread method vector, doubles) comes from the generator: the method's stage
// storage, at least nsp + 16 when T(rho, u) uses mixture coefficients

extern "C" __global__ void __launch_bounds__(GDTK_BLOCK, GDTK_MIN_BLOCKS) gdtk_chem_fast(const __grid_constant__ FastArgs a) {
    extern __shared__ double smem[];
    double* TH = smem;                                   // thermo table, nsp * stride
    double* ETAB = smem + GDTK_NSP * GDTK_TH_STRIDE;     // exp table, GDTK_EXP2_TABLE_SIZE
    const CellBlock* BLK = a.blocks;
    double* S = ETAB + GDTK_EXP2_TABLE_SIZE;             // per-thread vectors
    for (int k = threadIdx.x; k < GDTK_NSP * GDTK_TH_STRIDE; k += blockDim.x) TH[k] = a.thermo[k];
    for (int k = threadIdx.x; k < GDTK_EXP2_TABLE_SIZE; k += blockDim.x) ETAB[k] = a.exp_table[k];
    __syncthreads();
    const int ks = blockDim.x;
    double* K = S + threadIdx.x;                         // kf[NR], kb[NR]
    double* V = K + 2 * GDTK_NR * ks;                    // method vectors; also G/RT and Y_i R_i scratch
#if GDTK_PHASE_CLOCKS
    if ((threadIdx.x & 31) == 0) gdtk_pc_ph[threadIdx.x >> 5] = -1;
    __syncwarp();
#endif

    unsigned g = 0;
    int b = 0, ci = 0;
    bool have = false, alive = true, retried = false, need_kc = false;
    int phase = 0, cycle = 0, attempt = 0, err = 0;
    double rho = 0, rrho = 0, u = 0, T = 0, lnT = 0, p = 0, dtS = 0, dtS0 = 0, dtSave = 0, h = 0, t = 0, tI = 0;
    double y0[GDTK_NSP];
    int n_steps = 0, n_rhs = 0, n_kc = 0, n_newton = 0, n_rej = 0, n_est = 0;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;

    // All 32 lanes of a warp stay in this loop until the whole warp is out of work, so that
    // every iteration can re-converge them (__syncwarp) and lanes that refill with a new cell
    // run the same iteration as their neighbours instead of splitting the warp.
    unsigned q_lo = 0, q_hi = 0;   // visit positions this warp has reserved and not yet handed out
    while (true) {
        const unsigned need = __ballot_sync(FULL, alive && !have);
        if (need) {   // refill: at most one atomic per warp for all lanes that need a cell
            const int leader = __ffs(need) - 1;
            const unsigned n_need = __popc(need), rank = __popc(need & ((1u << lane) - 1u));
            unsigned pos;
            if (a.refill_chunk <= 1) {
                unsigned base = 0;
                if (lane == leader) base = atomicAdd(a.counter, n_need);
                pos = __shfl_sync(FULL, base, leader) + rank;
            } else {   // chunks of refill_chunk (>= 32) positions: the reserve, then a new chunk
                const unsigned left = q_hi - q_lo;
                unsigned nb = 0;
                if (left < n_need) {
                    if (lane == leader) nb = atomicAdd(a.counter, (unsigned)a.refill_chunk);
                    nb = __shfl_sync(FULL, nb, leader);
                }
                pos = rank < left ? q_lo + rank : nb + (rank - left);
                if (left < n_need) {
                    q_lo = nb + (n_need - left);
                    q_hi = nb + (unsigned)a.refill_chunk;
                } else {
                    q_lo += n_need;
                }
            }
            if (alive && !have) {
                g = pos;
                if (g >= (unsigned)a.total) {
                    alive = false;
                } else {
                    if (a.order) g = (unsigned)a.order[g];
                    int lo = 0, hi = a.nblocks - 1;          // last block with first <= g
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if ((unsigned)BLK[mid].first <= g) lo = mid; else hi = mid - 1;
                    }
                    b = lo;
                    ci = (int)(g - (unsigned)BLK[b].first);
                    const CellBlock& B = BLK[b];
                    rho = B.rho[ci]; u = B.u[ci]; tI = B.t_interval; dtS0 = B.dt_chem[ci];
                    if (B.T[ci] <= a.T_frozen) {
                        if (B.status) B.status[ci] = ST_FROZEN;
                    } else if (isnan(rho) || rho <= 0.0) {
                        if (B.status) B.status[ci] = ST_BAD;
                    } else {
                        have = true;
                        retried = false;
                        rrho = gdtk_div(1.0, rho);
                        n_steps = n_rhs = n_kc = n_newton = n_rej = n_est = 0;
                        phase = -1;
                    }
                }
            }
        }
        const unsigned hm = __ballot_sync(FULL, have);
        if (need) lane_stat(a.lane_stats, 6);
        if (!__any_sync(FULL, alive || have)) break;
        if (have) {
        lane_stat(a.lane_stats, 0);
        if (phase == -1) {   // (re)start from the stored input state
            const CellBlock& B = BLK[b];
            T = B.T[ci]; p = B.p[ci]; dtS = dtS0; t = 0.0; err = 0;
            lnT = log(T);
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double v = B.massf[(size_t)i * B.ncell + ci] * rho * GDTK_RM[i];
                y0[i] = (v < MIN_MOLES) ? 0.0 : v;
            }
            need_kc = true;
            phase = 0;
        }
        if (need_kc) {
            lane_stat(a.lane_stats, 1);
            if (GDTK_NFALLOFF) gen_falloff_M(y0, V + GDTK_NSP * ks, ks);
            rate_constants(TH, T, lnT, K, ks, ETAB, V, &err);
            ++n_kc;
            need_kc = false;
        }
        __syncwarp(hm);
        ++n_steps;
        double yn[GDTK_NSP];   // stage input, then the step's result
        bool ok = false;
#if GDTK_METHOD == 0
        // Runge-Kutta-Fehlberg with Cash-Karp coefficients, chemistry_update.d:404-478.
        // V holds k_1..k_6; all six right-hand sides share one call site.
        double errn = 0.0;
#pragma unroll 1
        for (int s = 0; s < 6; ++s) {
            double q[GDTK_NSP], L[GDTK_NSP];
            {
                double cin[GDTK_NSP];
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) cin[i] = (s == 0) ? y0[i] : yn[i];
                gen_rhs(cin, q, L, K, ks);
            }
            ++n_rhs;
            if (s == 0) {
                if (phase == 0) {
                    if (dtS > tI) h = tI;
                    else if (dtS <= 0.0) { h = estimate_step(y0, q, L); ++n_est; ++n_rhs; }
                    else h = dtS;
                    cycle = 0;
                    phase = 1;
                }
                if (phase == 1) { dtSave = dtS; h = fmin(h, tI - t); attempt = 0; phase = 2; }
            }
            double* kv = V + s * GDTK_NSP * ks;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) kv[i * ks] = q[i] - L[i];
            if (s < 5) {
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double acc = RKF_A[s][0] * V[i * ks];
                    for (int j = 1; j <= s; ++j) acc = fma(RKF_A[s][j], V[(j * GDTK_NSP + i) * ks], acc);
                    yn[i] = fma(h, acc, y0[i]);
                }
            } else {
                const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771.,
                    b41 = 2825. / 27648., b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336.,
                    b46 = 1.0 / 4.0;
                double err2 = 0.0;
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double K1 = V[i * ks], K3 = V[(2 * GDTK_NSP + i) * ks], K4 = V[(3 * GDTK_NSP + i) * ks],
                           K5 = V[(4 * GDTK_NSP + i) * ks], K6 = V[(5 * GDTK_NSP + i) * ks];
                    double o = fma(h, fma(b56, K6, fma(b54, K4, fma(b53, K3, b51 * K1))), y0[i]);
                    double o4 = fma(h, fma(b46, K6, fma(b45, K5, fma(b44, K4, fma(b43, K3, b41 * K1)))), y0[i]);
                    double sk = fma(GDTK_ERRTOL, fmax(fabs(y0[i]), fabs(o)), GDTK_ERRTOL);
                    double e = gdtk_div(o - o4, sk);
                    err2 = fma(e, e, err2);
                    yn[i] = o;
                }
                errn = sqrt(err2 * (1.0 / GDTK_NSP));
            }
        }
        {
            double scale;
            if (errn <= 1.0) {
                scale = (errn == 0.0) ? 10.0 : fmin(fmax(0.9 * gdtk_exp(-0.2 * log(errn), ETAB), 0.2), 10.0);
                ok = true;
            } else {
                scale = fmax(0.9 * gdtk_exp(-0.2 * log(errn), ETAB), 0.2);
            }
            dtS = scale * h;
        }
#else
        // alpha-QSS, chemistry_update.d:533-655.  Iteration 0 is the predictor, 1..maxIters the
        // correctors; with q0 = q and p0 = p the corrector formula reduces to the predictor's, so
        // one update (and one right-hand-side call site) serves both.  V holds q0, p0, yp0.
        {
            double* Q0 = V;
            double* P0 = V + GDTK_NSP * ks;
            double* YP0 = V + 2 * GDTK_NSP * ks;
            bool conv = false;
#pragma unroll 1
            for (int s = 0; s <= GDTK_MAX_ITERS; ++s) {
                double q[GDTK_NSP], L[GDTK_NSP];
                {
                    double cin[GDTK_NSP];
#pragma unroll
                    for (int i = 0; i < GDTK_NSP; ++i) cin[i] = (s == 0) ? y0[i] : yn[i];
                    lane_stat(a.lane_stats, 2);
                    gen_rhs(cin, q, L, K, ks);
                }
                lane_stat(a.lane_stats, 7);
                ++n_rhs;
                if (s == 0) {
                    if (phase == 0) {
                        if (dtS > tI) h = tI;
                        else if (dtS <= 0.0) { h = estimate_step(y0, q, L); ++n_est; ++n_rhs; }
                        else h = dtS;
                        cycle = 0;
                        phase = 1;
                    }
                    if (phase == 1) { dtSave = dtS; h = fmin(h, tI - t); attempt = 0; phase = 2; }
                }
                conv = true;
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    const double y = y0[i];
                    const double ci_ = (s == 0) ? y : yn[i];
                    const double pp = gdtk_div_nr(L[i], ci_ + ZERO_EPS);
                    double N, D;
                    alpha_nd(pp * h, N, D);
                    const double q0 = (s == 0) ? q[i] : Q0[i * ks];
                    const double pb = (s == 0) ? pp : fma(0.5, pp, P0[i * ks]);   // P0 holds p0 / 2
                    // y + h (N (q - q0) + D (q0 - pb y)) / (N h pb + D)
                    const double num = h * fma(N, q[i] - q0, D * fma(-pb, y, q0));
                    const double v = gdtk_add_div(y, num, fma(N, h * pb, D));
                    if (s == 0) {
                        Q0[i * ks] = q[i];
                        P0[i * ks] = 0.5 * pp;
                        YP0[i * ks] = v;
                    } else if (!lt_pos(v, ZERO_EPS) &&
                               ge_nn(abs_bits(v - YP0[i * ks]), fma(GDTK_EPS1, v, GDTK_EPS1 * GDTK_DELTA))) {
                        conv = false;
                    }
                    yn[i] = v;
                }
                if (s > 0 && conv) break;
            }
            // sigma = max_i |yc - yp0| / (eps2 (yc + delta)), the largest ratio found by comparing
            // cross products (denominators are positive), then one division
            double snum = 0.0, sden = 1.0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double yc = yn[i];
                if (lt_pos(yc, ZERO_EPS)) continue;
                const double num = abs_bits(yc - YP0[i * ks]), den = fma(GDTK_EPS2, yc, GDTK_EPS2 * GDTK_DELTA);
                if (gt_nn(num * sden, snum * den)) { snum = num; sden = den; }
            }
            const double sigma = gdtk_div(snum, sden);
            if (!nonzero(sigma)) dtS = 10.0 * h;   // sigma <= 0 (sigma is >= 0 or NaN)
            else {
                double x = sigma;
                x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
                x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
                x = x - 0.5 * gdtk_div_nr(x * x - sigma, x);
                dtS = h * (gdtk_div(1.0, x) + 0.005);
            }
            ok = conv;
        }
#endif
        __syncwarp(hm);
        lane_stat(a.lane_stats, 3);
        if (ok) {   // mass-fraction test (chemistry_update.d:175-185); the Y_i go to V for the thermo update
            double tot = sum_pairwise([&](int i) {
                double v = yn[i] * GDTK_M[i] * rrho;
                v = lt_pos(v, 1.0e-30) ? 0.0 : v;
                V[i * ks] = v;
                return v;
            });
            if (gt_pos(abs_bits(tot - 1.0), ALLOWABLE_MASSF_ERROR)) ok = false;
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
            {   // chemistry_update.d:265-269; Y_i (from the mass-fraction test) -> Y_i R_i in V, free until the next step
                double Rm = 0.0;
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double yr = V[i * ks] * GDTK_R[i];
                    V[i * ks] = yr;
                    Rm += yr;
                }
                T = T_from_u(TH, V, ks, V + GDTK_NSP * ks, u, T, Rm, &lnT, &err, &n_newton, a.lane_stats);
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
            if ((a.flags & F_RETRY) && retryable && !retried) {   // fluidfvcell.d:924-941
                retried = true;
                dtS0 = -1.0;
                phase = -1;
            } else {
                if (BLK[b].status) BLK[b].status[ci] = fail;
                have = false;
            }
        }
        if (done) {   // chemistry_update.d:290-325, then fluidfvcell.d:956
            lane_stat(a.lane_stats, 5);
            auto mf_of = [&](int i) {
                double v = y0[i] * GDTK_M[i] * rrho;
                return lt_pos(v, 1.0e-30) ? 0.0 : v;
            };
            double rtot = gdtk_div(1.0, sum_pairwise(mf_of));
            double Rm = 0.0;
#pragma unroll
            for (int i = 0; i < GDTK_NSP; ++i) {
                double yr = mf_of(i) * rtot * GDTK_R[i];
                V[i * ks] = yr;
                Rm += yr;
            }
            int st = 0;
            if (a.flags & F_UPDATE_THERMO) {
                T = T_from_u(TH, V, ks, V + GDTK_NSP * ks, u, T, Rm, &lnT, &st, &n_newton, a.lane_stats);
                p = rho * Rm * T;
            }
            const CellBlock& B = BLK[b];
            if (st) {
                if (B.status) B.status[ci] = st;
            } else {
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) B.massf[(size_t)i * B.ncell + ci] = mf_of(i) * rtot;
                B.T[ci] = T;
                B.p[ci] = p;
                B.dt_chem[ci] = dtSave;
                if (B.status) B.status[ci] = ST_OK;
            }
            have = false;
        }
        if (!have) {
            if (a.cell_counters) {
                const size_t n = (size_t)a.total;
                a.cell_counters[0 * n + g] = n_steps;
                a.cell_counters[1 * n + g] = n_rhs;
                a.cell_counters[2 * n + g] = n_kc;
                a.cell_counters[3 * n + g] = n_newton;
                a.cell_counters[4 * n + g] = n_rej;
                a.cell_counters[5 * n + g] = n_est;
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
        }   // if (have)
        __syncwarp(FULL);
    }
}

// Expected cost of each cell, for longest-first scheduling of the persistent kernel: the
// number of steps the 10%-per-step growth limit alone imposes (chemistry_update.d:204-219)
// from the cell's first step size -- dt_chem when the cell carries one, otherwise the
// estimate of reaction_mechanism.d:161-203 (rate constants + one right-hand side).
extern "C" __global__ void __launch_bounds__(GDTK_BLOCK, GDTK_MIN_BLOCKS) gdtk_chem_cost(const __grid_constant__ FastArgs a,
                                                                                     float* key) {
    extern __shared__ double smem[];
    double* TH = smem;
    double* ETAB = smem + GDTK_NSP * GDTK_TH_STRIDE;
    double* S = ETAB + GDTK_EXP2_TABLE_SIZE;
    for (int k = threadIdx.x; k < GDTK_NSP * GDTK_TH_STRIDE; k += blockDim.x) TH[k] = a.thermo[k];
    for (int k = threadIdx.x; k < GDTK_EXP2_TABLE_SIZE; k += blockDim.x) ETAB[k] = a.exp_table[k];
    __syncthreads();
    const int ks = blockDim.x;
    double* K = S + threadIdx.x;
    double* V = K + 2 * GDTK_NR * ks;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < a.total; g += gridDim.x * blockDim.x) {
        int lo = 0, hi = a.nblocks - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (a.blocks[mid].first <= g) lo = mid; else hi = mid - 1;
        }
        const CellBlock& B = a.blocks[lo];
        const int ci = g - B.first;
        const double rho = B.rho[ci], T = B.T[ci], dtc = B.dt_chem[ci], tI = B.t_interval;
        float k = 0.0f;
        if (T > a.T_frozen && rho > 0.0) {
            double h;
            if (dtc > 0.0) {
                h = fmin(dtc, tI);
            } else {
                double y[GDTK_NSP], q[GDTK_NSP], L[GDTK_NSP];
#pragma unroll
                for (int i = 0; i < GDTK_NSP; ++i) {
                    double v = B.massf[(size_t)i * B.ncell + ci] * rho * GDTK_RM[i];
                    y[i] = (v < MIN_MOLES) ? 0.0 : v;
                }
                int err = 0;
                if (GDTK_NFALLOFF) gen_falloff_M(y, V + GDTK_NSP * ks, ks);
                rate_constants(TH, T, log(T), K, ks, ETAB, V, &err);
                gen_rhs(y, q, L, K, ks);
                h = estimate_step(y, q, L);
            }
            k = (float)(log1p(0.1 * tI / h) * 10.492058687799444);   // / ln 1.1
        }
        key[g] = k;
    }
}

}  // namespace gdtk_fast
