// codegen.cpp -- writes the mechanism as CUDA, compiles it with NVRTC for the device at hand, and
// launches it.
//
// The generated part is small: compile-time sizes and tolerances, the species constants, and
// two functions -- gen_kc (rate constants: a loop over a __constant__ table of the Arrhenius
// reactions, the pressure-dependent ones straight-line) and gen_rhs (production/loss rates,
// straight-line) -- in which every species index, stoichiometric coefficient, third-body
// efficiency and Arrhenius parameter is a literal or a table entry.  The integrator around them is chem_fast.cuh.  The reference
// interprets its reaction objects at run time (kinetics/reaction_mechanism.d:82-96,
// reaction.d:145-149, 267-311, 394-456); its legacy GPU path generated source in a similar
// spirit, from prep-chem's compact notation (eilmer/utils/prep-cuda-gpu-chem-kernel.py).
#include "codegen.h"

#include <cuda.h>
#include <nvrtc.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>
#include <unistd.h>

#include "cea_thermo.h"
#include "chem_types.h"
#include "fast_exp.h"
#include "chem_launch.h"

namespace gdtk {

extern const char* const kFastCuhSource;
extern const char* const kFastExpSource;

namespace {

constexpr double R_universal = 8.31451;

std::string lit(double v) {   // exact double literal
    char buf[64];
    std::snprintf(buf, sizeof buf, "%a", v);
    std::string s(buf);
    if (v == 0.0) return "0.0";
    return s;
}

// ---- driver entry points, resolved through the runtime (no link-time libcuda dependency)
struct Driver {
    CUresult (*moduleLoadData)(CUmodule*, const void*) = nullptr;
    CUresult (*moduleUnload)(CUmodule) = nullptr;
    CUresult (*moduleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*funcSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*launchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
    CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
    CUresult (*getErrorString)(CUresult, const char**) = nullptr;
};

template <typename F>
void resolve(const char* name, F& fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
        throw std::runtime_error(std::string("cannot resolve driver entry point ") + name);
    fn = reinterpret_cast<F>(p);
}

Driver& driver() {
    static Driver d;
    static std::once_flag once;
    static std::string failure;
    std::call_once(once, [] {
        try {
            resolve("cuModuleLoadData", d.moduleLoadData);
            resolve("cuModuleUnload", d.moduleUnload);
            resolve("cuModuleGetFunction", d.moduleGetFunction);
            resolve("cuFuncSetAttribute", d.funcSetAttribute);
            resolve("cuLaunchKernel", d.launchKernel);
            resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", d.occupancy);
            resolve("cuGetErrorString", d.getErrorString);
        } catch (std::exception& e) {
            failure = e.what();
        }
    });
    if (!failure.empty()) throw std::runtime_error(failure);
    return d;
}

void cu_check(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return;
    const char* s = "unknown";
    if (driver().getErrorString) driver().getErrorString(r, &s);
    throw std::runtime_error(std::string(what) + ": " + s);
}

// Integer power of a symbol, in the order of D's std.math pow(x, int) (binary exponentiation).
std::string ipow_expr(const std::string& x, int n) {
    if (n == 1) return x;
    if (n == 2) return "(" + x + " * " + x + ")";
    std::string p, v = x;
    unsigned m = (unsigned)n;
    bool have = false;
    while (true) {
        if (m & 1u) { p = have ? "(" + p + " * " + v + ")" : v; have = true; }
        m >>= 1;
        if (!m) break;
        v = "(" + v + " * " + v + ")";
    }
    return p;
}

struct Part { int isp; int nu; };

std::vector<Part> participants(const ReactionHost& r) {
    std::vector<int> sp;
    for (auto& x : r.reac) sp.push_back(x.first);
    for (auto& x : r.prod) sp.push_back(x.first);
    std::sort(sp.begin(), sp.end());
    sp.erase(std::unique(sp.begin(), sp.end()), sp.end());
    std::vector<Part> out;
    for (int isp : sp) {
        int nu1 = 0, nu2 = 0;
        for (auto& x : r.reac) if (x.first == isp) { nu1 = x.second; break; }
        for (auto& x : r.prod) if (x.first == isp) { nu2 = x.second; break; }
        out.push_back({isp, nu2 - nu1});
    }
    return out;
}

// ln k = ln A + n ln T - C / T as an expression; empty if A == 0.
std::string log_arrhenius(const RateConstHost& rc) {
    if (rc.model == RATE_ARRHENIUS2) {   // ln k = logA + B T - C/T (rate_constant.d:112-115)
        std::string e = lit(rc.A);
        if (rc.n != 0.0) e = "fma(" + lit(rc.n) + ", T, " + e + ")";
        if (rc.C != 0.0) e = "fma(" + lit(-rc.C) + ", rT, " + e + ")";
        return e;
    }
    if (rc.A <= 0.0) return "";
    std::string e = lit(std::log(rc.A));
    if (rc.n != 0.0) e = "fma(" + lit(rc.n) + ", lnT, " + e + ")";
    if (rc.C != 0.0) e = "fma(" + lit(-rc.C) + ", rT, " + e + ")";
    return e;
}

// k = A T^n as products when C == 0 and n is a small integer (no exponential needed).
bool power_arrhenius(const RateConstHost& rc, std::string& out) {
    if (rc.model != RATE_ARRHENIUS || rc.C != 0.0 || rc.n != std::floor(rc.n) || std::fabs(rc.n) > 4) return false;
    int n = (int)rc.n;
    if (n == 0) { out = lit(rc.A); return true; }
    out = lit(rc.A) + " * " + ipow_expr(n > 0 ? "T" : "rT", n > 0 ? n : -n);
    return true;
}

// k = A T^n exp(-C/T) as an expression (products, one exponential, or 0).
std::string arrhenius_expr(double A, double n, double C) {
    RateConstHost rc;
    rc.A = A; rc.n = n; rc.C = C;
    std::string e;
    if (power_arrhenius(rc, e)) return e;
    e = log_arrhenius(rc);
    return e.empty() ? std::string("0.0") : "gdtk_exp(" + e + ", etab)";
}

// Forward rate constant of a pressure-dependent reaction (rate_constant.d:155-160, 258-287,
// 338-350) as statements ending in `kf`, from the third-body concentration `Mc`.  log10 and
// pow(10, x) are written as ln x / ln 10 and exp(x ln 10).
std::string pressure_dependent_code(const RateConstHost& f) {
    std::ostringstream o;
    o << "    const double kinf = " << arrhenius_expr(f.A, f.n, f.C) << ";\n";
    o << "    const double k0 = " << arrhenius_expr(f.A0, f.n0, f.C0) << ";\n";
    o << "    const double klh = k0 * kinf * Mc / fma(k0, Mc, kinf);\n";
    if (f.model == RATE_LH) {
        o << "    const double kf = klh;\n";
    } else if (f.model == RATE_TROE) {
        const double INV_LN10 = 1.0 / std::log(10.0);
        o << "    const double pr = k0 * Mc / kinf;\n";
        o << "    const double lpr = log(fmax(pr, 1.0e-30)) * " << lit(INV_LN10) << ";\n";
        if (f.troe_flags & TROE_FCENT) {
            const double lfc = std::log10(std::max(f.Fcent, 1.0e-30));
            o << "    const double lfc = " << lit(lfc) << ", cc = " << lit(-0.4 - 0.67 * lfc)
              << ", nn = " << lit(0.75 - 1.27 * lfc) << ";\n";
        } else {
            o << "    double fcent = " << lit(1.0 - f.a) << " * gdtk_exp(" << lit(-1.0 / f.T3) << " * T, etab);\n";
            if (f.troe_flags & TROE_T1)
                o << "    fcent = fma(" << lit(f.a) << ", gdtk_exp(" << lit(-1.0 / f.T1) << " * T, etab), fcent);\n";
            if (f.troe_flags & TROE_T2) o << "    fcent += gdtk_exp(" << lit(-f.T2) << " * rT, etab);\n";
            o << "    const double lfc = log(fmax(fcent, 1.0e-30)) * " << lit(INV_LN10) << ";\n";
            o << "    const double cc = fma(-0.67, lfc, -0.4), nn = fma(-1.27, lfc, 0.75);\n";
        }
        o << "    const double numer = lpr + cc;\n";
        o << "    const double frac = numer / fma(-0.14, numer, nn);\n";
        o << "    const double kf = gdtk_exp(lfc / fma(frac, frac, 1.0) * " << lit(std::log(10.0)) << ", etab) * klh;\n";
    } else {   // Yungster-Rabinowitz: a, b, c in a, T1, T2
        o << "    const double pr = k0 * Mc / kinf;\n";
        o << "    const double lpr = log(pr);\n";
        o << "    const double fc = fma(" << lit(f.a) << ", gdtk_exp(" << lit(-f.T1) << " * rT, etab), " << lit(1.0 - f.a)
          << " * gdtk_exp(" << lit(-f.T2) << " * rT, etab));\n";
        o << "    const double kf = kinf * (pr / (1.0 + pr)) * fc / fma(lpr, lpr, 1.0);\n";
    }
    return o.str();
}

}  // namespace

FastKernel::~FastKernel() {
    if (module) driver().moduleUnload((CUmodule)module);
    if (d_thermo) cudaFree(d_thermo);
    if (d_exp) cudaFree(d_exp);
}

std::vector<double> fast_thermo_table(const GasModelHost& gm) {
    const int nsp = gm.n_species();
    PackedMech pm = pack(gm, nullptr);   // reference-form curve ends (cea_thermo_curves.d:46-53)
    MechView v;
    v.bind(pm.I.data(), pm.D.data());
    std::vector<double> t((size_t)nsp * 120, 0.0);
    for (int i = 0; i < nsp; ++i) {
        const CeaCurveHost& c = gm.curves[i];
        const double* s = v.sp(i);
        const double R = R_universal / gm.M[i];
        double* th = t.data() + (size_t)i * 120;
        th[0] = s[SP_TLOW];
        th[1] = s[SP_THIGH];
        th[2] = s[SP_HLOW] / R;
        th[3] = s[SP_HHIGH] / R;
        th[4] = s[SP_CPLOW] / R;
        th[5] = s[SP_CPHIGH] / R;
        th[6] = s[SP_SLOW] / R;
        th[7] = s[SP_SHIGH] / R;
        th[8] = std::log(s[SP_TLOW]);
        th[9] = std::log(s[SP_THIGH]);
        // segment count as integer bits; per break k = 1..nseg-1 the blend window [lo, hi] of
        // cea_thermo_curves.d:150-182 (break -/+ blend/2, the reference's arithmetic) and 1 / blend
        const int64_t nseg_bits = c.nseg;
        std::memcpy(&th[10], &nseg_bits, sizeof nseg_bits);
        for (int k = 1; k < c.nseg; ++k) {
            th[10 + k] = c.breaks[k] - 0.5 * c.blends[k - 1];
            th[13 + k] = c.breaks[k] + 0.5 * c.blends[k - 1];
            th[16 + k] = 1. / c.blends[k - 1];
            if (!(th[10 + k] > 0.0)) throw std::runtime_error("thermo curve blend window below 0 K");
        }
        for (int sg = 0; sg < c.nseg; ++sg) {
            const double* a = c.coeffs.data() + 9 * sg;
            double* h = th + 24 + 24 * sg;
            // H/R = -a0/T + a1 lnT + a7 + T (a2 + T (a3/2 + T (a4/3 + T (a5/4 + T a6/5))))
            h[0] = -a[0]; h[1] = a[1]; h[2] = a[2]; h[3] = a[3] / 2.0; h[4] = a[4] / 3.0; h[5] = a[5] / 4.0;
            h[6] = a[6] / 5.0; h[7] = a[7];
            // Cp/R = a0/T^2 + a1/T + a2 + T (a3 + T (a4 + T (a5 + T a6)))
            for (int k = 0; k < 7; ++k) h[8 + k] = a[k];
            // G/RT = H/RT - S/R
            h[15] = -a[0] / 2.0; h[16] = a[1]; h[17] = a[7]; h[18] = a[2]; h[19] = -a[8];
            h[20] = -a[3] / 2.0; h[21] = -a[4] / 6.0; h[22] = -a[5] / 12.0; h[23] = -a[6] / 20.0;
        }
    }
    return t;
}

// The temperature range where every species takes the same curve segment and blend of
// cea_thermo_curves.d:150-182 (so that the mixture's H/R is one polynomial there): species curves
// with at least two segments and equal first three breaks and first blend range.
// Unroll factors of the rate-constant loops (reaction table, species G/RT): two independent
// iterations in flight give the FP64 pipe work while one waits on its table loads.
int env_int(const char* name, int dflt) {
    const char* e = std::getenv(name);
    return (e && *e) ? std::max(1, std::atoi(e)) : dflt;
}
int kc_unroll() { return env_int("GDTK_KC_UNROLL", 1); }
int g_unroll() { return env_int("GDTK_G_UNROLL", 1); }
// Reactions between compiler fences in gen_rhs (0: none); the fences bound how far the scheduler
// hoists the k_f, k_b loads, and with them the registers held.
int rhs_fence() {
    const char* e = std::getenv("GDTK_RHS_FENCE");
    return (e && *e) ? std::max(0, std::atoi(e)) : 4;
}

bool mix_thermo_range(const GasModelHost& gm, double& tlo, double& thi) {
    const int nsp = gm.n_species();
    if (nsp == 0) return false;
    PackedMech pm = pack(gm, nullptr);
    MechView v;
    v.bind(pm.I.data(), pm.D.data());
    const CeaCurveHost& c0 = gm.curves[0];
    tlo = -1e300;
    thi = 1e300;
    for (int i = 0; i < nsp; ++i) {
        const CeaCurveHost& c = gm.curves[i];
        if (c.nseg < 2 || c0.nseg < 2 || c.breaks[0] != c0.breaks[0] || c.breaks[1] != c0.breaks[1] ||
            c.breaks[2] != c0.breaks[2] || c.blends[0] != c0.blends[0])
            return false;
        tlo = std::max(tlo, v.sp(i)[SP_TLOW]);
        thi = std::min(thi, v.sp(i)[SP_THIGH]);
        if (c.nseg > 2) thi = std::min(thi, c.breaks[2] - 0.5 * c.blends[1]);
    }
    return thi > tlo;
}

// Largest |G_i / R T| of each species over [tlo, thi] (log-spaced samples plus the curve breaks),
// from the same NASA-9 curves, blends and extrapolation the kernels use.
std::vector<double> species_g_bound(const GasModelHost& gm, double tlo, double thi) {
    const int nsp = gm.n_species();
    PackedMech pm = pack(gm, nullptr);
    MechView v;
    v.bind(pm.I.data(), pm.D.data());
    std::vector<double> Ts;
    const int n = 4000;
    for (int k = 0; k <= n; ++k) Ts.push_back(tlo * std::pow(thi / tlo, (double)k / n));
    for (auto& c : gm.curves)
        for (double b : c.breaks)
            if (b > tlo && b < thi) { Ts.push_back(b); Ts.push_back(b * (1 - 1e-9)); Ts.push_back(b * (1 + 1e-9)); }
    std::vector<double> out(nsp, 0.0);
    for (int i = 0; i < nsp; ++i) {
        const double Ri = R_universal / gm.M[i];
        for (double T : Ts) {
            int err = 0;
            const double lT = std::log(T);
            const double g = (cea_h(v, i, T, lT, err) - T * cea_s(v, i, T, lT, err)) / (Ri * T);
            out[i] = (err || !std::isfinite(g)) ? 1e300 : std::max(out[i], std::fabs(g));
        }
    }
    return out;
}

// Reactions whose k_b = k_f / K_c is formed as k_f (R T / P_atm)^(sum nu) prod_i E_i^nu_i with
// E_i = exp(G_i / R T) formed once per species (GDTK_KB_EXP=1 keeps one exp per reaction).  Only where
// every partial product stays inside exp(+-600) over the mechanism's temperature limits, so that no
// product can overflow or underflow.
std::vector<bool> kb_product_reactions(const GasModelHost& gm, const MechanismHost& mh) {
    std::vector<bool> out(mh.reactions.size(), false);
    const char* e = std::getenv("GDTK_KB_EXP");
    if (e && e[0] == '1') return out;
    const std::vector<double> gb = species_g_bound(gm, mh.T_lower, mh.T_upper);
    const double lcf = std::max(std::fabs(std::log(mh.T_lower * R_universal / 101325.0)),
                                std::fabs(std::log(mh.T_upper * R_universal / 101325.0)));
    for (size_t ir = 0; ir < mh.reactions.size(); ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        if (r.frc.pressure_dependent() || r.frc.model != RATE_ARRHENIUS || r.brc.model != RATE_FROM_EQ) continue;
        double bound = 0.0;
        int nusum = 0, np = 0;
        for (auto& pp : participants(r)) {
            bound += std::abs(pp.nu) * gb[pp.isp];
            nusum += pp.nu;
            np += pp.nu != 0;
        }
        bound += std::abs(nusum) * lcf;
        out[ir] = np <= 8 && bound <= 600.0;
    }
    return out;
}

bool any_kb_products(const GasModelHost& gm, const MechanismHost& mh) {
    for (bool b : kb_product_reactions(gm, mh)) if (b) return true;
    return false;
}

// Per-thread method vector (doubles): the ODE method's stage storage, and room for the
// species' Y_i R_i plus two sets of 12 mixture coefficients during T(rho, u).
int fast_vec_doubles(const GasModelHost& gm, const MechanismHost& mh) {
    const int nsp = gm.n_species();
    int vec = (mh.method == METHOD_RKF ? 6 : 3) * nsp;
    double tlo, thi;
    if (mix_thermo_range(gm, tlo, thi)) vec = std::max(vec, nsp + 24);
    int nfall = 0;   // third-body concentrations of pressure-dependent rates, beside G/RT
    for (auto& r : mh.reactions) nfall += r.frc.pressure_dependent() ? 1 : 0;
    // G/RT, the falloff concentrations, then E_i and 1/E_i for the product-form k_b
    return std::max(vec, (any_kb_products(gm, mh) ? 3 * nsp : nsp) + nfall);
}

std::string generate_fast_source(const GasModelHost& gm, const MechanismHost& mh, int block, int min_blocks) {
    if (gm.n_species() > GDTK_MAX_SPECIES || (int)mh.reactions.size() > GDTK_MAX_REACTIONS)
        throw std::runtime_error("the mechanism-specialised kernel takes up to " + std::to_string(GDTK_MAX_SPECIES) +
                                 " species and " + std::to_string(GDTK_MAX_REACTIONS) +
                                 " reactions; larger mechanisms run one warp per cell");
    const int nsp = gm.n_species();
    const int nr = (int)mh.reactions.size();
    std::ostringstream o;
    o << "// generated: " << nsp << " species, " << nr << " reactions\n";
    o << "#define GDTK_NSP " << nsp << "\n#define GDTK_NR " << nr << "\n";
    o << "#define GDTK_METHOD " << mh.method << "\n#define GDTK_TIGHT " << (mh.tight ? 1 : 0) << "\n";
    o << "#define GDTK_MAX_ITERS " << mh.maxIters << "\n#define GDTK_MAX_SUBCYCLES " << mh.maxSubcycles << "\n";
    o << "#define GDTK_MAX_ATTEMPTS " << mh.maxAttempts << "\n";
    o << "#define GDTK_T_LOWER " << lit(mh.T_lower) << "\n#define GDTK_T_UPPER " << lit(mh.T_upper) << "\n";
    o << "#define GDTK_LN_T_LOWER " << lit(std::log(mh.T_lower)) << "\n#define GDTK_LN_T_UPPER "
      << lit(std::log(mh.T_upper)) << "\n";
    o << "#define GDTK_ERRTOL " << lit(mh.errTol) << "\n#define GDTK_EPS1 " << lit(mh.eps1) << "\n";
    o << "#define GDTK_EPS2 " << lit(mh.eps2) << "\n#define GDTK_DELTA " << lit(mh.delta) << "\n";
    o << "#define GDTK_BLOCK " << block << "\n#define GDTK_MIN_BLOCKS " << min_blocks << "\n";
    {
        double tlo = 0.0, thi = 0.0;
        const bool mix = mix_thermo_range(gm, tlo, thi);
        o << "#define GDTK_MIX_THERMO " << (mix ? 1 : 0) << "\n";
        if (mix) o << "#define GDTK_MIX_TLO " << lit(tlo) << "\n#define GDTK_MIX_THI " << lit(thi) << "\n";
        o << "#define GDTK_VEC " << fast_vec_doubles(gm, mh) << "\n";
        o << "#define GDTK_G_UNROLL _Pragma(\"unroll " << g_unroll() << "\")\n";
        const char* pc = std::getenv("GDTK_PHASE_CLOCKS");
        o << "#define GDTK_PHASE_CLOCKS " << ((pc && pc[0] == '1') ? 1 : 0) << "\n";
    }
    o << kFastExpSource << "\n";
    auto arr = [&](const char* name, std::function<double(int)> f) {
        o << "__constant__ double " << name << "[" << nsp << "] = {";
        for (int i = 0; i < nsp; ++i) o << (i ? ", " : "") << lit(f(i));
        o << "};\n";
    };
    arr("GDTK_M", [&](int i) { return gm.M[i]; });
    arr("GDTK_RM", [&](int i) { return 1.0 / gm.M[i]; });
    arr("GDTK_R", [&](int i) { return R_universal / gm.M[i]; });
    o << "namespace gdtk_fast {\nusing gdtk::gdtk_exp;\nusing gdtk::gdtk_div_nr;\n";

    // ---- third-body concentrations of the pressure-dependent rate constants (rate_constant.d:114-121),
    // from the concentrations at which the rate constants are evaluated
    int nfall = 0;
    o << "__device__ __forceinline__ void gen_falloff_M(const double (&c)[GDTK_NSP], double* Mv, int ms) {\n";
    o << "  (void)c; (void)Mv; (void)ms;\n";
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        if (!r.frc.pressure_dependent()) continue;
        o << "  Mv[" << nfall << " * ms] = 0.0";
        for (auto& e : r.eff) o << " + " << lit(e.second) << " * c[" << e.first << "]";
        o << ";\n";
        ++nfall;
    }
    o << "}\n#define GDTK_NFALLOFF " << nfall << "\n";

    // ---- rate constants.  In table form (the default) the Arrhenius reactions are one loop over a
    // __constant__ table, which keeps the code the warps cycle through each step small (the kernel is
    // otherwise often stalled on instruction fetch); pressure-dependent reactions stay unrolled.
    const char* kc_env = std::getenv("GDTK_KC_UNROLLED");
    const bool kc_table = !(kc_env && kc_env[0] == '1');
    std::vector<int> table_rx;
    // 256 records of 208 bytes = 53 KB of the 64 KB constant bank, leaving room for the species constants;
    // reactions beyond them stay straight-line
    for (int ir = 0; ir < nr && (int)table_rx.size() < 256; ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        int np = 0;
        for (auto& pp : participants(r)) np += pp.nu != 0;
        // the table holds ln A, n, C records; Arrhenius2 rate constants stay straight-line
        const bool arr2 = r.frc.model == RATE_ARRHENIUS2 || r.brc.model == RATE_ARRHENIUS2;
        if (kc_table && !r.frc.pressure_dependent() && !arr2 && np <= 8) table_rx.push_back(ir);
    }
    const std::vector<bool> kbp = kb_product_reactions(gm, mh);
    bool any_kbp = false;
    for (int ir : table_rx) any_kbp = any_kbp || kbp[ir];
    if (!table_rx.empty()) {
        // pw: k_f = A T^pw by multiplication (C = 0, integer |n| <= 4); 99: by exp of its logarithm
        o << "struct KcRec { double lnA, n, mC, lnAb, nb, mCb, A; int mode, np, nusum, idx, pw; int sp[8], anu[8]; "
             "double nu[8]; };\n";
        o << "__constant__ KcRec GDTK_KC_TAB[" << table_rx.size() << "] = {\n";
        for (int ir : table_rx) {
            const ReactionHost& r = mh.reactions[ir];
            auto parts = participants(r);
            int np = 0, nusum = 0;
            std::ostringstream sp, nu, anu;
            for (auto& pp : parts) {
                if (pp.nu == 0) continue;
                sp << (np ? ", " : "") << pp.isp;
                nu << (np ? ", " : "") << lit((double)pp.nu);
                anu << (np ? ", " : "") << pp.nu;   // signed: > 0 products, < 0 reactants
                nusum += pp.nu;
                ++np;
            }
            if (np == 0) { sp << "0"; nu << "0.0"; anu << "0"; }
            // mode 0: k_f Arrhenius, k_b from K_c; 1: both Arrhenius; 2: k_b Arrhenius, k_f from K_c;
            // 3: as 0, with k_b = k_f / K_c from the species' E_i
            int mode = r.frc.model == RATE_ARRHENIUS ? (r.brc.model == RATE_FROM_EQ ? 0 : 1) : 2;
            if (mode == 0 && kbp[ir]) mode = 3;
            auto lnA = [](const RateConstHost& rc) { return rc.A > 0.0 ? std::log(rc.A) : -1.0e300; };
            std::string pws;
            const int pw = power_arrhenius(r.frc, pws) ? (int)r.frc.n : 99;
            o << "  {" << lit(lnA(r.frc)) << ", " << lit(r.frc.n) << ", " << lit(-r.frc.C) << ", " << lit(lnA(r.brc))
              << ", " << lit(r.brc.n) << ", " << lit(-r.brc.C) << ", " << lit(r.frc.A) << ", " << mode << ", " << np
              << ", " << nusum << ", " << ir << ", " << pw << ", {" << sp.str() << "}, {" << anu.str() << "}, {"
              << nu.str() << "}},   // "
              << (r.equation.empty() ? std::string("reaction") : r.equation) << "\n";
        }
        o << "};\n";
    }
    o << "__device__ __forceinline__ void gen_kc(double T, double lnT, double rT, const double* g, int gs, double* K, "
         "int ks, const double* etab, const double* Mv, int ms) {\n";
    o << "  (void)T; (void)Mv; (void)ms;\n";
    if (any_kbp) {   // E_i = exp(G_i / R T) and its reciprocal, after G/RT and the falloff concentrations
        o << "  const double* E = g + (" << nsp << " + " << nfall << ") * gs;\n";
        o << "  const double* Ei = E + " << nsp << " * gs;\n";
        o << "#pragma unroll 1\n";
        o << "  for (int i = 0; i < " << nsp << "; ++i) {\n";
        o << "    const double e = gdtk_exp(g[i * gs], etab);\n";
        o << "    const_cast<double*>(E)[i * gs] = e;\n";
        o << "    const_cast<double*>(Ei)[i * gs] = gdtk_div_nr(1.0, e);\n  }\n";
        o << "  const double cf = T * " << lit(R_universal / 101325.0) << ", rcf = rT * " << lit(101325.0 / R_universal)
          << ";   // R T / P_atm and its reciprocal\n";
    }
    if (!table_rx.empty()) {
        o << "#pragma unroll " << kc_unroll() << "\n";
        o << "  for (int t = 0; t < " << table_rx.size() << "; ++t) {   // reaction.d:26-52, 94-143\n";
        o << "    const KcRec& R = GDTK_KC_TAB[t];\n";
        if (any_kbp) {
            o << "    if (R.mode == 3) {   // k_b = k_f (R T / P_atm)^(sum nu) prod E_i^nu_i\n";
            o << "      double kf;\n";
            o << "      if (R.pw != 99) {   // A T^n, C = 0, integer n\n";
            o << "        const double b = R.pw > 0 ? T : rT;\n        kf = R.A;\n";
            o << "        for (int m = 0; m < abs(R.pw); ++m) kf *= b;\n";
            o << "      } else {\n        kf = gdtk_exp(fma(R.mC, rT, fma(R.n, lnT, R.lnA)), etab);\n      }\n";
            o << "      double P = 1.0;\n";
            o << "      const double c = R.nusum > 0 ? cf : rcf;\n";
            o << "      for (int m = 0; m < abs(R.nusum); ++m) P *= c;\n";
            o << "      for (int k = 0; k < R.np; ++k) {\n";
            o << "        const int nk = R.anu[k];\n";
            o << "        const double v = (nk > 0 ? E : Ei)[R.sp[k] * gs];\n";
            o << "        for (int m = 0; m < abs(nk); ++m) P *= v;\n      }\n";
            o << "      K[R.idx * ks] = kf;\n      K[(" << nr << " + R.idx) * ks] = kf * P;\n      continue;\n    }\n";
        }
        bool all_kbp = true;
        for (int ir : table_rx) all_kbp = all_kbp && kbp[ir];
        if (all_kbp) o << "#if 0   // every table reaction takes the product form\n";
        o << "    double dg = 0.0;\n";
        o << "    for (int k = 0; k < R.np; ++k) dg = fma(R.nu[k], g[R.sp[k] * gs], dg);\n";
        o << "    const double lnKc = fma((double)R.nusum, " << lit(std::log(101325.0 / R_universal)) << " - lnT, -dg);\n";
        o << "    double kf, kb;\n";
        o << "    if (R.mode != 2) {\n";
        o << "      const double lkf = fma(R.mC, rT, fma(R.n, lnT, R.lnA));\n";
        o << "      kf = gdtk_exp(lkf, etab);\n";
        o << "      kb = R.mode == 0 ? gdtk_exp(lkf - lnKc, etab) : gdtk_exp(fma(R.mCb, rT, fma(R.nb, lnT, R.lnAb)), etab);\n";
        o << "    } else {\n";
        o << "      const double lkb = fma(R.mCb, rT, fma(R.nb, lnT, R.lnAb));\n";
        o << "      kb = gdtk_exp(lkb, etab);\n";
        o << "      kf = gdtk_exp(lkb + lnKc, etab);\n";
        o << "    }\n";
        o << "    K[R.idx * ks] = kf;\n    K[(" << nr << " + R.idx) * ks] = kb;\n";
        if (all_kbp) o << "#endif\n";
        o << "  }\n";
    }
    int ifall = 0;
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        if (std::find(table_rx.begin(), table_rx.end(), ir) != table_rx.end()) continue;
        auto parts = participants(r);
        if (ir > 0 && ir % 4 == 0) o << "  asm volatile(\"\" ::: \"memory\");\n";
        std::ostringstream dg;   // sum nu * G/RT
        int nusum = 0;
        for (auto& p : parts) {
            if (p.nu == 0) continue;
            nusum += p.nu;
            std::string term = "g[" + std::to_string(p.isp) + " * gs]";
            if (dg.tellp() == 0) {
                if (p.nu == 1) dg << term;
                else dg << lit((double)p.nu) << " * " << term;
            } else {
                if (p.nu == 1) dg << " + " << term;
                else if (p.nu == -1) dg << " - " << term;
                else dg << " + " << lit((double)p.nu) << " * " << term;
            }
        }
        std::string dgs = dg.tellp() == 0 ? std::string("0.0") : dg.str();
        // ln K_c = -sum(nu G/RT) + sum(nu) ln(P_atm / R T)   (reaction.d:26-52)
        std::string lnKc = "(-(" + dgs + ")" +
                           (nusum ? " + " + lit((double)nusum) + " * (" + lit(std::log(101325.0 / R_universal)) + " - lnT)" : std::string("")) + ")";
        o << "  { // " << (r.equation.empty() ? std::string("reaction") : r.equation) << "\n";
        if (r.frc.pressure_dependent()) {   // backward from K_c (checked when the mechanism is read)
            o << "    const double Mc = Mv[" << ifall++ << " * ms];\n";
            o << pressure_dependent_code(r.frc);
            o << "    const double kb = kf * gdtk_exp(-" << lnKc << ", etab);\n";
        } else if (r.frc.simple()) {
            std::string pw;
            if (power_arrhenius(r.frc, pw)) {
                o << "    const double kf = " << pw << ";\n";
                if (r.brc.model == RATE_FROM_EQ) o << "    const double kb = kf * gdtk_exp(-" << lnKc << ", etab);\n";
            } else {
                std::string l = log_arrhenius(r.frc);
                if (l.empty()) o << "    const double lkf = -1.0e300; const double kf = 0.0;\n";
                else o << "    const double lkf = " << l << ";\n    const double kf = gdtk_exp(lkf, etab);\n";
                if (r.brc.model == RATE_FROM_EQ) o << "    const double kb = gdtk_exp(lkf - " << lnKc << ", etab);\n";
            }
            if (r.brc.simple()) {
                std::string pb;
                if (power_arrhenius(r.brc, pb)) o << "    const double kb = " << pb << ";\n";
                else {
                    std::string l = log_arrhenius(r.brc);
                    o << "    const double kb = " << (l.empty() ? std::string("0.0") : "gdtk_exp(" + l + ", etab)")
                      << ";\n";
                }
            }
        } else {   // forward from K_c and a given backward rate constant
            std::string l = log_arrhenius(r.brc);
            if (l.empty()) o << "    const double kb = 0.0; const double kf = 0.0;\n";
            else o << "    const double lkb = " << l << ";\n    const double kb = gdtk_exp(lkb, etab);\n"
                   << "    const double kf = gdtk_exp(lkb + " << lnKc << ", etab);\n";
        }
        o << "    K[" << ir << " * ks] = kf;\n    K[" << (nr + ir) << " * ks] = kb;\n  }\n";
    }
    o << "}\n";

    // ---- production / loss rates
    o << "__device__ __forceinline__ void gen_rhs(const double* c, double* q, double* L, const double* K, int ks) {\n";
    // distinct third-body lists
    std::vector<std::vector<std::pair<int, double>>> sets;
    std::vector<int> set_of(nr, -1);
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        if (!r.collider) continue;
        int f = -1;
        for (size_t s = 0; s < sets.size(); ++s) if (sets[s] == r.eff) { f = (int)s; break; }
        if (f < 0) { sets.push_back(r.eff); f = (int)sets.size() - 1; }
        set_of[ir] = f;
    }
    for (size_t s = 0; s < sets.size(); ++s) {
        o << "  double M" << s << " = 0.0;\n";
        bool first = true;
        for (auto& e : sets[s]) {
            std::string cc = "c[" + std::to_string(e.first) + "]";
            if (first) {
                o << "  M" << s << " = " << (e.second == 1.0 ? cc : lit(e.second) + " * " + cc) << ";\n";
                first = false;
            } else if (e.second == 1.0) {
                o << "  M" << s << " += " << cc << ";\n";
            } else {
                o << "  M" << s << " = fma(" << lit(e.second) << ", " << cc << ", M" << s << ");\n";
            }
        }
    }
    std::vector<bool> qset(nsp, false), lset(nsp, false);
    auto acc = [&](std::vector<bool>& set, const char* arr, int isp, int coeff, const char* w) {
        std::string dst = std::string(arr) + "[" + std::to_string(isp) + "]";
        std::string val = coeff == 1 ? std::string(w) : lit((double)coeff) + " * " + w;
        if (!set[isp]) { o << "    " << dst << " = " << val << ";\n"; set[isp] = true; }
        else if (coeff == 1) o << "    " << dst << " += " << w << ";\n";
        else o << "    " << dst << " = fma(" << lit((double)coeff) << ", " << w << ", " << dst << ");\n";
    };
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh.reactions[ir];
        // A compiler barrier every few reactions stops the scheduler from hoisting every k_f/k_b
        // load to the top, which would hold 2 NR doubles live and spill registers.
        if (ir > 0 && rhs_fence() > 0 && ir % rhs_fence() == 0) o << "  asm volatile(\"\" ::: \"memory\");\n";
        o << "  {\n    double wf = K[" << ir << " * ks], wb = K[" << (nr + ir) << " * ks];\n";
        if (r.collider) o << "    wf *= M" << set_of[ir] << "; wb *= M" << set_of[ir] << ";\n";
        for (auto& x : r.reac) o << "    wf *= " << ipow_expr("c[" + std::to_string(x.first) + "]", x.second) << ";\n";
        for (auto& x : r.prod) o << "    wb *= " << ipow_expr("c[" + std::to_string(x.first) + "]", x.second) << ";\n";
        for (auto& p : participants(r)) {
            if (p.nu > 0) { acc(qset, "q", p.isp, p.nu, "wf"); acc(lset, "L", p.isp, p.nu, "wb"); }
            else if (p.nu < 0) { acc(qset, "q", p.isp, -p.nu, "wb"); acc(lset, "L", p.isp, -p.nu, "wf"); }
        }
        o << "  }\n";
    }
    for (int i = 0; i < nsp; ++i) {
        if (!qset[i]) o << "  q[" << i << "] = 0.0;\n";
        if (!lset[i]) o << "  L[" << i << "] = 0.0;\n";
    }
    o << "}\n}  // namespace gdtk_fast\n";
    o << kFastCuhSource;
    return o.str();
}

namespace {

std::string cache_dir() {
    const char* env = std::getenv("GDTK_JIT_CACHE");
    if (env && *env) return env;
    const char* home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/gdtk_gb300";
}

std::string arch_option(int major, int minor) {
    return "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + (major >= 9 ? "a" : "");
}
const char* const kJitOptions[] = {"--std=c++17", "--fmad=true", "-default-device", "-lineinfo",
                                   "--ptxas-options=-v"};

// Key of the in-process and on-disk cubin caches: the source, the target, NVRTC's version and
// every compile option, so a toolkit upgrade or an option change never loads a stale cubin.
std::string cubin_cache_key(const std::string& src, int major, int minor) {
    int vmaj = 0, vmin = 0;
    nvrtcVersion(&vmaj, &vmin);
    std::string opts = arch_option(major, minor);
    for (const char* o : kJitOptions) opts += std::string(" ") + o;
    const size_t h = std::hash<std::string>{}(src) ^ (std::hash<std::string>{}(opts) * 0x9e3779b97f4a7c15ull);
    return std::to_string(h) + "_sm" + std::to_string(major) + std::to_string(minor) + "_nvrtc" +
           std::to_string(vmaj) + "." + std::to_string(vmin);
}

std::string compile_cubin(const std::string& src, int major, int minor, std::string& log) {
    const std::string arch = arch_option(major, minor);
    std::vector<const char*> opts{arch.c_str()};
    for (const char* o : kJitOptions) opts.push_back(o);
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "gdtk_chem_fast.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        throw std::runtime_error("nvrtcCreateProgram failed");
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    log.assign(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &log[0]);
    while (!log.empty() && log.back() == '\0') log.pop_back();
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        throw std::runtime_error(std::string("NVRTC compilation of the mechanism kernel failed: ") +
                                 nvrtcGetErrorString(rc) + "\n" + log);
    }
    size_t cn = 0;
    nvrtcGetCUBINSize(prog, &cn);
    std::string cubin(cn, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return cubin;
}

std::mutex g_jit_mu;
std::map<std::string, std::string> g_cubins;   // source hash key -> cubin (this process)

}  // namespace

std::string compile_fast_check(const GasModelHost& gm, const MechanismHost& mh, int major, int minor) {
    std::string log;
    std::string src = generate_fast_source(gm, mh, 256, 1);
    std::string cubin = compile_cubin(src, major, minor, log);
    return log + "\ncubin bytes: " + std::to_string(cubin.size()) + "\n";
}

FastKernel* build_fast_kernel(const GasModelHost& gm, const MechanismHost& mh, int req_block, int req_min_blocks) {
    int dev = 0, major = 0, minor = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int nsp = gm.n_species(), nr = (int)mh.reactions.size();
    if (nsp > GDTK_MAX_SPECIES || nr > GDTK_MAX_REACTIONS) generate_fast_source(gm, mh, 32, 1);   // throws the reason
    const int per_thread = 2 * nr + fast_vec_doubles(gm, mh);
    const int table = nsp * 120 + GDTK_EXP2_TABLE_SIZE;
    // Block size: as many resident threads as shared memory allows, up to 256 per SM.  Each resident
    // block also holds the kernel's static shared arrays (at most kStaticSmem bytes, the phase-clock
    // instrumentation) and the 1 KB the hardware reserves per block; one block may use up to 227 KB.
    constexpr double kStaticSmem = 512.0, kReserved = 1024.0, kSmPerSm = 228.0 * 1024, kSmPerBlock = 227.0 * 1024;
    auto fits = [&](int blk, int nblk) {
        const double dyn = (table + (double)per_thread * blk) * 8.0;
        return dyn + kStaticSmem <= kSmPerBlock && nblk * (dyn + kStaticSmem + kReserved) <= kSmPerSm;
    };
    int block = 256, min_blocks = 1;
    while (block > 32 && !fits(block, 1)) block -= 32;
    if (!fits(block, 1)) throw std::runtime_error("mechanism too large for shared memory");
    if (block <= 128 && fits(block, 2)) min_blocks = 2;
    if (req_block > 0) {   // an explicit launch shape (autotuning)
        if (req_block % 32 || req_block > 1024) throw std::runtime_error("block size must be a multiple of 32, <= 1024");
        int mb = req_min_blocks > 0 ? req_min_blocks : 1;
        if (!fits(req_block, mb)) throw std::runtime_error("requested block shape does not fit in shared memory");
        block = req_block;
        min_blocks = mb;
    }

    auto k = std::make_unique<FastKernel>();
    k->block = block;
    k->min_blocks = min_blocks;
    k->per_thread_doubles = per_thread;
    k->table_doubles = table;
    k->source = generate_fast_source(gm, mh, block, min_blocks);
    std::string key = cubin_cache_key(k->source, major, minor);
    std::string cubin;
    {
        std::lock_guard<std::mutex> lk(g_jit_mu);
        auto it = g_cubins.find(key);
        if (it != g_cubins.end()) cubin = it->second;
    }
    std::string dir = cache_dir(), path = dir + "/" + key + ".cubin";
    if (cubin.empty()) {
        std::ifstream f(path, std::ios::binary);
        if (f) {
            std::ostringstream ss;
            ss << f.rdbuf();
            cubin = ss.str();
            k->log = "loaded from " + path;
        }
    }
    if (cubin.empty()) {
        cubin = compile_cubin(k->source, major, minor, k->log);
        std::string tmp = path + ".tmp" + std::to_string((long)getpid());
        ::mkdir((dir.substr(0, dir.rfind('/'))).c_str(), 0755);
        ::mkdir(dir.c_str(), 0755);
        std::ofstream f(tmp, std::ios::binary);
        if (f) {
            f.write(cubin.data(), (std::streamsize)cubin.size());
            f.close();
            std::rename(tmp.c_str(), path.c_str());
        }
    }
    {
        std::lock_guard<std::mutex> lk(g_jit_mu);
        g_cubins[key] = cubin;
    }
    Driver& d = driver();
    CUmodule mod;
    cu_check(d.moduleLoadData(&mod, cubin.data()), "cuModuleLoadData");
    k->module = mod;
    CUfunction fn;
    cu_check(d.moduleGetFunction(&fn, mod, "gdtk_chem_fast"), "cuModuleGetFunction");
    k->function = fn;
    CUfunction cfn;
    cu_check(d.moduleGetFunction(&cfn, mod, "gdtk_chem_cost"), "cuModuleGetFunction");
    k->cost_function = cfn;
    const size_t smem_max = (size_t)(table + per_thread * block) * 8;
    cu_check(d.funcSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem_max),
             "cuFuncSetAttribute");
    cu_check(d.funcSetAttribute(cfn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem_max),
             "cuFuncSetAttribute");
    cu_check(d.occupancy(&k->blocks_per_sm, fn, block, smem_max), "cuOccupancyMaxActiveBlocksPerMultiprocessor");
    if (k->blocks_per_sm < 1) throw std::runtime_error("fast kernel cannot be resident (registers/shared memory)");
    std::vector<double> th = fast_thermo_table(gm);
    static const double etab[GDTK_EXP2_TABLE_SIZE] = GDTK_EXP2_TABLE_INIT;
    if (cudaMalloc(&k->d_thermo, th.size() * 8) != cudaSuccess || cudaMalloc(&k->d_exp, sizeof etab) != cudaSuccess)
        throw std::runtime_error("cudaMalloc failed");
    cudaMemcpy(k->d_thermo, th.data(), th.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(k->d_exp, etab, sizeof etab, cudaMemcpyHostToDevice);
    (void)sms;
    return k.release();
}

cudaError_t launch_fast(FastKernel& k, FastArgs& a, int sm_count, cudaStream_t stream, int* grid_out, int* block_out,
                        int* smem_out) {
    a.thermo = k.d_thermo;
    a.exp_table = k.d_exp;
    int block = k.block;
    while (block > 32 && ((long long)a.total + block - 1) / block < sm_count) block -= 32;
    long long want = ((long long)a.total + block - 1) / block;
    long long grid = (long long)sm_count * k.blocks_per_sm * (k.block / block);
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    size_t smem = (size_t)(k.table_doubles + k.per_thread_doubles * block) * 8;
    void* params[] = {&a};
    CUresult r = driver().launchKernel((CUfunction)k.function, (unsigned)grid, 1, 1, (unsigned)block, 1, 1,
                                       (unsigned)smem, (CUstream)stream, params, nullptr);
    if (grid_out) *grid_out = (int)grid;
    if (block_out) *block_out = block;
    if (smem_out) *smem_out = (int)smem;
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorLaunchFailure;
}

cudaError_t launch_order(FastKernel& k, FastArgs& a, int sm_count, float* key, int* order, int* hist,
                         cudaStream_t stream) {
    a.thermo = k.d_thermo;
    a.exp_table = k.d_exp;
    const int block = k.block;
    long long grid = ((long long)a.total + block - 1) / block;
    if (grid > (long long)sm_count * k.blocks_per_sm) grid = (long long)sm_count * k.blocks_per_sm;
    if (grid < 1) grid = 1;
    size_t smem = (size_t)(k.table_doubles + k.per_thread_doubles * block) * 8;
    void* params[] = {&a, &key};
    CUresult r = driver().launchKernel((CUfunction)k.cost_function, (unsigned)grid, 1, 1, (unsigned)block, 1, 1,
                                       (unsigned)smem, (CUstream)stream, params, nullptr);
    if (r != CUDA_SUCCESS) return cudaErrorLaunchFailure;
    return launch_bucket_order(key, a.total, order, hist, sm_count, stream);
}

}  // namespace gdtk
