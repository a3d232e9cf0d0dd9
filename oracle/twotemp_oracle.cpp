// twotemp_oracle.cpp -- TEST INFRASTRUCTURE ONLY: a compiled restatement of the reference's
// multi-temperature thermochemical reactor for a two-temperature gas, operation for operation as
// oracle/two_temperature_reactor.py (the checker, which cites the reference's file:line for each
// part), so that the CPU side of the two-temperature workload can be timed at compiled speed.
// Nothing in the product links it; tests/ check it against the Python restatement and bench.py
// times it as the CPU baseline.
//
//   kinetics/multi_temperature_thermochemical_reactor.d:137-294, 334-431   opCall, RKF (Cash-Karp)
//   kinetics/reaction.d:26-52, 94-149, 290-311                          K_c, rate constants, tick rates
//   kinetics/rate_constant.d:72-75, 364-566                             Arrhenius, Park, (modified) Marrone-Treanor
//   kinetics/reaction_mechanism.d:74-96, 161-203                        q, L, initial step
//   kinetics/energy_exchange_system.d:93-104, energy_exchange_mechanism.d:56-101, 195-253
//   kinetics/relaxation_time.d:27-175, exchange_chemistry_coupling.d:41-227
//   gas/thermo/two_temperature_gas.d:45-124, 427-590, 656-700           2-T thermo, T and T_ve from (rho, u)
// The CEA curves are the one-temperature oracle's (chem_oracle.cpp), through its C entry points.
#include <algorithm>
#include <cmath>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" int oracle_species_h(void* m, int isp, double T, double logT, double* h);
extern "C" int oracle_species_cp(void* m, int isp, double T, double* cp);
extern "C" int oracle_species_thermo(void* m, int isp, double T, double* Cp, double* hh, double* s);

namespace {

constexpr double R_UNIVERSAL = 8.31451;        // gas/physical_constants.d:13
constexpr double P_ATM = 101325.0;
constexpr double AVOGADRO = 6.02214e23;        // gas/physical_constants.d:19
constexpr double BOLTZMANN = 1.380658e-23;     // gas/physical_constants.d:18
constexpr double PI = 3.141592653589793;
constexpr double T_REF = 298.15;               // two_temperature_gas.d:26
constexpr double SMALL_MOLE_FRACTION = 1.0e-15;
constexpr double IGAMMA_SWITCH = 1.0e-7, IGAMMA_OVERFLOW = 0.001;
constexpr double H_MIN = 1.0e-15, ALLOWABLE_MASSF_ERROR = 1.0e-3;

struct Failure { int code; };

enum { RC_ARRHENIUS = 0, RC_FROM_EQ = 1, RC_PARK = 6, RC_MT = 7, RC_MMT = 8 };
enum { EEM_LT = 0, EEM_MT = 1 };
enum { RT_MW = 0, RT_PARK_HTC = 1, RT_PARK_HTC2 = 2 };
enum { CPL_IMPARTIAL = 0, CPL_MT = 1, CPL_MMT = 2 };

struct Rate {
    int model = RC_ARRHENIUS, base = RC_ARRHENIUS, rct = -1;
    double A = 0, n = 0, C = 0, s = 0, TD = 0, U = 0, theta = 0, aU = 0, Ustar = 0, nb = 1;
};

double pow_int(double x, int n) {
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

double Qmt(double T, double D, double theta) { return (1 - std::exp(-D / T)) / (1 - std::exp(-theta / T)); }

// rate_constant.d at (T, T_mode)
double rate_constant(const Rate& rc, int model, double T, double Tm) {
    if (model == RC_ARRHENIUS) {
        const double Tr = rc.rct == -1 ? T : Tm;
        return rc.A * std::pow(Tr, rc.n) * std::exp(-rc.C / Tr);
    }
    if (model == RC_PARK) {
        const double Tr = std::pow(T, rc.s) * std::pow(Tm, 1.0 - rc.s);
        return rc.A * std::pow(Tr, rc.n) * std::exp(-rc.C / Tr);
    }
    const double kEQ = rate_constant(rc, rc.base, T, Tm);
    if (model == RC_MT) {
        const double Gamma = 1. / (1. / Tm - 1. / T - 1. / rc.U);
        return kEQ * Qmt(T, rc.TD, rc.theta) * Qmt(Gamma, rc.TD, rc.theta) /
               (Qmt(Tm, rc.TD, rc.theta) * Qmt(-rc.U, rc.TD, rc.theta));
    }
    const double Tinv = 1. / T, Tvinv = 1. / Tm;
    const double Uinv = rc.aU * Tinv + 1. / rc.Ustar;
    const double U = 1. / Uinv;
    const double TF = 1. / (Tvinv - Tinv - Uinv);
    return rc.nb * kEQ * Qmt(T, rc.TD, rc.theta) * Qmt(TF, rc.TD, rc.theta) /
           (Qmt(Tm, rc.TD, rc.theta) * Qmt(-U, rc.TD, rc.theta));
}

struct Reaction {
    bool collider = false;
    std::vector<std::pair<int, int>> reac, prod;
    std::vector<int> part, nu;
    std::vector<std::pair<int, double>> eff;
    Rate frc, brc;
    double kf = 0, kb = 0, wf = 0, wb = 0;
    double production(int isp) const {
        const int n = nu[isp];
        return n > 0 ? n * wf : (n < 0 ? -n * wb : 0.0);
    }
    double loss(int isp) const {
        const int n = nu[isp];
        return n > 0 ? n * wb : (n < 0 ? -n * wf : 0.0);
    }
};

struct Relax {
    int model = RT_MW, q = 0;
    double a = 0, b = 0, sigma = 0, mu = 0, sub_a = 0, sub_b = 0;
};

struct Eem {
    int kind = EEM_LT, p = 0, q = 0, r = 0, coupling = CPL_IMPARTIAL;
    Relax rt;
    double D = 0, Thetav = 0, U = 0, TD = 0, aU = 0, Ustar = 0, nb = 0;
};

struct State {
    double rho, T, Tve, p;
    std::vector<double> Y;
};

struct Reactor {
    void* curves = nullptr;   // one-temperature oracle model of the gas (CEA curves)
    int nsp = 0, electron = -1;
    std::vector<double> M, R, cp_tr, h_f;
    double T_lower = 300, T_upper = 50000, tol = 1e-3;
    int max_subcycles = 10000, max_attempts = 4;
    std::vector<Reaction> rx;
    std::vector<Eem> eem;

    double h(int i, double T) const {
        double v;
        if (oracle_species_h(curves, i, T, std::log(T), &v)) throw Failure{7};
        return v;
    }
    double cp(int i, double T) const {
        double v;
        if (oracle_species_cp(curves, i, T, &v)) throw Failure{7};
        return v;
    }
    // two_temperature_gas.d:427-445, 538-545, 558-590
    double e_tr(int i, double T) const { return i == electron ? 0.0 : cp_tr[i] * (T - T_REF) + h_f[i] - R[i] * T; }
    double e_ve(int i, double Tve) const {
        return i == electron ? 1.5 * R[i] * Tve : h(i, Tve) - cp_tr[i] * (Tve - T_REF) - h_f[i];
    }
    double cv_ve(int i, double Tve) const { return i == electron ? 1.5 * R[i] : cp(i, Tve) - cp_tr[i]; }
    double e_tr_mix(const std::vector<double>& Y, double T) const {
        double e = 0.0;
        for (int i = 0; i < nsp; ++i)
            if (i != electron) e += Y[i] * e_tr(i, T);
        return e;
    }
    double e_ve_mix(const std::vector<double>& Y, double Tve) const {
        double e = 0.0;
        for (int i = 0; i < nsp; ++i) e += Y[i] * e_ve(i, Tve);
        return e;
    }
    double cv_ve_mix(const std::vector<double>& Y, double Tve) const {
        double c = 0.0;
        for (int i = 0; i < nsp; ++i) c += Y[i] * cv_ve(i, Tve);
        return c;
    }
    // two_temperature_gas.d:95-117, 656-700
    void from_rhou(State& st, double u, double u_ve) const {
        double sumA = 0.0, sumB = 0.0;
        for (int i = 0; i < nsp; ++i)
            if (i != electron) sumA += st.Y[i] * (cp_tr[i] * T_REF - h_f[i]);
        for (int i = 0; i < nsp; ++i)
            if (i != electron) sumB += st.Y[i] * (cp_tr[i] - R[i]);
        const double T = (u + sumA) / sumB;
        double Tve = st.Tve;
        double f = e_ve_mix(st.Y, Tve) - u_ve;
        if (std::fabs(f) >= 1e-5) {
            int count = 0;
            double dT = 0.0;
            for (int it = 0; it < 40; ++it) {
                dT = -f / cv_ve_mix(st.Y, Tve);
                Tve += dT;
                if (std::fabs(dT) < 1.0e-9) break;
                f = e_ve_mix(st.Y, Tve) - u_ve;
                ++count;
            }
            if (count == 40 && std::fabs(dT) > 1e-3) throw Failure{4};
        }
        double p = 0.0;
        for (int i = 0; i < nsp; ++i) p += st.rho * st.Y[i] * R[i] * (i == electron ? Tve : T);
        st.T = T;
        st.Tve = Tve;
        st.p = p;
    }

    void rate_constants(const State& st) {
        const double T = std::min(std::max(st.T, T_lower), T_upper);
        std::vector<double> g(nsp);
        for (int i = 0; i < nsp; ++i) {
            double Cp, hh, s;
            if (oracle_species_thermo(curves, i, T, &Cp, &hh, &s)) throw Failure{7};
            g[i] = hh - T * s;
        }
        const double Tm = st.Tve;
        for (Reaction& r : rx) {
            auto Kc = [&]() {
                double dG = 0.0, nuSum = 0.0;
                for (int isp : r.part) {
                    dG += r.nu[isp] * g[isp] * M[isp];
                    nuSum += r.nu[isp];
                }
                const double K_p = std::exp(-dG / (R_UNIVERSAL * T));
                return K_p * std::pow(P_ATM / (R_UNIVERSAL * T), nuSum);
            };
            if (r.frc.model != RC_FROM_EQ) {
                r.kf = rate_constant(r.frc, r.frc.model, T, Tm);
                if (r.brc.model == RC_FROM_EQ) {
                    const double Tb = r.brc.rct < 0 ? T : Tm;
                    const double K = Kc();
                    r.kb = rate_constant(r.frc, r.frc.model, Tb, Tb) / K;
                } else {
                    r.kb = rate_constant(r.brc, r.brc.model, T, Tm);
                }
            } else {
                r.kb = rate_constant(r.brc, r.brc.model, T, Tm);
                const double K = Kc();
                r.kf = rate_constant(r.brc, r.brc.model, T, Tm) * K;
            }
        }
    }

    double tau_of(const Relax& t, int model, double a, double b, double T, double p, const std::vector<double>& molef,
                  const std::vector<double>& numden) const {
        if (molef[t.q] <= SMALL_MOLE_FRACTION) return -1.0;
        if (model == RT_MW) {
            const double pBath = molef[t.q] * p / P_ATM;
            return (1.0 / pBath) * std::exp(a * (std::pow(T, -1.0 / 3.0) - b) - 18.42);
        }
        const double tau_sub = tau_of(t, RT_MW, t.sub_a, t.sub_b, T, p, molef, numden);
        const double sigma = model == RT_PARK_HTC ? t.sigma : t.sigma * (50e3 / T) * (50e3 / T);
        const double cs = std::sqrt(8.0 * BOLTZMANN * T / PI / t.mu);
        return tau_sub + 1.0 / (sigma * cs * numden[t.q]);
    }

    std::vector<double> relaxation_times(const State& st) const {
        std::vector<double> mol(nsp), molef(nsp), numden(nsp), taus(eem.size(), 0.0);
        double tot = 0.0;
        for (int i = 0; i < nsp; ++i) { mol[i] = st.Y[i] / M[i]; tot += mol[i]; }
        for (int i = 0; i < nsp; ++i) {
            molef[i] = mol[i] / tot;
            numden[i] = AVOGADRO * st.Y[i] * st.rho / M[i];
        }
        for (size_t k = 0; k < eem.size(); ++k)
            if (eem[k].kind == EEM_LT) taus[k] = tau_of(eem[k].rt, eem[k].rt.model, eem[k].rt.a, eem[k].rt.b, st.T, st.p,
                                                        molef, numden);
        return taus;
    }

    static double L_knab(double iG, double D, double th) {
        if (std::fabs(iG) < IGAMMA_SWITCH)
            return 0.5 * (D - th * R_UNIVERSAL) + iG * (th * th * R_UNIVERSAL * R_UNIVERSAL - D * D) / 12.0 / R_UNIVERSAL;
        if (iG > IGAMMA_OVERFLOW)
            return R_UNIVERSAL * th / (std::exp(th * iG) - 1.0) - D * std::exp(-D / R_UNIVERSAL * iG);
        return R_UNIVERSAL * th / (std::exp(th * iG) - 1.0) - D / (std::exp(D / R_UNIVERSAL * iG) - 1.0);
    }

    static void coupling(const Eem& m, double T, double Tv, double& ga, double& gv) {
        const double th = m.Thetav;
        if (m.coupling == CPL_IMPARTIAL) {
            ga = 0.5 * (m.D - th * R_UNIVERSAL);
            gv = L_knab((T - Tv) / (T * Tv), m.D, th);
        } else if (m.coupling == CPL_MT) {
            gv = L_knab(1. / Tv - 1. / T - 1. / m.U, m.D, th);
            const double T_F_inv = -1. / m.U;
            ga = R_UNIVERSAL * th / (std::exp(th * T_F_inv) - 1.) - m.D / (std::exp(m.D / R_UNIVERSAL * T_F_inv) - 1.);
        } else {
            const double TD = m.TD;
            const double Uinv = m.aU / T + 1 / m.Ustar;
            double T_F_inv = 1. / Tv - 1. / T - Uinv;
            gv = R_UNIVERSAL * (th / (std::exp(th * T_F_inv) - 1.) - TD / (std::exp(TD * T_F_inv) - 1.)) +
                 m.nb * R_UNIVERSAL * TD;
            T_F_inv = -m.aU / T - 1 / m.Ustar;
            ga = R_UNIVERSAL * (th / (std::exp(th * T_F_inv) - 1.) - TD / (std::exp(TD * T_F_inv) - 1.));
        }
    }

    void split_rates(const double* conc, std::vector<double>& q, std::vector<double>& L) {
        std::fill(q.begin(), q.end(), 0.0);
        std::fill(L.begin(), L.end(), 0.0);
        for (Reaction& r : rx) {
            double m = 1.0;
            if (r.collider) {
                m = 0.0;
                for (auto& e : r.eff) m += e.second * conc[e.first];
            }
            double wf = r.kf * m;
            for (auto& x : r.reac) wf *= pow_int(conc[x.first], x.second);
            double wb = r.kb * m;
            for (auto& x : r.prod) wb *= pow_int(conc[x.first], x.second);
            r.wf = wf;
            r.wb = wb;
        }
        for (const Reaction& r : rx)
            for (int isp : r.part) {
                q[isp] += r.production(isp);
                L[isp] += r.loss(isp);
            }
    }

    double ees_rate(const State& st, const std::vector<double>& taus) const {
        double rate = 0.0;
        for (size_t k = 0; k < eem.size(); ++k) {
            const Eem& m = eem[k];
            if (m.kind == EEM_LT) {
                if (taus[k] < 0.0) continue;
                const double ev_star = e_ve(m.p, st.T), ev = e_ve(m.p, st.Tve);
                rate += st.Y[m.p] * (ev_star - ev) / taus[k];
            } else {
                const Reaction& r = rx[m.r];
                double ga, gv;
                coupling(m, st.T, st.Tve, ga, gv);
                rate += (r.production(m.p) * ga - r.loss(m.p) * gv) / st.rho;
            }
        }
        return rate;
    }

    void rates(const State& st, const std::vector<double>& taus, const std::vector<double>& y, std::vector<double>& out,
               std::vector<double>& q, std::vector<double>& L) {
        split_rates(y.data(), q, L);
        for (int i = 0; i < nsp; ++i) out[i] = q[i] - L[i];
        out[nsp] = ees_rate(st, taus);
    }

    double estimate_step(const std::vector<double>& conc) {
        std::vector<double> q(nsp), L(nsp);
        split_rates(conc.data(), q, L);
        double min_dt = 1.0e6;
        for (int i = 0; i < nsp; ++i)
            if (conc[i] > 0.0 && std::fabs(q[i] - L[i]) > 1.0e-30) {
                const double dt = q[i] > 10000.0 * L[i] ? conc[i] / (L[i] + 1.0e-50) : std::fabs(conc[i] / (q[i] - L[i]));
                min_dt = std::min(min_dt, dt);
            }
        return std::max(std::min(1.0e-3 * min_dt, 1.0e-10), 1.0e-15);
    }

    // Cash-Karp step (multi_temperature_thermochemical_reactor.d:334-431); returns ok, yOut, dt_suggest
    bool step(const State& st, const std::vector<double>& taus, const std::vector<double>& y0, double h,
              std::vector<double>& yOut, double& dt_sug) {
        const int nv = nsp + 1;
        const double a21 = 1. / 5., a31 = 3. / 40., a32 = 9. / 40., a41 = 3. / 10., a42 = -9. / 10., a43 = 6. / 5.,
                     a51 = -11. / 54., a52 = 5. / 2., a53 = -70. / 27., a54 = 35. / 27., a61 = 1631. / 55296.,
                     a62 = 175. / 512., a63 = 575. / 13824., a64 = 44275. / 110592., a65 = 253. / 4096.;
        const double b51 = 37. / 378., b53 = 250. / 621., b54 = 125. / 594., b56 = 512. / 1771.,
                     b41 = 2825. / 27648., b43 = 18575. / 48384., b44 = 13525. / 55296., b45 = 277. / 14336.,
                     b46 = 1.0 / 4.0;
        std::vector<double> k1(nv), k2(nv), k3(nv), k4(nv), k5(nv), k6(nv), yT(nv), q(nsp), L(nsp);
        rates(st, taus, y0, k1, q, L);
        for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * a21 * k1[i];
        rates(st, taus, yT, k2, q, L);
        for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * (a31 * k1[i] + a32 * k2[i]);
        rates(st, taus, yT, k3, q, L);
        for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
        rates(st, taus, yT, k4, q, L);
        for (int i = 0; i < nv; ++i) yT[i] = y0[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
        rates(st, taus, yT, k5, q, L);
        for (int i = 0; i < nv; ++i)
            yT[i] = y0[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
        rates(st, taus, yT, k6, q, L);
        double err = 0.0;
        for (int i = 0; i < nv; ++i) {
            yOut[i] = y0[i] + h * (b51 * k1[i] + b53 * k3[i] + b54 * k4[i] + b56 * k6[i]);
            const double yErr = yOut[i] - (y0[i] + h * (b41 * k1[i] + b43 * k3[i] + b44 * k4[i] + b45 * k5[i] + b46 * k6[i]));
            const double sk = tol + tol * std::max(std::fabs(y0[i]), std::fabs(yOut[i]));
            err += (yErr / sk) * (yErr / sk);
        }
        err = std::sqrt(err / nv);
        if (err <= 1.0) {
            const double scale = err == 0.0 ? 10.0 : std::min(std::max(0.9 * std::pow(err, -0.2), 0.2), 10.0);
            dt_sug = scale * h;
            return true;
        }
        dt_sug = std::max(0.9 * std::pow(err, -0.2), 0.2) * h;
        return false;
    }

    // opCall for one cell (multi_temperature_thermochemical_reactor.d:137-294); throws Failure with the
    // input left alone.
    void update(State& in, double t_interval, double& dt_suggest, double& u_out, double& uve_out, long long& steps) {
        State st = in;
        std::vector<double> conc0(nsp);
        for (int i = 0; i < nsp; ++i) {
            const double c = st.Y[i] * st.rho / M[i];
            conc0[i] = c < 1.0e-30 ? 0.0 : c;
        }
        const double u_total = e_tr_mix(st.Y, st.T) + e_ve_mix(st.Y, st.Tve);
        rate_constants(st);
        std::vector<double> taus = relaxation_times(st);
        double t = 0.0, h;
        if (dt_suggest > t_interval) h = t_interval;
        else if (dt_suggest <= 0.0) h = estimate_step(conc0);
        else h = dt_suggest;
        std::vector<double> y0(nsp + 1), yOut(nsp + 1);
        for (int i = 0; i < nsp; ++i) y0[i] = conc0[i];
        y0[nsp] = e_ve_mix(st.Y, st.Tve);
        double dtSave = dt_suggest, u = 0.0, u_ve = 0.0;
        int cycle = 0;
        while (cycle < max_subcycles) {
            rate_constants(st);
            taus = relaxation_times(st);
            dtSave = dt_suggest;
            h = std::min(h, t_interval - t);
            int attempt = 0;
            while (attempt < max_attempts) {
                const bool ok = step(st, taus, y0, h, yOut, dt_suggest);
                ++steps;
                bool passed = true;
                if (ok) {
                    double tot = 0.0;
                    for (int i = 0; i < nsp; ++i) {
                        double mf = yOut[i] * M[i] / st.rho;
                        mf = mf < 1.0e-30 ? 0.0 : mf;
                        st.Y[i] = mf;
                        tot += mf;
                    }
                    if (std::fabs(tot - 1.0) > ALLOWABLE_MASSF_ERROR) passed = false;
                }
                if (ok && passed) {
                    t += h;
                    y0 = yOut;
                    const double hMax = h * (1.0 + 10.0 / 100.0);
                    if (dt_suggest > h) h = std::min(dt_suggest, hMax);
                    break;
                }
                h /= 10.0;
                if (h < H_MIN) throw Failure{1};
                ++attempt;
            }
            if (attempt == max_attempts) throw Failure{2};
            u_ve = y0[nsp];
            u = u_total - u_ve;
            from_rhou(st, u, u_ve);
            if (t >= t_interval) {
                if (cycle == 0) dtSave = dt_suggest;
                break;
            }
            ++cycle;
        }
        if (cycle == max_subcycles) throw Failure{3};
        double tot = 0.0;
        for (int i = 0; i < nsp; ++i) tot += st.Y[i];
        for (int i = 0; i < nsp; ++i) st.Y[i] /= tot;
        in = st;
        dt_suggest = dtSave;
        u_out = u;
        uve_out = u_ve;
    }
};

}  // namespace

extern "C" {

void* oracle2t_new(void* curves, int nsp, const double* M, const double* cp_tr, const double* h_f, int electron,
                   double T_lower, double T_upper, double tol, int max_subcycles, int max_attempts) {
    if (!curves || nsp < 1) return nullptr;
    Reactor* r = new Reactor();
    r->curves = curves;
    r->nsp = nsp;
    r->M.assign(M, M + nsp);
    r->R.resize(nsp);
    for (int i = 0; i < nsp; ++i) r->R[i] = R_UNIVERSAL / M[i];
    r->cp_tr.assign(cp_tr, cp_tr + nsp);
    r->h_f.assign(h_f, h_f + nsp);
    r->electron = electron;
    r->T_lower = T_lower; r->T_upper = T_upper; r->tol = tol;
    r->max_subcycles = max_subcycles; r->max_attempts = max_attempts;
    return r;
}

void oracle2t_free(void* h) { delete (Reactor*)h; }

// rate[k]: model, base model, rctIndex, A, n, C, s, T_D, U, theta, aU, Ustar, non-Boltzmann factor (13 values)
static Rate rate_from(const double* v) {
    Rate r;
    r.model = (int)v[0]; r.base = (int)v[1]; r.rct = (int)v[2];
    r.A = v[3]; r.n = v[4]; r.C = v[5]; r.s = v[6]; r.TD = v[7]; r.U = v[8]; r.theta = v[9];
    r.aU = v[10]; r.Ustar = v[11]; r.nb = v[12];
    return r;
}

int oracle2t_add_reaction(void* h, int collider, int nreac, const int* reac_idx, const int* reac_coeff, int nprod,
                          const int* prod_idx, const int* prod_coeff, int neff, const int* eff_idx,
                          const double* eff_val, const double* frc, const double* brc) {
    Reactor* r = (Reactor*)h;
    Reaction x;
    x.collider = collider != 0;
    for (int k = 0; k < nreac; ++k) x.reac.push_back({reac_idx[k], reac_coeff[k]});
    for (int k = 0; k < nprod; ++k) x.prod.push_back({prod_idx[k], prod_coeff[k]});
    x.nu.assign(r->nsp, 0);
    for (auto& p : x.reac) x.nu[p.first] -= p.second;
    for (auto& p : x.prod) x.nu[p.first] += p.second;
    for (auto& p : x.reac) x.part.push_back(p.first);
    for (auto& p : x.prod) x.part.push_back(p.first);
    std::sort(x.part.begin(), x.part.end());
    x.part.erase(std::unique(x.part.begin(), x.part.end()), x.part.end());
    for (int k = 0; k < neff; ++k) x.eff.push_back({eff_idx[k], eff_val[k]});
    x.frc = rate_from(frc);
    x.brc = rate_from(brc);
    r->rx.push_back(x);
    return (int)r->rx.size() - 1;
}

// v: kind, p, q, rt model, a, b, sigma, mu, sub a, sub b, reaction, coupling, D, Thetav, U, T_D, aU, Ustar, nb
int oracle2t_add_eem(void* h, const double* v) {
    Reactor* r = (Reactor*)h;
    Eem e;
    e.kind = (int)v[0]; e.p = (int)v[1]; e.q = (int)v[2];
    e.rt.model = (int)v[3]; e.rt.q = e.q; e.rt.a = v[4]; e.rt.b = v[5]; e.rt.sigma = v[6]; e.rt.mu = v[7];
    e.rt.sub_a = v[8]; e.rt.sub_b = v[9];
    e.r = (int)v[10]; e.coupling = (int)v[11]; e.D = v[12]; e.Thetav = v[13]; e.U = v[14]; e.TD = v[15];
    e.aU = v[16]; e.Ustar = v[17]; e.nb = v[18];
    r->eem.push_back(e);
    return (int)r->eem.size() - 1;
}

// A batch of cells, OpenMP over cells (nthreads 0: all).  massf is [n][nsp].  status 0, or the failure
// code with the cell left as it was; steps[c] = RKF attempts.
int oracle2t_update(void* h, int n, const double* rho, double* T, double* Tve, double* p, double* massf,
                    double t_interval, double* dt_suggest, double* u, double* u_ve, int* status, long long* steps,
                    int nthreads) {
    Reactor* proto = (Reactor*)h;
#ifdef _OPENMP
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
    {
        Reactor r = *proto;   // per-thread copy: the reactions hold per-cell rate constants
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int c = 0; c < n; ++c) {
            State st;
            st.rho = rho[c]; st.T = T[c]; st.Tve = Tve[c]; st.p = p[c];
            st.Y.assign(massf + (size_t)c * r.nsp, massf + (size_t)(c + 1) * r.nsp);
            long long s = 0;
            try {
                double uu = 0, uv = 0;
                r.update(st, t_interval, dt_suggest[c], uu, uv, s);
                T[c] = st.T; Tve[c] = st.Tve; p[c] = st.p;
                for (int i = 0; i < r.nsp; ++i) massf[(size_t)c * r.nsp + i] = st.Y[i];
                if (u) u[c] = uu;
                if (u_ve) u_ve[c] = uv;
                status[c] = 0;
            } catch (Failure& f) {
                status[c] = f.code;
            }
            if (steps) steps[c] = s;
        }
    }
    return 0;
}

}  // extern "C"
