// mechanism.cpp -- reading gas-model and mechanism files, and packing them for the device.
#include "mechanism.h"

#include <map>

#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "cea_thermo.h"
#include "chem_types.h"

namespace gdtk {

namespace {
constexpr double R_universal = 8.31451;   // gas/physical_constants.d:13

std::vector<std::string> species_list(const LuaValue& v) {
    std::vector<std::string> out;
    for (auto& s : v.sequence()) out.push_back(s.string());
    return out;
}

void arrhenius_params(const LuaValue& t, double& A, double& n, double& C) {   // rate_constant.d:60-66
    A = t.get("A").number();
    n = t.get("n").number();
    C = t.get("C").number();
    if (t.has("rctIndex") && t.get("rctIndex").number() != -1)
        throw std::runtime_error("rate constants on a temperature other than T need a multi-temperature gas");
}

// createRateConstant, kinetics/rate_constant.d:570-597, for a single-temperature gas.
RateConstHost rate_const(const LuaValue& t) {
    RateConstHost r;
    const std::string& model = t.get("model").string();
    if (model == "Arrhenius") {
        r.model = RATE_ARRHENIUS;
        arrhenius_params(t, r.A, r.n, r.C);
    } else if (model == "Arrhenius2" || model == "Arrhenius-logA") {   // rate_constant.d:82-121, 574-577
        r.model = RATE_ARRHENIUS2;
        r.A = t.get("logA").number();
        r.n = t.get("B").number();
        r.C = t.get("C").number();
        if (t.has("rctIndex") && t.get("rctIndex").number() != -1)
            throw std::runtime_error("rate constants on a temperature other than T need a multi-temperature gas");
    } else if (model == "Park") {   // rate_constant.d:364-393, rate-controlling T^s T_mode^(1-s)
        r.model = RATE_PARK;
        r.A = t.get("A").number();
        r.n = t.get("n").number();
        r.C = t.get("C").number();
        r.s = t.has("s") ? t.get("s").number() : std::nan("");   // checked with the gas model below
        if (t.has("mode") && t.get("mode").number() != 0)
            throw std::runtime_error("Park rate constants on an energy mode other than 0 need more than two temperatures");
    } else if (model == "Marrone-Treanor" || model == "Modified-Marrone-Treanor") {   // rate_constant.d:395-566
        RateConstHost b = rate_const(t.get("rate"));
        if (b.model != RATE_ARRHENIUS && b.model != RATE_PARK)
            throw std::runtime_error("a Marrone-Treanor rate constant needs an Arrhenius or Park rate beneath it");
        r = b;
        r.base = b.model;
        r.model = model == "Marrone-Treanor" ? RATE_MT : RATE_MMT;
        r.TD = t.get("T_D").number();
        r.theta = t.get("theta").number();
        if (r.model == RATE_MT) {
            r.U = t.get("U").number();
        } else {
            r.aU = t.get("aU").number();
            r.Ustar = t.get("Ustar").number();
            if (t.has("non_boltzmann_correction")) {   // rate_constant.d:470-492: only the constant model
                const LuaValue& nb = t.get("non_boltzmann_correction");
                if (nb.get("model").string() != "constant")
                    throw std::runtime_error("Invalid non Boltzmann correction factor for MMT");
                r.nb = nb.get("factor").number();
            }
        }
        if (t.has("mode") && t.get("mode").number() != 0)
            throw std::runtime_error("Marrone-Treanor rate constants on an energy mode other than 0 need more than "
                                     "two temperatures");
    } else if (model == "fromEqConst") {
        r.model = RATE_FROM_EQ;
    } else if (model == "Lindemann-Hinshelwood" || model == "Troe" || model == "Yungster-Rabinowitz") {
        arrhenius_params(t.get("kInf"), r.A, r.n, r.C);
        arrhenius_params(t.get("k0"), r.A0, r.n0, r.C0);
        if (model == "Lindemann-Hinshelwood") {
            r.model = RATE_LH;
        } else if (model == "Troe") {   // rate_constant.d:190-229
            r.model = RATE_TROE;
            if (t.has("F_cent")) {
                r.troe_flags = TROE_FCENT;
                r.Fcent = t.get("F_cent").number();
            } else {
                r.a = t.get("a").number();
                r.T3 = t.get("T3").number();
                if (t.get("T1").kind == LuaValue::NUMBER) { r.troe_flags |= TROE_T1; r.T1 = t.get("T1").number(); }
                if (t.get("T2").kind == LuaValue::NUMBER) { r.troe_flags |= TROE_T2; r.T2 = t.get("T2").number(); }
            }
        } else {   // rate_constant.d:321-333
            r.model = RATE_YR;
            r.a = t.get("a").number();
            r.T1 = t.get("b").number();
            r.T2 = t.get("c").number();
        }
    } else {
        // kinetics/rate_constant.d:570-597 also knows Park, Marrone-Treanor and MMT, which take the
        // rate-controlling temperature of a multi-temperature gas
        throw std::runtime_error("rate-constant model '" + model + "' is not supported by this engine");
    }
    return r;
}
}  // namespace

GasModelHost load_gas_model(const std::string& path, bool allow_two_temperature) {
    LuaValue g = read_lua_file(path);
    GasModelHost gm;
    std::string model = g.has("model") ? g.get("model").string() : "";
    if (model == "CompositeGas") {
        std::string phys = g.get("physical_model").string();
        if (phys == "two-temperature-gas" && allow_two_temperature) {
            gm.two_temperature = true;
        } else if (phys != "thermally-perfect-gas") {
            throw std::runtime_error("physical model '" + phys + "' is not supported here (thermally-perfect-gas" +
                                     std::string(allow_two_temperature ? " or two-temperature-gas)" : ")"));
        }
        gm.type_str = "CompositeGas";
    } else if (model == "ThermallyPerfectGas") {
        gm.type_str = "ThermallyPerfectGas";
    } else if (model.empty() && g.get("physical_model").kind == LuaValue::STRING &&
               g.get("physical_model").string() == "thermally-perfect-gas") {
        gm.type_str = "CompositeGas";
    } else {
        throw std::runtime_error("gas model '" + model + "' is not supported (thermally perfect gas only)");
    }
    gm.names = species_list(g.get("species"));
    if (gm.names.empty() || (int)gm.names.size() > GDTK_MAX_SPECIES_ANY)
        throw std::runtime_error("species count out of range (1.." + std::to_string(GDTK_MAX_SPECIES_ANY) + ")");
    const LuaValue& db = g.get("db");
    for (auto& name : gm.names) {
        const LuaValue& e = db.get(name);
        if (e.is_nil()) throw std::runtime_error("no database entry for species " + name);
        gm.M.push_back(e.get("M").number());
        if (gm.two_temperature) {   // two_temperature_gas.d:45-80: the particle kind sets the heat capacity
            const std::string kind = e.get("type").kind == LuaValue::STRING ? e.get("type").string() : "";
            if (name == "e-" || kind == "electron") gm.particle.push_back(PARTICLE_ELECTRON);
            else if (kind == "atom") gm.particle.push_back(PARTICLE_ATOM);
            else if (kind == "molecule")
                gm.particle.push_back(e.get("molecule_type").kind == LuaValue::STRING &&
                                      e.get("molecule_type").string() == "linear" ? PARTICLE_LINEAR : PARTICLE_NONLINEAR);
            else throw std::runtime_error("TwoTemperatureGas: unknown particle type for species " + name);
        }
        std::map<std::string, int> comp;   // atomicConstituents = { H=2, O=1 } (prep-gas species record)
        const LuaValue& ac = e.get("atomicConstituents");
        if (ac.kind == LuaValue::TABLE)
            for (auto& kv : *ac.tab)
                if (kv.second.kind == LuaValue::NUMBER) comp[kv.first] = (int)kv.second.number();
        for (auto& kv : comp)
            if (std::find(gm.elements.begin(), gm.elements.end(), kv.first) == gm.elements.end())
                gm.elements.push_back(kv.first);
        gm.composition.push_back(comp);
        const LuaValue& th = e.get("thermoCoeffs");
        CeaCurveHost c;
        c.nseg = (int)th.get("nsegments").number();
        if (c.nseg < 1 || c.nseg > GDTK_MAX_SEGMENTS) throw std::runtime_error("bad nsegments for " + name);
        c.breaks = th.get("T_break_points").numbers();
        c.blends = th.get("T_blend_ranges").numbers();
        if ((int)c.breaks.size() != c.nseg + 1 || (int)c.blends.size() < c.nseg - 1)
            throw std::runtime_error("inconsistent CEA curve for " + name);
        for (int s = 0; s < c.nseg; ++s) {
            std::vector<double> seg = th.get("segment" + std::to_string(s)).numbers();
            if (seg.size() != 9) throw std::runtime_error("CEA segment needs 9 coefficients for " + name);
            c.coeffs.insert(c.coeffs.end(), seg.begin(), seg.end());
        }
        gm.curves.push_back(c);
    }
    return gm;
}

MechanismHost load_mechanism(const std::string& path, const GasModelHost& gm, bool with_config) {
    LuaValue c = read_lua_file(path);
    MechanismHost mh;
    if (c.has("species")) {   // chemistry_update.d:54-73
        std::vector<std::string> sp = species_list(c.get("species"));
        if (sp.size() != gm.names.size())
            throw std::runtime_error("species count differs between gas model and chemistry input");
        for (size_t i = 0; i < sp.size(); ++i)
            if (sp[i] != gm.names[i])
                throw std::runtime_error("Species order is incompatible between gas model and chemistry input: index " +
                                         std::to_string(i) + " is '" + gm.names[i] + "' in the gas model and '" +
                                         sp[i] + "' in the chemistry input");
    } else if (with_config) {
        throw std::runtime_error("There is no species listing in the chemistry input file " + path);
    }
    if (with_config) {
        const LuaValue& cfg = c.get("config");
        mh.T_lower = cfg.get("tempLimits").get("lower").number();
        mh.T_upper = cfg.get("tempLimits").get("upper").number();
        const LuaValue& ode = cfg.get("odeStep");
        std::string method = ode.get("method").string();
        if (method == "rkf") {
            mh.method = METHOD_RKF;
            mh.errTol = ode.get("errTol").number();
        } else if (method == "alpha-qss") {
            mh.method = METHOD_ALPHA_QSS;
            mh.eps1 = ode.get("eps1").number();
            mh.eps2 = ode.get("eps2").number();
            mh.delta = ode.get("delta").number();
            mh.maxIters = (int)ode.get("maxIters").number();
        } else {
            throw std::runtime_error("ERROR: The odeStep '" + method + "' is unknown.");
        }
        mh.tight = cfg.get("tightTempCoupling").boolean();
        mh.maxSubcycles = (int)cfg.get("maxSubcycles").number();
        mh.maxAttempts = (int)cfg.get("maxAttempts").number();
    }
    const LuaValue& rt = c.get("reaction");
    const int nsp = gm.n_species();
    for (long k : rt.int_keys()) {
        const LuaValue& r = rt.at(k);
        ReactionHost rh;
        std::string type = r.get("type").string();
        if (type == "anonymous_collider") rh.collider = true;
        else if (type != "elementary") throw std::runtime_error("The reaction type: " + type + " is not known.");
        if (r.has("equation")) rh.equation = r.get("equation").string();
        rh.frc = rate_const(r.get("frc"));
        rh.brc = rate_const(r.get("brc"));
        auto two_t = [](const RateConstHost& c) {
            return c.model == RATE_PARK || c.model == RATE_MT || c.model == RATE_MMT;
        };
        if (two_t(rh.frc) || two_t(rh.brc)) {
            if (!gm.two_temperature)
                throw std::runtime_error("rate-constant model '" +
                                         std::string(rh.frc.model == RATE_PARK || rh.brc.model == RATE_PARK
                                                         ? "Park" : "Marrone-Treanor") +
                                         "' is not supported for a one-temperature gas: it needs a two-temperature "
                                         "gas model (rate_constant.d:364-566)");
            if (!std::isfinite(rh.frc.s) && (rh.frc.model == RATE_PARK || rh.frc.base == RATE_PARK))
                throw std::runtime_error("Park rate constant without its exponent s");
            if (two_t(rh.brc))
                throw std::runtime_error("Park and Marrone-Treanor backward rate constants are not supported "
                                         "(forward with k_b from K_c)");
        }
        if (rh.frc.model == RATE_FROM_EQ && rh.brc.model == RATE_FROM_EQ)
            throw std::runtime_error("a reaction needs at least one Arrhenius rate constant");
        if (rh.brc.pressure_dependent() || (rh.frc.pressure_dependent() && rh.brc.model != RATE_FROM_EQ))
            throw std::runtime_error("pressure-dependent rate constants are supported as the forward rate with a "
                                     "backward rate from K_c");
        std::vector<int> ri = r.get("reacIdx").ints(), rc = r.get("reacCoeffs").ints();
        std::vector<int> pi = r.get("prodIdx").ints(), pc = r.get("prodCoeffs").ints();
        if (ri.size() != rc.size() || pi.size() != pc.size())
            throw std::runtime_error("reacIdx/reacCoeffs or prodIdx/prodCoeffs lengths differ");
        if ((int)ri.size() > GDTK_MAX_TERMS || (int)pi.size() > GDTK_MAX_TERMS)
            throw std::runtime_error("too many reactant or product terms in one reaction");
        for (size_t i = 0; i < ri.size(); ++i) {
            if (ri[i] < 0 || ri[i] >= nsp) throw std::runtime_error("species index out of range");
            rh.reac.push_back({ri[i], rc[i]});
        }
        for (size_t i = 0; i < pi.size(); ++i) {
            if (pi[i] < 0 || pi[i] >= nsp) throw std::runtime_error("species index out of range");
            rh.prod.push_back({pi[i], pc[i]});
        }
        // kinetics/reaction.d:484-495 reads the efficiency table with lua_next; for the integer
        // keys 0..n-1 of these constructors Lua 5.4 visits them in ascending order.
        const LuaValue& eff = r.get("efficiencies");
        for (long key : eff.int_keys()) {
            if (key < 0 || key >= nsp) throw std::runtime_error("efficiency species index out of range");
            rh.eff.push_back({(int)key, eff.at(key).number()});
        }
        mh.reactions.push_back(rh);
    }
    if ((int)mh.reactions.size() > GDTK_MAX_REACTIONS_ANY)
        throw std::runtime_error("too many reactions (max " + std::to_string(GDTK_MAX_REACTIONS_ANY) + ")");
    return mh;
}

PackedMech pack(const GasModelHost& gm, const MechanismHost* mh) {
    PackedMech pm;
    const int nsp = gm.n_species();
    const int nr = mh ? (int)mh->reactions.size() : 0;
    // distinct efficiency lists
    std::vector<std::vector<std::pair<int, double>>> sets;
    std::vector<int> set_of(nr, -1);
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh->reactions[ir];
        if (!r.collider && !r.frc.pressure_dependent()) continue;   // third bodies of the reaction or its rate
        int found = -1;
        for (size_t s = 0; s < sets.size(); ++s)
            if (sets[s] == r.eff) { found = (int)s; break; }
        if (found < 0) { sets.push_back(r.eff); found = (int)sets.size() - 1; }
        set_of[ir] = found;
    }
    if ((int)sets.size() > GDTK_MAX_EFFSETS) throw std::runtime_error("too many distinct efficiency lists");
    const int neff = (int)sets.size();
    pm.nsp = nsp; pm.nr = nr; pm.neff = neff; pm.method = mh ? mh->method : 0;
    pm.I.assign(mech_n_ints(nsp, nr, neff), 0);
    pm.D.assign(mech_n_doubles(nsp, nr, neff), 0.0);
    int* I = pm.I.data();
    double* D = pm.D.data();
    I[0] = nsp; I[1] = nr; I[2] = neff;
    if (mh) {
        I[3] = mh->method; I[4] = mh->maxIters; I[5] = mh->tight ? 1 : 0;
        I[6] = mh->maxSubcycles; I[7] = mh->maxAttempts;
        D[0] = mh->T_lower; D[1] = mh->T_upper; D[2] = mh->errTol; D[3] = mh->eps1; D[4] = mh->eps2; D[5] = mh->delta;
    }
    MechView v;
    v.bind(I, D);
    for (int isp = 0; isp < nsp; ++isp) {
        const CeaCurveHost& c = gm.curves[isp];
        I[HI + isp] = c.nseg;
        double* s = D + HD + SPD * isp;
        s[SP_M] = gm.M[isp];
        s[SP_R] = R_universal / gm.M[isp];   // therm_perf_gas_mix.d:40
        for (int k = 0; k <= c.nseg; ++k) s[SP_BREAKS + k] = c.breaks[k];
        for (int k = 0; k < c.nseg - 1; ++k) s[SP_BLENDS + k] = c.blends[k];
        for (int k = 0; k < c.nseg * 9; ++k) s[SP_COEFFS + k] = c.coeffs[k];
        // cea_thermo_curves.d:46-53: values at the ends of the curve, used beyond them.
        s[SP_TLOW] = c.breaks.front();
        s[SP_THIGH] = c.breaks.back();
        int err = 0;
        const double Tl = s[SP_TLOW], Th = s[SP_THIGH];
        double Cp_low = cea_Cp(v, isp, Tl, err), Cp_high = cea_Cp(v, isp, Th, err);
        double h_low = cea_h(v, isp, Tl, std::log(Tl), err), h_high = cea_h(v, isp, Th, std::log(Th), err);
        double s_low = cea_s(v, isp, Tl, std::log(Tl), err), s_high = cea_s(v, isp, Th, std::log(Th), err);
        if (err) throw std::runtime_error("CEA curve of " + gm.names[isp] + " cannot be evaluated at its end points");
        s[SP_CPLOW] = Cp_low; s[SP_CPHIGH] = Cp_high; s[SP_HLOW] = h_low; s[SP_HHIGH] = h_high;
        s[SP_SLOW] = s_low; s[SP_SHIGH] = s_high;
    }
    for (int ir = 0; ir < nr; ++ir) {
        const ReactionHost& r = mh->reactions[ir];
        int* ri = I + HI + nsp + RXI * ir;
        double* rd = D + HD + SPD * nsp + RXD * ir;
        ri[RX_COLLIDER] = r.collider ? 1 : 0;
        ri[RX_FRC] = r.frc.model;
        ri[RX_BRC] = r.brc.model;
        ri[RX_EFFSET] = set_of[ir] < 0 ? 0 : set_of[ir];
        ri[RX_NREAC] = (int)r.reac.size();
        ri[RX_NPROD] = (int)r.prod.size();
        for (size_t k = 0; k < r.reac.size(); ++k) { ri[RX_REAC_IDX + k] = r.reac[k].first; ri[RX_REAC_COEFF + k] = r.reac[k].second; }
        for (size_t k = 0; k < r.prod.size(); ++k) { ri[RX_PROD_IDX + k] = r.prod[k].first; ri[RX_PROD_COEFF + k] = r.prod[k].second; }
        // participants: sorted distinct species of both sides; nu = first product coeff - first
        // reactant coeff (kinetics/reaction.d:211-238)
        std::vector<int> part;
        for (auto& x : r.reac) part.push_back(x.first);
        for (auto& x : r.prod) part.push_back(x.first);
        std::sort(part.begin(), part.end());
        part.erase(std::unique(part.begin(), part.end()), part.end());
        if ((int)part.size() > GDTK_MAX_PARTICIPANTS) throw std::runtime_error("too many participants in a reaction");
        ri[RX_NPART] = (int)part.size();
        for (size_t k = 0; k < part.size(); ++k) {
            int isp = part[k], nu1 = 0, nu2 = 0;
            for (auto& x : r.reac) if (x.first == isp) { nu1 = x.second; break; }
            for (auto& x : r.prod) if (x.first == isp) { nu2 = x.second; break; }
            ri[RX_PART + k] = isp;
            ri[RX_PART_NU + k] = nu2 - nu1;
        }
        rd[0] = r.frc.A; rd[1] = r.frc.n; rd[2] = r.frc.C;
        rd[3] = r.brc.A; rd[4] = r.brc.n; rd[5] = r.brc.C;
        rd[RD_K0A] = r.frc.A0; rd[RD_K0N] = r.frc.n0; rd[RD_K0C] = r.frc.C0;
        rd[RD_FCENT] = r.frc.Fcent; rd[RD_TA] = r.frc.a; rd[RD_T1] = r.frc.T1; rd[RD_T2] = r.frc.T2;
        rd[RD_T3] = r.frc.T3; rd[RD_TFLAGS] = r.frc.troe_flags;
        rd[RD_S] = r.frc.s;
        if (r.frc.model == RATE_MT || r.frc.model == RATE_MMT) {
            ri[RX_BASE] = r.frc.base;
            rd[RD_MT_TD] = r.frc.TD;
            rd[RD_MT_U] = r.frc.model == RATE_MT ? r.frc.U : r.frc.aU;
            rd[RD_MT_THETA] = r.frc.theta;
            rd[RD_MT_USTAR] = r.frc.Ustar;
            rd[RD_MT_NB] = r.frc.nb;
        }
    }
    for (int s = 0; s < neff; ++s) {
        int* ei = I + HI + nsp + RXI * nr + (1 + nsp) * s;
        double* ed = D + HD + SPD * nsp + RXD * nr + nsp * s;
        ei[0] = (int)sets[s].size();
        for (size_t k = 0; k < sets[s].size(); ++k) {
            ei[1 + k] = sets[s][k].first;
            ed[sets[s][k].first] = sets[s][k].second;
        }
    }
    return pm;
}

// Operation counts of the reference expressions, term by term (add/sub/mul/div/sqrt = 1,
// exp/log = 20, pow = 40; comparisons and copies are free).
void flop_model(const GasModelHost& gm, const MechanismHost& mh, double out[5]) {
    const double EXP = 20, LOG = 20, POW = 40;
    const int nsp = gm.n_species();
    // eval_rate_constants: log T, log(p/P_atm) and its division; per species eval_h (29),
    // eval_s with the pressure term (28) and g = h - T s (2) (therm_perf_gas_mix.d:354-364).
    double kc = 2 * LOG + 1 + 59.0 * nsp;
    // eval_split_rates: distinct third-body sums (2 per efficiency), then per reaction the
    // collider products, the concentration powers and four operations per participant.
    std::vector<std::vector<std::pair<int, double>>> sets;
    double rhs = 0;
    for (auto& r : mh.reactions) {
        std::vector<int> part;
        for (auto& x : r.reac) part.push_back(x.first);
        for (auto& x : r.prod) part.push_back(x.first);
        std::sort(part.begin(), part.end());
        part.erase(std::unique(part.begin(), part.end()), part.end());
        // rate constants (rate_constant.d:72-75, 112-115, reaction.d:26-52, 94-143)
        auto arr_of = [&](const RateConstHost& rc) { return rc.model == RATE_ARRHENIUS2 ? EXP + 4 : POW + EXP + 3; };
        const double arr = POW + EXP + 3;
        // pressure-dependent forward rates (rate_constant.d:114-121, 155-160, 258-287, 338-350): two
        // Arrhenius terms, the third-body sum (4 per efficiency) and the blending
        double fwd = arr;
        const double tb = 2 * arr + 4.0 * r.eff.size() + 5;
        if (r.frc.model == RATE_LH) {
            fwd = tb;
        } else if (r.frc.model == RATE_TROE) {
            double fc = 0;
            if (!(r.frc.troe_flags & TROE_FCENT))
                fc = (EXP + 4) + ((r.frc.troe_flags & TROE_T1) ? EXP + 3 : 0) + ((r.frc.troe_flags & TROE_T2) ? EXP + 2 : 0);
            fwd = tb + 2 + LOG + fc + LOG + 4 + 7 + POW + 1;
        } else if (r.frc.model == RATE_YR) {
            fwd = tb + 2 + LOG + 2 * EXP + 7 + 3 + 4;
        }
        if (r.frc.model == RATE_ARRHENIUS2) fwd = arr_of(r.frc);
        if (r.frc.model == RATE_FROM_EQ || r.brc.model == RATE_FROM_EQ)
            kc += (r.frc.model == RATE_FROM_EQ ? arr_of(r.brc) : fwd) + 4.0 * part.size() + (EXP + 2) + 3 + 1 + 1;
        else
            kc += fwd + arr_of(r.brc);
        if (r.collider) {
            if (std::find(sets.begin(), sets.end(), r.eff) == sets.end()) {
                sets.push_back(r.eff);
                rhs += 2.0 * r.eff.size();
            }
            rhs += 2;
        }
        for (auto& x : r.reac) rhs += x.second;
        for (auto& x : r.prod) rhs += x.second;
        for (int isp : part) {
            int nu1 = 0, nu2 = 0;
            for (auto& x : r.reac) if (x.first == isp) { nu1 = x.second; break; }
            for (auto& x : r.prod) if (x.first == isp) { nu2 = x.second; break; }
            if (nu2 != nu1) rhs += 4;
        }
    }
    double step, corr = 0;
    if (mh.method == METHOD_RKF) {
        rhs += nsp;                              // rates = q - L
        step = 62.0 * nsp + 2 + POW + 2 + 3.0 * nsp;   // chemistry_update.d:417-477 + mass test
    } else {
        step = 32.0 * nsp + 4.0 * nsp + 18 + 3.0 * nsp;   // predictor, step_suggest, mass test
        corr = 41.0 * nsp;                       // chemistry_update.d:546-558 per corrector
    }
    step += 2;                                   // t += h, hMax
    // update_temperature_from_energy: per iteration Cv (23 per species), log T and u(T)
    // (33 per species) and the update/convergence arithmetic.
    double newton = 56.0 * nsp + LOG + 4;
    out[0] = kc; out[1] = rhs; out[2] = step; out[3] = corr; out[4] = newton;
}

}  // namespace gdtk
