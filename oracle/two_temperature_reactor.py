"""CPU restatement of the reference's multi-temperature thermochemical reactor for a two-temperature
gas (TEST INFRASTRUCTURE ONLY).

Follows kinetics/multi_temperature_thermochemical_reactor.d (RKF Cash-Karp on the species
concentrations and the vibrational-electronic energy, one rate-constant and relaxation-time
evaluation per subcycle, T and T_ve from (rho, u, u_ve) after each successful step), with
  * rate constants, reaction.d:94-143 (multi-temperature branch) and rate_constant.d:52-80,
    364-393 (Arrhenius; Park 2-T, T_eff = T^s T_ve^(1-s)), 395-452 (Marrone-Treanor) and 494-566
    (modified Marrone-Treanor) over an Arrhenius or Park rate; backward rates from K_c at T with the
    forward rate constant re-evaluated at T_ve = T; Gibbs energies at p = P_atm and T_ve = T
    (reaction_mechanism.d:49-63, 204-218; two_temperature_gas.d:469-482);
  * tick rates, reaction.d:267-311, 394-456 (pow(conc, coeff), anonymous colliders), and species
    rates q - L (reaction_mechanism.d:74-96);
  * energy exchange, energy_exchange_system.d:70-104 and energy_exchange_mechanism.d: Landau-Teller
    (:56-101) with Millikan-White, ParkHTC and ParkHTC2 relaxation times (relaxation_time.d:27-175),
    and the Marrone-Treanor chemistry-vibration coupling (:195-253) with impartial, Marrone-Treanor or
    modified Marrone-Treanor dissociation (exchange_chemistry_coupling.d:18-227); within a step the
    exchange sees the gas state of the
    step's start (T, T_ve, p, mass fractions), as the reference's does;
  * the two-temperature thermo of oracle/two_temperature.py (two_temperature_gas.d), pinned to the
    reference's known-answer test.
No reference test holds numbers for this reactor; tests/test_oracle_kat.py checks this restatement
against a tight implicit integration of the same ODE system.  Plain Python, one cell at a time.
"""
import math

import numpy as np

from .luatable import read_lua_file
from .two_temperature import TwoTemperatureGas, R_UNIVERSAL

P_ATM = 101325.0
AVOGADRO = 6.02214e23           # gas/physical_constants.d:19
BOLTZMANN = 1.380658e-23        # gas/physical_constants.d:18
SMALL_MOLE_FRACTION = 1.0e-15   # gas/gas_model.d:42
IGAMMA_SWITCH = 1.0e-7          # exchange_chemistry_coupling.d:24
IGAMMA_OVERFLOW = 0.001         # exchange_chemistry_coupling.d:25
# multi_temperature_thermochemical_reactor.d:24-33
DT_INCREASE_PERCENT = 10.0
DT_REDUCTION_FACTOR = 10.0
H_MIN = 1.0e-15
ALLOWABLE_MASSF_ERROR = 1.0e-3


class ReactorFailure(Exception):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _ints(t):
    return [int(t[k]) for k in sorted(t)] if isinstance(t, dict) else [int(v) for v in t]


def _Qmt(T, D, theta):
    """rate_constant.d:397-404: the partition-function ratio of the Marrone-Treanor rates."""
    return (1 - math.exp(-D / T)) / (1 - math.exp(-theta / T))


def _pow_int(x, n):
    """D's pow(number, int) for the small positive stoichiometric coefficients here."""
    r = 1.0
    for _ in range(n):
        r *= x
    return r


class Reaction:
    def __init__(self, r, nsp):
        self.collider = r["type"] == "anonymous_collider"
        self.reac = list(zip(_ints(r["reacIdx"]), _ints(r["reacCoeffs"])))
        self.prod = list(zip(_ints(r["prodIdx"]), _ints(r["prodCoeffs"])))
        self.nu = np.zeros(nsp, dtype=np.int64)
        for i, c in self.reac:
            self.nu[i] -= c
        for i, c in self.prod:
            self.nu[i] += c
        self.participants = sorted({i for i, _ in self.reac} | {i for i, _ in self.prod})
        eff = r.get("efficiencies") or {}
        self.eff = [(int(k), float(eff[k])) for k in sorted(eff) if float(eff[k]) != 0.0]
        self.frc, self.brc = r["frc"], r["brc"]
        self.kf = self.kb = self.wf = self.wb = 0.0

    @staticmethod
    def rate_constant(rc, T, T_modes):
        """rate_constant.d: Arrhenius at T (or T_modes[rctIndex]), Park at T^s T_mode^(1-s)."""
        m = rc["model"]
        if m == "Arrhenius":
            idx = int(rc.get("rctIndex", -1))
            Tr = T if idx == -1 else T_modes[idx]
            return rc["A"] * math.pow(Tr, rc["n"]) * math.exp(-rc["C"] / Tr)
        if m == "Park":
            Tr = math.pow(T, rc["s"]) * math.pow(T_modes[int(rc["mode"])], 1.0 - rc["s"])
            return rc["A"] * math.pow(Tr, rc["n"]) * math.exp(-rc["C"] / Tr)
        if m == "Marrone-Treanor":   # rate_constant.d:438-447
            kEQ = Reaction.rate_constant(rc["rate"], T, T_modes)
            Tv, TD, th, U = T_modes[int(rc["mode"])], rc["T_D"], rc["theta"], rc["U"]
            Gamma = 1. / (1. / Tv - 1. / T - 1. / U)
            return kEQ * _Qmt(T, TD, th) * _Qmt(Gamma, TD, th) / (_Qmt(Tv, TD, th) * _Qmt(-U, TD, th))
        if m == "Modified-Marrone-Treanor":   # rate_constant.d:541-554
            kEQ = Reaction.rate_constant(rc["rate"], T, T_modes)
            Tv, TD, th = T_modes[int(rc["mode"])], rc["T_D"], rc["theta"]
            Tinv = 1. / T
            Tvinv = 1. / Tv
            Uinv = rc["aU"] * Tinv + 1. / rc["Ustar"]
            U = 1. / Uinv
            TF = 1. / (Tvinv - Tinv - Uinv)
            nbc = rc.get("non_boltzmann_correction")
            nb = float(nbc["factor"]) if nbc else 1.0
            return nb * kEQ * _Qmt(T, TD, th) * _Qmt(TF, TD, th) / (_Qmt(Tv, TD, th) * _Qmt(-U, TD, th))
        raise ValueError("rate-constant model %s is outside the two-temperature path" % m)

    def eval_rate_constants(self, T, T_modes, gibbs, M):
        """reaction.d:94-143, multi-temperature branch; T is the clamped T."""
        def Kc():   # reaction.d:26-52 with the Gibbs energies at T (rate-controlling index -1)
            dG = 0.0
            nuSum = 0.0
            for isp in self.participants:
                dG += self.nu[isp] * gibbs[isp] * M[isp]
                nuSum += self.nu[isp]
            K_p = math.exp(-dG / (R_UNIVERSAL * T))
            return K_p * math.pow(P_ATM / (R_UNIVERSAL * T), nuSum)
        if self.frc["model"] != "fromEqConst":
            self.kf = self.rate_constant(self.frc, T, T_modes)
            if self.brc["model"] == "fromEqConst":
                Tb = T if int(self.brc.get("rctIndex", -1)) < 0 else T_modes[int(self.brc["rctIndex"])]
                K = Kc()
                kf_rct = self.rate_constant(self.frc, Tb, [Tb] * len(T_modes))
                self.kb = kf_rct / K
            else:
                self.kb = self.rate_constant(self.brc, T, T_modes)
        else:
            self.kb = self.rate_constant(self.brc, T, T_modes)
            K = Kc()
            kb_rct = self.rate_constant(self.brc, T, T_modes)   # evaluated at Q, as reaction.d:131
            self.kf = kb_rct * K

    def eval_rates(self, conc):
        """reaction.d:145-149, 290-311, 416-440."""
        m = 1.0
        if self.collider:
            m = 0.0
            for isp, e in self.eff:
                m += e * conc[isp]
        wf = self.kf * m
        for isp, c in self.reac:
            wf *= _pow_int(conc[isp], c)
        wb = self.kb * m
        for isp, c in self.prod:
            wb *= _pow_int(conc[isp], c)
        self.wf, self.wb = wf, wb

    def production(self, isp):
        n = self.nu[isp]
        return n * self.wf if n > 0 else (-n * self.wb if n < 0 else 0.0)

    def loss(self, isp):
        n = self.nu[isp]
        return n * self.wb if n > 0 else (-n * self.wf if n < 0 else 0.0)


class TwoTemperatureReactor:
    """multi_temperature_thermochemical_reactor.d for a two-temperature gas (one energy mode)."""

    def __init__(self, gas_file, chem_file, eem_file):
        self.gas = TwoTemperatureGas(gas_file)
        self.nsp = self.gas.nsp
        self.M = self.gas.M
        c = read_lua_file(chem_file)
        self.reactions = [Reaction(c["reaction"][k], self.nsp) for k in sorted(c["reaction"])]
        cfg = c["config"]
        self.T_lower, self.T_upper = float(cfg["tempLimits"]["lower"]), float(cfg["tempLimits"]["upper"])
        ode = cfg["odeStep"]
        if ode["method"] != "rkf":
            raise ValueError("the multi-temperature reactor takes the rkf step only")
        self.tol = float(ode.get("errTol", 1e-3))
        self.max_subcycles = int(cfg.get("maxSubcycles", 10000))
        self.max_attempts = int(cfg.get("maxAttempts", 4))
        e = read_lua_file(eem_file)
        idx = {n: i for i, n in enumerate(self.gas.names)}
        self.mechs = []
        for k in sorted(e["mechanism"]):
            m = e["mechanism"][k]
            if m["rate"] == "Landau-Teller":
                p, q = idx[m["p"]], idx[m["q"]]
                self.mechs.append(dict(kind="LT", p=p, q=q, rt=self._relaxation(m["relaxation_time"], p, q)))
            elif m["rate"] == "Marrone-Treanor":
                cm = m["coupling_model"]
                mech = dict(kind="MT", p=idx[m["p"]], r=int(m["reaction_index"]), coupling=cm["model"],
                            Thetav=float(cm["Thetav"]))
                if cm["model"] == "ImpartialDissociation":
                    mech.update(D=float(cm["D"]))
                elif cm["model"] == "MarroneTreanorDissociation":
                    mech.update(D=float(cm["D"]), U=float(cm["U"]))
                elif cm["model"] == "ModifiedMarroneTreanorDissociation":
                    mech.update(T_D=float(cm["T_D"]), aU=float(cm["aU"]), Ustar=float(cm["Ustar"]),
                                nb=float(cm.get("non_boltzmann", 0.0)))
                else:
                    raise ValueError("coupling model %s is outside this restatement" % cm["model"])
                self.mechs.append(mech)
            else:
                raise ValueError("energy exchange rate %s is outside this restatement" % m["rate"])

    def _relaxation(self, t, p, q):
        model = t["model"]
        if model == "Millikan-White":
            return dict(model="MW", q=q, a=float(t["a"]), b=float(t["b"]))
        if model in ("ParkHTC", "ParkHTC2"):
            mq, mp = self.M[q] / AVOGADRO, self.M[p] / AVOGADRO
            return dict(model=model, q=q, sigma=float(t["sigma"]), mu=mq * mp / (mq + mp),
                        sub=self._relaxation(t["submodel"], p, q))
        raise ValueError("relaxation time %s is outside this restatement" % model)

    # ---- relaxation times (relaxation_time.d:27-175)
    def _tau(self, rt, T, p, molef, numden):
        if molef[rt["q"]] <= SMALL_MOLE_FRACTION:
            return -1.0
        if rt["model"] == "MW":
            pBath = molef[rt["q"]] * p / P_ATM
            return (1.0 / pBath) * math.exp(rt["a"] * (math.pow(T, -1.0 / 3.0) - rt["b"]) - 18.42)
        tau_sub = self._tau(rt["sub"], T, p, molef, numden)
        sigma = rt["sigma"] if rt["model"] == "ParkHTC" else rt["sigma"] * (50e3 / T) * (50e3 / T)
        cs = math.sqrt(8.0 * BOLTZMANN * T / math.pi / rt["mu"])
        return tau_sub + 1.0 / (sigma * cs * numden[rt["q"]])

    # ---- chemistry-vibration coupling (exchange_chemistry_coupling.d:41-227)
    @staticmethod
    def _coupling(m, T, Tv):
        """(G_appear, G_vanish) of a Marrone-Treanor mechanism at (T, T_ve)."""
        th = m["Thetav"]
        if m["coupling"] == "ImpartialDissociation":   # :94-126
            return 0.5 * (m["D"] - th * R_UNIVERSAL), TwoTemperatureReactor._gvanish(T, Tv, m["D"], th)
        if m["coupling"] == "MarroneTreanorDissociation":   # :152-174
            D, U = m["D"], m["U"]
            iG = 1. / Tv - 1. / T - 1. / U
            gv = TwoTemperatureReactor._L(iG, D, th)
            T_F_inv = -1. / U
            ga = R_UNIVERSAL * th / (math.exp(th * T_F_inv) - 1.) - D / (math.exp(D / R_UNIVERSAL * T_F_inv) - 1.)
            return ga, gv
        TD = m["T_D"]   # ModifiedMarroneTreanorDissociation, :204-220
        Uinv = m["aU"] / T + 1 / m["Ustar"]
        T_F_inv = 1. / Tv - 1. / T - Uinv
        gv = R_UNIVERSAL * (th / (math.exp(th * T_F_inv) - 1.) - TD / (math.exp(TD * T_F_inv) - 1.)) \
            + m["nb"] * R_UNIVERSAL * TD
        T_F_inv = - m["aU"] / T - 1 / m["Ustar"]
        ga = R_UNIVERSAL * (th / (math.exp(th * T_F_inv) - 1.) - TD / (math.exp(TD * T_F_inv) - 1.))
        return ga, gv

    @staticmethod
    def _L(iG, D, Thetav):
        """Equation (39) of Knab 1995 with its small-iG and overflow forms (exchange_chemistry_coupling.d:41-69)."""
        if abs(iG) < IGAMMA_SWITCH:
            return 0.5 * (D - Thetav * R_UNIVERSAL) + iG * (Thetav * Thetav * R_UNIVERSAL * R_UNIVERSAL - D * D) / 12.0 \
                / R_UNIVERSAL
        if iG > IGAMMA_OVERFLOW:
            return R_UNIVERSAL * Thetav / (math.exp(Thetav * iG) - 1.0) - D * math.exp(-D / R_UNIVERSAL * iG)
        return R_UNIVERSAL * Thetav / (math.exp(Thetav * iG) - 1.0) - D / (math.exp(D / R_UNIVERSAL * iG) - 1.0)

    # ---- Marrone-Treanor, impartial dissociation (exchange_chemistry_coupling.d:27-121)
    @staticmethod
    def _gvanish(T, Tv, D, Thetav):
        iG = (T - Tv) / (T * Tv)
        if abs(iG) < IGAMMA_SWITCH:
            return 0.5 * (D - Thetav * R_UNIVERSAL) + iG * (Thetav * Thetav * R_UNIVERSAL * R_UNIVERSAL - D * D) / 12.0 \
                / R_UNIVERSAL
        if iG > IGAMMA_OVERFLOW:
            return R_UNIVERSAL * Thetav / (math.exp(Thetav * iG) - 1.0) - D * math.exp(-D / R_UNIVERSAL * iG)
        return R_UNIVERSAL * Thetav / (math.exp(Thetav * iG) - 1.0) - D / (math.exp(D / R_UNIVERSAL * iG) - 1.0)

    def _ees_rate(self, st, taus):
        """energy_exchange_system.d:93-104: J/kg/s into the vibrational-electronic mode."""
        T, Tv, Y, rho = st["T"], st["Tve"], st["massf"], st["rho"]
        rate = 0.0
        for m, tau in zip(self.mechs, taus):
            if m["kind"] == "LT":
                if tau < 0.0:
                    continue
                ev_star = self.gas.e_ve(m["p"], T)
                ev = self.gas.e_ve(m["p"], Tv)
                rate += Y[m["p"]] * (ev_star - ev) / tau
            else:
                r = self.reactions[m["r"]]
                ga, gv = self._coupling(m, T, Tv)
                rate += (r.production(m["p"]) * ga - r.loss(m["p"]) * gv) / rho
        return rate

    # ---- state
    def _gibbs(self, T):
        out = np.empty(self.nsp)
        for i in range(self.nsp):
            _, h, s = self.gas.curves.species_thermo(i, T)
            out[i] = h - T * s
        return out

    def _rate_constants(self, st):
        T = min(max(st["T"], self.T_lower), self.T_upper)
        g = self._gibbs(T)
        for r in self.reactions:
            r.eval_rate_constants(T, [st["Tve"]], g, self.M)

    def _relaxation_times(self, st):
        Y, rho = st["massf"], st["rho"]
        mol = Y / self.M
        molef = mol / mol.sum()
        numden = AVOGADRO * Y * rho / self.M
        return [self._tau(m["rt"], st["T"], st["p"], molef, numden) if m["kind"] == "LT" else 0.0 for m in self.mechs]

    def _split_rates(self, conc):
        q = np.zeros(self.nsp)
        L = np.zeros(self.nsp)
        for r in self.reactions:
            r.eval_rates(conc)
        for r in self.reactions:   # reaction_mechanism.d:82-95
            for isp in r.participants:
                q[isp] += r.production(isp)
                L[isp] += r.loss(isp)
        return q, L

    def _rates(self, st, taus, y):
        q, L = self._split_rates(y[:self.nsp])
        out = np.empty(self.nsp + 1)
        out[:self.nsp] = q - L
        out[self.nsp] = self._ees_rate(st, taus)
        return out

    def _step(self, st, taus, y0, h):
        """multi_temperature_thermochemical_reactor.d:334-431 (Cash-Karp RKF)."""
        a21, a31, a32 = 1. / 5., 3. / 40., 9. / 40.
        a41, a42, a43 = 3. / 10., -9. / 10., 6. / 5.
        a51, a52, a53, a54 = -11. / 54., 5. / 2., -70. / 27., 35. / 27.
        a61, a62, a63, a64, a65 = 1631. / 55296., 175. / 512., 575. / 13824., 44275. / 110592., 253. / 4096.
        b51, b53, b54, b56 = 37. / 378., 250. / 621., 125. / 594., 512. / 1771.
        b41, b43, b44, b45, b46 = 2825. / 27648., 18575. / 48384., 13525. / 55296., 277. / 14336., 1.0 / 4.0
        k1 = self._rates(st, taus, y0)
        k2 = self._rates(st, taus, y0 + h * a21 * k1)
        k3 = self._rates(st, taus, y0 + h * (a31 * k1 + a32 * k2))
        k4 = self._rates(st, taus, y0 + h * (a41 * k1 + a42 * k2 + a43 * k3))
        k5 = self._rates(st, taus, y0 + h * (a51 * k1 + a52 * k2 + a53 * k3 + a54 * k4))
        k6 = self._rates(st, taus, y0 + h * (a61 * k1 + a62 * k2 + a63 * k3 + a64 * k4 + a65 * k5))
        yOut = y0 + h * (b51 * k1 + b53 * k3 + b54 * k4 + b56 * k6)
        yErr = yOut - (y0 + h * (b41 * k1 + b43 * k3 + b44 * k4 + b45 * k5 + b46 * k6))
        err = 0.0
        for i in range(len(y0)):
            sk = self.tol + self.tol * max(abs(y0[i]), abs(yOut[i]))
            err += (yErr[i] / sk) * (yErr[i] / sk)
        err = math.sqrt(err / len(y0))
        if err <= 1.0:
            scale = 10.0 if err == 0.0 else min(max(0.9 * math.pow(err, -0.2), 0.2), 10.0)
            return True, yOut, scale * h
        return False, yOut, max(0.9 * math.pow(err, -0.2), 0.2) * h

    def estimate_step(self, conc):
        """reaction_mechanism.d:161-203 from the tick rates at conc."""
        q, L = self._split_rates(conc)
        min_dt = 1.0e6
        for i in range(self.nsp):
            if conc[i] > 0.0 and abs(q[i] - L[i]) > 1.0e-30:
                dt = conc[i] / (L[i] + 1.0e-50) if q[i] > 10000.0 * L[i] else abs(conc[i] / (q[i] - L[i]))
                min_dt = min(min_dt, dt)
        dt_chem = min(1.0e-3 * min_dt, 1.0e-10)
        return max(dt_chem, 1.0e-15)

    def update(self, rho, T, Tve, p, massf, t_interval, dt_suggest=-1.0):
        """opCall for one cell (multi_temperature_thermochemical_reactor.d:137-294).  Returns dict(T, Tve,
        p, u, u_ve, massf, dt_suggest, steps) or raises ReactorFailure with the input state left alone."""
        nsp = self.nsp
        Y = np.array(massf, dtype=np.float64)
        st = dict(rho=rho, T=T, Tve=Tve, p=p, massf=Y.copy())
        conc0 = Y * rho / self.M
        conc0 = np.where(conc0 < 1.0e-30, 0.0, conc0)   # gas_model.d:237-256 massf2conc
        u_total = self.gas.e_tr_mix(Y, T) + self.gas.e_ve_mix(Y, Tve)
        self._rate_constants(st)
        taus = self._relaxation_times(st)
        t = 0.0
        if dt_suggest > t_interval:
            h = t_interval
        elif dt_suggest <= 0.0:
            h = self.estimate_step(conc0)
        else:
            h = dt_suggest
        y0 = np.empty(nsp + 1)
        y0[:nsp] = conc0
        y0[nsp] = self.gas.e_ve_mix(Y, Tve)
        dtSave = dt_suggest
        steps = 0
        cycle = 0
        u = u_ve = 0.0
        while cycle < self.max_subcycles:
            self._rate_constants(st)
            taus = self._relaxation_times(st)
            dtSave = dt_suggest
            h = min(h, t_interval - t)
            attempt = 0
            while attempt < self.max_attempts:
                ok, yOut, dt_suggest = self._step(st, taus, y0, h)
                steps += 1
                passed = True
                if ok:
                    c = yOut[:nsp]
                    mf = c * self.M / rho
                    mf = np.where(mf < 1.0e-30, 0.0, mf)   # conc2massf (gas_model.d:258-271)
                    st["massf"] = mf
                    if abs(math.fsum(mf) - 1.0) > ALLOWABLE_MASSF_ERROR:
                        passed = False
                if ok and passed:
                    t += h
                    y0 = yOut.copy()
                    hMax = h * (1.0 + DT_INCREASE_PERCENT / 100.0)
                    if dt_suggest > h:
                        h = min(dt_suggest, hMax)
                    break
                h /= DT_REDUCTION_FACTOR
                if h < H_MIN:
                    raise ReactorFailure(1, "Hit the minimum allowable timestep in 2-T thermochemical update.")
                attempt += 1
            if attempt == self.max_attempts:
                raise ReactorFailure(2, "Hit maxmium number of step attempts within a subcycle.")
            u_ve = y0[nsp]
            u = u_total - u_ve
            try:
                Tn, Tven, pn = self.gas.update_from_rhou(rho, u, u_ve, st["massf"], st["Tve"])
            except ArithmeticError:
                raise ReactorFailure(4, "Failed to update thermodynamic state in multi-T thermochemical update.")
            st["T"], st["Tve"], st["p"] = Tn, Tven, pn
            if t >= t_interval:
                if cycle == 0:
                    dtSave = dt_suggest
                break
            cycle += 1
        if cycle == self.max_subcycles:
            raise ReactorFailure(3, "Hit maximum number of subcycles while attempting 2-T thermochemical update.")
        mf = st["massf"] / math.fsum(st["massf"])
        return dict(T=st["T"], Tve=st["Tve"], p=st["p"], u=u, u_ve=u_ve, massf=mf, dt_suggest=dtSave, steps=steps)


# ---- the compiled restatement (oracle/twotemp_oracle.cpp), for timing the CPU side at compiled speed
_RC_CODE = {"Arrhenius": 0, "fromEqConst": 1, "Park": 6, "Marrone-Treanor": 7, "Modified-Marrone-Treanor": 8}
_RT_CODE = {"MW": 0, "ParkHTC": 1, "ParkHTC2": 2}
_CPL_CODE = {"ImpartialDissociation": 0, "MarroneTreanorDissociation": 1, "ModifiedMarroneTreanorDissociation": 2}


def _rate_vec(rc):
    """model, base model, rctIndex, A, n, C, s, T_D, U, theta, aU, Ustar, non-Boltzmann factor."""
    m = rc["model"]
    v = np.zeros(13)
    v[0], v[1], v[2], v[12] = _RC_CODE[m], 0, -1, 1.0
    base = rc
    if m in ("Marrone-Treanor", "Modified-Marrone-Treanor"):
        base = rc["rate"]
        v[1] = _RC_CODE[base["model"]]
        v[7], v[9] = rc["T_D"], rc["theta"]
        if m == "Marrone-Treanor":
            v[8] = rc["U"]
        else:
            v[10], v[11] = rc["aU"], rc["Ustar"]
            nbc = rc.get("non_boltzmann_correction")
            v[12] = float(nbc["factor"]) if nbc else 1.0
    if base["model"] in ("Arrhenius", "fromEqConst"):
        v[2] = int(base.get("rctIndex", -1))
    if base["model"] in ("Arrhenius", "Park"):
        v[3], v[4], v[5] = base["A"], base["n"], base["C"]
    if base["model"] == "Park":
        v[6] = base["s"]
    return v


class CompiledTwoTemperatureReactor:
    """The same reactor in C++ (oracle/twotemp_oracle.cpp), built from a parsed TwoTemperatureReactor;
    update_cells runs a batch of cells on the host's threads."""

    def __init__(self, r):
        from . import lib, _dp, _ip
        self.r = r
        self.nsp = r.nsp
        M, cp_tr, h_f = (np.ascontiguousarray(x, np.float64) for x in (r.M, r.gas.cp_tr, r.gas.h_f))
        self.h = lib().oracle2t_new(r.gas.curves.h, r.nsp, _dp(M), _dp(cp_tr), _dp(h_f), r.gas.electron,
                                    r.T_lower, r.T_upper, r.tol, r.max_subcycles, r.max_attempts)
        if not self.h:
            raise ValueError("oracle2t_new failed")
        for x in r.reactions:
            ri = np.array([i for i, _ in x.reac], np.int32); rc = np.array([c for _, c in x.reac], np.int32)
            pi = np.array([i for i, _ in x.prod], np.int32); pc = np.array([c for _, c in x.prod], np.int32)
            ei = np.array([i for i, _ in x.eff], np.int32); ev = np.array([e for _, e in x.eff], np.float64)
            fv, bv = _rate_vec(x.frc), _rate_vec(x.brc)
            lib().oracle2t_add_reaction(self.h, int(x.collider), len(ri), _ip(ri), _ip(rc), len(pi), _ip(pi), _ip(pc),
                                        len(ei), _ip(ei), _dp(ev), _dp(fv), _dp(bv))
        for m in r.mechs:
            v = np.zeros(19)
            if m["kind"] == "LT":
                rt = m["rt"]
                v[0], v[1], v[2], v[3] = 0, m["p"], m["q"], _RT_CODE[rt["model"]]
                if rt["model"] == "MW":
                    v[4], v[5] = rt["a"], rt["b"]
                else:
                    v[6], v[7], v[8], v[9] = rt["sigma"], rt["mu"], rt["sub"]["a"], rt["sub"]["b"]
            else:
                v[0], v[1], v[10], v[11] = 1, m["p"], m["r"], _CPL_CODE[m["coupling"]]
                v[13] = m["Thetav"]
                v[12] = m.get("D", 0.0)
                v[14] = m.get("U", 0.0)
                v[15] = m.get("T_D", 0.0)
                v[16], v[17], v[18] = m.get("aU", 0.0), m.get("Ustar", 0.0), m.get("nb", 0.0)
            lib().oracle2t_add_eem(self.h, _dp(v))

    def __del__(self):
        from . import _lib
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle2t_free(self.h)
            self.h = None

    def update_cells(self, rho, T, Tve, p, massf, t_interval, dt_suggest=None, nthreads=0):
        """massf (n, nsp).  Returns dict(T, Tve, p, massf, u, u_ve, dt_suggest, status, steps)."""
        from . import lib, _dp, _ip, _l
        n = len(rho)
        rho = np.ascontiguousarray(rho, np.float64)
        T, Tve, p = (np.array(x, np.float64, copy=True) for x in (T, Tve, p))
        mf = np.array(massf, np.float64, order="C", copy=True).reshape(n, self.nsp)
        dt = np.full(n, -1.0) if dt_suggest is None else np.array(dt_suggest, np.float64, copy=True)
        u, uve = np.zeros(n), np.zeros(n)
        st = np.zeros(n, np.int32)
        steps = np.zeros(n, np.int64)
        lib().oracle2t_update(self.h, n, _dp(rho), _dp(T), _dp(Tve), _dp(p), _dp(mf), t_interval, _dp(dt), _dp(u),
                              _dp(uve), _ip(st), steps.ctypes.data_as(_l), nthreads)
        return dict(T=T, Tve=Tve, p=p, massf=mf, u=u, u_ve=uve, dt_suggest=dt, status=st, steps=steps)
