"""Pins the CPU oracle against every known-answer test the reference holds for this path.

Each expected value and tolerance below is the reference's own assertion (file:line in
the gdtk source tree).  The oracle must reproduce all of them before it is trusted as
the checker for the CUDA kernels.
"""
import math
import os

import numpy as np
import pytest

import oracle
from conftest import mech, GOLDEN

R_universal = 8.31451


def close(a, b, rel):
    return math.isclose(a, b, rel_tol=rel)


def approx_equal_numbers(a, b, tol):
    # nm/number.d approxEqualNumbers: relative test with the same tolerance as absolute floor
    return abs(a - b) <= tol * max(abs(a), abs(b)) or abs(a - b) <= tol


@pytest.fixture(scope="module")
def o_thermo(tmp_path_factory):
    # cea_thermo_curves.d:194-199: a single curve for O with R = 8.31451/0.0159994.
    from oracle.luatable import read_lua_file, array
    t = read_lua_file(mech("O-thermo.lua"))['CEA_coeffs']
    d = tmp_path_factory.mktemp("othermo")
    body = ["species = {'O', }", "db = {}", "db['O'] = {}", "db['O'].M = 0.0159994", "db['O'].thermoCoeffs = {",
            "  nsegments = %d," % t['nsegments'],
            "  T_break_points = {%s}," % ", ".join(repr(x) for x in array(t['T_break_points'])),
            "  T_blend_ranges = {%s}," % ", ".join(repr(x) for x in array(t['T_blend_ranges']))]
    for s in range(t['nsegments']):
        body.append("  segment%d = {%s}," % (s, ", ".join(repr(x) for x in array(t['segment%d' % s]))))
    body.append("}")
    path = d / "O-gas.lua"
    path.write_text("\n".join(body) + "\n")
    return oracle.Oracle(str(path))


def test_cea_curve_oxygen(o_thermo):
    # cea_thermo_curves.d:201-206
    cp, _, _ = o_thermo.species_thermo(0, 500.0)
    assert close(1328.627, cp, 1.0e-6)
    _, h, _ = o_thermo.species_thermo(0, 3700.0)
    assert close(20_030_794.683, h, 1.0e-6)
    _, _, s = o_thermo.species_thermo(0, 10_000.0)
    assert close(14_772.717, s, 1.0e-3)


def test_thermally_perfect_air5():
    # therm_perf_gas_mix.d:491-504 (and composite_gas.d:281-288)
    o = oracle.Oracle(mech("tpg-air5-gas.lua"))
    mf = np.full((1, 5), 0.2)
    rho, u = o.update_thermo_from_pT([1.0e6], [2000.0], mf)
    assert approx_equal_numbers(11801825.6, u[0], 1.0e-6)
    assert approx_equal_numbers(1.2840117, rho[0], 1.0e-6)
    T, p, st = o.update_thermo_from_rhou([2.0], [14.0e6], mf, [2000.0])
    assert st[0] == 0
    assert approx_equal_numbers(3373757.4, p[0], 1.0e-6)
    assert approx_equal_numbers(4331.944, T[0], 1.0e-6)
    # updateFromRhoT (therm_perf_gas_mix.d:506-510): p = rho R T and u(T)
    rho2, u2 = o.update_thermo_from_pT([5841068.3], [10000.0], mf)
    assert approx_equal_numbers(1.5, rho2[0], 1.0e-6)
    assert approx_equal_numbers(20340105.9, u2[0], 1.0e-6)


def test_arrhenius_rate_constants(tmp_path):
    # rate_constant.d:604-617.  Test 2 reads sample-input/N2-diss.lua.
    from oracle.luatable import read_lua_file
    r = read_lua_file(mech("n2-diss-rate.lua"))['rate']
    A, n, C = r['A'], r['n'], r['C']
    chem = tmp_path / "chem.lua"
    chem.write_text(
        "species = {[0]='H2', [1]='I2', [2]='HI', }\n"
        "config = {maxSubcycles=50, maxAttempts=2, tightTempCoupling=false,\n"
        "  tempLimits={lower=100.0, upper=1.0e5}, odeStep={method='rkf', errTol=1.0e-3}}\n"
        "reaction = {}\n"
        "reaction[1] = {type='elementary', frc={model='Arrhenius', A=%r, n=0.0, C=20620.0},\n"
        "  brc={model='Arrhenius', A=%r, n=%r, C=%r}, reacIdx={0,1}, reacCoeffs={1,1}, prodIdx={2}, prodCoeffs={2}}\n"
        % (1.94e14 * 1e-6, A, n, C))
    o = oracle.Oracle(mech("h2i2-gas.lua"), str(chem))
    kf, _ = o.rate_constants(700.0)
    assert close(3.10850956e-5, kf[0], 1.0e-2)
    _, kb = o.rate_constants(4000.0)
    assert close(0.00159439, kb[0], 1.0e-5)


def test_reaction_mechanism_rates():
    # reaction_mechanism.d:264-283 and reaction.d:538-556
    o = oracle.Oracle(mech("h2i2-gas.lua"), os.path.join(GOLDEN, "inputs", "h2i2-kat-chem.lua"))
    q, L, wf, wb = o.split_rates(700.0, np.array([4.54, 4.54, 0.0]))
    rates = q - L
    for got, want in zip(rates, [-643.9303, -643.9303, 1287.8606]):
        assert close(want, got, 1.0e-6)
    # production(2) = 2 w_f, loss(0) = loss(1) = w_f, production(0) = loss(2) = 0 (w_b = 0)
    assert close(1287.8606, q[2], 1.0e-6) and close(643.9303, L[0], 1.0e-6) and close(643.9303, L[1], 1.0e-6)
    assert q[0] == 0.0 and q[1] == 0.0 and L[2] == 0.0


@pytest.fixture(scope="module")
def h2i2():
    return oracle.Oracle(mech("h2i2-gas.lua"), mech("h2i2-chem.lua"))


def test_rkf_order(h2i2):
    # chemistry_update.d:695-713: error ratio 1.96809 when dt shrinks by 2^(-1/5)
    analytical = 7.1420197868416215
    c0 = 4.54
    y0, _ = h2i2.integrate_fixed('rkf', 700.0, [c0, c0, 0.0], 287.175, 60_000.0)
    y1, _ = h2i2.integrate_fixed('rkf', 700.0, [c0, c0, 0.0], 287.175 * 2.0 ** (-1.0 / 5.0), 60_000.0)
    assert close(1.96809, (analytical - y0[2]) / (analytical - y1[2]), 1.0e-4)


def test_alpha_qss_order(h2i2):
    # chemistry_update.d:715-734 (the reference constructs the step with eps1 1e-3, eps2 5e-4,
    # delta 1e-10, maxIters 10, the defaults this oracle uses for alpha-qss)
    analytical = 7.1420197868416215
    c0 = 4.54
    y0, _ = h2i2.integrate_fixed('alpha-qss', 700.0, [c0, c0, 0.0], 2.0, 60_000.0)
    y1, _ = h2i2.integrate_fixed('alpha-qss', 700.0, [c0, c0, 0.0], 1.0, 60_000.0)
    assert close(7.1420197868416215, y1[2], 1.0e-4)
    assert close(4.001, (analytical - y0[2]) / (analytical - y1[2]), 1.0e-4)


def test_full_chemistry_update(h2i2):
    # chemistry_update.d:736-750: the complete update over 60,000 s from dtSuggest = 200
    T = 700.0
    c0 = 4.54
    p = 2.0 * c0 * R_universal * T
    M = h2i2.M
    molef = np.array([0.5, 0.5, 0.0])
    mix = float(np.dot(molef, M))
    massf = molef * M / mix
    rho, u = h2i2.update_thermo_from_pT([p], [T], massf[None, :])
    out = h2i2.chem_update(rho, u, [T], [p], massf[None, :], [200.0], 60_000.0,
                           update_thermo=False, retry=False)
    assert out['status'][0] == 0
    conc = out['massf'][0] * rho[0] / M
    assert close(7.14201983840, conc[2], 1.0e-9)


def test_fixed_volume_reactor_n2():
    # examples/kinetics/fixed-volume-reactor-n2/test_fvreactor.py:30-55: N2/N with backward
    # rates from K_c, 300 us in 1 us updates, each followed by update_thermo_from_rhou.
    o = oracle.Oracle(mech("n2-gas.lua"), mech("n2-chem.lua"))
    M = o.M
    molef = np.array([2 / 3, 1 / 3])
    massf = molef * M / float(np.dot(molef, M))
    p, T = 1.0e5, 4000.0
    rho, u = o.update_thermo_from_pT([p], [T], massf[None, :])
    state = dict(T=np.array([T]), p=np.array([p]), massf=massf[None, :])
    t, dt, dt_suggest, t_final = 0.0, 1.0e-6, 1.0e-11, 300.0e-6
    while t <= t_final:
        out = o.chem_update(rho, u, state['T'], state['p'], state['massf'], [dt_suggest], dt, retry=False)
        assert out['status'][0] == 0
        state = out
        dt_suggest = out['dt_chem'][0]
        t = t + dt
    assert close(t, t_final, 1.0e-6)
    assert close(state['T'][0], 6177.3, 1.0e-4)
    assert close(state['p'][0], 145.518e3, 1.0e-4)
    assert close(state['massf'][0][0], 8.692812671003e-01, 1.0e-4)
    assert close(state['massf'][0][1], 1.307187328997e-01, 1.0e-4)
    conc = state['massf'][0] * rho[0] / M
    assert close(conc[0], 2.178123112237e+00, 1.0e-4)
    assert close(conc[1], 6.550733441684e-01, 1.0e-4)


def drm19_fixed_volume_reactor(update, nsteps=1999):
    """The DRM19 example's fixed-volume reactor (examples/kinetics/methane-combustion-w-drm19/
    fixed-volume-reactor.lua): CH4:O2:N2 = 1:2:7.52 by mole at 2000 K and 1 atm, nsteps updates of
    2e-7 s with dt_chem carried, each followed by update_thermo_from_rhou.  `update(rho, u, T, p, Y,
    dt_chem, dt)` -> (T, p, Y, dt_chem).  Returns the temperature history."""
    orc = oracle.Oracle(mech("drm19-gas.lua"), mech("drm19-chem.lua"))
    names = orc.names
    X = np.zeros(len(names))
    total = 1 + 2 + 7.52
    X[names.index('CH4')], X[names.index('O2')], X[names.index('N2')] = 1 / total, 2 / total, 7.52 / total
    Y = X * orc.M / (X * orc.M).sum()
    T, p = np.array([2000.0]), np.array([101.325e3])
    rho, u = orc.update_thermo_from_pT(p, T, Y[None, :])
    dtc = np.array([-1.0])
    Ts = [T[0]]
    for _ in range(nsteps):
        T, p, Y, dtc = update(rho, u, T, p, Y, dtc, 4.0e-4 / 2000)
        Ts.append(T[0])
    return np.array(Ts)


def compare_with_eilmer3(Ts):
    ref = np.loadtxt(os.path.join(GOLDEN, "drm19-fvr-eilmer3-T.txt"))
    rel = np.abs(Ts - ref[:, 1]) / ref[:, 1]
    t_ign = ref[np.argmax(np.diff(Ts)), 0]
    t_ign_ref = ref[np.argmax(np.diff(ref[:, 1])), 0]
    return rel, t_ign, t_ign_ref


def test_troe_falloff_fixed_volume_reactor_against_eilmer3():
    """Pins the pressure-dependent (Troe) rate constants: the DRM19 methane reactor against the
    example's Eilmer3 result (the reference's plot comparison).  The ignition time agrees to 1%
    and the temperature history to 3% at the steepest point and 0.2% at the end; with Lindemann
    blending (F = 1) in place of Troe's, ignition moves 8% earlier and T differs by 25%."""
    orc = oracle.Oracle(mech("drm19-gas.lua"), mech("drm19-chem.lua"))

    def update(rho, u, T, p, Y, dtc, dt):
        o = orc.chem_update(rho, u, T, p, Y[None, :], dtc, dt)
        assert o["status"][0] == 0
        return o["T"], o["p"], o["massf"][0], o["dt_chem"]

    Ts = drm19_fixed_volume_reactor(update)
    rel, t_ign, t_ign_ref = compare_with_eilmer3(Ts)
    assert abs(t_ign - t_ign_ref) <= 0.01 * t_ign_ref
    assert rel.max() < 0.03
    assert rel[-1] < 2e-3


def test_two_temperature_air5():
    """gas/thermo/two_temperature_gas.d:704-738: five-species air, Y = 0.2 each, at p = 1 MPa and
    T = T_ve = 2000 K has u + u_ve = 11,801,825.6 J/kg and rho = 1.2840117 kg/m^3; the (rho, u)
    update returns T, T_ve and p (all to 1e-6).  Groundwork of the multi-temperature reactor."""
    from oracle.two_temperature import TwoTemperatureGas
    g = TwoTemperatureGas(mech("air5-2T-gas.lua"))
    Y = np.full(5, 0.2)
    rho, u, u_ve = g.update_from_pT(1.0e6, 2000.0, 2000.0, Y)
    assert u + u_ve == pytest.approx(11_801_825.6, rel=1e-6)
    assert rho == pytest.approx(1.2840117, rel=1e-6)
    for guess in (2000.0, 1500.0):
        T, T_ve, p = g.update_from_rhou(rho, u, u_ve, Y, guess)
        assert T == pytest.approx(2000.0, rel=1e-6)
        assert T_ve == pytest.approx(2000.0, rel=1e-6)
        assert p == pytest.approx(1.0e6, rel=1e-6)


def test_arrhenius2_and_falloff_forms_restated():
    """The oracle's Arrhenius2 (rate_constant.d:112-115), Lindemann-Hinshelwood (155-160) and
    Yungster-Rabinowitz (338-350) forward rate constants, from the formulas with the fixture's
    parameters as prep_chem wrote them."""
    from oracle.luatable import read_lua_file
    o = oracle.Oracle(mech("h2o2forms-gas.lua"), mech("h2o2forms-chem.lua"))
    rx = read_lua_file(mech("h2o2forms-chem.lua"))["reaction"]
    T = 1700.0
    conc = np.linspace(0.5, 6.5, o.nsp)            # mol/m^3, any positive state
    kf, kb = o.rate_constants(T, conc)
    for k in (1, 2, 8):                            # r1, r2, r11: Arrhenius2
        f = rx[k]["frc"]
        assert f["model"] == "Arrhenius2"
        assert close(np.exp(f["logA"] + f["B"] * T - f["C"] / T), kf[k - 1], 1e-14)

    def arr(d):
        return d["A"] * T ** d["n"] * np.exp(-d["C"] / T)

    def third_body(r):
        eff = r["efficiencies"]
        return sum(eff[i] * conc[i] for i in eff)

    lh, yr = rx[10], rx[11]
    assert lh["frc"]["model"] == "Lindemann-Hinshelwood" and yr["frc"]["model"] == "Yungster-Rabinowitz"
    kinf, k0, M = arr(lh["frc"]["kInf"]), arr(lh["frc"]["k0"]), third_body(lh)
    assert close(k0 * kinf * M / (k0 * M + kinf), kf[9], 1e-13)
    f = yr["frc"]
    kinf, k0, M = arr(f["kInf"]), arr(f["k0"]), third_body(yr)
    pr = k0 * M / kinf
    fc = f["a"] * np.exp(-f["b"] / T) + (1.0 - f["a"]) * np.exp(-f["c"] / T)
    assert close(kinf * (pr / (1.0 + pr)) * fc / (1.0 + np.log(pr) ** 2), kf[10], 1e-13)


@pytest.mark.parametrize("chem,eem", [("park2t-chem.lua", "park2t-eem.lua"), ("park2tmt-chem.lua", "park2tmt-eem.lua")],
                         ids=["impartial", "marrone-treanor"])
def test_two_temperature_reactor_against_a_tight_integration(chem, eem):
    """The two-temperature reactor restatement (oracle/two_temperature_reactor.py) on Park 2-T air
    against a Radau integration (rtol 1e-9) of the same system with every rate at the instantaneous
    state.  The reference algorithm freezes the rate constants and the exchange terms over each RKF
    step (errTol 1e-3), so it agrees to that order only; total energy is conserved exactly."""
    from scipy.integrate import solve_ivp
    from oracle.two_temperature_reactor import TwoTemperatureReactor
    r = TwoTemperatureReactor(mech("park2t-gas.lua"), mech(chem), mech(eem))
    rng = np.random.default_rng(0)
    for _ in range(4):
        T, p = rng.uniform(4000.0, 12000.0), 10.0 ** rng.uniform(3.0, 4.5)
        Tve = rng.uniform(500.0, 1.2 * T)
        Y = rng.dirichlet([2.0, 1.0, 0.3, 0.3, 0.3])
        rho, u, uve = r.gas.update_from_pT(p, T, Tve, Y)
        o = r.update(rho, T, Tve, p, Y, 1.0e-6)
        assert close(o["u"] + o["u_ve"], u + uve, 1e-12)
        c0 = Y * rho / r.M
        guess = {"Tve": Tve}

        def rhs(t, y):
            c = np.maximum(y[:r.nsp], 0.0)
            Ym = c * r.M / rho
            Tn, Tven, pn = r.gas.update_from_rhou(rho, u + uve - y[r.nsp], y[r.nsp], Ym, guess["Tve"])
            guess["Tve"] = Tven
            st = dict(rho=rho, T=Tn, Tve=Tven, p=pn, massf=Ym)
            r._rate_constants(st)
            return r._rates(st, r._relaxation_times(st), np.concatenate([c, [y[r.nsp]]]))

        sol = solve_ivp(rhs, (0.0, 1.0e-6), np.concatenate([c0, [uve]]), method="Radau", rtol=1e-9,
                        atol=np.concatenate([np.full(r.nsp, 1e-14 * c0.max()), [1e-6]]))
        y = sol.y[:, -1]
        Yt = np.maximum(y[:r.nsp], 0.0) * r.M / rho
        Yt /= Yt.sum()
        Tt, Tvt, _ = r.gas.update_from_rhou(rho, u + uve - y[r.nsp], y[r.nsp], Yt, guess["Tve"])
        assert abs(o["T"] - Tt) / Tt < 1.5e-2 and abs(o["Tve"] - Tvt) / Tvt < 1.5e-2
        assert np.abs(o["massf"] - Yt).max() < 5e-3


def test_marrone_treanor_forms_at_thermal_equilibrium():
    """At T_ve = T the Marrone-Treanor factor of rate_constant.d:438-447 is 1 and the modified form's
    (:541-554) is its non-Boltzmann factor; the Marrone-Treanor coupling's G_vanish equals its G_appear,
    and the modified coupling's exceeds it by non_boltzmann R T_D (exchange_chemistry_coupling.d:152-220).
    The parameters are those prep_chem / prep_kinetics wrote (T_D from the species' heats of formation,
    U from T_D / U = 3)."""
    from oracle.two_temperature_reactor import TwoTemperatureReactor, Reaction
    from oracle.two_temperature import R_UNIVERSAL
    r = TwoTemperatureReactor(mech("park2t-gas.lua"), mech("park2tmt-chem.lua"), mech("park2tmt-eem.lua"))
    mt, mmt = r.reactions[0].frc, r.reactions[1].frc
    assert mt["model"] == "Marrone-Treanor" and mmt["model"] == "Modified-Marrone-Treanor"
    assert close(mt["U"], mt["T_D"] / 3.0, 1e-9)
    for T in (3000.0, 7000.0, 12000.0):
        assert close(Reaction.rate_constant(mt, T, [T]), Reaction.rate_constant(mt["rate"], T, [T]), 1e-12)
        assert close(Reaction.rate_constant(mmt, T, [T]), 0.9 * Reaction.rate_constant(mmt["rate"], T, [T]), 1e-12)
        # out of equilibrium the factors move the rate (cold vibration slows dissociation)
        assert Reaction.rate_constant(mt, T, [0.5 * T]) < Reaction.rate_constant(mt["rate"], T, [0.5 * T])
    kinds = {m["coupling"]: m for m in r.mechs if m["kind"] == "MT"}
    assert set(kinds) == {"ImpartialDissociation", "MarroneTreanorDissociation", "ModifiedMarroneTreanorDissociation"}
    for T in (3000.0, 9000.0):
        ga, gv = r._coupling(kinds["MarroneTreanorDissociation"], T, T)
        assert close(gv, ga, 1e-9)
        m = kinds["ModifiedMarroneTreanorDissociation"]
        ga, gv = r._coupling(m, T, T)
        assert close(gv - ga, m["nb"] * R_UNIVERSAL * m["T_D"], 1e-9)


@pytest.mark.parametrize("chem,eem", [("park2t-chem.lua", "park2t-eem.lua"), ("park2tmt-chem.lua", "park2tmt-eem.lua")],
                         ids=["impartial", "marrone-treanor"])
def test_compiled_two_temperature_reactor_equals_the_restatement(chem, eem):
    """oracle/twotemp_oracle.cpp (the two-temperature workload's CPU timing reference) against the
    Python restatement it transcribes: same status and RKF attempts per cell, T and T_ve to 1e-14,
    mass fractions to 1e-15 (only the final normalising sum is taken differently)."""
    from oracle.two_temperature_reactor import TwoTemperatureReactor, CompiledTwoTemperatureReactor, ReactorFailure
    from gdtk_gb300.workloads import air2t_cells
    r = TwoTemperatureReactor(mech("park2t-gas.lua"), mech(chem), mech(eem))
    c = CompiledTwoTemperatureReactor(r)
    n = 24
    T, Tve, p, Y = air2t_cells(n, seed=13)
    rho = np.array([r.gas.update_from_pT(p[k], T[k], Tve[k], Y[:, k])[0] for k in range(n)])
    o = c.update_cells(rho, T, Tve, p, Y.T, 1e-6, nthreads=2)
    for k in range(n):
        try:
            py = r.update(rho[k], T[k], Tve[k], p[k], Y[:, k], 1e-6)
        except ReactorFailure as f:
            assert o["status"][k] == f.code
            continue
        assert o["status"][k] == 0 and o["steps"][k] == py["steps"]
        assert close(o["T"][k], py["T"], 1e-14) and close(o["Tve"][k], py["Tve"], 1e-14)
        assert np.abs(o["massf"][k] - py["massf"]).max() <= 1e-15
        assert close(o["u_ve"][k], py["u_ve"], 1e-13) and close(o["dt_suggest"][k], py["dt_suggest"], 1e-14)
