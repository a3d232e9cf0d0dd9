"""Tight-tolerance FP64 integration of the chemistry ODE (TEST INFRASTRUCTURE ONLY).

The reference's update is an adaptive explicit integration with loose tolerances (RKF
errTol 1e-3, or alpha-QSS eps1 1e-3).  This module integrates the same ODE with scipy's
implicit Radau IIA method at rtol 1e-12, to state how far the reference algorithm -- and the
GPU engine that reproduces it -- are from the exact solution, per workload.

The ODE is the one the reference approximates (kinetics/chemistry_update.d:139-326):
  * without tight temperature coupling: dc/dt = q(c) - L(c) with the rate constants frozen at
    the initial (clamped) temperature (chemistry_update.d:148);
  * with tight coupling: the rate constants follow T(rho, u, Y(c)) continuously, where the
    reference re-evaluates them once per subcycle (chemistry_update.d:265-269).
Rates and rate constants come from the oracle (oracle/chem_oracle.cpp).
"""
import numpy as np
from scipy.integrate import solve_ivp


def integrate_cell(orc, rho, u, T0, massf, t_end, rtol=1e-12, tight=None):
    """Returns (massf_final renormalised, T_final) for one cell."""
    M = orc.M
    c0 = massf * rho / M
    c0 = np.where(c0 < 1e-30, 0.0, c0)
    if tight is None:
        tight = bool(orc.config and orc.config.get('tightTempCoupling'))
    state = {"T": T0}

    def temperature(c):
        mf = np.maximum(c, 0.0) * M / rho
        T, _, st = orc.update_thermo_from_rhou([rho], [u], mf[None, :], [state["T"]])
        if st[0] == 0:
            state["T"] = T[0]
        return state["T"]

    def rhs(t, c):
        T = temperature(c) if tight else T0
        q, L, _, _ = orc.split_rates(T, np.maximum(c, 0.0))
        return q - L

    scale = max(c0.max(), 1e-30)
    sol = solve_ivp(rhs, (0.0, t_end), c0, method="Radau", rtol=rtol, atol=1e-14 * scale, dense_output=False)
    if not sol.success:
        raise RuntimeError(sol.message)
    c = np.maximum(sol.y[:, -1], 0.0)
    mf = c * M / rho
    mf = np.where(mf < 1e-30, 0.0, mf)
    mf = mf / mf.sum()
    T, _, st = orc.update_thermo_from_rhou([rho], [u], mf[None, :], [state["T"] if tight else T0])
    return mf, T[0]


def errors_vs_tight(orc, rho, u, T0, massf, massf_out, T_out, t_end, rtol=1e-12):
    """max |dY| and max relative dT of (massf_out, T_out) against the tight integration.

    massf is (n, nsp); returns (max_abs_dY, max_rel_dT, per-cell arrays)."""
    n = len(rho)
    dY = np.zeros(n)
    dT = np.zeros(n)
    for k in range(n):
        mf, T = integrate_cell(orc, rho[k], u[k], T0[k], massf[k], t_end, rtol=rtol)
        dY[k] = np.abs(massf_out[k] - mf).max()
        dT[k] = abs(T_out[k] - T) / T
    return float(dY.max()), float(dT.max()), dY, dT
