"""CPU restatement of the reference's two-temperature gas thermo (TEST INFRASTRUCTURE ONLY).

Follows gas/thermo/two_temperature_gas.d (TwoTemperatureGasMixture): translation and rotation at T
with fully excited heat capacities, vibration and electronic excitation at T_ve, taken as the NASA-9
(CEA) enthalpy at T_ve less the translational-rotational part.  This module is the groundwork of the
multi-temperature reactor, which the GPU engine does not implement yet; it is pinned to the
reference's known-answer test (two_temperature_gas.d:704-738) by tests/test_oracle_kat.py.  The CEA
curves are the oracle's own (oracle/chem_oracle.cpp, pinned to cea_thermo_curves.d).
"""
import numpy as np

from . import Oracle
from .luatable import read_lua_file

R_UNIVERSAL = 8.31451   # gas/physical_constants.d:13
T_REF = 298.15          # two_temperature_gas.d:26


def _array(t):
    return [t[k] for k in sorted(t)] if isinstance(t, dict) else list(t)


class TwoTemperatureGas:
    """Per-species constants of two_temperature_gas.d:45-80 and the state updates of :84-124."""

    def __init__(self, gas_file):
        self.curves = Oracle(gas_file)
        g = read_lua_file(gas_file)
        self.names = _array(g["species"])
        self.nsp = len(self.names)
        self.M = np.array([float(g["db"][n]["M"]) for n in self.names])
        self.R = R_UNIVERSAL / self.M
        self.electron = -1
        cp_tr = []
        for i, n in enumerate(self.names):
            e = g["db"][n]
            kind = e.get("type")
            if n == "e-":
                self.electron = i
            if kind == "electron":
                cp_tr.append(0.0)
            elif kind == "atom":
                cp_tr.append(2.5 * self.R[i])
            elif kind == "molecule":
                cp_tr.append((3.5 if e.get("molecule_type") == "linear" else 4.0) * self.R[i])
            else:
                raise ValueError("TwoTemperatureGas: unknown particle type %r for %s" % (kind, n))
        self.cp_tr = np.array(cp_tr)
        self.h_f = np.array([self._h(i, T_REF) for i in range(self.nsp)])

    def _h(self, i, T):
        return self.curves.species_thermo(i, T)[1]

    def _cp(self, i, T):
        return self.curves.species_thermo(i, T)[0]

    # ---- per species (two_temperature_gas.d:427-445, 538-545, 558-590)
    def e_tr(self, i, T):
        if i == self.electron:
            return 0.0
        return self.cp_tr[i] * (T - T_REF) + self.h_f[i] - self.R[i] * T

    def e_ve(self, i, Tve):
        if i == self.electron:
            return 1.5 * self.R[i] * Tve
        return self._h(i, Tve) - self.cp_tr[i] * (Tve - T_REF) - self.h_f[i]

    def cv_ve(self, i, Tve):
        if i == self.electron:
            return 1.5 * self.R[i]
        return self._cp(i, Tve) - self.cp_tr[i]

    # ---- mixtures
    def e_tr_mix(self, Y, T):
        return sum(Y[i] * self.e_tr(i, T) for i in range(self.nsp) if i != self.electron)

    def e_ve_mix(self, Y, Tve):
        return sum(Y[i] * self.e_ve(i, Tve) for i in range(self.nsp))

    def cv_ve_mix(self, Y, Tve):
        return sum(Y[i] * self.cv_ve(i, Tve) for i in range(self.nsp))

    # ---- state updates (two_temperature_gas.d:84-124, 497-520, 656-700)
    def update_from_pT(self, p, T, Tve, Y):
        """(rho, u, u_ve) of a state given p, T, T_ve and mass fractions Y."""
        denom = sum(Y[i] * self.R[i] * (Tve if i == self.electron else T) for i in range(self.nsp))
        rho = p / denom
        return rho, self.e_tr_mix(Y, T), self.e_ve_mix(Y, Tve)

    def update_from_rhou(self, rho, u, u_ve, Y, Tve_guess):
        """(T, T_ve, p): T by direct inversion of the fully excited translation-rotation energy, T_ve by
        the reference's Newton iteration from Tve_guess (40 iterations at most, |dT| < 1e-9 K, or the
        guess itself when its energy is within 1e-5 J/kg)."""
        sumA = sum(Y[i] * (self.cp_tr[i] * T_REF - self.h_f[i]) for i in range(self.nsp) if i != self.electron)
        sumB = sum(Y[i] * (self.cp_tr[i] - self.R[i]) for i in range(self.nsp) if i != self.electron)
        T = (u + sumA) / sumB
        Tve = Tve_guess
        f = self.e_ve_mix(Y, Tve) - u_ve
        if abs(f) >= 1e-5:
            count, dT = 0, 0.0
            for _ in range(40):
                dT = -f / self.cv_ve_mix(Y, Tve)
                Tve += dT
                if abs(dT) < 1.0e-9:
                    break
                f = self.e_ve_mix(Y, Tve) - u_ve
                count += 1
            if count == 40 and abs(dT) > 1e-3:
                raise ArithmeticError("vibElecTemperature failed to converge")
        p = sum(rho * Y[i] * self.R[i] * (Tve if i == self.electron else T) for i in range(self.nsp))
        return T, Tve, p
