"""CPU oracle for the chemistry update (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package, and only as the checker or as the timed CPU baseline; the product path in
gdtk_gb300/ never calls it.  `Oracle` loads a gas-model file and a mechanism file
written by gdtk's prep-gas / prep-chem (read here by oracle/luatable.py), and drives
the C++ restatement in oracle/chem_oracle.cpp through ctypes.
"""
import ctypes
import os
import subprocess

import numpy as np

from .luatable import read_lua_file, array

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_l = ctypes.POINTER(ctypes.c_long)
_lib = None

# Status codes shared with the product (include/gdtk_chem.h).
ST_OK, ST_H_MIN, ST_MAX_ATTEMPTS, ST_MAX_SUBCYCLES, ST_NEWTON_FAIL, ST_BAD_INPUT, ST_FROZEN = range(7)


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_model_new.restype = ctypes.c_void_p
        L.oracle_model_new.argtypes = [ctypes.c_int]
        L.oracle_model_free.argtypes = [ctypes.c_void_p]
        L.oracle_set_species.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, _d, _d, _d]
        L.oracle_add_reaction.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, _i, _i, ctypes.c_int, _i, _i, ctypes.c_int, _i, _d]
        L.oracle_set_config.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_n_reactions.argtypes = [ctypes.c_void_p]
        L.oracle_species_thermo.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, _d, _d, _d]
        L.oracle_rate_constants.argtypes = [ctypes.c_void_p, ctypes.c_double, _d, _d, _d]
        L.oracle_set_pressure_dependent.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_double] * 8 + \
            [ctypes.c_int]
        L.oracle_split_rates.argtypes = [ctypes.c_void_p, ctypes.c_double, _d, _d, _d, _d, _d]
        L.oracle_estimate_step.restype = ctypes.c_double
        L.oracle_estimate_step.argtypes = [ctypes.c_void_p, ctypes.c_double, _d]
        L.oracle_ode_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, _d, ctypes.c_double, _d, _d]
        L.oracle_update_thermo_from_pT.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d, _d, _d, _d]
        L.oracle_update_thermo_from_rhou.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d, _d, _d, _d, _i]
        L.oracle_chem_update.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d, _d, _d, _d, _d, _i,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _l]
        L.oracle_integrate_fixed.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, _d, ctypes.c_double, ctypes.c_double]
        L.oracle_max_threads.restype = ctypes.c_int
        # the compiled two-temperature reactor (twotemp_oracle.cpp; see two_temperature_reactor.compiled)
        L.oracle2t_new.restype = ctypes.c_void_p
        L.oracle2t_new.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d, _d, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.oracle2t_free.argtypes = [ctypes.c_void_p]
        L.oracle2t_add_reaction.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _i, _i, ctypes.c_int, _i, _i,
                                            ctypes.c_int, _i, _d, _d, _d]
        L.oracle2t_add_eem.argtypes = [ctypes.c_void_p, _d]
        L.oracle2t_update.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d, _d, _d, _d, ctypes.c_double, _d, _d, _d,
                                      _i, _l, ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_d)


def _ip(a):
    return a.ctypes.data_as(_i)


def load_gas(path):
    """(species names, molar masses, CEA curves) from a prep-gas file (composite_gas.d:45-71)."""
    g = read_lua_file(path)
    names = array(g['species'])
    species = []
    for name in names:
        entry = g['db'][name]
        th = entry['thermoCoeffs']
        nseg = th['nsegments']
        species.append(dict(name=name, M=float(entry['M']), nseg=nseg,
                            breaks=np.array(array(th['T_break_points']), dtype=np.float64),
                            blends=np.array(array(th['T_blend_ranges']), dtype=np.float64),
                            coeffs=np.array([array(th['segment%d' % s]) for s in range(nseg)], dtype=np.float64)))
    return names, species


def load_mechanism(path, names):
    """Reactions and the `config` table of a prep-chem file (chemistry_update.d:42-137)."""
    c = read_lua_file(path)
    sp = array(c['species'])
    if sp != names:
        raise ValueError("species order differs between gas model and mechanism: %s vs %s" % (names, sp))
    reactions = []
    for k in sorted(c['reaction']):
        r = c['reaction'][k]
        eff = r.get('efficiencies') or {}
        # Lua's next() visits the integer keys 0..n-1 of these constructors in ascending order.
        keys = sorted(eff)
        reactions.append(dict(
            collider=(r['type'] == 'anonymous_collider'),
            frc=r['frc'], brc=r['brc'],
            reac=list(zip(array(r['reacIdx']), array(r['reacCoeffs']))),
            prod=list(zip(array(r['prodIdx']), array(r['prodCoeffs']))),
            eff=[(int(i), float(eff[i])) for i in keys]))
    return reactions, c['config']


class Oracle:
    """The reference algorithm on the CPU, for one gas model + mechanism pair."""

    def __init__(self, gas_file, chem_file=None, T_limits=None):
        L = lib()
        self.names, self.species = load_gas(gas_file)
        self.nsp = len(self.names)
        self.M = np.array([s['M'] for s in self.species])
        self.h = L.oracle_model_new(self.nsp)
        if not self.h:
            raise ValueError("the oracle takes 1..128 species")
        for isp, s in enumerate(self.species):
            rc = L.oracle_set_species(self.h, isp, s['M'], s['nseg'], _dp(s['breaks']), _dp(s['blends']),
                                      _dp(np.ascontiguousarray(s['coeffs'].ravel())))
            if rc != 0:
                raise ValueError("bad thermo curve for %s" % s['name'])
        self.config = None
        if chem_file is not None:
            reactions, cfg = load_mechanism(chem_file, self.names)
            pd_models = {'Lindemann-Hinshelwood': 2, 'Troe': 3, 'Yungster-Rabinowitz': 4}
            for r in reactions:
                def rcm(d):
                    if d['model'] == 'Arrhenius':
                        return 0, float(d['A']), float(d['n']), float(d['C'])
                    if d['model'] == 'fromEqConst':
                        return 1, 0.0, 0.0, 0.0
                    if d['model'] in ('Arrhenius2', 'Arrhenius-logA'):   # rate_constant.d:82-121
                        return 5, float(d['logA']), float(d['B']), float(d['C'])
                    if d['model'] in pd_models:   # k_inf here, k_0 and the blending below
                        k = d['kInf']
                        return pd_models[d['model']], float(k['A']), float(k['n']), float(k['C'])
                    raise ValueError("rate-constant model %s is outside this path" % d['model'])
                fm, fA, fn, fC = rcm(r['frc'])
                bm, bA, bn, bC = rcm(r['brc'])
                ri = np.array([i for i, _ in r['reac']], np.int32); rcf = np.array([k for _, k in r['reac']], np.int32)
                pi = np.array([i for i, _ in r['prod']], np.int32); pcf = np.array([k for _, k in r['prod']], np.int32)
                ei = np.array([i for i, _ in r['eff']], np.int32); ev = np.array([v for _, v in r['eff']], np.float64)
                ir = L.oracle_add_reaction(self.h, int(r['collider']), fm, fA, fn, fC, bm, bA, bn, bC,
                                           len(ri), _ip(ri), _ip(rcf), len(pi), _ip(pi), _ip(pcf), len(ei), _ip(ei),
                                           _dp(ev))
                if ir < 0:
                    raise ValueError("the oracle takes up to 1024 reactions")
                if fm in pd_models.values():   # rate_constant.d:135-145, 181-229, 310-333
                    d = r['frc']
                    k0 = d['k0']
                    flags = 0
                    Fc = a = T1 = T2 = T3 = 0.0
                    if fm == 3:
                        if d.get('F_cent') is not None:
                            flags, Fc = 1, float(d['F_cent'])
                        else:
                            a, T3 = float(d['a']), float(d['T3'])
                            if d.get('T1') is not None:
                                flags |= 2; T1 = float(d['T1'])
                            if d.get('T2') is not None:
                                flags |= 4; T2 = float(d['T2'])
                    elif fm == 4:
                        a, T1, T2 = float(d['a']), float(d['b']), float(d['c'])
                    L.oracle_set_pressure_dependent(self.h, ir, float(k0['A']), float(k0['n']), float(k0['C']), Fc, a,
                                                    T1, T2, T3, flags)
            ode = cfg['odeStep']
            lim = cfg['tempLimits']
            T_lo, T_hi = (lim['lower'], lim['upper']) if T_limits is None else T_limits
            method = 0 if ode['method'] == 'rkf' else 1
            L.oracle_set_config(self.h, T_lo, T_hi, method, float(ode.get('errTol', 1e-3)),
                                float(ode.get('eps1', 1e-3)), float(ode.get('eps2', 5e-4)),
                                float(ode.get('delta', 1e-10)), int(ode.get('maxIters', 10)),
                                int(bool(cfg['tightTempCoupling'])), int(cfg['maxSubcycles']), int(cfg['maxAttempts']))
            self.config = cfg
            self.nr = L.oracle_n_reactions(self.h)

    def __del__(self):
        if getattr(self, 'h', None) and _lib is not None:
            _lib.oracle_model_free(self.h)
            self.h = None

    # --- thermo -------------------------------------------------------------------------
    def species_thermo(self, isp, T):
        cp, h, s = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = lib().oracle_species_thermo(self.h, isp, T, ctypes.byref(cp), ctypes.byref(h), ctypes.byref(s))
        if rc:
            raise ValueError("thermo evaluation failed (%d)" % rc)
        return cp.value, h.value, s.value

    def update_thermo_from_pT(self, p, T, massf):
        p = np.ascontiguousarray(p, np.float64); T = np.ascontiguousarray(T, np.float64)
        mf = np.array(massf, np.float64, order='C').reshape(len(p), self.nsp)
        rho = np.empty_like(p); u = np.empty_like(p)
        rc = lib().oracle_update_thermo_from_pT(self.h, len(p), _dp(p), _dp(T), _dp(mf), _dp(rho), _dp(u))
        if rc:
            raise ValueError("update_thermo_from_pT failed (%d)" % rc)
        return rho, u

    def update_thermo_from_rhou(self, rho, u, massf, T_guess, p=None):
        rho = np.ascontiguousarray(rho, np.float64); u = np.ascontiguousarray(u, np.float64)
        mf = np.array(massf, np.float64, order='C').reshape(len(rho), self.nsp)
        T = np.array(T_guess, np.float64, copy=True).reshape(len(rho))
        pp = np.zeros_like(rho) if p is None else np.array(p, np.float64, copy=True)
        st = np.zeros(len(rho), np.int32)
        lib().oracle_update_thermo_from_rhou(self.h, len(rho), _dp(rho), _dp(u), _dp(mf), _dp(T), _dp(pp), _ip(st))
        return T, pp, st

    # --- kinetics -----------------------------------------------------------------------
    def rate_constants(self, T, conc=None):
        """k_f, k_b at T; conc (mol/m^3) gives the third bodies of pressure-dependent rates."""
        kf = np.empty(self.nr); kb = np.empty(self.nr)
        c = None if conc is None else _dp(np.ascontiguousarray(conc, np.float64))
        rc = lib().oracle_rate_constants(self.h, T, c, _dp(kf), _dp(kb))
        if rc:
            raise ValueError("rate constants failed (%d)" % rc)
        return kf, kb

    def split_rates(self, T, conc):
        conc = np.ascontiguousarray(conc, np.float64)
        q = np.empty(self.nsp); L = np.empty(self.nsp); wf = np.empty(self.nr); wb = np.empty(self.nr)
        rc = lib().oracle_split_rates(self.h, T, _dp(conc), _dp(q), _dp(L), _dp(wf), _dp(wb))
        if rc:
            raise ValueError("split rates failed (%d)" % rc)
        return q, L, wf, wb

    def estimate_step(self, T, conc):
        conc = np.ascontiguousarray(conc, np.float64)
        return lib().oracle_estimate_step(self.h, T, _dp(conc))

    def ode_step(self, method, T, y0, h):
        y0 = np.ascontiguousarray(y0, np.float64)
        y1 = np.empty_like(y0)
        hs = ctypes.c_double()
        ok = lib().oracle_ode_step(self.h, 0 if method == 'rkf' else 1, T, _dp(y0), h, _dp(y1), ctypes.byref(hs))
        return bool(ok), y1, hs.value

    def integrate_fixed(self, method, T, y0, dt, t_max):
        y = np.array(y0, np.float64, copy=True)
        n = lib().oracle_integrate_fixed(self.h, 0 if method == 'rkf' else 1, T, _dp(y), dt, t_max)
        return y, n

    def chem_update(self, rho, u, T, p, massf, dt_chem, t_interval, T_frozen=0.0, update_thermo=True,
                    retry=True, nthreads=0, counters=False):
        """Batch of thermochemical increments.  massf is (ncell, nsp).  Returns a dict."""
        n = len(rho)
        rho = np.ascontiguousarray(rho, np.float64); u = np.ascontiguousarray(u, np.float64)
        T = np.array(T, np.float64, copy=True); p = np.array(p, np.float64, copy=True)
        mf = np.array(massf, np.float64, order='C', copy=True).reshape(n, self.nsp)
        dt = np.array(dt_chem, np.float64, copy=True).reshape(n)
        st = np.zeros(n, np.int32)
        cnt = np.zeros((n, 5), np.int64) if counters else None
        flags = (1 if update_thermo else 0) | (2 if retry else 0)
        nfail = lib().oracle_chem_update(self.h, n, _dp(rho), _dp(u), _dp(T), _dp(p), _dp(mf), _dp(dt), _ip(st),
                                         t_interval, T_frozen, flags, nthreads,
                                         cnt.ctypes.data_as(_l) if counters else None)
        out = dict(T=T, p=p, massf=mf, dt_chem=dt, status=st, nfail=nfail)
        if counters:
            out['counters'] = cnt
        return out


def max_threads():
    return lib().oracle_max_threads()
