"""CPU restatement of the surrogate's FP64 gate (TEST INFRASTRUCTURE ONLY).

The checks that gdtk_gb300/csrc/surrogate_kernels.cu (gate_kernel) applies to each predicted
increment before a cell takes it -- training domain, element balance and its projection,
non-negativity, T from (rho, u) by the reference's Newton iteration
(gas/thermo/therm_perf_gas_mix.d:426-468, through the oracle) and energy consistency -- written
independently in numpy, for the gate's parity test.  The surrogate has no counterpart in the
reference.
"""
import numpy as np

from .luatable import array, read_lua_file

ATOMIC_MASS = {"H": 1.00794e-3, "He": 4.002602e-3, "C": 12.0107e-3, "N": 14.0067e-3, "O": 15.9994e-3,
               "Ar": 39.948e-3}

ACCEPTED, FROZEN, BAD_INPUT, DOMAIN, ELEMENTS, NEGATIVE, ENERGY, NEWTON, MAGNITUDE, PREDICTED_ERROR = range(10)


def element_matrix(gas_file):
    """(element names, E (ne, nsp) = atoms per kg of species, element molar masses), elements in
    the order of first appearance over the species list (each species' constituents sorted by
    name)."""
    g = read_lua_file(gas_file)
    names = array(g["species"])
    comp = []
    els = []
    for nm in names:
        ac = g["db"][nm].get("atomicConstituents") or {}
        c = {k: int(v) for k, v in sorted(ac.items())}
        comp.append(c)
        for k in c:
            if k not in els and k not in ("e-", "e"):
                els.append(k)
    M = np.array([float(g["db"][nm]["M"]) for nm in names])
    E = np.array([[comp[s].get(e, 0) / M[s] for s in range(len(names))] for e in els])
    return els, E, np.array([ATOMIC_MASS[e] for e in els])


def gate(orc, E, EM, rho, u, T, p, Y, dY, dT, x_min, x_max, dt, T_frozen, elem_tol, neg_tol, T_tol, max_dY=0.0):
    """Per cell (Y, dY: (n, nsp)): gate code, Y_new, T_new, p_new (the last three meaningful where
    the code is ACCEPTED)."""
    n, nsp = Y.shape
    codes = np.zeros(n, np.int32)
    Y1 = Y.copy()
    T1 = T.copy()
    p1 = p.copy()
    feats = np.concatenate([np.log(T)[:, None], np.log(p)[:, None], Y, np.full((n, 1), np.log(dt))], axis=1)
    feats = feats.astype(np.float32).astype(np.float64)   # the domain test sees float features
    for c in range(n):
        if T[c] <= T_frozen:
            codes[c] = FROZEN
            continue
        if not (rho[c] > 0):
            codes[c] = BAD_INPUT
            continue
        f = feats[c]
        if np.any(f < x_min[:nsp + 3]) or np.any(f > x_max[:nsp + 3]):
            codes[c] = DOMAIN
            continue
        d = dY[c].astype(np.float64).copy()
        if max_dY > 0 and np.abs(d).max() > max_dY:
            codes[c] = MAGNITUDE
            continue
        r = E @ d
        if np.max(np.abs(r) * EM) > elem_tol:
            codes[c] = ELEMENTS
            continue
        w = np.maximum(Y[c], Y[c] + d) + 1e-12
        G = (E * w[None, :]) @ E.T
        lam = np.linalg.solve(G, r)
        d = d - w * (E.T @ lam)
        y = Y[c] + d
        if y.min() < -neg_tol:
            codes[c] = NEGATIVE
            continue
        if y.min() < 0.0:
            # clip, then restore the element balance moving only the species present
            y = np.maximum(y, 0.0)
            w2 = y + 1e-300
            G2 = (E * w2[None, :]) @ E.T
            lam2 = np.linalg.solve(G2, E @ (y - Y[c]))
            y = np.maximum(y - w2 * (E.T @ lam2), 0.0)
        y = y / y.sum()
        guess = T[c] + dT[c]
        if not guess > 0:
            guess = T[c]
        Tn, pn, st = orc.update_thermo_from_rhou([rho[c]], [u[c]], y[None, :], [guess])
        if st[0] != 0 or not Tn[0] > 0:
            codes[c] = NEWTON
            continue
        if abs(Tn[0] - (T[c] + dT[c])) > T_tol * Tn[0]:
            codes[c] = ENERGY
            continue
        Y1[c], T1[c], p1[c] = y, Tn[0], pn[0]
    return codes, Y1, T1, p1
