"""Chemical equilibrium at fixed (p, T) for an ideal-gas mixture, batched over cells (host side).

The H2-air workloads blend unburnt stoichiometric H2-air with its equilibrium products at each
cell's (p, T).  The reference computes such compositions with its equilibrium library
(extern/eqc/source/pt.c:328 solve_pt), a Gordon-McBride (NASA RP-1311) Newton iteration on the
species moles.  This module finds the same Gibbs-energy minimum by the element-potential form of
that problem, vectorised over all cells with numpy:

    x_j = exp(c_j + sum_i a_ij pi_i),   c_j = -G0_j/(R T) - ln(p / 1 bar)
    n sum_j a_ij x_j = b_i   (element balance, i = 1..nel),   sum_j x_j = 1

with unknowns the element potentials pi_i and y = ln n (n = moles of mixture per kg, b_i = moles of
element i per kg).  Each Newton step solves the (nel + 1) x (nel + 1) system by pseudo-inverse, so
that the direction left undetermined by trace species (a cold stoichiometric mixture, where the
split between trace H2 and O2 is below double precision of the balances) gets no step; steps are
limited and backtracked on the scaled residual.  Standard-state G0/RT comes from each species'
NASA-9 curves with the segment choice of the reference's equilibrium library (T <= 1000 K, then
<= 6000 K, then the third range; extern/eqc/source/thermo.c:25-104).

Inputs are the species of a gdtk gas file (read by `species_data`).  `tests/golden/eq_h2air.json`
holds compositions from the reference's own solve_pt for the same species data; the CPU test
`tests/test_equilibrium_cpu.py` checks this solver against them.
"""
import re

import numpy as np

P_STD = 1.0e5   # the standard pressure of the NASA-9 curves (1 bar)

_SPECIES = re.compile(r"species\s*=\s*\{(.*?)\}", re.S)
_NAME = re.compile(r"'([^']+)'")


def _block(text, start):
    """The text of the brace-balanced table constructor that opens at text[start] == '{'."""
    depth = 0
    for k in range(start, len(text)):
        if text[k] == '{':
            depth += 1
        elif text[k] == '}':
            depth -= 1
            if depth == 0:
                return text[start:k + 1]
    raise ValueError("unbalanced table constructor")


def species_data(gas_file):
    """Species names, atomic constituents and NASA-9 segments (T breaks, [nseg][9] coefficients)
    of a gas file written by gdtk's prep-gas (thermally perfect gas, CEA curves)."""
    text = open(gas_file).read()
    names = _NAME.findall(_SPECIES.search(text).group(1))
    out = []
    for s in names:
        key = "db['%s']" % s
        k = text.index(key + ".atomicConstituents")
        atoms = dict((a, int(v)) for a, v in re.findall(r"(\w+)\s*=\s*(\d+)", _block(text, text.index('{', k))))
        k = text.index(key + ".thermoCoeffs")
        tc = _block(text, text.index('{', k))
        breaks = [float(v) for v in re.search(r"T_break_points\s*=\s*\{([^}]*)\}", tc).group(1).split(',') if
                  v.strip()]
        nseg = int(re.search(r"nsegments\s*=\s*(\d+)", tc).group(1))
        segs = []
        for i in range(nseg):
            body = re.search(r"segment%d\s*=\s*\{([^}]*)\}" % i, tc).group(1)
            segs.append([float(v) for v in body.split(',') if v.strip()])
        out.append(dict(name=s, atoms=atoms, breaks=breaks, coeffs=np.array(segs)))
    return out


def g0_rt(sp, T):
    """G0/RT of one species at temperatures T (array) from its NASA-9 curves, choosing the range
    T <= 1000 K, <= 6000 K, else the third, with T clamped to [1, 20000] K."""
    T = np.clip(np.asarray(T, dtype=np.float64), 1.0, 20000.0)
    seg = np.where(T <= 1000.0, 0, np.where(T <= 6000.0, 1, 2))
    seg = np.minimum(seg, sp["coeffs"].shape[0] - 1)
    a = sp["coeffs"][seg]                       # (n, 9)
    lnT = np.log(T)
    h = (-a[:, 0] / T ** 2 + a[:, 1] * lnT / T + a[:, 2] + a[:, 3] * T / 2 + a[:, 4] * T ** 2 / 3 +
         a[:, 5] * T ** 3 / 4 + a[:, 6] * T ** 4 / 5 + a[:, 7] / T)
    s = (-a[:, 0] / T ** 2 / 2 - a[:, 1] / T + a[:, 2] * lnT + a[:, 3] * T + a[:, 4] * T ** 2 / 2 +
         a[:, 5] * T ** 3 / 3 + a[:, 6] * T ** 4 / 4 + a[:, 8])
    return h - s


def element_matrix(species):
    """Element names (sorted) and a[nel][nsp], atoms of each element per molecule."""
    elems = sorted({e for sp in species for e in sp["atoms"]})
    a = np.array([[sp["atoms"].get(e, 0) for sp in species] for e in elems], dtype=np.float64)
    return elems, a


def equilibrium_pT(species, p, T, b, guess=None, tol=1e-12, max_iter=100):
    """Equilibrium mole fractions x (n, nsp) at pressures p (n,) and temperatures T (n,) for
    element amounts b (nel,) or (n, nel) [mol per kg], by element-potential Newton iteration.

    guess: optional (n, nsp) mole fractions to start from (each species' ln x then sets the
    initial potentials by least squares); the default starts from the species with the largest
    share of each element in a uniform mixture.  Raises if a cell does not converge."""
    p = np.atleast_1d(np.asarray(p, dtype=np.float64))
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    n = T.shape[0]
    elems, a = element_matrix(species)
    nel, nsp = a.shape
    b = np.broadcast_to(np.asarray(b, dtype=np.float64), (n, nel)).copy()
    c = -np.stack([g0_rt(sp, T) for sp in species], axis=1) - np.log(p / P_STD)[:, None]   # (n, nsp)
    if guess is None:
        guess = np.full((n, nsp), 1.0 / nsp)
    guess = np.asarray(guess, dtype=np.float64)
    lx = np.log(np.maximum(guess, 1e-300))
    # Initial potentials.  (1) The minimum-norm least-squares fit of c_j + a_j . pi = ln x_j over the
    # guess's major species.  (2) Along the directions V that the majors leave open (a_major . V = 0),
    # the minimum of ln sum_j x_j, a convex function of t in pi + V t: its stationarity condition
    # sum_j (a_j . V) x_j = 0 balances the remaining species' elements as the exact solution does.
    w = (guess > 1e-3 * guess.max(axis=1, keepdims=True)).astype(np.float64)
    A = a.T[None, :, :] * w[:, :, None]                    # (n, nsp, nel)
    U, sv, Vt = np.linalg.svd(A, full_matrices=True)
    rank = (sv > 1e-10 * sv[:, :1]).sum(axis=1)
    rhs = (lx - c) * w
    coef = np.einsum("nji,nj->ni", U[:, :, :nel], rhs) / np.where(sv > 1e-10 * sv[:, :1], sv, np.inf)
    pi = np.einsum("nki,nk->ni", Vt, coef)                  # minimum-norm solution (n, nel)
    for r_ in np.unique(rank):
        if r_ >= nel:
            continue
        rows = np.flatnonzero(rank == r_)
        V = np.transpose(Vt[rows, r_:, :], (0, 2, 1))       # (m, nel, k): the open directions
        aV = np.einsum("ij,mik->mjk", a, V)                 # (m, nsp, k): a_j . V
        t = np.zeros((rows.size, nel - r_))
        base = c[rows] + pi[rows] @ a

        def lnz(t):
            e = base + np.einsum("mjk,mk->mj", aV, t)
            emax = e.max(axis=1, keepdims=True)
            return np.log(np.exp(e - emax).sum(axis=1)) + emax[:, 0], e

        f, e = lnz(t)
        live = np.ones(rows.size, dtype=bool)
        for _ in range(60):
            xt = np.exp(e - e.max(axis=1, keepdims=True))
            xt /= xt.sum(axis=1, keepdims=True)
            g = np.einsum("mjk,mj->mk", aV, xt)
            live &= np.abs(g).max(axis=1) > 1e-12
            if not live.any():
                break
            H = np.einsum("mjk,mjl,mj->mkl", aV, aV, xt) - g[:, :, None] * g[:, None, :]
            H += 1e-12 * np.eye(nel - r_)[None]
            d = -np.linalg.solve(H, g[:, :, None])[:, :, 0]
            d *= np.minimum(1.0, 10.0 / np.maximum(np.abs(d).max(axis=1), 1e-300))[:, None]
            d[~live] = 0.0
            lam = np.ones(rows.size)
            slope = (g * d).sum(axis=1)
            for _ in range(40):
                fn, en = lnz(t + lam[:, None] * d)
                ok = (fn <= f + 1e-4 * lam * slope + 1e-13 * (1.0 + np.abs(f))) | ~live
                if ok.all():
                    break
                lam = np.where(ok, lam, 0.5 * lam)
            t = t + lam[:, None] * d
            f, e = fn, en
        pi[rows] += np.einsum("mik,mk->mi", V, t)
    y = np.log(b.sum(axis=1) / np.maximum((a.sum(axis=0)[None, :] * guess).sum(axis=1), 1e-300))

    def resid(pi, y, rows):
        e = np.clip(c[rows] + pi @ a, -745.0, 300.0)
        x = np.exp(e)
        ax = x @ a.T                                        # (rows, nel)
        r = np.empty((pi.shape[0], nel + 1))
        r[:, :nel] = (np.exp(y)[:, None] * ax - b[rows]) / b[rows]
        r[:, nel] = x.sum(axis=1) - 1.0
        return r, x, ax

    r, x, ax = resid(pi, y, np.arange(n))
    norm = np.abs(r).max(axis=1)
    active = norm > tol
    for _ in range(max_iter):
        if not active.any():
            break
        ia = np.flatnonzero(active)
        old_norm = norm[ia].copy()
        xa, axa, ya, ra = x[ia], ax[ia], y[ia], r[ia]
        nn = np.exp(ya)
        J = np.zeros((ia.size, nel + 1, nel + 1))
        J[:, :nel, :nel] = nn[:, None, None] * np.einsum("ij,kj,nj->nik", a, a, xa) / b[ia][:, :, None]
        J[:, :nel, nel] = nn[:, None] * axa / b[ia]
        J[:, nel, :nel] = axa
        # Levenberg-Marquardt normal equations: directions whose singular value is below ~1e-7 of the
        # largest (left open by trace species, e.g. the trace H2 : O2 split of a cold stoichiometric
        # mixture) get almost no step; the rest take the Newton step
        JtJ = np.einsum("nki,nkj->nij", J, J)
        mu = 1e-14 * np.einsum("nii->n", JtJ)
        d = -np.linalg.solve(JtJ + mu[:, None, None] * np.eye(nel + 1)[None],
                             np.einsum("nki,nk->ni", J, ra)[:, :, None])[:, :, 0]
        big = np.abs(d).max(axis=1)
        d *= np.minimum(1.0, 4.0 / np.maximum(big, 1e-300))[:, None]
        # backtracking on the largest scaled residual
        step = np.ones(ia.size)
        best_pi, best_y = pi[ia].copy(), ya.copy()
        done = np.zeros(ia.size, dtype=bool)
        for _ in range(30):
            tpi = best_pi + step[:, None] * d[:, :nel]
            ty = best_y + step * d[:, nel]
            tr, tx, tax = resid(tpi, ty, ia)
            tn = np.abs(tr).max(axis=1)
            good = (tn < norm[ia]) & ~done
            if good.any():
                gi = ia[good]
                pi[gi], y[gi], r[gi], x[gi], ax[gi], norm[gi] = tpi[good], ty[good], tr[good], tx[good], tax[good], \
                    tn[good]
                done |= good
            if done.all():
                break
            step = np.where(done, step, step * 0.5)
        # a cell whose residual no longer falls, or falls by under a tenth near rounding level, is done
        slow = np.zeros(n, dtype=bool)
        slow[ia] = ~done | ((norm[ia] > 0.9 * old_norm) & (norm[ia] < 1e-10))
        active = (norm > tol) & ~slow
    if np.any(norm > 1e-9):
        bad = int(np.argmax(norm))
        raise RuntimeError("equilibrium did not converge at p=%g T=%g (residual %g)" % (p[bad], T[bad], norm[bad]))
    return x / x.sum(axis=1, keepdims=True)


def products_massf(species, M, Y_products, p, T):
    """Equilibrium mass fractions (nsp, n) at each (p, T) of the mixture whose elements are those of
    the mass fractions Y_products (nsp,), started from Y_products as the mole-fraction guess."""
    M = np.asarray(M, dtype=np.float64)
    elems, a = element_matrix(species)
    moles = np.asarray(Y_products, dtype=np.float64) / M
    b = a @ moles                                           # mol of each element per kg
    x0 = moles / moles.sum()
    guess = np.broadcast_to(x0, (np.atleast_1d(T).shape[0], len(species)))
    x = equilibrium_pT(species, p, T, b, guess=guess)
    y = x * M[None, :]
    return np.ascontiguousarray((y / y.sum(axis=1, keepdims=True)).T)


class ProductsTable:
    """Equilibrium mass fractions of one element composition over a (T, log10 p) rectangle.

    The exact solver (`products_massf`) runs once on a grid of T_step K by logp_step decades; each
    species' ln x is then a bicubic spline in (T, log10 p), evaluated at any cell's (p, T).  A node
    sits on the 1000 K break of the curves.  tests/test_equilibrium_cpu.py bounds the interpolation
    error against the exact solver."""

    def __init__(self, gas_file, Y_products, M, T_range=(250.0, 3000.0), logp_range=(3.5, 6.5), T_step=5.0,
                 logp_step=0.05):
        from scipy.interpolate import RectBivariateSpline
        self.species = species_data(gas_file)
        self.M = np.asarray(M, dtype=np.float64)
        self.T = np.arange(T_range[0], T_range[1] + 0.5 * T_step, T_step)
        self.logp = np.arange(logp_range[0], logp_range[1] + 0.5 * logp_step, logp_step)
        TT, PP = np.meshgrid(self.T, self.logp, indexing="ij")
        Y = products_massf(self.species, self.M, Y_products, 10.0 ** PP.ravel(), TT.ravel())   # (nsp, nT*np)
        x = Y / self.M[:, None]
        x /= x.sum(axis=0, keepdims=True)
        lnx = np.log(np.maximum(x, 1e-300)).reshape(len(self.species), len(self.T), len(self.logp))
        self.splines = [RectBivariateSpline(self.T, self.logp, lnx[j], kx=3, ky=3) for j in range(len(self.species))]
        self.T_range, self.logp_range = (self.T[0], self.T[-1]), (self.logp[0], self.logp[-1])

    def massf(self, p, T):
        """(nsp, n) equilibrium mass fractions at each cell's (p, T)."""
        T = np.asarray(T, dtype=np.float64)
        lp = np.log10(np.asarray(p, dtype=np.float64))
        if T.min() < self.T_range[0] or T.max() > self.T_range[1] or lp.min() < self.logp_range[0] or \
                lp.max() > self.logp_range[1]:
            raise ValueError("(p, T) outside the equilibrium table")
        x = np.exp(np.stack([s.ev(T, lp) for s in self.splines]))
        y = x * self.M[:, None]
        return np.ascontiguousarray(y / y.sum(axis=0, keepdims=True))


_TABLES = {}


def products_table(gas_file, Y_products, M):
    """The (cached) ProductsTable of gas_file for the element composition of Y_products."""
    key = (gas_file, tuple(np.round(np.asarray(Y_products, dtype=np.float64), 15)))
    if key not in _TABLES:
        _TABLES[key] = ProductsTable(gas_file, Y_products, M)
    return _TABLES[key]
