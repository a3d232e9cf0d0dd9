"""Seeded synthetic cell states for the reference's chemistry workloads.

No benchmark data set exists for this path; every input is drawn from a numpy PCG64
generator with a fixed seed, on the host, so the GPU engine and the CPU oracle see the
same bits.  Densities and energies are then obtained from (p, T, Y) by the gas model
(update_thermo_from_pT).
"""
import numpy as np

AIR5_SPECIES = ['N2', 'O2', 'NO', 'N', 'O']
H2AIR_RADICALS = ['H', 'O', 'OH', 'HO2', 'H2O2', 'N', 'NO', 'NO2', 'HNO']


def air5_cells(n, seed=0):
    """4096-cell air workload: T ~ U[2000, 8000] K, p = 10^U[3, 5] Pa, Y ~ Dirichlet(1) over
    (N2, O2, NO, N, O).  Returns T (n,), p (n,), Y (5, n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    T = rng.uniform(2000.0, 8000.0, n)
    p = 10.0 ** rng.uniform(3.0, 5.0, n)
    Y = rng.dirichlet(np.ones(5), n)
    Y = Y / Y.sum(axis=1, keepdims=True)
    return T, p, np.ascontiguousarray(Y.T)


def air2t_cells(n, seed=7):
    """Two-temperature (thermal non-equilibrium) air behind a shock, Park's 5 species (N2, O2, N, O, NO):
    T ~ U[3000, 12000] K, T_ve ~ U[300 K, 1.2 T], p = 10^U[3, 4.7] Pa, Y ~ Dirichlet(2, 1, 0.3, 0.3, 0.3).
    Returns T, T_ve, p (n,) and Y (5, n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    T = rng.uniform(3000.0, 12000.0, n)
    Tve = rng.uniform(300.0, 1.2 * T)
    p = 10.0 ** rng.uniform(3.0, 4.7, n)
    Y = rng.dirichlet([2.0, 1.0, 0.3, 0.3, 0.3], n)
    return T, Tve, p, np.ascontiguousarray(Y.T)


def h2air_cells(names, mol_masses, n, seed=1, frozen_fraction=0.5, T_cold=(300.0, 600.0), T_hot=(1100.0, 2800.0),
                p_range=(2.0e4, 5.0e5), gas_file=None, subset=None):
    """H2-air workload of uneven stiffness.

    A fraction `frozen_fraction` of the cells is cold (T ~ U[T_cold]), the rest hot
    (T ~ U[T_hot]); p = 10^U[log10 p_range].  Composition: a blend, weight lambda ~ U[0, 1],
    of stoichiometric H2-air (X_H2 : X_O2 : X_N2 = 2 : 1 : 3.76) and its equilibrium products at
    the cell's (p, T) (the element composition of X_H2O : X_N2 = 2 : 3.76, by
    gdtk_gb300.equilibrium from the NASA-9 data of `gas_file`), plus radicals (H, O, OH, HO2,
    H2O2, N, NO, NO2, HNO) whose total mass fraction is 10^U[-6, -2] split by Dirichlet(0.5);
    renormalised.  Returns T (n,), p (n,), Y (nsp, n).  With `subset` (indices into the n cells),
    only those cells are returned, and the equilibrium products are evaluated for them alone; the
    random draws are the same as for all n cells.
    """
    if gas_file is None:
        raise ValueError("h2air_cells needs the gas file (species thermo data) for the equilibrium products")
    from .equilibrium import products_table
    rng = np.random.Generator(np.random.PCG64(seed))
    idx = {s: i for i, s in enumerate(names)}
    M = np.asarray(mol_masses, dtype=np.float64)
    nsp = len(names)
    hot = rng.uniform(0.0, 1.0, n) >= frozen_fraction
    T = np.where(hot, rng.uniform(T_hot[0], T_hot[1], n), rng.uniform(T_cold[0], T_cold[1], n))
    p = 10.0 ** rng.uniform(np.log10(p_range[0]), np.log10(p_range[1]), n)

    def massf_of(molef):
        x = np.zeros(nsp)
        for s, v in molef.items():
            x[idx[s]] = v
        y = x * M
        return y / y.sum()

    unburnt = massf_of({'H2': 2.0, 'O2': 1.0, 'N2': 3.76})
    lam = rng.uniform(0.0, 1.0, n)
    rad_idx = [idx[s] for s in H2AIR_RADICALS if s in idx]
    share = 10.0 ** rng.uniform(-6.0, -2.0, n)
    w = rng.dirichlet(np.full(len(rad_idx), 0.5), n)
    if subset is not None:
        subset = np.asarray(subset, dtype=np.int64)
        T, p, lam, share, w = T[subset], p[subset], lam[subset], share[subset], w[subset]
    burnt = products_table(gas_file, massf_of({'H2O': 2.0, 'N2': 3.76}), M).massf(p, T).T   # (n, nsp)
    Y = (1.0 - lam)[:, None] * unburnt[None, :] + lam[:, None] * burnt
    Y *= (1.0 - share)[:, None]
    Y[:, rad_idx] += share[:, None] * w
    Y = Y / Y.sum(axis=1, keepdims=True)
    return T, p, np.ascontiguousarray(Y.T)


def h2air_blocks(names, mol_masses, nblocks=64, seed=2, n_min=2048, n_max=524288, dts=(1.0e-7, 1.0e-6, 1.0e-5),
                 gas_file=None, pick=None):
    """Uneven multi-block H2-air workload.

    Block sizes are log-uniform in [n_min, n_max]; each block draws its own update interval from
    `dts`, its own cold fraction, and its own sub-ranges of the cold (300-600 K) and hot
    (1100-2800 K) temperatures and of the pressure (2e4-5e5 Pa), and then its cells as in
    h2air_cells.  Returns a list of dicts with T, p, Y (nsp, n) and dt.  With `pick(b, n)` -> indices,
    block b holds only those of its n cells (and 'n' and 'cells' record the full size and the indices).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.round(10.0 ** rng.uniform(np.log10(n_min), np.log10(n_max), nblocks)).astype(np.int64)
    out = []
    for b in range(nblocks):
        dt = float(rng.choice(dts))
        cold = np.sort(rng.uniform(300.0, 600.0, 2))
        hot = np.sort(rng.uniform(1100.0, 2800.0, 2))
        lp = np.sort(rng.uniform(np.log10(2.0e4), np.log10(5.0e5), 2))
        frac = float(rng.uniform(0.0, 1.0))
        nb = int(sizes[b])
        sub = None if pick is None else np.asarray(pick(b, nb), dtype=np.int64)
        T, p, Y = h2air_cells(names, mol_masses, nb, seed=seed * 1000 + b, frozen_fraction=frac,
                              T_cold=(cold[0], cold[1] + 1e-9), T_hot=(hot[0], hot[1] + 1e-9),
                              p_range=(10.0 ** lp[0], 10.0 ** lp[1] * (1 + 1e-12)), gas_file=gas_file, subset=sub)
        out.append(dict(T=T, p=p, Y=Y, dt=dt, n=nb, cells=sub))
    return out


def h2air_mixing_layer(names, mol_masses, nx=2048, ny=1024, seed=4, thickness=16.0, T_fuel=300.0, T_ox=1500.0,
                       p=1.0e5, radical_share=0.10):
    """A 2-D structured block (nx x ny cells, cell index i + nx*j) holding a tanh mixing layer
    across j: fuel stream (pure H2 at T_fuel) on one side, oxidiser stream (air at T_ox) on the
    other, mixture fraction f = (1 + tanh((j - ny/2) / thickness)) / 2.  The oxidiser carries a
    seeded radical share (O, OH, H, HO2, NO, N) of up to `radical_share` of its mass per cell.
    T and Y blend linearly in f.  Returns T (n,), p (n,), Y (nsp, n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    idx = {s: i for i, s in enumerate(names)}
    M = np.asarray(mol_masses, dtype=np.float64)
    nsp = len(names)
    n = nx * ny
    j = np.repeat(np.arange(ny), nx)
    f = 0.5 * (1.0 + np.tanh((j - ny / 2.0) / thickness))
    fuel = np.zeros(nsp)
    fuel[idx['H2']] = 1.0
    air = np.zeros(nsp)
    air[idx['O2']] = 1.0 * M[idx['O2']]
    air[idx['N2']] = 3.76 * M[idx['N2']]
    air /= air.sum()
    rad = [idx[s] for s in ('O', 'OH', 'H', 'HO2', 'NO', 'N') if s in idx]
    share = rng.uniform(0.0, radical_share, n)
    w = rng.dirichlet(np.full(len(rad), 0.5), n)
    ox = np.repeat(air[None, :], n, axis=0) * (1.0 - share)[:, None]
    ox[:, rad] += share[:, None] * w
    Y = f[:, None] * fuel[None, :] + (1.0 - f)[:, None] * ox
    Y /= Y.sum(axis=1, keepdims=True)
    T = f * T_fuel + (1.0 - f) * T_ox
    return T, np.full(n, p), np.ascontiguousarray(Y.T)


ACETYLENE_MIXTURE = {'C2H2': 0.02, 'O2': 0.025, 'Ar': 0.955}   # mole fractions, shock-tube mixture 25


def acetylene_cells(names, mol_masses, n, seed=5, T_range=(1150.0, 1750.0), p_atm=0.6, share=(-6.0, -2.0)):
    """Shock-tube ignition states of the 75-species C2H2/C2H4 mechanism (the reference's
    examples/kinetics/acetylene-ignition-delay: the mixture above at 0.6 atm, 1150-1750 K).  Each
    cell carries a 10^U[share] mass share of the other 72 species (Dirichlet(0.5)), standing for
    cells at different stages of induction; T ~ U[T_range], p = p_atm atm.  Returns T, p, Y (nsp, n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    M = np.asarray(mol_masses, dtype=np.float64)
    x = np.zeros(len(names))
    for s, v in ACETYLENE_MIXTURE.items():
        x[names.index(s)] = v
    y0 = x * M / (x * M).sum()
    minor = [i for i, s in enumerate(names) if s not in ACETYLENE_MIXTURE]
    Y = np.repeat(y0[None, :], n, axis=0)
    w = 10.0 ** rng.uniform(share[0], share[1], n)
    Y *= (1.0 - w)[:, None]
    Y[:, minor] += w[:, None] * rng.dirichlet(np.full(len(minor), 0.5), n)
    T = rng.uniform(T_range[0], T_range[1], n)
    p = np.full(n, p_atm * 101325.0)
    return T, p, np.ascontiguousarray(Y.T)
