"""The equilibrium products of the H2-air workloads (gdtk_gb300.equilibrium) against the reference's
own equilibrium library, extern/eqc/source/pt.c:328 solve_pt, whose results for the same species
data are the fixture tests/golden/eq_h2air.json (written by tests/golden/make_equilibrium_fixture.py
from the reference's C sources, built by 'make -C oracle eqc')."""
import json
import os

import numpy as np

from conftest import GOLDEN, mech


def _fixture():
    with open(os.path.join(GOLDEN, "eq_h2air.json")) as f:
        return json.load(f)


def _setup():
    from gdtk_gb300 import equilibrium as eq
    sp = eq.species_data(mech("j92-gas.lua"))
    d = _fixture()
    assert [s["name"] for s in sp] == d["species"]
    import oracle
    M = np.asarray(oracle.Oracle(mech("j92-gas.lua")).M)
    X0 = np.asarray(d["products_molef"])
    Y0 = X0 * M / (X0 * M).sum()
    return eq, sp, d, M, Y0


def test_equilibrium_matches_reference_solve_pt():
    eq, sp, d, M, Y0 = _setup()
    p = np.array([r["p"] for r in d["points"]])
    T = np.array([r["T"] for r in d["points"]])
    Xr = np.array([r["X"] for r in d["points"]])
    assert all(r["rc"] == 0 for r in d["points"])
    Y = eq.products_massf(sp, M, Y0, p, T)
    X = Y.T / M
    X /= X.sum(axis=1, keepdims=True)
    err = np.abs(X - Xr)
    # every mole fraction to 1e-12 absolute; relative 1e-9 above 1e-6 and 1e-11 above 1e-2 (the
    # reference iterates to a residual of 1e-11, trace species below ~1e-10 are only roughly set there)
    assert err.max() <= 1e-12, err.max()
    for lo, rel in ((1e-2, 1e-11), (1e-6, 1e-9), (1e-8, 1e-6)):
        m = Xr > lo
        assert (err[m] / Xr[m]).max() <= rel, (lo, (err[m] / Xr[m]).max())
    # the hot points dissociate: at 2800 K and 1e5 Pa the products hold percent-level OH and H2
    k = [i for i, r in enumerate(d["points"]) if r["p"] == 1.0e5 and r["T"] == 3400.0][0]
    assert X[k, d["species"].index("OH")] > 0.05


def test_products_table_interpolates_the_exact_solver():
    eq, sp, d, M, Y0 = _setup()
    tab = eq.products_table(mech("j92-gas.lua"), Y0, M)
    rng = np.random.default_rng(3)
    T = rng.uniform(300.0, 2900.0, 1500)
    p = 10.0 ** rng.uniform(np.log10(1.0e4), np.log10(1.0e6), 1500)
    Ye = eq.products_massf(sp, M, Y0, p, T)
    Yt = tab.massf(p, T)
    assert np.abs(Yt - Ye).max() <= 1e-8
    big = Ye > 1e-6
    assert (np.abs(Yt - Ye)[big] / Ye[big]).max() <= 1e-5


def test_h2air_cells_blend_equilibrium_products():
    from gdtk_gb300.workloads import h2air_cells
    eq, sp, d, M, Y0 = _setup()
    names = d["species"]
    T, p, Y = h2air_cells(names, M, 4096, seed=5, gas_file=mech("j92-gas.lua"))
    assert Y.shape == (len(names), 4096)
    assert (Y >= 0.0).all() and np.allclose(Y.sum(axis=0), 1.0, atol=1e-14)
    assert ((T >= 300.0) & (T <= 600.0) | (T >= 1100.0) & (T <= 2800.0)).all()
    # element balance: H and O stay in the 2:1 ratio of stoichiometric H2-air, apart from the
    # radical share (at most 1e-2 of the mass) that is added afterwards
    _, a = eq.element_matrix(sp)
    el = a @ (Y / M[:, None])
    e = {n: i for i, n in enumerate(sorted({k for s in sp for k in s["atoms"]}))}
    ratio = el[e["H"]] / el[e["O"]]
    assert np.median(np.abs(ratio - 2.0)) < 0.05
