"""CPU checks of the surrogate's oracles: the FP64 network gradient against central
differences, the BF16 rounding helper, the element matrix read from the gas file, and the
gate restatement on hand-made increments."""
import numpy as np
import pytest

import oracle
from oracle import mlp
from oracle import surrogate_gate as sgate
from conftest import mech


def _layers(dims, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [(rng.uniform(-1, 1, (dims[l + 1], dims[l])) / np.sqrt(dims[l]), rng.uniform(-0.1, 0.1, dims[l + 1]))
            for l in range(len(dims) - 1)]


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(1))
    layers = _layers([16, 24, 24, 16], 2)
    X = rng.normal(size=(32, 16))
    Y = rng.normal(size=(32, 16))
    w = np.ones(16)
    w[14:] = 0.0
    assert mlp.finite_difference_check(layers, X, Y, w, n_probe=40) < 1e-6


def test_oracle_pinball_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(4))
    layers = _layers([24, 16, 8], 6)
    X = rng.normal(size=(64, 24))
    Y = np.zeros((64, 8))
    Y[:, 0] = rng.normal(size=64) * 3.0   # away from the kinks of the piecewise-linear loss
    assert mlp.finite_difference_check(layers, X, Y, np.ones(8), n_probe=40, quantile=0.9) < 1e-5


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-5, 0.0])
    r = mlp.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                     # tie -> even
    assert r[2] == 1.0 + 4 * 2 ** -8       # tie -> even (up)
    assert r[3] == 1.0
    assert r[4] == -2.5 and r[6] == 0.0
    assert abs(r[5] - 3.0e-5) <= 3.0e-5 * 2 ** -8


def test_element_matrix_of_h2_air():
    els, E, EM = sgate.element_matrix(mech("j92-gas.lua"))
    assert sorted(els) == ["H", "N", "O"]
    names, species = oracle.load_gas(mech("j92-gas.lua"))
    M = np.array([s["M"] for s in species])
    h2o = names.index("H2O")
    assert E[els.index("H"), h2o] * M[h2o] == pytest.approx(2.0)
    assert E[els.index("O"), h2o] * M[h2o] == pytest.approx(1.0)
    # each species' mass is the sum of its atoms' masses (so element balance implies mass balance)
    assert np.allclose((E * EM[:, None]).sum(axis=0), 1.0, rtol=1e-6)


def test_gate_restatement_projects_onto_element_conservation():
    orc = oracle.Oracle(mech("j92-gas.lua"))
    els, E, EM = sgate.element_matrix(mech("j92-gas.lua"))
    names = orc.names
    Y = np.zeros((1, len(names)))
    Y[0, names.index("H2")] = 0.03
    Y[0, names.index("O2")] = 0.22
    Y[0, names.index("N2")] = 0.75
    T = np.array([1500.0])
    p = np.array([1.0e5])
    rho, u = orc.update_thermo_from_pT(p, T, Y)
    # a balanced increment (2 H2 + O2 -> 2 H2O, 1e-3 kg/kg of H2O) plus a small imbalance
    d = np.zeros((1, len(names)))
    mH2O = 1e-3
    nH2O = mH2O / orc.M[names.index("H2O")]
    d[0, names.index("H2O")] = mH2O
    d[0, names.index("H2")] = -nH2O * orc.M[names.index("H2")]
    d[0, names.index("O2")] = -0.5 * nH2O * orc.M[names.index("O2")] + 5e-7
    lo, hi = np.full(16, -1e300), np.full(16, 1e300)
    codes, Y1, T1, p1 = sgate.gate(orc, E, EM, rho, u, T, p, Y, d, np.array([0.0]), lo, hi, 1e-6, 0.0,
                                   elem_tol=1e-6, neg_tol=1e-9, T_tol=1.0)
    assert codes[0] == sgate.ACCEPTED
    assert np.abs(E @ (Y1[0] - Y[0])).max() < 1e-12 * np.abs(E @ Y[0]).max()
    assert T1[0] > T[0]   # heat release
    codes, *_ = sgate.gate(orc, E, EM, rho, u, T, p, Y, d, np.array([0.0]), lo, hi, 1e-6, 0.0,
                           elem_tol=1e-8, neg_tol=1e-9, T_tol=1.0)
    assert codes[0] == sgate.ELEMENTS
