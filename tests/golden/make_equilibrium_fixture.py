"""Writes tests/golden/eq_h2air.json: equilibrium compositions of the products of stoichiometric
H2-air (X_H2O : X_N2 = 2 : 3.76 in the 13 species of the Jachimowski-1992 gas file) at a grid of
(p, T), computed by the reference's own equilibrium library, extern/eqc/source/pt.c:328 solve_pt.

Test infrastructure.  Run where the reference sources are present:
    make -C oracle eqc        # builds oracle/_ref/libeqc.so from the reference's C sources
    python tests/golden/make_equilibrium_fixture.py
The species data (NASA-9 segments, molar masses, atoms) come from tests/golden/mech/j92-gas.lua, read
by the oracle's Lua reader; solve_pt takes them as its 'lewis' array [nsp][3][9] (the first three
curve segments: 200-1000, 1000-6000, 6000-20000 K; the grid stays below 6000 K) and its element
matrix a[nel][nsp].
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.luatable import read_lua_file   # noqa: E402

TEMPS = [300.0, 450.0, 600.0, 800.0, 1000.0, 1100.0, 1300.0, 1500.0, 1700.0, 1900.0, 2100.0, 2300.0, 2500.0,
         2650.0, 2800.0, 3000.0, 3400.0]
PRESSURES = [2.0e4, 1.0e5, 5.0e5]


def main():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libeqc.so"))
    d = ctypes.POINTER(ctypes.c_double)
    lib.solve_pt.restype = ctypes.c_int
    lib.solve_pt.argtypes = [ctypes.c_double, ctypes.c_double, d, ctypes.c_int, ctypes.c_int, d, d, d, d,
                             ctypes.c_int]
    g = read_lua_file(os.path.join(HERE, "mech", "j92-gas.lua"))
    names = [g["species"][k] for k in sorted(g["species"])]
    db = g["db"]
    elems = sorted({e for s in names for e in db[s]["atomicConstituents"]})
    nsp, nel = len(names), len(elems)
    a = np.array([[db[s]["atomicConstituents"].get(e, 0) for s in names] for e in elems], dtype=np.float64)
    M = np.array([db[s]["M"] for s in names], dtype=np.float64)
    lewis = np.zeros((nsp, 3, 9))
    for i, s in enumerate(names):
        tc = db[s]["thermoCoeffs"]
        for k in range(3):   # two-segment species repeat their second curve above 6000 K (unused here)
            seg = tc["segment%d" % min(k, int(tc["nsegments"]) - 1)]
            lewis[i, k] = [seg[j + 1] for j in range(9)]
    X0 = np.zeros(nsp)
    X0[names.index("H2O")] = 2.0
    X0[names.index("N2")] = 3.76
    X0 /= X0.sum()
    P = lambda v: np.ascontiguousarray(v, dtype=np.float64).ctypes.data_as(d)
    rows = []
    for p in PRESSURES:
        for T in TEMPS:
            X1 = np.zeros(nsp)
            rc = lib.solve_pt(p, T, P(X0), nsp, nel, P(lewis.ravel()), P(M), P(a.ravel()),
                              X1.ctypes.data_as(d), 0)
            rows.append({"p": p, "T": T, "rc": int(rc), "X": X1.tolist()})
    out = {"source": "extern/eqc/source/pt.c:328 solve_pt, built by 'make -C oracle eqc'",
           "gas_file": "tests/golden/mech/j92-gas.lua", "species": names, "elements": elems,
           "products_molef": X0.tolist(), "points": rows}
    with open(os.path.join(HERE, "eq_h2air.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote %d points" % len(rows))


if __name__ == "__main__":
    main()
