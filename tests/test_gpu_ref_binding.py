"""The reference's own Python binding, unmodified, over this library (GPU).

src/lib/gdtk/gas.py (copied verbatim to tests/golden/ref_gdtk/gdtk/gas.py by make_fixtures.sh) opens
its C library with cffi's ffi.dlopen("libgas.so").  Here a directory holding libgas.so as a link to
gdtk_gb300/libgdtk_chem.so is put on LD_LIBRARY_PATH of a fresh interpreter, which then runs the body
of the reference's examples/kinetics/fixed-volume-reactor-n2/test_fvreactor.py:26-55 with its
known answers (rel 1e-4).  The prep-gas / prep-chem outputs that test makes are the committed
fixtures n2-gas.lua / n2-chem.lua (made from the same inputs by make_fixtures.sh).  Where cffi is
not installed, tests/golden/cffi_standin provides the part of it that gas.py uses.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, MECH, ROOT

pytestmark = pytest.mark.gpu

FVREACTOR = r'''
import json
from math import isclose
from gdtk.gas import GasModel, PyGasState as GasState, ThermochemicalReactor
gm = GasModel("n2-gas.lua")
reactor = ThermochemicalReactor(gm, "n2-chem.lua")
gs = GasState(gm)
gs.p = 1.0e5 # Pa
gs.T = 4000.0 # degree K
gs.molef = {'N2':2/3, 'N':1/3}
gs.update_thermo_from_pT()
tFinal = 300.0e-6 # s
t = 0.0
dt = 1.0e-6
dtSuggest = 1.0e-11
while t <= tFinal:
    dtSuggest = reactor.update_state(gs, dt, dtSuggest)
    t = t + dt
    gs.update_thermo_from_rhou()
print(json.dumps(dict(t=t, T=gs.T, p=gs.p, massf=list(gs.massf), conc=list(gs.conc))))
'''


def run_with_reference_binding(script, tmp_path, standin=None):
    """Runs `script` in a fresh interpreter that imports the reference's gdtk.gas over this library."""
    import gdtk_gb300
    libdir = tmp_path / "lib"
    libdir.mkdir()
    os.symlink(os.path.abspath(gdtk_gb300.LIB_PATH), str(libdir / "libgas.so"))
    if standin is None:
        try:
            import cffi   # noqa: F401
            standin = False
        except ImportError:
            standin = True
    paths = [os.path.join(GOLDEN, "ref_gdtk")] + ([os.path.join(GOLDEN, "cffi_standin")] if standin else [])
    env = dict(os.environ, LD_LIBRARY_PATH=str(libdir) + os.pathsep + os.environ.get("LD_LIBRARY_PATH", ""),
               PYTHONPATH=os.pathsep.join(paths + [ROOT]), PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", script], cwd=MECH, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_reference_gas_py_runs_the_fixed_volume_reactor_test(tmp_path):
    from math import isclose
    out = run_with_reference_binding(FVREACTOR, tmp_path)
    assert isclose(out["t"], 300.0e-6, rel_tol=1.0e-6)
    assert isclose(out["T"], 6177.3, rel_tol=1.0e-4)
    assert isclose(out["p"], 145.518e3, rel_tol=1.0e-4)
    assert isclose(out["massf"][0], 8.692812671003e-01, rel_tol=1.0e-4)
    assert isclose(out["massf"][1], 1.307187328997e-01, rel_tol=1.0e-4)
    assert isclose(out["conc"][0], 2.178123112237e+00, rel_tol=1.0e-4)
    assert isclose(out["conc"][1], 6.550733441684e-01, rel_tol=1.0e-4)
