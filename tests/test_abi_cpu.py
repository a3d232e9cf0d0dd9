"""CPU-only checks of the C ABI library: it loads, exports what include/gdtk_chem.h declares,
reads the reference's gas/mechanism files like the oracle's independent reader, compiles its
mechanism kernels with NVRTC, and refuses GPU work loudly when there is no GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import gdtk_gb300
import oracle
from conftest import mech, ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared_functions():
    text = "\n".join(open(h).read() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    L = gdtk_gb300.lib()
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding table covers all of them
    assert sorted(gdtk_gb300.SIGNATURES) == names


@pytest.mark.parametrize("name", ["park5", "j92", "gupta5", "n2", "h2i2", "stanford", "drm19", "c2h2"])
def test_gas_model_reader_matches_oracle_reader(name):
    from gdtk_gb300.gas import GasModel
    gm = GasModel(mech(name + "-gas.lua"))
    names, species = oracle.load_gas(mech(name + "-gas.lua"))
    assert gm.species_names == names
    assert np.array_equal(np.array(gm.mol_masses), np.array([s["M"] for s in species]))
    assert gm.n_modes == 0


def test_reader_rejects_wrong_species_order(tmp_path):
    from gdtk_gb300.gas import GasModel
    src = open(mech("park5-chem.lua")).read().replace("[0]='N2', [1]='O2'", "[0]='O2', [1]='N2'")
    bad = tmp_path / "bad.lua"
    bad.write_text(src)
    L = gdtk_gb300.lib()
    gm = GasModel(mech("park5-gas.lua"))
    assert L.thermochemical_reactor_new(gm.id, str(bad).encode(), b"") == -1
    assert "Species order" in gdtk_gb300.last_error() or "CUDA" in gdtk_gb300.last_error()


def test_unsupported_rate_model_is_refused(tmp_path):
    src = open(mech("park5-chem.lua")).read().replace("model='Arrhenius', A=7.0", "model='Park', A=7.0", 1)
    bad = tmp_path / "park.lua"
    bad.write_text(src)
    L = gdtk_gb300.lib()
    n = L.gdtk_generate_fast_source(mech("park5-gas.lua").encode(), str(bad).encode(), None, 0)
    assert n == -1 and "not supported" in gdtk_gb300.last_error()


def test_large_mechanism_is_read_and_routed_to_the_warp_kernel():
    """The 75-species, 474-reaction acetylene model: both readers take it, the oracle holds all of
    it, and the mechanism-specialised (thread-per-cell) generator refuses it with the reason."""
    gas, chem = mech("c2h2-gas.lua"), mech("c2h2-chem.lua")
    names, _ = oracle.load_gas(gas)
    assert len(names) == 75
    rx, _ = oracle.load_mechanism(chem, names)
    assert len(rx) == 474
    orc = oracle.Oracle(gas, chem)
    kf, kb = orc.rate_constants(1500.0, np.full(75, 1e-3))
    assert kf.shape == (474,) and np.isfinite(kf).all() and np.isfinite(kb).all()
    L = gdtk_gb300.lib()
    assert L.gdtk_generate_fast_source(gas.encode(), chem.encode(), None, 0) == -1
    assert "one warp per cell" in gdtk_gb300.last_error()


def test_gpu_work_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gdtk_gb300.gas import GasModel, GasState
    gm = GasModel(mech("park5-gas.lua"))
    gs = GasState(gm)
    gs.p, gs.T = 1e5, 3000.0
    gs.massf = [0.2] * 5
    with pytest.raises(gdtk_gb300.ChemError, match="GPU"):
        gm.update_thermo_from_pT(gs)


def test_table_driven_exp_accuracy():
    rng = np.random.Generator(np.random.PCG64(3))
    x = np.concatenate([rng.uniform(-745.0, 709.7, 200000), rng.uniform(-40.0, 40.0, 200000),
                        np.array([0.0, 1.0, -1.0, 709.78, -745.0, -708.4, 1e-300, -1e-300])])
    y = np.empty_like(x)
    gdtk_gb300.lib().gdtk_exp_host(len(x), x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    ref = np.exp(x.astype(np.longdouble))
    ok = np.isfinite(y) & (ref > np.finfo(np.float64).tiny)
    ulp = np.spacing(ref[ok].astype(np.float64))
    err = np.abs((y[ok].astype(np.longdouble) - ref[ok]) / ulp.astype(np.longdouble))
    assert float(err.max()) <= 1.5, float(err.max())
    assert y[-8] == 1.0


@pytest.mark.parametrize("name", ["park5", "j92", "stanford", "drm19"])
def test_mechanism_kernel_compiles_for_sm103a(name):
    log = gdtk_gb300.compile_fast_source_check(mech(name + "-gas.lua"), mech(name + "-chem.lua"))
    assert "sm_103a" in log
    m = re.search(r"Used (\d+) registers", log)
    assert m and int(m.group(1)) <= 255


def _kc_modes(source):
    """Mode of every record of the generated rate-constant table (0: k_b from K_c by exp, 1: both
    Arrhenius, 2: k_f from K_c, 3: k_b from the species' exp(G/RT) products)."""
    if "GDTK_KC_TAB" not in source:
        return []
    tab = source[source.index("GDTK_KC_TAB"):source.index("};", source.index("GDTK_KC_TAB"))]
    return [int(m) for m in re.findall(r"^\s*\{(?:[^,{]*,){7}\s*(\d),", tab, flags=re.M)]


def _source(gas, chem):
    L = gdtk_gb300.lib()
    buf = ctypes.create_string_buffer(1 << 22)
    assert L.gdtk_generate_fast_source(gas.encode(), chem.encode(), buf, len(buf)) > 0
    return buf.value.decode()


def test_rate_constant_table_forms(monkeypatch):
    # H2-air: every reaction's k_b from the species' exp(G/RT) products; the exp form is compiled out
    src = _source(mech("j92-gas.lua"), mech("j92-chem.lua"))
    assert _kc_modes(src) == [3] * 33
    assert "#if 0   // every table reaction takes the product form" in src
    # both directions Arrhenius stay in the exp form
    assert set(_kc_modes(_source(mech("gupta5-gas.lua"), mech("gupta5-chem.lua")))) == {1}
    monkeypatch.setenv("GDTK_KB_EXP", "1")
    assert _kc_modes(_source(mech("j92-gas.lua"), mech("j92-chem.lua"))) == [0] * 33
    monkeypatch.delenv("GDTK_KB_EXP")
    monkeypatch.setenv("GDTK_KC_UNROLLED", "1")
    assert _kc_modes(_source(mech("j92-gas.lua"), mech("j92-chem.lua"))) == []


def test_product_form_refused_where_it_could_overflow(tmp_path):
    """At 300 K the N atom's G/RT is about 170, so N2 <=> 2N stays inside exp(+-600); with the lower
    temperature limit at 20 K it reaches about 2,800 and the reaction keeps the exp form."""
    assert set(_kc_modes(_source(mech("n2-gas.lua"), mech("n2-chem.lua")))) == {3}
    cold = tmp_path / "n2-cold-chem.lua"
    cold.write_text(open(mech("n2-chem.lua")).read().replace("lower=300.000000", "lower=20.000000"))
    assert set(_kc_modes(_source(mech("n2-gas.lua"), str(cold)))) == {0}


def test_rate_forms_fixture_generates_and_compiles():
    """Arrhenius2 (rate_constant.d:82-121), Lindemann-Hinshelwood and Yungster-Rabinowitz forms: the
    reader takes them, Arrhenius2 stays out of the ln A / n / C table, and the kernel compiles."""
    gas, chem = mech("h2o2forms-gas.lua"), mech("h2o2forms-chem.lua")
    src = _source(gas, chem)
    assert len(_kc_modes(src)) == 6              # r3..r7 and r13 in the table; r1, r2, r11, lh, yr straight-line
    assert "fma(%s, T, " % float.hex(2.0e-5) in src            # the B T term of r2 (hex literal)
    assert "#define GDTK_NFALLOFF 2" in src
    log = gdtk_gb300.compile_fast_source_check(gas, chem)
    assert "sm_103a" in log


def test_arrhenius_logA_is_the_same_model(tmp_path):
    # createRateConstant (rate_constant.d:574-577) maps 'Arrhenius-logA' and 'Arrhenius2' to one class
    alias = tmp_path / "alias-chem.lua"
    alias.write_text(open(mech("h2o2forms-chem.lua")).read().replace("model='Arrhenius2'", "model='Arrhenius-logA'"))
    gas = mech("h2o2forms-gas.lua")
    assert _source(gas, str(alias)) == _source(gas, mech("h2o2forms-chem.lua"))
    conc = np.linspace(0.5, 6.5, 13)
    a = oracle.Oracle(gas, str(alias)).rate_constants(1500.0, conc)
    b = oracle.Oracle(gas, mech("h2o2forms-chem.lua")).rate_constants(1500.0, conc)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


GAS_MODEL_INFO = r'''
import json
from gdtk.gas import GasModel
gm = GasModel("j92-gas.lua")
print(json.dumps(dict(type=gm.type_str, n=gm.n_species, modes=gm.n_modes, names=gm.species_names,
                      M=list(gm.mol_masses))))
'''


@pytest.mark.parametrize("standin", [False, True])
def test_reference_gas_py_opens_this_library(tmp_path, standin):
    """The reference's unmodified gdtk/gas.py loads this library as its libgas.so and reads a gas model
    (the calls that need no GPU), with the real cffi and with the stand-in the GPU machines use."""
    if not standin:
        pytest.importorskip("cffi")
    from test_gpu_ref_binding import run_with_reference_binding
    out = run_with_reference_binding(GAS_MODEL_INFO, tmp_path, standin=standin)
    names, species = oracle.load_gas(mech("j92-gas.lua"))
    assert out["names"] == names and out["n"] == 13 and out["modes"] == 0
    assert np.array_equal(np.array(out["M"]), np.array([s["M"] for s in species]))
    assert out["type"] in ("CompositeGas", "ThermallyPerfectGas")
