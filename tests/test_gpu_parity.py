"""Parity of the CUDA chemistry path with the CPU oracle, cell by cell, through the C ABI.

Bars (from the engine's specification): every mass fraction within 1e-8 absolute and T, p
within 1e-7 relative of the oracle, which restates the reference's CPU chemistry update
and is itself pinned to the reference's known-answer tests (tests/test_oracle_kat.py).
"""
import os

import numpy as np
import pytest

import oracle
from conftest import mech

pytestmark = pytest.mark.gpu

Y_ABS = 1.0e-8
TP_REL = 1.0e-7


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


@pytest.fixture(scope="module")
def park5():
    from gdtk_gb300.cells import ReactorCells
    return ReactorCells(mech("park5-gas.lua"), mech("park5-chem.lua")), oracle.Oracle(mech("park5-gas.lua"),
                                                                                        mech("park5-chem.lua"))


@pytest.fixture(scope="module")
def j92():
    from gdtk_gb300.cells import ReactorCells
    return ReactorCells(mech("j92-gas.lua"), mech("j92-chem.lua")), oracle.Oracle(mech("j92-gas.lua"),
                                                                                    mech("j92-chem.lua"))


def to_dev(torch, *arrs):
    return [torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda") for a in arrs]


KERNELS = {"fast": 0, "reference_order": 4}


def run_pair(rc, orc, T, p, Y, dt, dt_chem0=-1.0, T_frozen=0.0, flags=3, kernel="fast"):
    """Same inputs through the GPU and the oracle; returns (gpu dict, oracle dict, rho, u)."""
    torch = torch_cuda()
    n = T.shape[0]
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    torch.cuda.synchronize()
    rho_h, u_h = rho.cpu().numpy(), u.cpu().numpy()
    dtc = torch.full((n,), dt_chem0, dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros((6, n), dtype=torch.int32, device="cuda")
    rc.update(rho, u, dT, dp, dY, dtc, dt, status=st, T_frozen=T_frozen, flags=flags | KERNELS[kernel],
              cell_counters=cnt)
    torch.cuda.synchronize()
    g = dict(T=dT.cpu().numpy(), p=dp.cpu().numpy(), Y=dY.cpu().numpy(), dt_chem=dtc.cpu().numpy(),
             status=st.cpu().numpy(), counters=cnt.cpu().numpy())
    o = orc.chem_update(rho_h, u_h, T, p, Y.T, np.full(n, dt_chem0), dt, T_frozen=T_frozen,
                        update_thermo=bool(flags & 1), retry=bool(flags & 2), counters=True)
    return g, o, rho_h, u_h


def assert_parity(g, o, min_same_path=0.99):
    assert np.array_equal(g["status"], o["status"]), "per-cell status differs"
    ok = g["status"] == 0
    dY = np.abs(g["Y"] - o["massf"].T)[:, ok]
    relT = np.abs(g["T"] - o["T"])[ok] / np.abs(o["T"][ok])
    relp = np.abs(g["p"] - o["p"])[ok] / np.abs(o["p"][ok])
    assert dY.max(initial=0.0) <= Y_ABS, "max |dY| = %g" % dY.max()
    assert relT.max(initial=0.0) <= TP_REL, "max rel dT = %g" % relT.max()
    assert relp.max(initial=0.0) <= TP_REL, "max rel dp = %g" % relp.max()
    # The integrators take the same path (same attempts and right-hand-side evaluations)
    # on nearly every cell; a differing path comes only from a step-acceptance test that
    # sits within rounding of its threshold.
    same = (g["counters"][0] == o["counters"][:, 0]) & (g["counters"][1] == o["counters"][:, 1])
    assert same.mean() >= min_same_path, "only %.4f of cells took the oracle's path" % same.mean()


def test_thermo_pT_and_rhou(park5):
    from gdtk_gb300.workloads import air5_cells
    torch = torch_cuda()
    rc, orc = park5
    T, p, Y = air5_cells(2048, seed=11)
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    rho_o, u_o = orc.update_thermo_from_pT(p, T, Y.T)
    assert np.allclose(rho.cpu().numpy(), rho_o, rtol=1e-13, atol=0)
    assert np.allclose(u.cpu().numpy(), u_o, rtol=1e-12, atol=1e-6)
    # round trip: T from (rho, u) starting 5% off
    T2 = dT * 1.05
    p2 = torch.zeros_like(dp)
    st = torch.zeros(2048, dtype=torch.int32, device="cuda")
    rc.thermo_from_rhou(rho, u, dY, T2, p2, status=st)
    torch.cuda.synchronize()
    assert int(st.abs().sum()) == 0
    assert np.allclose(T2.cpu().numpy(), T, rtol=1e-9)
    assert np.allclose(p2.cpu().numpy(), p, rtol=1e-9)
    To, po, sto = orc.update_thermo_from_rhou(rho.cpu().numpy(), u.cpu().numpy(), Y.T, T * 1.05)
    assert np.allclose(T2.cpu().numpy(), To, rtol=1e-12)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_air5_rkf_parity(park5, kernel):
    from gdtk_gb300.workloads import air5_cells
    rc, orc = park5
    T, p, Y = air5_cells(1024, seed=0)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert (g["status"] == 0).all()
    assert_parity(g, o)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_air5_warm_start_parity(park5, kernel):
    from gdtk_gb300.workloads import air5_cells
    rc, orc = park5
    T, p, Y = air5_cells(512, seed=5)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, dt_chem0=1.0e-9, kernel=kernel)
    assert_parity(g, o)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_h2air_alpha_qss_tight_parity(j92, kernel):
    from gdtk_gb300.workloads import h2air_cells
    rc, orc = j92
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 512, seed=3, gas_file=rc.gmodel.file_name)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert (g["status"] == 0).mean() > 0.95
    assert_parity(g, o)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_gupta_given_backward_rates_parity(kernel):
    from gdtk_gb300.cells import ReactorCells
    rc = ReactorCells(mech("gupta5-gas.lua"), mech("gupta5-chem.lua"))
    orc = oracle.Oracle(mech("gupta5-gas.lua"), mech("gupta5-chem.lua"))
    rng = np.random.Generator(np.random.PCG64(7))
    n = 256
    T = rng.uniform(3000.0, 9000.0, n)
    p = 10.0 ** rng.uniform(3.0, 5.0, n)
    Y = np.ascontiguousarray(rng.dirichlet(np.ones(5), n).T)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert_parity(g, o)


def test_frozen_and_bad_cells(park5):
    from gdtk_gb300.workloads import air5_cells
    torch = torch_cuda()
    rc, orc = park5
    T, p, Y = air5_cells(64, seed=2)
    T[:8] = 250.0            # at or below T_frozen -> untouched
    g, o, rho, u = run_pair(rc, orc, T, p, Y, 1.0e-6, T_frozen=300.0)
    assert (g["status"][:8] == oracle.ST_FROZEN).all()
    assert np.array_equal(g["T"][:8], T[:8]) and np.array_equal(g["Y"][:, :8], Y[:, :8])
    assert_parity(g, o)
    # invalid density: status BAD_INPUT, state untouched
    dT, dp, dY = to_dev(torch, T, p, Y)
    drho, du = to_dev(torch, rho, u)
    drho[10] = -1.0
    drho[11] = float("nan")
    st = torch.zeros(64, dtype=torch.int32, device="cuda")
    dtc = torch.full((64,), -1.0, dtype=torch.float64, device="cuda")
    rc.update(drho, du, dT, dp, dY, dtc, 1.0e-6, status=st, T_frozen=300.0)
    torch.cuda.synchronize()
    s = st.cpu().numpy()
    assert s[10] == oracle.ST_BAD_INPUT and s[11] == oracle.ST_BAD_INPUT
    assert dT[10].item() == T[10] and dT[11].item() == T[11]


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_temperature_edges_match_the_oracle(j92, kernel):
    # The fast kernel compares doubles on their bit patterns (rate-constant clamp, curve segment and blend
    # window, the mixture-coefficient range, the extrapolation beyond the curves): cells that start exactly
    # on, just below and just above each of those edges take the oracle's branch.  J92: T limits 300 K and
    # 50,000 K; CEA breaks 200 / 1000 / 6000 K with blend windows [800, 1200] and [5500, 6500]; the
    # mixture-coefficient range ends at 5,500 K.
    from gdtk_gb300.workloads import h2air_cells
    rc, orc = j92
    edges = [150.0, 199.99999, 200.0, 250.0, 300.0, 300.00001, 799.99999, 800.0, 800.00001, 1199.99999, 1200.0,
             1200.00001, 5499.99999, 5500.0, 5500.00001, 6499.99999, 6500.0, 6500.00001]
    per = 4
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, len(edges) * per, seed=23, gas_file=rc.gmodel.file_name)
    T = np.repeat(np.array(edges), per)
    p = np.full(T.shape, 1.0e5)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-7, kernel=kernel)
    assert_parity(g, o, min_same_path=0.9)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_failure_restores_state_and_retry(tmp_path, kernel):
    # A mechanism allowed only 3 subcycles cannot finish 1e-6 s from a fresh start: both the
    # first try and the dt_chem = -1 retry hit maxSubcycles; the cell is left as it was.
    from gdtk_gb300.cells import ReactorCells
    from gdtk_gb300.workloads import air5_cells
    src = open(mech("park5-chem.lua")).read().replace("maxSubcycles = 10000", "maxSubcycles = 3")
    chem = tmp_path / "park5-short.lua"
    chem.write_text(src)
    rc = ReactorCells(mech("park5-gas.lua"), str(chem))
    orc = oracle.Oracle(mech("park5-gas.lua"), str(chem))
    T, p, Y = air5_cells(64, seed=9)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert (g["status"] == oracle.ST_MAX_SUBCYCLES).all()
    assert np.array_equal(g["T"], T) and np.array_equal(g["Y"], Y) and np.array_equal(g["p"], p)
    assert np.array_equal(g["status"], o["status"])


def test_empty_batch(park5):
    torch = torch_cuda()
    rc, _ = park5
    z = torch.zeros(0, dtype=torch.float64, device="cuda")
    rc.update(z, z, z.clone(), z.clone(), torch.zeros((5, 0), dtype=torch.float64, device="cuda"), z.clone(), 1e-6)
    torch.cuda.synchronize()


def test_host_entry_point_matches_device(park5):
    from gdtk_gb300.workloads import air5_cells
    torch = torch_cuda()
    rc, _ = park5
    T, p, Y = air5_cells(300, seed=4)
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    rho_h, u_h = rho.cpu().numpy(), u.cpu().numpy()
    dtc = torch.full((300,), -1.0, dtype=torch.float64, device="cuda")
    rc.update(rho, u, dT, dp, dY, dtc, 1e-6)
    torch.cuda.synchronize()
    Th, ph, Yh, dth = T.copy(), p.copy(), Y.copy(), np.full(300, -1.0)
    nfail = rc.update_host(rho_h, u_h, Th, ph, Yh, dth, 1e-6)
    assert nfail == 0
    assert np.array_equal(Th, dT.cpu().numpy()) and np.array_equal(Yh, dY.cpu().numpy())
    assert np.array_equal(dth, dtc.cpu().numpy())


def test_source_terms(j92):
    from gdtk_gb300.workloads import h2air_cells
    torch = torch_cuda()
    rc, orc = j92
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 128, seed=8, gas_file=rc.gmodel.file_name)
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, _ = rc.thermo_from_pT(dp, dT, dY)
    src = rc.source_terms(rho, dT, dY).cpu().numpy()
    rho_h = rho.cpu().numpy()
    for c in range(0, 128, 7):
        conc = Y[:, c] * rho_h[c] / orc.M
        conc[conc < 1e-30] = 0.0
        q, L, _, _ = orc.split_rates(T[c], conc)
        want = (q - L) * orc.M
        scale = np.abs(want).max() + 1e-300
        assert np.abs(src[:, c] - want).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", ["park5", "c2h2"])
def test_gas_state_properties_match_oracle(name):
    """Cv, Cp, gamma, R, u, h, s, the frozen sound speed and per-species h, s, g of a gas state
    (gas_cwrap.d:610-824 over therm_perf_gas_mix.d:230-364) from the oracle's species curves, and
    the (rho, p) update (therm_perf_gas_mix.d:75-79)."""
    from gdtk_gb300.gas import GasModel, GasState
    gm = GasModel(mech(name + "-gas.lua"))
    orc = oracle.Oracle(mech(name + "-gas.lua"))
    nsp = gm.n_species
    Y = np.random.default_rng(3).dirichlet(np.full(nsp, 0.5))
    gs = GasState(gm)
    gs.massf = list(Y)
    T, p = 2345.0, 2.5e5
    gs.T, gs.p = T, p
    gs.update_thermo_from_pT()
    R_i = 8.31451 / orc.M
    th = np.array([orc.species_thermo(i, T) for i in range(nsp)])   # Cp, h, s per species
    lp = np.log(p / 101325.0)
    cv, cp = np.sum(Y * (th[:, 0] - R_i)), np.sum(Y * th[:, 0])
    R = np.sum(Y * R_i)
    want = dict(Cv=cv, Cp=cp, gamma=cp / cv, R=R, internal_energy=np.sum(Y * (th[:, 1] - R_i * T)),
                enthalpy=np.sum(Y * th[:, 1]), entropy=np.sum(Y * (th[:, 2] - R_i * lp)),
                a=np.sqrt(cp / cv * R * T))
    for k, v in want.items():
        assert np.isclose(getattr(gs, k), v, rtol=1e-12, atol=0), k
    assert np.isclose(gm.dpdrho_const_T(gs), R * T, rtol=1e-12, atol=0)
    for i in range(0, nsp, max(1, nsp // 9)):
        h, s = gm.enthalpy_isp(gs, i), gm.entropy_isp(gs, i)
        assert np.isclose(h, th[i, 1], rtol=1e-13, atol=0)
        assert np.isclose(s, th[i, 2] - R_i[i] * lp, rtol=1e-13, atol=0)
        assert gm.gibbs_free_energy_isp(gs, i) == h - T * s
    g2 = GasState(gm)
    g2.massf = list(Y)
    g2.rho, g2.p = gs.rho, gs.p
    g2.update_thermo_from_rhop()
    assert np.isclose(g2.T, T, rtol=1e-13) and np.isclose(g2.u, gs.u, rtol=1e-12)
    assert g2.a == gs.a or np.isclose(g2.a, gs.a, rtol=1e-13)


def test_fixed_volume_reactor_through_gas_api():
    # examples/kinetics/fixed-volume-reactor-n2/test_fvreactor.py through the mirrored gdtk.gas API
    from gdtk_gb300.gas import GasModel, PyGasState as GasState, ThermochemicalReactor
    from math import isclose
    gm = GasModel(mech("n2-gas.lua"))
    reactor = ThermochemicalReactor(gm, mech("n2-chem.lua"))
    gs = GasState(gm)
    gs.p = 1.0e5
    gs.T = 4000.0
    gs.molef = {'N2': 2 / 3, 'N': 1 / 3}
    gs.update_thermo_from_pT()
    tFinal = 300.0e-6
    t = 0.0
    dt = 1.0e-6
    dtSuggest = 1.0e-11
    while t <= tFinal:
        dtSuggest = reactor.update_state(gs, dt, dtSuggest)
        t = t + dt
        gs.update_thermo_from_rhou()
    assert isclose(t, tFinal, rel_tol=1.0e-6)
    assert isclose(gs.T, 6177.3, rel_tol=1.0e-4)
    assert isclose(gs.p, 145.518e3, rel_tol=1.0e-4)
    assert isclose(gs.massf[0], 8.692812671003e-01, rel_tol=1.0e-4)
    assert isclose(gs.massf[1], 1.307187328997e-01, rel_tol=1.0e-4)
    assert isclose(gs.conc[0], 2.178123112237e+00, rel_tol=1.0e-4)
    assert isclose(gs.conc[1], 6.550733441684e-01, rel_tol=1.0e-4)


def test_h2_i2_full_update_kat():
    # kinetics/chemistry_update.d:736-750 through the per-state C ABI
    from gdtk_gb300.gas import GasModel, GasState, ThermochemicalReactor
    from math import isclose
    gm = GasModel(mech("h2i2-gas.lua"))
    reactor = ThermochemicalReactor(gm, mech("h2i2-chem.lua"))
    gs = GasState(gm)
    gs.T = 700.0
    gs.p = 2.0 * 4.54 * 8.31451 * 700.0
    gs.molef = [0.5, 0.5, 0.0]
    gs.update_thermo_from_pT()
    reactor.update_state(gs, 60_000.0, 200.0)
    assert isclose(7.14201983840, gs.conc[2], rel_tol=1.0e-9)


def test_tickrates_match_oracle():
    from gdtk_gb300.gas import GasModel, GasState, ReactionMechanism
    gm = GasModel(mech("j92-gas.lua"))
    rm = ReactionMechanism(gm, mech("j92-chem.lua"))
    orc = oracle.Oracle(mech("j92-gas.lua"), mech("j92-chem.lua"), T_limits=(300.0, 30000.0))
    gs = GasState(gm)
    gs.T = 1500.0
    gs.p = 1.0e5
    gs.molef = {'H2': 0.25, 'O2': 0.15, 'N2': 0.5, 'H2O': 0.05, 'OH': 0.02, 'H': 0.02, 'O': 0.01}
    gs.update_thermo_from_pT()
    f = np.array(rm.forward_tickrates(gs))
    b = np.array(rm.backward_tickrates(gs))
    conc = np.array(gs.conc)
    _, _, wf, wb = orc.split_rates(1500.0, conc)
    assert np.allclose(f, wf, rtol=1e-13, atol=0) and np.allclose(b, wb, rtol=1e-13, atol=0)


def test_block_batch_equals_per_block_updates(j92):
    # Cells are independent: one launch over uneven blocks with their own intervals gives each
    # cell exactly the result of updating its block alone.
    from gdtk_gb300.workloads import h2air_cells
    torch = torch_cuda()
    rc, _ = j92
    sizes, dts = [300, 37, 1200], [1e-7, 1e-5, 1e-6]
    blocks, solo = [], []
    for k, (n, dt) in enumerate(zip(sizes, dts)):
        T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, n, seed=20 + k, gas_file=rc.gmodel.file_name)
        dT, dp, dY = to_dev(torch, T, p, Y)
        rho, u = rc.thermo_from_pT(dp, dT, dY)
        mk = lambda: dict(rho=rho, u=u, T=dT.clone(), p=dp.clone(), massf=dY.clone(),
                          dt_chem=torch.full((n,), -1.0, dtype=torch.float64, device="cuda"),
                          status=torch.zeros(n, dtype=torch.int32, device="cuda"), t_interval=dt)
        blocks.append(mk())
        solo.append(mk())
    rc.update_blocks(blocks)
    for b in solo:
        rc.update(b["rho"], b["u"], b["T"], b["p"], b["massf"], b["dt_chem"], b["t_interval"], status=b["status"])
    torch.cuda.synchronize()
    for b, s in zip(blocks, solo):
        for key in ("T", "p", "massf", "dt_chem", "status"):
            assert torch.equal(b[key], s[key]), key


def test_block_batch_graph_replay_matches_direct_calls(j92):
    # One split step captured once as a CUDA graph and replayed twice (dt_chem carried) gives the
    # same cells as two direct calls.
    from gdtk_gb300.workloads import h2air_cells
    torch = torch_cuda()
    rc, _ = j92
    def make():
        out = []
        for k, (n, dt) in enumerate(zip([200, 50], [1e-6, 1e-5])):
            T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, n, seed=60 + k, gas_file=rc.gmodel.file_name)
            dT, dp, dY = to_dev(torch, T, p, Y)
            rho, u = rc.thermo_from_pT(dp, dT, dY)
            out.append(dict(rho=rho, u=u, T=dT, p=dp, massf=dY,
                            dt_chem=torch.full((n,), -1.0, dtype=torch.float64, device="cuda"),
                            status=torch.zeros(n, dtype=torch.int32, device="cuda"), t_interval=dt))
        return out
    direct, graphed = make(), make()
    rc.update_blocks(direct)
    rc.update_blocks(direct)
    warm = make()
    rc.update_blocks(warm)            # sizes the scratch before capture
    torch.cuda.synchronize()
    table = rc.block_table(graphed)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc.update_blocks(graphed, table=table)
        g.replay()
        g.replay()
    torch.cuda.synchronize()
    for a, b in zip(direct, graphed):
        for key in ("T", "p", "massf", "dt_chem", "status"):
            assert torch.equal(a[key], b[key]), key


def test_autotuner_picks_a_fitting_shape(j92, tmp_path, monkeypatch):
    from gdtk_gb300 import autotune
    from gdtk_gb300.workloads import h2air_cells
    torch = torch_cuda()
    monkeypatch.setenv("GDTK_JIT_CACHE", str(tmp_path))
    monkeypatch.setattr(autotune, "SHAPES", [(256, 1), (128, 1)])
    rc, orc = j92
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 2048, seed=70, gas_file=rc.gmodel.file_name)
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    sample = dict(rho=rho, u=u, T=dT, p=dp, massf=dY, dt_chem=torch.full((2048,), -1.0, dtype=torch.float64,
                                                                         device="cuda"))
    choice, oflag, results = autotune.tune(rc, sample, 1e-6, tag="test")
    # 2 shapes x 2 orders, 2 refill chunks on the best, one warp per cell
    assert len(results) == 7
    assert sorted({r["refill_chunk"] for r in results}) == [0] + autotune.CHUNKS
    assert [r["cells_per_warp"] for r in results].count(1) == 1
    if choice["cells_per_warp"] == 32:
        assert (choice["block"], choice["min_blocks"]) in [(256, 1), (128, 1)]
    assert os.path.exists(os.path.join(str(tmp_path), "tune.json"))
    again, again_flag, _ = autotune.tune(rc, sample, 1e-6, tag="test")     # from the cache
    assert again["block"] == choice["block"] and again_flag == oflag
    # results still match the oracle under the tuned variant
    g, o, _, _ = run_pair(rc, orc, T[:256], p[:256], np.ascontiguousarray(Y[:, :256]), 1.0e-6, flags=3 | oflag)
    assert_parity(g, o)
    thread_only, tflag, tres = autotune.tune(rc, sample, 1e-6, tag="test", allow_warp=False)
    assert thread_only["cells_per_warp"] == 32 and not tflag & autotune.WARP_PER_CELL and len(tres) == 6
    autotune.check_shape(rc, 0, 0)   # back to the default shape and refill for later tests
    autotune.set_refill_chunk(rc, 0)


@pytest.mark.parametrize("chunk", [32, 128, 4096])
def test_refill_chunk_changes_no_result(j92, chunk):
    """The refill chunk only changes which warp takes which cell: bitwise the same cells."""
    from gdtk_gb300 import autotune
    from gdtk_gb300.workloads import h2air_cells
    torch = torch_cuda()
    rc, _ = j92
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 5000, seed=72, gas_file=rc.gmodel.file_name)
    outs = []
    for cells in (0, chunk):
        autotune.set_refill_chunk(rc, cells)
        dT, dp, dY = to_dev(torch, T, p, Y)
        rho, u = rc.thermo_from_pT(dp, dT, dY)
        dtc = torch.full((5000,), -1.0, dtype=torch.float64, device="cuda")
        st = torch.zeros(5000, dtype=torch.int32, device="cuda")
        rc.update(rho, u, dT, dp, dY, dtc, 1.0e-6, status=st)
        torch.cuda.synchronize()
        outs.append((dT, dp, dY, dtc, st))
    autotune.set_refill_chunk(rc, 0)
    for a, b in zip(*outs):
        assert torch.equal(a, b)


def test_mixing_layer_split_steps_track_the_oracle(j92):
    # In-loop use: 10 split steps of 5e-7 s with dt_chem carried and T_frozen = 300 K on a
    # small mixing-layer block; every step's output feeds the next, on the GPU and in the oracle.
    from gdtk_gb300.workloads import h2air_mixing_layer
    torch = torch_cuda()
    rc, orc = j92
    T, p, Y = h2air_mixing_layer(rc.species_names, rc.mol_masses, nx=4, ny=128, seed=9, thickness=4.0)
    n = T.shape[0]
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    rho_h, u_h = rho.cpu().numpy(), u.cpu().numpy()
    cT, cp, cY, cdt = T.copy(), p.copy(), Y.T.copy(), np.full(n, -1.0)
    for _ in range(10):
        rc.update(rho, u, dT, dp, dY, dtc, 5.0e-7, status=st, T_frozen=300.0)
        o = orc.chem_update(rho_h, u_h, cT, cp, cY, cdt, 5.0e-7, T_frozen=300.0)
        cT, cp, cY, cdt = o["T"], o["p"], o["massf"], o["dt_chem"]
    torch.cuda.synchronize()
    assert np.array_equal(st.cpu().numpy(), o["status"])
    assert np.abs(dY.cpu().numpy() - cY.T).max() <= Y_ABS
    assert (np.abs(dT.cpu().numpy() - cT) / cT).max() <= TP_REL
    assert (o["status"] == 0).any()


def _premixed_cells(names, M, n, seed, majors, T_range=(1100.0, 2500.0), logp=(4.0, 6.0)):
    """Seeded cells: the premixed `majors` (mole ratios) with a 10^U[-6, -2] share of the other
    species (Dirichlet(0.5)), T ~ U[T_range], p = 10^U[logp]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = np.zeros(len(names))
    for s, v in majors.items():
        x[names.index(s)] = v
    y0 = x * M / (x * M).sum()
    minor = [i for i, s in enumerate(names) if s not in majors]
    Y = np.repeat(y0[None, :], n, axis=0)
    share = 10.0 ** rng.uniform(-6.0, -2.0, n)
    Y *= (1.0 - share)[:, None]
    Y[:, minor] += share[:, None] * rng.dirichlet(np.full(len(minor), 0.5), n)
    T = rng.uniform(T_range[0], T_range[1], n)
    p = 10.0 ** rng.uniform(logp[0], logp[1], n)
    return T, p, np.ascontiguousarray(Y.T)


FALLOFF = {"stanford": {'H2': 2.0, 'O2': 1.0, 'N2': 3.76},          # Troe with F_cent given
           "drm19": {'CH4': 1.0, 'O2': 2.0, 'N2': 7.52}}            # Troe with a, T3, T1, T2 (tight coupling)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", sorted(FALLOFF))
def test_pressure_dependent_rates_parity(name, kernel):
    """Troe falloff reactions (third-body concentration from the cell's own composition)."""
    from gdtk_gb300.cells import ReactorCells
    rc = ReactorCells(mech(name + "-gas.lua"), mech(name + "-chem.lua"))
    orc = oracle.Oracle(mech(name + "-gas.lua"), mech(name + "-chem.lua"))
    T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, 384, seed=31, majors=FALLOFF[name])
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert (g["status"] == 0).mean() > 0.95
    assert_parity(g, o)


def test_pressure_dependent_tickrates_match_oracle():
    from gdtk_gb300.gas import GasModel, GasState, ReactionMechanism
    gm = GasModel(mech("drm19-gas.lua"))
    rm = ReactionMechanism(gm, mech("drm19-chem.lua"))
    orc = oracle.Oracle(mech("drm19-gas.lua"), mech("drm19-chem.lua"))
    gs = GasState(gm)
    gs.T = 1800.0
    gs.p = 3.0e5
    gs.molef = {'CH4': 0.08, 'O2': 0.17, 'N2': 0.62, 'H2O': 0.05, 'CO': 0.03, 'CH3': 0.02, 'H': 0.02, 'OH': 0.01}
    gs.update_thermo_from_pT()
    f = np.array(rm.forward_tickrates(gs))
    b = np.array(rm.backward_tickrates(gs))
    conc = np.array(gs.conc)
    _, _, wf, wb = orc.split_rates(1800.0, conc)
    assert np.allclose(f, wf, rtol=1e-12, atol=0) and np.allclose(b, wb, rtol=1e-12, atol=0)


def test_troe_fixed_volume_reactor_on_the_gpu_against_eilmer3():
    """The DRM19 reactor of tests/test_oracle_kat.py, 1,999 chained updates through the GPU's
    mechanism-specialised kernel: same bounds against the Eilmer3 history as the oracle's."""
    import test_oracle_kat as kat
    from gdtk_gb300.cells import ReactorCells
    torch = torch_cuda()
    rc = ReactorCells(mech("drm19-gas.lua"), mech("drm19-chem.lua"))
    st = torch.zeros(1, dtype=torch.int32, device="cuda")

    def update(rho, u, T, p, Y, dtc, dt):
        drho, du, dT, dp, ddt = to_dev(torch, rho, u, T, p, dtc)
        dY = torch.tensor(np.ascontiguousarray(Y[:, None]), dtype=torch.float64, device="cuda")
        rc.update(drho, du, dT, dp, dY, ddt, dt, status=st)
        assert int(st.item()) == 0
        return dT.cpu().numpy(), dp.cpu().numpy(), dY.cpu().numpy()[:, 0], ddt.cpu().numpy()

    Ts = kat.drm19_fixed_volume_reactor(update)
    rel, t_ign, t_ign_ref = kat.compare_with_eilmer3(Ts)
    assert abs(t_ign - t_ign_ref) <= 0.01 * t_ign_ref
    assert rel.max() < 0.03
    assert rel[-1] < 2e-3


def test_kernel_division_against_ieee_division():
    """gdtk_div (Newton-Raphson refinement of the hardware's approximate reciprocal with one
    quotient correction) is within 1 ulp of the IEEE quotient over the whole normal range, and
    gdtk_div_nr (without the correction) within 2 ulp; both equal it for zero, subnormal and
    infinite quotients (which take the IEEE division) and give NaN where it does."""
    import gdtk_gb300
    torch = torch_cuda()
    rng = np.random.Generator(np.random.PCG64(17))
    n = 1 << 20
    a = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-1000, 1000, n)) * rng.choice([-1.0, 1.0], n)
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-1000, 1000, n)) * rng.choice([-1.0, 1.0], n)
    # the chemistry kernels' operand ranges: concentrations, rates, (c + 1e-50), positive denominators
    a[: n // 4] = rng.uniform(0.0, 1.0, n // 4) * 10.0 ** rng.uniform(-40, 10, n // 4)
    b[: n // 4] = rng.uniform(0.0, 1.0, n // 4) * 10.0 ** rng.uniform(-40, 10, n // 4) + 1e-50
    special = np.array([0.0, -0.0, 5e-324, -3e-310, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf,
                        np.nan, 1.0, -1.0, 3.0, 2.0 ** -999, 2.0 ** 1000])
    sa, sb = np.meshgrid(special, special)
    a = np.concatenate([a, sa.ravel()])
    b = np.concatenate([b, sb.ravel()])
    da, db = to_dev(torch, a, b)
    qf, qn, qi = torch.empty_like(da), torch.empty_like(da), torch.empty_like(da)
    assert gdtk_gb300.lib().gdtk_div_device(len(a), da.data_ptr(), db.data_ptr(), qf.data_ptr(), qn.data_ptr(),
                                            qi.data_ptr()) == 0
    qi = qi.cpu().numpy()
    fin = ~np.isnan(qi)
    edge = fin & ((qi == 0.0) | np.isinf(qi) | (np.abs(qi) < 2.2250738585072014e-308))
    for q, bound, exact in ((qf.cpu().numpy(), 1, 0.99), (qn.cpu().numpy(), 2, 0.5)):
        assert np.array_equal(np.isnan(q), np.isnan(qi))
        ulp = np.abs(q[fin].view(np.int64) - qi[fin].view(np.int64))
        assert np.all((np.sign(q[fin]) == np.sign(qi[fin])) | (qi[fin] == 0.0))
        print("max %d ulp, %.4f exact" % (ulp.max(), (ulp == 0).mean()))
        assert ulp.max() <= bound, "largest difference %d ulp" % ulp.max()
        assert (ulp == 0).mean() > exact
        # zero, subnormal and infinite quotients come from the IEEE division itself
        assert np.array_equal(q[edge].view(np.int64), qi[edge].view(np.int64))


@pytest.mark.parametrize("form", [{"GDTK_KB_EXP": "1"}, {"GDTK_KC_UNROLLED": "1"}, {"GDTK_PHASE_CLOCKS": "1"}])
def test_alternate_kernel_forms_parity(form, monkeypatch):
    """The generator's alternate forms (k_b by one exp per reaction, straight-line rate constants,
    phase clocks compiled in) keep parity; the variables are read when a reactor's kernel is
    generated, so each form gets a fresh reactor."""
    from gdtk_gb300.cells import ReactorCells
    from gdtk_gb300.workloads import h2air_cells
    for k, v in form.items():
        monkeypatch.setenv(k, v)
    rc = ReactorCells(mech("j92-gas.lua"), mech("j92-chem.lua"))
    orc = oracle.Oracle(mech("j92-gas.lua"), mech("j92-chem.lua"))
    torch = torch_cuda()
    stats = torch.zeros(24, dtype=torch.int64, device="cuda")
    rc.set_lane_stats(stats)
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 512, seed=3, gas_file=rc.gmodel.file_name)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6)
    rc.set_lane_stats(None)
    assert (g["status"] == 0).mean() > 0.95
    assert_parity(g, o)
    s = stats.cpu().numpy()
    assert s[2] > 0 and s[4] > 0                       # rate-constant and right-hand-side executions counted
    if "GDTK_PHASE_CLOCKS" in form:
        assert (s[16:24][[1, 2, 4, 7]] > 0).all()      # cycles in rate constants, RHS, Newton, alpha update
    else:
        assert (s[16:24] == 0).all()


def test_full_size_h2air_update_properties(j92):
    """The benchmark's full workload (1,048,576 H2-air cells, one update of 1 us from a fresh step
    size) through the fast kernel, checked by properties that do not depend on its size: every cell
    completes, mass fractions are non-negative and sum to 1, p = rho R_mix T, and u recomputed from
    (p, T, Y) is the input u (the update holds rho and u fixed, and T solves u(T) = u to |dT|/T < 1e-10);
    plus cell-by-cell parity with the oracle on a strided sample of 2,000 cells."""
    import bench
    torch = torch_cuda()
    rc, orc = j92
    w = bench.WORKLOADS["h2air-1M"]
    T0, p0, Y0 = bench.make_cells(w, rc.species_names, rc.mol_masses)
    n = T0.shape[0]
    assert n == 1 << 20
    dT, dp = to_dev(torch, T0, p0)
    dY = torch.tensor(np.ascontiguousarray(Y0), dtype=torch.float64, device="cuda")
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc.update(rho, u, dT, dp, dY, dtc, w["dt"], status=st)
    torch.cuda.synchronize()
    assert int((st != 0).sum()) == 0
    assert float(dY.min()) >= 0.0
    assert float((dY.sum(dim=0) - 1.0).abs().max()) <= 1e-13
    R = torch.tensor(8.31451 / np.asarray(rc.mol_masses), dtype=torch.float64, device="cuda")
    p_eos = rho * (dY * R[:, None]).sum(dim=0) * dT
    assert float(((p_eos - dp).abs() / dp).max()) <= 1e-12
    rho2, u2 = rc.thermo_from_pT(dp, dT, dY)
    assert float(((rho2 - rho).abs() / rho).max()) <= 1e-12
    assert float((u2 - u).abs().max()) <= 1e-2   # J/kg: c_v |dT| with |dT| below 1e-10 T
    idx = np.linspace(0, n - 1, 2000).astype(np.int64)
    o = orc.chem_update(rho.cpu().numpy()[idx], u.cpu().numpy()[idx], T0[idx], p0[idx], Y0[:, idx].T,
                        np.full(len(idx), -1.0), w["dt"], counters=True)
    g = dict(T=dT.cpu().numpy()[idx], p=dp.cpu().numpy()[idx], Y=dY.cpu().numpy()[:, idx],
             status=st.cpu().numpy()[idx], counters=None)
    assert np.array_equal(g["status"], o["status"])
    assert np.abs(g["Y"] - o["massf"].T).max() <= Y_ABS
    assert (np.abs(g["T"] - o["T"]) / o["T"]).max() <= TP_REL
    assert (np.abs(g["p"] - o["p"]) / o["p"]).max() <= TP_REL


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_arrhenius2_lindemann_yungster_rabinowitz_parity(kernel):
    # the h2o2forms fixture: Arrhenius2 (one with a B T term), Lindemann-Hinshelwood and
    # Yungster-Rabinowitz forward rates beside Arrhenius and third-body reactions (rate_constant.d:82-355)
    from gdtk_gb300.cells import ReactorCells
    from gdtk_gb300.workloads import h2air_cells
    gas, chem = mech("h2o2forms-gas.lua"), mech("h2o2forms-chem.lua")
    rc, orc = ReactorCells(gas, chem), oracle.Oracle(gas, chem)
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, 512, seed=13, gas_file=gas)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel=kernel)
    assert (g["status"] == 0).mean() > 0.95
    assert_parity(g, o)


def test_rate_forms_tickrates_match_oracle():
    from gdtk_gb300.gas import GasModel, GasState, ReactionMechanism
    gm = GasModel(mech("h2o2forms-gas.lua"))
    rm = ReactionMechanism(gm, mech("h2o2forms-chem.lua"))
    orc = oracle.Oracle(mech("h2o2forms-gas.lua"), mech("h2o2forms-chem.lua"))
    gs = GasState(gm)
    gs.T = 1700.0
    gs.p = 2.0e5
    gs.molef = {'H2': 0.25, 'O2': 0.15, 'N2': 0.45, 'H2O': 0.05, 'OH': 0.02, 'H': 0.02, 'O': 0.01, 'HO2': 0.03,
                'H2O2': 0.02}
    gs.update_thermo_from_pT()
    f = np.array(rm.forward_tickrates(gs))
    b = np.array(rm.backward_tickrates(gs))
    _, _, wf, wb = orc.split_rates(1700.0, np.array(gs.conc))
    assert np.allclose(f, wf, rtol=1e-13, atol=0) and np.allclose(b, wb, rtol=1e-13, atol=0)
