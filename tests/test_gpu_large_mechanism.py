"""One warp per cell (GDTK_CHEM_WARP_PER_CELL, and every mechanism beyond the thread-per-cell
kernels' 32 species / 128 reactions) against the oracle, through the C ABI.

The warp kernel is the reference-order update with a cell's species and reactions spread over the
lanes; each sum the reference takes in order is still taken in that order, and it is compiled with
FMA contraction, so on the small mechanisms it gives the reference-order kernel's statuses and its
values to rounding (both are held to the oracle's bars).  The large mechanism is
the reference's examples/kinetics/acetylene-ignition-delay model (75 species, 474 reactions: 423
Arrhenius, 50 Troe, 1 Lindemann-Hinshelwood; alpha-QSS), converted by the reference's chemkin2eilmer
and prep_chem (tests/golden/make_fixtures.sh), at that example's mixture (C2H2 0.02, O2 0.025,
Ar 0.955 by mole).  Bars as in test_gpu_parity.py: 1e-8 absolute in Y, 1e-7 relative in T and p.
"""
import numpy as np
import pytest

import oracle
from conftest import mech
from test_gpu_parity import _premixed_cells, assert_parity, run_pair, to_dev, torch_cuda

pytestmark = pytest.mark.gpu

WARP_PER_CELL = 16      # GDTK_CHEM_WARP_PER_CELL
ACETYLENE = {'C2H2': 0.02, 'O2': 0.025, 'Ar': 0.955}


def pair(name):
    from gdtk_gb300.cells import ReactorCells
    return (ReactorCells(mech(name + "-gas.lua"), mech(name + "-chem.lua")),
            oracle.Oracle(mech(name + "-gas.lua"), mech(name + "-chem.lua")))


@pytest.fixture(scope="module")
def c2h2():
    return pair("c2h2")


def _cells(name, rc, n, seed):
    from gdtk_gb300.workloads import air5_cells, h2air_cells
    if name == "park5":
        return air5_cells(n, seed=seed)
    if name == "j92":
        return h2air_cells(rc.species_names, rc.mol_masses, n, seed=seed, gas_file=rc.gmodel.file_name)
    return _premixed_cells(rc.species_names, rc.mol_masses, n, seed=seed, majors={'CH4': 1.0, 'O2': 2.0, 'N2': 7.52})


@pytest.mark.parametrize("name", ["park5", "j92", "drm19"])   # RKF; alpha-QSS tight; Troe, tight coupling
def test_warp_per_cell_matches_the_reference_order_kernel(name):
    rc, orc = pair(name)
    T, p, Y = _cells(name, rc, 384, seed=17)
    g_w, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, flags=3 | WARP_PER_CELL)
    g_r, _, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, kernel="reference_order")
    assert np.array_equal(g_w["status"], g_r["status"])
    ok = g_w["status"] == 0
    assert np.abs(g_w["Y"] - g_r["Y"])[:, ok].max(initial=0.0) <= 1e-8
    for k in ("T", "p"):
        assert (np.abs(g_w[k] - g_r[k]) / np.abs(g_r[k]))[ok].max(initial=0.0) <= 1e-7, k
    same = (g_w["counters"][0] == g_r["counters"][0]) & (g_w["counters"][1] == g_r["counters"][1])
    assert same.mean() >= 0.99
    assert (g_w["status"] == 0).mean() > 0.95
    assert_parity(g_w, o)
    assert_parity(g_r, o)
    last = rc.last_launch()
    assert last["block"] % 32 == 0 and last["grid"] >= 1


@pytest.mark.parametrize("dt", [1.0e-7, 1.0e-6, 1.0e-5])
def test_acetylene_mechanism_parity(c2h2, dt):
    rc, orc = c2h2
    assert (rc.nsp, rc.nr, rc.method) == (75, 474, "alpha-qss")
    T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, 192, seed=41, majors=ACETYLENE,
                              T_range=(1150.0, 2500.0), logp=(4.0, 5.5))
    g, o, _, _ = run_pair(rc, orc, T, p, Y, dt)
    assert (g["status"] == 0).all()
    assert_parity(g, o)


def test_acetylene_warm_start_and_flags(c2h2):
    """A suggested dt_chem carried in, and the update without the thermo call (flags 2)."""
    rc, orc = c2h2
    T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, 96, seed=43, majors=ACETYLENE)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, 1.0e-6, dt_chem0=1.0e-9, flags=2)
    assert_parity(g, o)


def test_acetylene_source_terms_and_tickrates(c2h2):
    """Gas services of a mechanism whose vectors do not fit in shared memory (global scratch)."""
    from gdtk_gb300.gas import GasState, ReactionMechanism
    torch = torch_cuda()
    rc, orc = c2h2
    T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, 64, seed=47, majors=ACETYLENE)
    dT, dp, dY = to_dev(torch, T, p, Y)
    rho, _ = rc.thermo_from_pT(dp, dT, dY)
    src = rc.source_terms(rho, dT, dY).cpu().numpy()
    rho_h = rho.cpu().numpy()
    for c in range(0, 64, 5):
        conc = Y[:, c] * rho_h[c] / orc.M
        conc[conc < 1e-30] = 0.0
        q, L, _, _ = orc.split_rates(T[c], conc)
        want = (q - L) * orc.M
        assert np.abs(src[:, c] - want).max() <= 1e-12 * (np.abs(want).max() + 1e-300)
    rm = ReactionMechanism(rc.gmodel, mech("c2h2-chem.lua"))
    gs = GasState(rc.gmodel)
    gs.T, gs.p = 1650.0, 0.6 * 101325.0
    gs.molef = dict(ACETYLENE, H=1e-4, OH=1e-4, CO=1e-3)
    gs.update_thermo_from_pT()
    f, b = np.array(rm.forward_tickrates(gs)), np.array(rm.backward_tickrates(gs))
    _, _, wf, wb = orc.split_rates(1650.0, np.array(gs.conc))
    assert np.allclose(f, wf, rtol=1e-12, atol=0) and np.allclose(b, wb, rtol=1e-12, atol=0)


def test_acetylene_ignition_chain(c2h2):
    """The example's constant-volume ignition at 1250-1750 K, 0.6 atm: 120 chained 10-us updates on
    the GPU and in the oracle, each side from its own previous state; the time of the largest
    pressure rise and the final state agree."""
    torch = torch_cuda()
    rc, orc = c2h2
    names, M = rc.species_names, rc.mol_masses
    x = np.zeros(rc.nsp)
    for s, v in ACETYLENE.items():
        x[names.index(s)] = v
    y0 = x * M / (x * M).sum()
    T0 = np.array([1250.0, 1450.0, 1650.0, 1750.0])
    n = len(T0)
    p0 = np.full(n, 0.6 * 101325.0)
    Y0 = np.ascontiguousarray(np.repeat(y0[:, None], n, axis=1))
    dT, dp, dY = to_dev(torch, T0, p0, Y0)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    rho_h, u_h = rho.cpu().numpy(), u.cpu().numpy()
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    oT, op, oY, odt = T0.copy(), p0.copy(), Y0.T.copy(), np.full(n, -1.0)
    dt = 1.0e-5
    gp, opr = [p0.copy()], [p0.copy()]
    for _ in range(120):
        rc.update(rho, u, dT, dp, dY, dtc, dt, status=st)
        o = orc.chem_update(rho_h, u_h, oT, op, oY, odt, dt)
        assert int(st.abs().sum()) == 0 and (o["status"] == 0).all()
        oT, op, oY, odt = o["T"], o["p"], o["massf"], o["dt_chem"]
        gp.append(dp.cpu().numpy())
        opr.append(op.copy())
    gp, opr = np.array(gp), np.array(opr)
    assert np.array_equal(np.argmax(np.diff(gp, axis=0), axis=0), np.argmax(np.diff(opr, axis=0), axis=0))
    assert (gp[-1] > 1.4 * p0).all()   # every cell ignited within 1.2 ms (delays 70-470 us)
    assert np.allclose(dT.cpu().numpy(), oT, rtol=1e-6, atol=0)
    assert np.abs(dY.cpu().numpy() - oY.T).max() <= 1e-7


def test_acetylene_block_batch_equals_per_block_updates(c2h2):
    """The block API over three blocks of the large mechanism (one warp per cell, one launch per block)
    gives every block bitwise what a separate update of it gives, and a CUDA graph of that call
    replays it."""
    torch = torch_cuda()
    rc, orc = c2h2

    def make():
        out = []
        for k, (n, dt) in enumerate(zip([300, 40, 129], [1e-6, 1e-5, 1e-7])):
            T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, n, seed=50 + k, majors=ACETYLENE)
            dT, dp, dY = to_dev(torch, T, p, Y)
            rho, u = rc.thermo_from_pT(dp, dT, dY)
            out.append(dict(rho=rho, u=u, T=dT, p=dp, massf=dY,
                            dt_chem=torch.full((n,), -1.0, dtype=torch.float64, device="cuda"),
                            status=torch.zeros(n, dtype=torch.int32, device="cuda"), t_interval=dt))
        return out
    batch, single = make(), make()
    rc.update_blocks(batch)
    for b in single:
        rc.update(b["rho"], b["u"], b["T"], b["p"], b["massf"], b["dt_chem"], b["t_interval"], status=b["status"])
    torch.cuda.synchronize()
    for a, b in zip(batch, single):
        for key in ("T", "p", "massf", "dt_chem", "status"):
            assert torch.equal(a[key], b[key]), key
    graphed = make()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc.update_blocks(graphed)
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(graphed, single):
        for key in ("T", "p", "massf", "dt_chem", "status"):
            assert torch.equal(a[key], b[key]), key


def test_acetylene_results_do_not_depend_on_the_schedule(c2h2):
    # Warps take cells from a work counter, so which warp integrates a cell depends on the batch's order
    # and on timing; a cell's result must not.  The same cells in reversed order give bitwise the same
    # states, statuses and work counters.
    torch = torch_cuda()
    rc, _ = c2h2
    n = 512
    T, p, Y = _premixed_cells(rc.species_names, rc.mol_masses, n, seed=47, majors=ACETYLENE,
                              T_range=(1150.0, 2500.0), logp=(4.0, 5.5))

    def run(order):
        dT, dp, dY = to_dev(torch, T[order], p[order], Y[:, order])
        rho, u = rc.thermo_from_pT(dp, dT, dY)
        dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
        st = torch.zeros(n, dtype=torch.int32, device="cuda")
        cnt = torch.zeros((6, n), dtype=torch.int32, device="cuda")
        rc.update(rho, u, dT, dp, dY, dtc, 1.0e-6, status=st, cell_counters=cnt)
        torch.cuda.synchronize()
        back = np.argsort(order)
        return [a.cpu().numpy()[..., back] for a in (dT, dp, dY, dtc, st, cnt)]

    fwd = run(np.arange(n))
    rev = run(np.arange(n)[::-1].copy())
    for a, b, name in zip(fwd, rev, ("T", "p", "Y", "dt_chem", "status", "counters")):
        assert np.array_equal(a, b), name
    assert (fwd[4] == 0).all()
