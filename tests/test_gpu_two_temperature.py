"""The two-temperature reactor on the GPU (chem_reactor2t_*), cell by cell against the oracle
(oracle/two_temperature_reactor.py, restating kinetics/multi_temperature_thermochemical_reactor.d),
on Park's 5-species 2-T air with Landau-Teller exchange and Marrone-Treanor coupling (the inputs of
examples/lmr/3D/cylinder-larc through prep-gas, prep-chem and prep-kinetics).

Bars as for the one-temperature reactor: |dY| <= 1e-8, T, T_ve and p within 1e-7 relative.
"""
import numpy as np
import pytest

from conftest import mech
from test_gpu_parity import torch_cuda, to_dev

pytestmark = pytest.mark.gpu

FILES = (mech("park2t-gas.lua"), mech("park2t-chem.lua"), mech("park2t-eem.lua"))
# the same air with Marrone-Treanor / modified Marrone-Treanor dissociation rates and couplings
FILES_MT = (mech("park2t-gas.lua"), mech("park2tmt-chem.lua"), mech("park2tmt-eem.lua"))


def _cells(n, seed):
    """Non-equilibrium air (gdtk_gb300.workloads.air2t_cells, the bench's air2t workload)."""
    from gdtk_gb300.workloads import air2t_cells
    return air2t_cells(n, seed=seed)


def test_two_temperature_thermo_from_pT():
    from oracle.two_temperature import TwoTemperatureGas
    from gdtk_gb300.cells import ReactorCells2T
    torch = torch_cuda()
    rc = ReactorCells2T(*FILES)
    gas = TwoTemperatureGas(FILES[0])
    T, Tve, p, Y = _cells(256, seed=3)
    dT, dTve, dp, dY = to_dev(torch, T, Tve, p, Y)
    rho, u, uve = rc.thermo_from_pT(dp, dT, dTve, dY)
    torch.cuda.synchronize()
    ref = np.array([gas.update_from_pT(p[k], T[k], Tve[k], Y[:, k]) for k in range(256)])
    assert np.allclose(rho.cpu().numpy(), ref[:, 0], rtol=1e-13, atol=0)
    assert np.allclose(u.cpu().numpy(), ref[:, 1], rtol=1e-12, atol=1e-6)
    assert np.allclose(uve.cpu().numpy(), ref[:, 2], rtol=1e-12, atol=1e-6)


@pytest.mark.parametrize("files", [FILES, FILES_MT], ids=["impartial", "marrone-treanor"])
def test_two_temperature_update_matches_the_oracle(files):
    from oracle.two_temperature_reactor import TwoTemperatureReactor, ReactorFailure
    from gdtk_gb300.cells import ReactorCells2T
    torch = torch_cuda()
    rc = ReactorCells2T(*files)
    orc = TwoTemperatureReactor(*files)
    n, dt = 96, 1.0e-6
    T, Tve, p, Y = _cells(n, seed=7)
    dT, dTve, dp, dY = to_dev(torch, T, Tve, p, Y)
    rho, u0, uve0 = rc.thermo_from_pT(dp, dT, dTve, dY)
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    st = torch.full((n,), -9, dtype=torch.int32, device="cuda")
    u, uve = torch.empty_like(rho), torch.empty_like(rho)
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc.update(rho, dT, dTve, dp, dY, dtc, dt, status=st, u=u, u_ve=uve, steps=steps)
    torch.cuda.synchronize()
    g = dict(T=dT.cpu().numpy(), Tve=dTve.cpu().numpy(), p=dp.cpu().numpy(), Y=dY.cpu().numpy(),
             st=st.cpu().numpy(), u=u.cpu().numpy(), uve=uve.cpu().numpy(), dt=dtc.cpu().numpy())
    rho_h = rho.cpu().numpy()
    total = 0
    for k in range(n):
        try:
            o = orc.update(rho_h[k], T[k], Tve[k], p[k], Y[:, k], dt)
        except ReactorFailure as f:
            assert g["st"][k] == f.code
            continue
        total += o["steps"]
        assert g["st"][k] == 0
        assert np.abs(g["Y"][:, k] - o["massf"]).max() <= 1e-8
        for key, ok in (("T", "T"), ("Tve", "Tve"), ("p", "p")):
            assert abs(g[key][k] - o[ok]) <= 1e-7 * abs(o[ok]), (k, key, g[key][k], o[ok])
        assert abs(g["uve"][k] - o["u_ve"]) <= 1e-7 * max(abs(o["u_ve"]), 1.0)
        assert g["dt"][k] == pytest.approx(o["dt_suggest"], rel=1e-6)
    assert (g["st"] == 0).mean() > 0.95
    # total energy is carried over: u + u_ve after the update equals it before
    ok = g["st"] == 0
    assert np.allclose((g["u"] + g["uve"])[ok], (u0 + uve0).cpu().numpy()[ok], rtol=1e-12, atol=1e-3)
    assert int(steps.item()) >= total


def test_two_temperature_results_do_not_depend_on_the_schedule():
    # The update's persistent grid hands cells to lanes from a work counter, so which lane integrates a
    # cell, and beside which others, depends on the order of the batch and on timing.  A cell's result
    # must not: the same cells in reversed order give bitwise the same states, statuses and step counts.
    from gdtk_gb300.cells import ReactorCells2T
    torch = torch_cuda()
    rc = ReactorCells2T(*FILES)
    n, dt = 4096, 1.0e-6
    T, Tve, p, Y = _cells(n, seed=19)

    def run(order):
        dT, dTve, dp, dY = to_dev(torch, T[order], Tve[order], p[order], Y[:, order])
        rho, _, _ = rc.thermo_from_pT(dp, dT, dTve, dY)
        dtc = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
        st = torch.zeros(n, dtype=torch.int32, device="cuda")
        rc.update(rho, dT, dTve, dp, dY, dtc, dt, status=st)
        torch.cuda.synchronize()
        back = np.argsort(order)
        return [a.cpu().numpy()[..., back] for a in (dT, dTve, dp, dY, dtc, st)]

    fwd = run(np.arange(n))
    rev = run(np.arange(n)[::-1].copy())
    for a, b, name in zip(fwd, rev, ("T", "T_ve", "p", "Y", "dt_chem", "status")):
        assert np.array_equal(a, b), name
    assert (fwd[5] == 0).mean() > 0.95
