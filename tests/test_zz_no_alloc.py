"""The allocation-free entry point (chem_reactor_update_cells_noalloc).

It exists for callers that cannot allocate device memory where they run the chemistry (graph
capture, a fixed memory budget, no device-wide synchronisation mid-step).  It must give the
same cells the same results as chem_reactor_update_cells, on repeated calls that reuse its
static scratch, and refuse batches larger than that scratch.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import mech

pytestmark = pytest.mark.gpu


def _cells(torch, rc, n, seed):
    from gdtk_gb300.workloads import h2air_cells
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, n, seed=seed, gas_file=rc.gmodel.file_name)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    dT, dp, dY = dev(T), dev(p), dev(Y)
    rho, u = rc.thermo_from_pT(dp, dT, dY)
    return rho, u, dT, dp, dY


def _state(torch, base, n):
    rho, u, T, p, Y = base
    return dict(rho=rho, u=u, T=T.clone(), p=p.clone(), massf=Y.clone(),
                dt_chem=torch.full((n,), -1.0, dtype=torch.float64, device="cuda"),
                status=torch.full((n,), -7, dtype=torch.int32, device="cuda"))


def _noalloc(lib, rc, s, n, dt, flags=3):
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    import torch
    return lib.chem_reactor_update_cells_noalloc(
        rc.reactor.id, n, ptr(s["rho"]), ptr(s["u"]), ptr(s["T"]), ptr(s["p"]), ptr(s["massf"]), ptr(s["dt_chem"]),
        ptr(s["status"]), dt, 0.0, flags, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    import gdtk_gb300
    from gdtk_gb300.cells import ReactorCells
    assert torch.cuda.is_available()
    lib = gdtk_gb300.lib()
    rc = ReactorCells(mech("j92-gas.lua"), mech("j92-chem.lua"))
    n, dt = 3000, 1.0e-6
    base = _cells(torch, rc, n, seed=41)
    ref = _state(torch, base, n)
    # the ordinary entry point (it also loads the reactor's kernel)
    rc.update(ref["rho"], ref["u"], ref["T"], ref["p"], ref["massf"], ref["dt_chem"], dt, status=ref["status"])
    torch.cuda.synchronize()
    for _ in range(2):   # two calls in a row reuse (and must reset) the shared scratch
        s = _state(torch, base, n)
        assert _noalloc(lib, rc, s, n, dt) == 0, gdtk_gb300.last_error()
        torch.cuda.synchronize()
        assert torch.equal(s["status"], ref["status"])
        ok = ref["status"] == 0
        assert bool(ok.all())
        # the same generated kernel integrates each cell on its own, so only the visit order may
        # differ between the two calls, and no cell's result depends on it: bitwise equality
        for k in ("massf", "T", "p", "dt_chem"):
            assert torch.equal(s[k], ref[k]), k


def test_noalloc_rejects_batches_beyond_its_scratch():
    import torch
    import gdtk_gb300
    from gdtk_gb300.cells import ReactorCells
    lib = gdtk_gb300.lib()
    rc = ReactorCells(mech("j92-gas.lua"), mech("j92-chem.lua"))
    base = _cells(torch, rc, 64, seed=42)
    s = _state(torch, base, 64)
    rc.update(s["rho"], s["u"], s["T"].clone(), s["p"].clone(), s["massf"].clone(), s["dt_chem"].clone(), 1e-6)
    torch.cuda.synchronize()
    # the size is checked before any array is touched or any kernel is launched
    assert _noalloc(lib, rc, s, (1 << 20) + 1, 1e-6) == -1
    assert "exceed" in gdtk_gb300.last_error()
