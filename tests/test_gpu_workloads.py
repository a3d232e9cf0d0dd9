"""The benchmark workloads themselves, cell by cell against the oracle (GPU).

- the 4,096-cell Park-air workload exactly as bench.py builds it (bench.WORKLOADS["air5-4096"]),
  both kernels;
- the 64 uneven H2-air blocks of bench.py's h2air-blocks64 workload (block sizes log-uniform in
  [2,048, 524,288], dt in {1e-7, 1e-6, 1e-5} s per block): a sample drawn from every block goes
  through the 20 split steps as one multi-block launch per step, and every step is compared with
  the oracle started from the same state, with per-cell status equality (h_min cells included).

Bars as in test_gpu_parity.py: |dY| <= 1e-8, T and p within 1e-7 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import mech
from test_gpu_parity import KERNELS, Y_ABS, TP_REL, assert_parity, run_pair, to_dev, torch_cuda

pytestmark = pytest.mark.gpu

# (block, cell) of the h2air-blocks64 workload that end a split step with status h_min in the reference
# algorithm (the oracle run over the 20 split steps on 128 strided cells of every block).
BLOCKS64_HMIN_CELLS = [(6, 4455), (43, 2530), (43, 8096), (43, 8602), (43, 13409), (43, 24288), (43, 2024),
                       (43, 16445), (43, 27830), (55, 123865), (55, 130943), (55, 449453)]


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_air5_4096_bench_workload_parity(kernel):
    import bench
    from gdtk_gb300.cells import ReactorCells
    w = bench.WORKLOADS["air5-4096"]
    rc = ReactorCells(mech(w["gas"]), mech(w["chem"]))
    orc = oracle.Oracle(mech(w["gas"]), mech(w["chem"]))
    T, p, Y = bench.make_cells(w)
    assert T.shape == (4096,)
    g, o, _, _ = run_pair(rc, orc, T, p, Y, w["dt"], kernel=kernel)
    assert (g["status"] == 0).all()
    assert_parity(g, o)


def test_h2air_blocks64_split_steps_match_the_oracle_per_step():
    import bench
    from gdtk_gb300.cells import ReactorCells, UPDATE_THERMO, RETRY
    from gdtk_gb300.workloads import h2air_blocks
    torch = torch_cuda()
    w = bench.WORKLOADS["h2air-blocks64"]
    rc = ReactorCells(mech(w["gas"]), mech(w["chem"]))
    orc = oracle.Oracle(mech(w["gas"]), mech(w["chem"]))
    extra = {}
    for b, i in BLOCKS64_HMIN_CELLS:
        extra.setdefault(b, []).append(i)
    pick = lambda b, n: np.unique(np.concatenate([np.arange(0, n, max(n // 32, 1))[:32], extra.get(b, [])]))
    spec = h2air_blocks(rc.species_names, rc.mol_masses, nblocks=w["nblocks"], seed=w["seed"],
                        gas_file=rc.gmodel.file_name, pick=pick)
    blocks = []
    for s in spec:
        idx = s["cells"]
        dT, dp, dY = to_dev(torch, s["T"], s["p"], s["Y"])
        rho, u = rc.thermo_from_pT(dp, dT, dY)
        blocks.append(dict(rho=rho, u=u, T=dT, p=dp, massf=dY, t_interval=s["dt"],
                           dt_chem=torch.full((len(idx),), -1.0, dtype=torch.float64, device="cuda"),
                           status=torch.zeros(len(idx), dtype=torch.int32, device="cuda")))
    assert {b["t_interval"] for b in blocks} == {1e-7, 1e-6, 1e-5}
    flags = UPDATE_THERMO | RETRY
    seen = {}
    for step in range(w["split_steps"]):
        before = [{k: b[k].cpu().numpy().copy() for k in ("rho", "u", "T", "p", "massf", "dt_chem")} for b in blocks]
        rc.update_blocks(blocks, flags=flags)
        torch.cuda.synchronize()
        for b, h in zip(blocks, before):
            o = orc.chem_update(h["rho"], h["u"], h["T"], h["p"], h["massf"].T, h["dt_chem"], b["t_interval"],
                                update_thermo=True, retry=True)
            st = b["status"].cpu().numpy()
            assert np.array_equal(st, o["status"]), "split step %d: per-cell status differs" % step
            for v in np.unique(st):
                seen[int(v)] = seen.get(int(v), 0) + int((st == v).sum())
            ok = st == 0
            gY, gT, gp = b["massf"].cpu().numpy(), b["T"].cpu().numpy(), b["p"].cpu().numpy()
            assert np.abs(gY[:, ok] - o["massf"][ok].T).max(initial=0.0) <= Y_ABS
            assert (np.abs(gT[ok] - o["T"][ok]) / o["T"][ok]).max(initial=0.0) <= TP_REL
            assert (np.abs(gp[ok] - o["p"][ok]) / o["p"][ok]).max(initial=0.0) <= TP_REL
            # a failed cell keeps its input state, as the reference restores it
            bad = ~ok
            assert np.array_equal(gT[bad], h["T"][bad]) and np.array_equal(gY[:, bad], h["massf"][:, bad])
    assert seen.get(oracle.ST_H_MIN, 0) > 0, seen     # the sample does exercise the failure path
    assert seen.get(oracle.ST_OK, 0) > 0.95 * sum(seen.values())
