"""GPU tests of the chemistry surrogate (include/gdtk_surrogate.h): the BF16 tensor-core GEMM
against an FP64 product of the same BF16 values, the training gradient against the CPU oracle
(oracle/mlp.py), training on samples of the FP64 update, the FP64 gate against its CPU
restatement (oracle/surrogate_gate.py), the fallback cells against the plain update, the
held-out monitor, and what the trained network gains over the update without it."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import mlp
from oracle import surrogate_gate as sgate
from conftest import mech

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


@pytest.fixture(scope="module")
def rc():
    from gdtk_gb300.cells import ReactorCells
    return ReactorCells(mech("j92-gas.lua"), mech("j92-chem.lua"))


@pytest.fixture(scope="module")
def samples(rc):
    """4,194,304 samples of the FP64 update of seeded H2-air cells (dt log-uniform in [0.5, 2] us)."""
    from gdtk_gb300.surrogate import ChemSurrogate, generate_samples
    sg = ChemSurrogate(rc, width=256, depth=4, seed=1)
    X, Y, valid, _ = generate_samples(rc, sg, 4194304, seed=11)
    rows = torch.nonzero(valid).flatten().to(torch.int32)
    return X, Y, rows


@pytest.fixture(scope="module")
def trained(rc, samples):
    from gdtk_gb300.surrogate import ChemSurrogate
    X, Y, rows = samples
    n = rows.shape[0]
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    perm = rows[torch.randperm(n, generator=g, device="cuda")]
    hold = perm[: n // 20].contiguous()
    train = perm[n // 20:].contiguous()
    sg = ChemSurrogate(rc, width=256, depth=4, seed=2)
    sg.fit_normalisation(X, Y, train)
    before = sg.heldout_error(X, Y, hold)
    hist = sg.train(X, Y, train, epochs=20, batch=8192, lr=2e-3)
    after = sg.heldout_error(X, Y, hold)
    return sg, hist, before, after


@pytest.mark.parametrize("ta,tb", [(0, 1), (0, 0), (1, 0)])
@pytest.mark.parametrize("M,N,K,act,bias,splits", [(200, 256, 16, 1, True, 1), (1000, 256, 256, 1, True, 1),
                                                   (256, 16, 4104, 0, False, 4), (512, 24, 272, 0, True, 1)])
def test_gemm_matches_fp64_product_of_bf16_values(ta, tb, M, N, K, act, bias, splits):
    from gdtk_gb300 import lib, check
    g = torch.Generator(device="cuda")
    g.manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((K, N), generator=g, device="cuda").to(torch.bfloat16)
    b = torch.randn(N, generator=g, device="cuda") if bias else None
    As = A.t().contiguous() if ta else A.contiguous()
    Bs = B.t().contiguous() if tb else B.contiguous()
    lda = M if ta else K
    ldb = K if tb else N
    D = torch.empty((M, N), device="cuda")
    Dh = torch.empty((M, N), device="cuda", dtype=torch.bfloat16) if splits == 1 else None
    pre = torch.empty((M, N), device="cuda") if act else None
    check(lib().gdtk_mlp_gemm(M, N, K, _ptr(As), lda, ta, _ptr(Bs), ldb, tb, _ptr(b), act, _ptr(pre), _ptr(D),
                              _ptr(Dh), N, splits, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
          "gdtk_mlp_gemm")
    torch.cuda.synchronize()
    ref = A.double() @ B.double()
    if bias:
        ref = ref + b.double()
    scale = (A.double().abs() @ B.double().abs()).clamp_min(1e-30)
    if act:
        assert ((pre.double() - ref).abs() / scale).max().item() < 1e-6
        z = ref
        ref = 0.5 * z * (1.0 + torch.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))
        err = ((D.double() - ref).abs() / (scale + 1.0)).max().item()
        assert err < 2e-6
    else:
        assert ((D.double() - ref).abs() / scale).max().item() < 1e-6
    if Dh is not None:
        assert ((Dh.double() - D.double()).abs() <= D.double().abs() * 2 ** -8 + 1e-30).all()


def test_training_gradient_matches_cpu_oracle(rc, samples):
    from gdtk_gb300.surrogate import ChemSurrogate
    X, Y, rows = samples
    sg = ChemSurrogate(rc, width=256, depth=4, seed=3)
    sg.fit_normalisation(X, Y, rows)
    batch = rows[:1024].contiguous()
    grad, loss = sg.gradients(X, Y, batch)
    grad = grad.cpu().numpy().astype(np.float64)
    nrm = sg.get_normalisation()
    xb = X[batch.long()].cpu().numpy()
    yb = Y[batch.long()].cpu().numpy()
    Xs = ((xb - nrm["x_shift"]) / nrm["x_scale"]).astype(np.float32)
    Ys = ((yb - nrm["y_shift"]) / nrm["y_scale"]).astype(np.float32).astype(np.float64)
    w = np.zeros(sg.nout_pad)
    w[:sg.nout] = 1.0
    layers = [(W.astype(np.float64), b.astype(np.float64)) for W, b in sg.unpack(sg.get_params())]
    L_bf, g_bf = mlp.loss_and_grads(layers, Xs, Ys, w, bf=True)
    L_64, g_64 = mlp.loss_and_grads(layers, Xs.astype(np.float64), Ys, w, bf=False)
    rels = []
    for (dW, db), (oW, ob), (fW, fb) in zip(sg.unpack(grad), g_bf, g_64):
        for got, ref, ref64 in ((dW, oW, fW), (db, ob, fb)):
            rels.append((np.linalg.norm(got - ref) / np.linalg.norm(ref),
                         np.linalg.norm(got - ref64) / np.linalg.norm(ref64)))
    info = (loss / 1024, L_bf, L_64, rels)
    assert loss / 1024 == pytest.approx(L_bf, rel=1e-2), info
    assert loss / 1024 == pytest.approx(L_64, rel=2e-2), info
    assert max(r for r, _ in rels) < 1e-2, info
    assert max(r for _, r in rels) < 8e-2, info


def test_training_reduces_heldout_error(trained):
    sg, hist, before, after = trained
    assert hist[-1] < 0.05 * hist[0]
    assert np.median(after[0]) < 0.1 * np.median(before[0])
    assert np.median(after[0]) < 1e-3
    assert np.median(after[1]) < 1e-3


def _fresh_cells(rc, n, seed):
    from gdtk_gb300.workloads import h2air_cells
    T, p, Y = h2air_cells(rc.species_names, rc.mol_masses, n, seed=seed, gas_file=rc.gmodel.file_name)
    d = dict(T=torch.tensor(T, device="cuda"), p=torch.tensor(p, device="cuda"),
             massf=torch.tensor(np.ascontiguousarray(Y), device="cuda"))
    d["rho"], d["u"] = rc.thermo_from_pT(d["p"], d["T"], d["massf"])
    d["dt_chem"] = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    d["status"] = torch.zeros(n, dtype=torch.int32, device="cuda")
    return d


def _clone(d):
    return {k: v.clone() for k, v in d.items()}


def test_gate_matches_cpu_restatement(rc, trained):
    sg, *_ = trained
    sg.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=5e-3, max_dY=0.0)
    n = 4096
    d = _fresh_cells(rc, n, seed=21)
    d0 = _clone(d)
    # the raw predictions the gate sees (features rounded as in training)
    X, _, _ = sg.make_samples(d0["T"], d0["p"], d0["massf"], 1e-6, d0["T"], d0["massf"], None)
    pred = sg.predict(X).double().cpu().numpy()
    gate = torch.empty(n, dtype=torch.int32, device="cuda")
    res = sg.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"], gate=gate)
    codes = gate.cpu().numpy()
    assert sum(res["gate"].values()) == n
    orc = oracle.Oracle(mech("j92-gas.lua"))
    els, E, EM = sgate.element_matrix(mech("j92-gas.lua"))
    nrm = sg.get_normalisation()
    c0 = {k: v.cpu().numpy() for k, v in d0.items()}
    nsp = rc.nsp
    ref, Y1, T1, p1 = sgate.gate(orc, E, EM, c0["rho"], c0["u"], c0["T"], c0["p"], c0["massf"].T,
                                 pred[:, :nsp], pred[:, nsp], nrm["x_min"], nrm["x_max"], 1e-6, 0.0,
                                 elem_tol=1e-4, neg_tol=1e-5, T_tol=5e-3)
    agree = (codes == ref).mean()
    assert agree > 0.995, (agree, np.bincount(codes, minlength=9), np.bincount(ref, minlength=9))
    both = (codes == sgate.ACCEPTED) & (ref == sgate.ACCEPTED)
    assert both.sum() > 0.1 * n
    Yg = d["massf"].cpu().numpy().T
    assert np.abs(Yg[both] - Y1[both]).max() < 1e-8
    assert (np.abs(d["T"].cpu().numpy()[both] - T1[both]) / T1[both]).max() < 1e-7
    # accepted cells conserve every element to rounding and hold no negative mass fraction
    dE = (E @ (Yg[both] - c0["massf"].T[both]).T) * EM[:, None]
    assert np.abs(dE).max() < 1e-12
    assert Yg[both].min() >= 0.0


def test_fallback_cells_equal_the_plain_update(rc, trained):
    sg, *_ = trained
    sg.set_gate(elem_tol=1e-5, neg_tol=1e-6, T_tol=1e-3, max_dY=1e-3)
    n = 8192
    d = _fresh_cells(rc, n, seed=22)
    d["T"][:16] = 250.0                       # frozen cells
    d0 = _clone(d)
    gate = torch.empty(n, dtype=torch.int32, device="cuda")
    res = sg.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"], gate=gate,
                    T_frozen=300.0)
    rc.update(d0["rho"], d0["u"], d0["T"], d0["p"], d0["massf"], d0["dt_chem"], 1e-6, status=d0["status"],
              T_frozen=300.0)
    codes = gate.cpu().numpy()
    assert res["gate"]["frozen"] == 16 and (codes[:16] == sgate.FROZEN).all()
    fb = (codes != sgate.ACCEPTED) & (codes != sgate.FROZEN) & (codes != sgate.BAD_INPUT)
    assert fb.sum() == res["fallback"] > 0
    fbt = torch.tensor(fb, device="cuda")
    for k in ("T", "p", "dt_chem", "status"):
        assert torch.equal(d[k][fbt], d0[k][fbt]), k
    assert torch.equal(d["massf"][:, fbt], d0["massf"][:, fbt])
    assert torch.equal(d["status"][:16], d0["status"][:16])      # frozen flagged as the plain update does
    assert torch.equal(d["T"][:16], d0["T"][:16])


def test_monitor_reports_the_error_against_the_fp64_update(rc, trained):
    sg, *_ = trained
    sg.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=5e-3, max_dY=0.0)
    n = 4096
    d = _fresh_cells(rc, n, seed=23)
    d0 = _clone(d)
    gate = torch.empty(n, dtype=torch.int32, device="cuda")
    res = sg.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"], gate=gate,
                    monitor_stride=1)
    rc.update(d0["rho"], d0["u"], d0["T"], d0["p"], d0["massf"], d0["dt_chem"], 1e-6, status=d0["status"])
    acc = (gate == 0) & (d0["status"] == 0)
    eY = (d["massf"][:, acc] - d0["massf"][:, acc]).abs().amax(dim=0)
    eT = (d["T"][acc] - d0["T"][acc]).abs() / d0["T"][acc]
    m = res["monitor"]
    assert m["cells"] == int(acc.sum())
    assert m["max_dY"] == pytest.approx(eY.max().item(), rel=1e-12)
    assert m["max_rel_dT"] == pytest.approx(eT.max().item(), rel=1e-12)
    assert m["mean_max_dY"] == pytest.approx(eY.mean().item(), rel=1e-9)


def test_trained_network_gains_over_the_update_without_it(rc, trained):
    """At one gate setting (magnitude cap 2e-3): the trained network takes over cells that carry
    a share of the FP64 work, within an error bound checked against the FP64 update, while the
    same network untrained is rejected almost everywhere."""
    from gdtk_gb300.surrogate import ChemSurrogate
    sg, *_ = trained
    n = 16384
    base = _fresh_cells(rc, n, seed=24)
    ref = _clone(base)
    tot_plain = torch.zeros(6, dtype=torch.int64, device="cuda")
    rc.update(ref["rho"], ref["u"], ref["T"], ref["p"], ref["massf"], ref["dt_chem"], 1e-6, status=ref["status"],
              totals=tot_plain)
    results = {}
    for name, net in (("trained", sg), ("untrained", ChemSurrogate(rc, width=256, depth=4, seed=9))):
        if name == "untrained":
            net.load_state_dict(dict(sg.state_dict(), params=net.get_params()))
        net.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=1e-3, max_dY=2e-3)
        d = _clone(base)
        gate = torch.empty(n, dtype=torch.int32, device="cuda")
        res = net.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"],
                         gate=gate)
        acc = (gate == 0) & (ref["status"] == 0)
        rej = (gate != 0)
        # FP64 work left to the fallback: the plain update of the rejected cells alone
        sub = {k: (v[:, rej] if k == "massf" else v[rej]).contiguous() for k, v in base.items()}
        tot = torch.zeros(6, dtype=torch.int64, device="cuda")
        rc.update(sub["rho"], sub["u"], sub["T"], sub["p"], sub["massf"], sub["dt_chem"], 1e-6, status=sub["status"],
                  totals=tot)
        err = (d["massf"][:, acc] - ref["massf"][:, acc]).abs().amax(dim=0)
        errT = ((d["T"][acc] - ref["T"][acc]).abs() / ref["T"][acc])
        results[name] = dict(accepted=float(acc.float().mean()), work=float(tot[1]) / float(tot_plain[1]),
                             max_dY=float(err.max()) if acc.any() else 0.0,
                             max_dT=float(errT.max()) if acc.any() else 0.0, gate=res["gate"])
    t, u = results["trained"], results["untrained"]
    print(results)
    assert t["accepted"] > 0.2, results
    assert t["work"] < 0.9, results                # FP64 right-hand sides left to the fallback
    assert t["max_dY"] < 5e-3 and t["max_dT"] < 2e-2, results
    assert u["accepted"] < 0.1 * t["accepted"], results


def test_surrogate_on_another_mechanism():
    """The surrogate is mechanism-generic: 5-species air (elements N, O; RKF) trained briefly,
    then updated with the fallback; accepted cells conserve N and O, rejected ones equal the
    plain update."""
    from gdtk_gb300.cells import ReactorCells
    from gdtk_gb300.surrogate import ChemSurrogate, generate_samples
    from gdtk_gb300.workloads import air5_cells
    rc = ReactorCells(mech("park5-gas.lua"), mech("park5-chem.lua"))
    sg = ChemSurrogate(rc, width=64, depth=2, seed=5)
    assert (sg.nin, sg.nin_pad, sg.nout, sg.nout_pad, sg.n_elements) == (8, 8, 6, 8, 2)
    X, Y, valid, _ = generate_samples(rc, sg, 131072, seed=3, block=32768, blocks_per_launch=4,
                                      cells=lambda m, s: air5_cells(m, seed=s))
    rows = torch.nonzero(valid).flatten().to(torch.int32)
    sg.fit_normalisation(X, Y, rows)
    hist = sg.train(X, Y, rows, epochs=4, batch=4096)
    assert hist[-1] < hist[0]
    sg.set_gate(elem_tol=1e-3, neg_tol=1e-4, T_tol=1e-2, max_dY=0.0)
    T, p, Yc = air5_cells(4096, seed=99)
    d = {"T": torch.tensor(T, device="cuda"), "p": torch.tensor(p, device="cuda"),
         "massf": torch.tensor(np.ascontiguousarray(Yc), device="cuda")}
    d["rho"], d["u"] = rc.thermo_from_pT(d["p"], d["T"], d["massf"])
    d["dt_chem"] = torch.full((4096,), -1.0, dtype=torch.float64, device="cuda")
    d["status"] = torch.zeros(4096, dtype=torch.int32, device="cuda")
    d0 = _clone(d)
    gate = torch.empty(4096, dtype=torch.int32, device="cuda")
    res = sg.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"], gate=gate)
    assert sum(res["gate"].values()) == 4096
    rc.update(d0["rho"], d0["u"], d0["T"], d0["p"], d0["massf"], d0["dt_chem"], 1e-6, status=d0["status"])
    codes = gate.cpu().numpy()
    rej = torch.tensor(codes != 0, device="cuda")
    assert torch.equal(d["massf"][:, rej], d0["massf"][:, rej]) and torch.equal(d["T"][rej], d0["T"][rej])
    acc = codes == 0
    if acc.any():
        els, E, EM = sgate.element_matrix(mech("park5-gas.lua"))
        dE = (E @ (d["massf"].cpu().numpy()[:, acc] - Yc[:, acc])) * EM[:, None]
        assert np.abs(dE).max() < 1e-12


def test_largest_batch_indexing():
    """2^24 + 13 cells (a ragged size) in one call: a strided sample of cells, including the last,
    matches the oracle."""
    from gdtk_gb300.cells import ReactorCells
    from gdtk_gb300.workloads import air5_cells
    rc = ReactorCells(mech("park5-gas.lua"), mech("park5-chem.lua"))
    orc = oracle.Oracle(mech("park5-gas.lua"), mech("park5-chem.lua"))
    n = (1 << 24) + 13
    T, p, Y = air5_cells(n, seed=12)
    d = {"T": torch.tensor(T, device="cuda"), "p": torch.tensor(p, device="cuda"),
         "massf": torch.tensor(np.ascontiguousarray(Y), device="cuda")}
    d["rho"], d["u"] = rc.thermo_from_pT(d["p"], d["T"], d["massf"])
    d["dt_chem"] = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    d["status"] = torch.zeros(n, dtype=torch.int32, device="cuda")
    rho, u = d["rho"].cpu().numpy(), d["u"].cpu().numpy()
    rc.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"])
    idx = np.concatenate([np.arange(0, n, n // 2000), [n - 1]])
    o = orc.chem_update(rho[idx], u[idx], T[idx], p[idx], Y[:, idx].T, np.full(len(idx), -1.0), 1e-6)
    g_st = d["status"].cpu().numpy()[idx]
    assert np.array_equal(g_st, o["status"])
    ok = g_st == 0
    gY = d["massf"].cpu().numpy()[:, idx].T
    assert np.abs(gY[ok] - o["massf"][ok]).max() <= 1e-8
    gT = d["T"].cpu().numpy()[idx]
    assert (np.abs(gT[ok] - o["T"][ok]) / o["T"][ok]).max() <= 1e-7


@pytest.fixture(scope="module")
def with_error_model(rc, samples, trained):
    """The trained network with an error model trained on the same samples (quantile 0.9)."""
    sg, *_ = trained
    X, Y, rows = samples
    sg.add_error_model(width=128, depth=2, seed=4)
    hist = sg.train_error_model(X, Y, rows, epochs=4, batch=8192, quantile=0.9)
    return sg, hist


def test_error_model_gradient_matches_cpu_oracle(rc, samples):
    from gdtk_gb300.surrogate import ChemSurrogate
    X, Y, rows = samples
    sg = ChemSurrogate(rc, width=256, depth=4, seed=7)
    sg.fit_normalisation(X, Y, rows)
    sg.add_error_model(width=64, depth=2, seed=8)
    batch = rows[:1024].contiguous()
    grad, loss = sg.error_gradients(X, Y, batch, quantile=0.9)
    grad = grad.cpu().numpy().astype(np.float64)
    nrm = sg.get_normalisation()
    xb, yb = X[batch.long()].cpu().numpy(), Y[batch.long()].cpu().numpy()
    Xs = ((xb - nrm["x_shift"]) / nrm["x_scale"]).astype(np.float32)
    Ys = ((yb - nrm["y_shift"]) / nrm["y_scale"]).astype(np.float32).astype(np.float64)
    # the increment network's output as the GPU computed it (standardised back from predict)
    raw = sg.predict(X[batch.long()].contiguous()).cpu().numpy()
    out = ((raw - nrm["y_shift"]) / nrm["y_scale"]).astype(np.float32).astype(np.float64)
    nsp = rc.nsp
    err = np.abs((out[:, :nsp] - Ys[:, :nsp]) * nrm["y_scale"][:nsp]).max(axis=1)
    # with the temperature increment's error relative to T, weighted 0.1 (1e-3 in T counts as 1e-4 in Y)
    errT = np.abs((out[:, nsp] - Ys[:, nsp]) * nrm["y_scale"][nsp]) / np.exp(xb[:, 0].astype(np.float64))
    err = np.maximum(err, 0.1 * errT)
    tgt = np.zeros((1024, sg.err_nout_pad))
    tgt[:, 0] = np.log10(err + 1e-12)
    feat = np.concatenate([mlp.bf16(Xs), mlp.bf16(out)], axis=1)
    dims = sg.error_layer_dims()
    flat = sg.get_error_params().astype(np.float64)
    layers, off = [], 0
    ws = []
    for l in range(len(dims) - 1):
        ws.append(flat[off:off + dims[l] * dims[l + 1]].reshape(dims[l + 1], dims[l]))
        off += dims[l] * dims[l + 1]
    for l in range(len(dims) - 1):
        layers.append((ws[l], flat[off:off + dims[l + 1]]))
        off += dims[l + 1]
    L, g = mlp.loss_and_grads(layers, feat, tgt, np.ones(sg.err_nout_pad), bf=True, quantile=0.9)
    goff = 0
    gw = []
    for l in range(len(dims) - 1):
        gw.append(grad[goff:goff + dims[l] * dims[l + 1]].reshape(dims[l + 1], dims[l]))
        goff += dims[l] * dims[l + 1]
    rels = []
    for l in range(len(dims) - 1):
        gb = grad[goff:goff + dims[l + 1]]
        goff += dims[l + 1]
        for got, ref in ((gw[l], g[l][0]), (gb, g[l][1])):
            rels.append(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30))
    info = (loss / 1024, L, rels)
    assert loss / 1024 == pytest.approx(L, rel=2e-2), info
    assert max(rels) < 3e-2, info


def test_error_model_ranks_the_surrogate_errors(samples, with_error_model):
    """On held-out samples the error model's estimate follows the actual error, and a cell it
    accepts at 1e-3 has a smaller error than the magnitude cap alone guarantees."""
    sg, hist = with_error_model
    assert hist[-1] < hist[0]
    X, Y, rows = samples
    hold = rows[-20000:]
    Xh, Yh = X[hold.long()].contiguous(), Y[hold.long()]
    pred = sg.predict(Xh)
    eT = (pred[:, sg.nout - 1] - Yh[:, sg.nout - 1]).abs() / torch.exp(Xh[:, 0])
    actual = torch.log10(torch.maximum((pred[:, :sg.nout - 1] - Yh[:, :sg.nout - 1]).abs().amax(dim=1), 0.1 * eT)
                         + 1e-12).cpu().numpy()
    est = sg.predict_error(Xh).cpu().numpy()
    rank = lambda v: np.argsort(np.argsort(v))
    assert np.corrcoef(rank(est), rank(actual))[0, 1] > 0.6
    below = (actual <= est).mean()
    assert 0.75 < below < 0.98   # the 0.9 quantile, approximately


def test_error_gate_in_the_update(rc, with_error_model):
    sg, _ = with_error_model
    n = 16384
    base = _fresh_cells(rc, n, seed=25)
    ref = _clone(base)
    rc.update(ref["rho"], ref["u"], ref["T"], ref["p"], ref["massf"], ref["dt_chem"], 1e-6, status=ref["status"])
    out = {}
    for tol in (0.0, 1e-3):
        sg.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=1e-3, max_dY=0.0)
        sg.set_error_gate(tol)
        d = _clone(base)
        gate = torch.empty(n, dtype=torch.int32, device="cuda")
        res = sg.update(d["rho"], d["u"], d["T"], d["p"], d["massf"], d["dt_chem"], 1e-6, status=d["status"],
                        gate=gate)
        acc = (gate == 0) & (ref["status"] == 0)
        e = (d["massf"][:, acc] - ref["massf"][:, acc]).abs().amax(dim=0)
        out[tol] = dict(acc=float(acc.float().mean()), p999=float(torch.quantile(e.double(), 0.999)),
                        rejected_by_model=res["gate"]["predicted_error"])
    sg.set_error_gate(0.0)
    assert out[0.0]["rejected_by_model"] == 0 and out[1e-3]["rejected_by_model"] > 0
    assert out[1e-3]["acc"] > 0.3
    assert out[1e-3]["p999"] < out[0.0]["p999"], out
