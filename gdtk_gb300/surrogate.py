"""Learned surrogate of the chemistry update with FP64 fallback (include/gdtk_surrogate.h).

The network maps (ln T, ln p, Y, ln dt) of a cell to its increment (dY, dT) over dt.  Its
training samples are produced by the FP64 chemistry update itself (ReactorCells), its
training step (BF16 tensor-core forward and backward, AdamW) and its inference run in the
library's own kernels, and every prediction is checked in FP64 before it is used: cells that
fail a check are integrated by the plain update (chem_surrogate_update_cells).

This has no counterpart in the reference.
"""
import ctypes
import math
import time

import numpy as np

from . import lib, check
from .cells import ReactorCells, UPDATE_THERMO, RETRY, _ptr, _stream, _f64

GATE_NAMES = ["accepted", "frozen", "bad_input", "domain", "elements", "negative", "energy", "newton", "magnitude",
              "predicted_error"]


def _vp(a):
    return ctypes.c_void_p(a.ctypes.data)


class ChemSurrogate:
    """A surrogate network for the reactor of `rc` (a ReactorCells)."""

    def __init__(self, rc, width=256, depth=4, seed=0):
        self.rc = rc
        self.id = check(lib().chem_surrogate_new(rc.reactor.id, int(width), int(depth), ctypes.c_ulonglong(seed)),
                        "chem_surrogate_new")
        d = (ctypes.c_int * 8)()
        check(lib().chem_surrogate_dims(self.id, d), "chem_surrogate_dims")
        (self.nin, self.nin_pad, self.nout, self.nout_pad, self.width, self.depth, self.n_params,
         self.n_elements) = list(d)

    def __del__(self):
        try:
            lib().chem_surrogate_free(self.id)
        except Exception:
            pass

    # ---------------------------------------------------------------- parameters
    def layer_dims(self):
        return [self.nin_pad] + [self.width] * self.depth + [self.nout_pad]

    def get_params(self):
        out = np.empty(self.n_params, np.float32)
        check(lib().chem_surrogate_get_params(self.id, _vp(out)), "chem_surrogate_get_params")
        return out

    def set_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        assert params.shape == (self.n_params,)
        check(lib().chem_surrogate_set_params(self.id, _vp(params)), "chem_surrogate_set_params")

    def unpack(self, flat):
        """[(W_l, b_l)] views of a flat parameter (or gradient) vector."""
        dims = self.layer_dims()
        ws, off = [], 0
        for l in range(self.depth + 1):
            n = dims[l] * dims[l + 1]
            ws.append(flat[off:off + n].reshape(dims[l + 1], dims[l]))
            off += n
        out = []
        for l in range(self.depth + 1):
            out.append((ws[l], flat[off:off + dims[l + 1]]))
            off += dims[l + 1]
        return out

    def get_normalisation(self):
        xs, xd, xmin, xmax = (np.empty(self.nin_pad, t) for t in (np.float32, np.float32, np.float64, np.float64))
        ys, yd = (np.empty(self.nout_pad, np.float32) for _ in range(2))
        check(lib().chem_surrogate_get_normalisation(self.id, _vp(xs), _vp(xd), _vp(ys), _vp(yd), _vp(xmin),
                                                     _vp(xmax)), "chem_surrogate_get_normalisation")
        return dict(x_shift=xs, x_scale=xd, y_shift=ys, y_scale=yd, x_min=xmin, x_max=xmax)

    def set_normalisation(self, x_shift, x_scale, y_shift, y_scale, x_min, x_max):
        a = [np.ascontiguousarray(v, t) for v, t in ((x_shift, np.float32), (x_scale, np.float32),
                                                     (y_shift, np.float32), (y_scale, np.float32),
                                                     (x_min, np.float64), (x_max, np.float64))]
        check(lib().chem_surrogate_set_normalisation(self.id, *[_vp(v) for v in a]), "chem_surrogate_set_normalisation")

    def state_dict(self):
        return dict(params=self.get_params(), **self.get_normalisation())

    def load_state_dict(self, sd):
        self.set_params(sd["params"])
        self.set_normalisation(sd["x_shift"], sd["x_scale"], sd["y_shift"], sd["y_scale"], sd["x_min"], sd["x_max"])

    def set_loss_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.shape == (self.nout,)
        check(lib().chem_surrogate_set_loss_weights(self.id, _vp(w)), "chem_surrogate_set_loss_weights")

    def set_gate(self, elem_tol=1e-4, neg_tol=1e-5, T_tol=1e-3, max_dY=5e-4):
        check(lib().chem_surrogate_set_gate(self.id, float(elem_tol), float(neg_tol), float(T_tol), float(max_dY)),
              "chem_surrogate_set_gate")

    # ---------------------------------------------------------------- samples and training
    def make_samples(self, T0, p0, Y0, dt, T1, Y1, status, X=None, Y=None, valid=None):
        """Raw samples of n cells advanced by dt: X (n, nin_pad), Y (n, nout_pad) float32, valid (n,) int32."""
        import torch
        n = T0.shape[0]
        dev = T0.device
        X = X if X is not None else torch.empty((n, self.nin_pad), dtype=torch.float32, device=dev)
        Y = Y if Y is not None else torch.empty((n, self.nout_pad), dtype=torch.float32, device=dev)
        valid = valid if valid is not None else torch.empty(n, dtype=torch.int32, device=dev)
        check(lib().chem_surrogate_make_samples(self.id, n, _ptr(T0), _ptr(p0), _ptr(Y0), float(dt), _ptr(T1),
                                                _ptr(Y1), _ptr(status), _ptr(X), _ptr(Y), _ptr(valid), _stream()),
              "chem_surrogate_make_samples")
        return X, Y, valid

    def fit_normalisation(self, X, Y, rows):
        check(lib().chem_surrogate_fit_normalisation(self.id, int(rows.shape[0]), _ptr(X), _ptr(Y), _ptr(rows),
                                                     _stream()), "chem_surrogate_fit_normalisation")

    def train_step(self, X, Y, rows, lr, weight_decay=0.0, loss_sum=None):
        check(lib().chem_surrogate_train_step(self.id, int(rows.shape[0]), _ptr(X), _ptr(Y), _ptr(rows),
                                              ctypes.c_float(lr), ctypes.c_float(weight_decay), _ptr(loss_sum),
                                              _stream()), "chem_surrogate_train_step")

    def gradients(self, X, Y, rows):
        """(gradient (n_params,) float32 cuda tensor, summed weighted squared error)."""
        import torch
        g = torch.empty(self.n_params, dtype=torch.float32, device=X.device)
        loss = torch.zeros(1, dtype=torch.float32, device=X.device)
        check(lib().chem_surrogate_gradients(self.id, int(rows.shape[0]), _ptr(X), _ptr(Y), _ptr(rows), _ptr(g),
                                             _ptr(loss), _stream()), "chem_surrogate_gradients")
        return g, float(loss.item())

    def predict(self, X):
        """Raw predicted increments (n, nout_pad) of raw features X (n, nin_pad)."""
        import torch
        out = torch.empty((X.shape[0], self.nout_pad), dtype=torch.float32, device=X.device)
        check(lib().chem_surrogate_predict(self.id, int(X.shape[0]), _ptr(X), _ptr(out), _stream()),
              "chem_surrogate_predict")
        return out

    def train(self, X, Y, rows, epochs=10, batch=8192, lr=2e-3, lr_min=1e-5, warmup=0.03, weight_decay=0.0,
              seed=0, log=None):
        """AdamW with a linear warm-up and cosine decay over epochs x (rows // batch) steps; rows
        (int32 cuda tensor) are reshuffled each epoch.  Returns the mean loss of each epoch."""
        import torch
        n = int(rows.shape[0])
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        gen = torch.Generator(device=rows.device)
        gen.manual_seed(seed)
        loss = torch.zeros(1, dtype=torch.float32, device=rows.device)
        hist = []
        step = 0
        t0 = time.time()
        for ep in range(epochs):
            perm = rows[torch.randperm(n, generator=gen, device=rows.device)]
            loss.zero_()
            for i in range(steps_per_epoch):
                frac = step / max(1, total - 1)
                if frac < warmup:
                    cur = lr * (step + 1) / max(1, int(warmup * total))
                else:
                    q = (frac - warmup) / max(1e-12, 1.0 - warmup)
                    cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * q))
                self.train_step(X, Y, perm[i * batch:(i + 1) * batch], cur, weight_decay, loss)
                step += 1
            m = float(loss.item()) / (steps_per_epoch * batch)
            hist.append(m)
            if log:
                log("epoch %d loss %.4e (%.1fs)" % (ep, m, time.time() - t0))
        return hist

    def heldout_error(self, X, Y, rows, T_col=0):
        """Errors of the raw predictions on rows against the FP64 increments: per-row max |dY|
        and |dT| / T (numpy)."""
        import torch
        Xr, Yr = X[rows.long()], Y[rows.long()]
        pr = self.predict(Xr.contiguous())
        eY = (pr[:, :self.nout - 1] - Yr[:, :self.nout - 1]).abs().amax(dim=1)
        T = torch.exp(Xr[:, T_col].double())
        eT = (pr[:, self.nout - 1].double() - Yr[:, self.nout - 1].double()).abs() / (T + Yr[:, self.nout - 1].double())
        return eY.cpu().numpy(), eT.cpu().numpy()

    # ---------------------------------------------------------------- error model
    def add_error_model(self, width=128, depth=2, seed=0):
        """Attach the error network (include/gdtk_surrogate.h): an estimate of log10 of this network's
        prediction error (the larger of the largest |dY| error and 0.1 x the relative dT error), from
        its standardised input and output."""
        check(lib().chem_surrogate_error_model_new(self.id, int(width), int(depth), ctypes.c_ulonglong(seed)),
              "chem_surrogate_error_model_new")
        d = (ctypes.c_int * 5)()
        check(lib().chem_surrogate_error_dims(self.id, d), "chem_surrogate_error_dims")
        self.err_nin, self.err_nout_pad, self.err_width, self.err_depth, self.err_n_params = list(d)

    def error_layer_dims(self):
        return [self.err_nin] + [self.err_width] * self.err_depth + [self.err_nout_pad]

    def get_error_params(self):
        out = np.empty(self.err_n_params, np.float32)
        check(lib().chem_surrogate_error_get_params(self.id, _vp(out)), "chem_surrogate_error_get_params")
        return out

    def set_error_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        check(lib().chem_surrogate_error_set_params(self.id, _vp(params)), "chem_surrogate_error_set_params")

    def error_gradients(self, X, Y, rows, quantile=0.9):
        import torch
        g = torch.empty(self.err_n_params, dtype=torch.float32, device=X.device)
        loss = torch.zeros(1, dtype=torch.float32, device=X.device)
        check(lib().chem_surrogate_error_gradients(self.id, int(rows.shape[0]), _ptr(X), _ptr(Y), _ptr(rows),
                                                   ctypes.c_float(quantile), _ptr(g), _ptr(loss), _stream()),
              "chem_surrogate_error_gradients")
        return g, float(loss.item())

    def train_error_model(self, X, Y, rows, epochs=8, batch=8192, lr=2e-3, lr_min=1e-5, quantile=0.9, seed=1,
                          log=None):
        """AdamW on the error network's pinball loss, cosine schedule; returns the mean loss per epoch."""
        import torch
        n = int(rows.shape[0])
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        gen = torch.Generator(device=rows.device)
        gen.manual_seed(seed)
        loss = torch.zeros(1, dtype=torch.float32, device=rows.device)
        hist, step = [], 0
        for ep in range(epochs):
            perm = rows[torch.randperm(n, generator=gen, device=rows.device)]
            loss.zero_()
            for i in range(steps_per_epoch):
                q = step / max(1, total - 1)
                cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * q))
                check(lib().chem_surrogate_error_train_step(self.id, batch, _ptr(X), _ptr(Y),
                                                            _ptr(perm[i * batch:(i + 1) * batch]), ctypes.c_float(cur),
                                                            ctypes.c_float(0.0), ctypes.c_float(quantile), _ptr(loss),
                                                            _stream()), "chem_surrogate_error_train_step")
                step += 1
            hist.append(float(loss.item()) / (steps_per_epoch * batch))
            if log:
                log("error model epoch %d loss %.4e" % (ep, hist[-1]))
        return hist

    def predict_error(self, X):
        """The error network's estimate, log10 of the prediction error, per row of raw X."""
        import torch
        out = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        check(lib().chem_surrogate_predict_error(self.id, int(X.shape[0]), _ptr(X), _ptr(out), _stream()),
              "chem_surrogate_predict_error")
        return out

    def set_error_gate(self, tol):
        """Reject cells whose estimated |dY| error exceeds tol (<= 0: off)."""
        check(lib().chem_surrogate_set_error_gate(self.id, float(tol)), "chem_surrogate_set_error_gate")

    # ---------------------------------------------------------------- gated update
    def update(self, rho, u, T, p, massf, dt_chem, t_interval, status=None, T_frozen=0.0,
               flags=UPDATE_THERMO | RETRY, gate=None, monitor_stride=0):
        """Surrogate update with FP64 fallback, in place.  Returns dict(counts by gate code,
        fallback cells and failures, monitor statistics)."""
        n = rho.shape[0]
        for t in (rho, u, T, p, dt_chem):
            _f64(t, (n,))
        _f64(massf, (self.rc.nsp, n))
        counts = (ctypes.c_longlong * (len(GATE_NAMES) + 2))()
        mon = (ctypes.c_double * 4)()
        check(lib().chem_surrogate_update_cells(self.id, n, _ptr(rho), _ptr(u), _ptr(T), _ptr(p), _ptr(massf),
                                                _ptr(dt_chem), _ptr(status), float(t_interval), float(T_frozen),
                                                int(flags), _stream(), _ptr(gate), counts, int(monitor_stride), mon),
              "chem_surrogate_update_cells")
        c = list(counts)
        return dict(gate={GATE_NAMES[k]: c[k] for k in range(len(GATE_NAMES))}, fallback=c[-2], fallback_failed=c[-1],
                    monitor=dict(cells=int(mon[0]), max_dY=mon[1], max_rel_dT=mon[2], mean_max_dY=mon[3]))


def generate_samples(rc, sg, n, seed=0, dt_range=(0.5e-6, 2.0e-6), block=65536, blocks_per_launch=16,
                     cells=None, log=None, cost=None):
    """n training samples (rounded up to whole blocks) from the FP64 update of seeded cells.

    Cells come from `cells(n, seed)` -> (T, p, Y (nsp, n)) (default: the H2-air workload of
    uneven stiffness, gdtk_gb300.workloads.h2air_cells); each block of `block` cells gets its
    own dt, log-uniform in dt_range, and is advanced from a fresh step size (dt_chem = -1) by
    the plain update, blocks_per_launch blocks per persistent launch.  Returns (X, Y, valid,
    seconds spent in the FP64 update).  `cost` (int32 cuda tensor of the rounded-up size), when
    given, receives each sample's right-hand-side evaluations in the FP64 update."""
    import torch
    from .workloads import h2air_cells
    if cells is None:
        cells = lambda m, s: h2air_cells(rc.species_names, rc.mol_masses, m, seed=s,
                                              gas_file=rc.gmodel.file_name)
    nblk = (n + block - 1) // block
    dev = torch.device("cuda")
    X = torch.empty((nblk * block, sg.nin_pad), dtype=torch.float32, device=dev)
    Y = torch.empty((nblk * block, sg.nout_pad), dtype=torch.float32, device=dev)
    valid = torch.empty(nblk * block, dtype=torch.int32, device=dev)
    rng = np.random.Generator(np.random.PCG64(seed))
    t_update = 0.0
    for g0 in range(0, nblk, blocks_per_launch):
        group = []
        for b in range(g0, min(nblk, g0 + blocks_per_launch)):
            T, p, Yh = cells(block, seed * 100003 + b)
            dt = float(math.exp(rng.uniform(math.log(dt_range[0]), math.log(dt_range[1]))))
            d = dict(T=torch.tensor(T, device=dev), p=torch.tensor(p, device=dev),
                     massf=torch.tensor(np.ascontiguousarray(Yh), device=dev))
            d["rho"], d["u"] = rc.thermo_from_pT(d["p"], d["T"], d["massf"])
            d0 = dict(T=d["T"].clone(), p=d["p"].clone(), massf=d["massf"].clone())
            d["dt_chem"] = torch.full((block,), -1.0, dtype=torch.float64, device=dev)
            d["status"] = torch.zeros(block, dtype=torch.int32, device=dev)
            d["t_interval"] = dt
            group.append((b, d, d0))
        counters = None
        if cost is not None:
            counters = torch.empty((6, len(group) * block), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        t0 = time.time()
        rc.update_blocks([g[1] for g in group], cell_counters=counters)
        torch.cuda.synchronize()
        t_update += time.time() - t0
        if cost is not None:
            cost[g0 * block:g0 * block + len(group) * block] = counters[1]
        for b, d, d0 in group:
            sl = slice(b * block, (b + 1) * block)
            sg.make_samples(d0["T"], d0["p"], d0["massf"], d["t_interval"], d["T"], d["massf"], d["status"],
                            X=X[sl], Y=Y[sl], valid=valid[sl])
        if log:
            log("samples %d / %d" % (min(nblk, g0 + blocks_per_launch) * block, nblk * block))
    torch.cuda.synchronize()
    return X, Y, valid, t_update


def calibrate_error_gate(rc, sg, T0, p0, Y0, dt, max_dY=5.0e-5, max_rel_dT=5.0e-4, flags=UPDATE_THERMO | RETRY):
    """Sets the error-model gate from a calibration batch so that its accepted cells meet the bounds.

    The cells (device tensors T0, p0 (n,), Y0 (nsp, n), fresh step sizes) are updated by the plain
    FP64 update and by the surrogate with the error gate off.  Each accepted cell's error against
    the FP64 result (largest |dY|, and |dT| / T of the final temperature) is ranked by the error
    network's estimate for that cell; the gate is set to the largest estimate below which every
    calibration cell is within max_dY and max_rel_dT (split-conformal calibration of a maximum; the
    bounds are set below the target error so that unseen cells keep a margin).  Returns a dict
    with the threshold, the accepted fraction on the calibration cells and their largest errors."""
    import torch
    n = T0.shape[0]
    dev = T0.device
    rho, u = rc.thermo_from_pT(p0, T0, Y0)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    Tp, pp, Yp, dtc = T0.clone(), p0.clone(), Y0.clone(), torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    rc.update(rho, u, Tp, pp, Yp, dtc, dt, status=st, flags=flags)
    X, _, valid = sg.make_samples(T0, p0, Y0, dt, Tp, Yp, st)
    est = sg.predict_error(X).double()
    sg.set_error_gate(0.0)
    Ts, ps, Ys, dts = T0.clone(), p0.clone(), Y0.clone(), torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    gate = torch.empty(n, dtype=torch.int32, device=dev)
    sst = torch.zeros(n, dtype=torch.int32, device=dev)
    sg.update(rho, u, Ts, ps, Ys, dts, dt, status=sst, flags=flags, gate=gate)
    acc = (gate == 0) & (st == 0) & (valid != 0)
    eY = (Ys - Yp).abs().amax(dim=0)
    eT = (Ts - Tp).abs() / Tp
    idx = torch.nonzero(acc).flatten()
    order = idx[torch.argsort(est[idx])]
    bad = (eY[order] > max_dY) | (eT[order] > max_rel_dT)
    k = int(torch.nonzero(bad).flatten()[0]) if bool(bad.any()) else order.shape[0]
    if k == 0:
        log10_tol = -30.0
    else:   # between the last estimate kept and the first excluded
        hi = float(est[order[k]]) if k < order.shape[0] else float(est[order[k - 1]]) + 1e-6
        log10_tol = 0.5 * (float(est[order[k - 1]]) + hi)
    sg.set_error_gate(10.0 ** log10_tol)
    kept = order[:k]
    return dict(cells=n, log10_tol=log10_tol, tol=10.0 ** log10_tol, accepted_fraction=k / n,
                max_dY=float(eY[kept].max()) if k else 0.0, max_rel_dT=float(eT[kept].max()) if k else 0.0,
                bounds=dict(max_dY=max_dY, max_rel_dT=max_rel_dT))
