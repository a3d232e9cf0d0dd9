"""Batch chemistry updates over device-resident cell arrays (torch tensors on cuda).

Cells are structure-of-arrays, FP64, contiguous: rho, u, T, p, dt_chem of shape (n,) and
mass fractions of shape (nsp, n) (species-major), as the batch entry points of
include/gdtk_chem.h expect.  Launches go on torch's current CUDA stream.
"""
import ctypes

import numpy as np

from . import lib, check
from .gas import GasModel, ThermochemicalReactor

UPDATE_THERMO = 1
RETRY = 2

STATUS_NAMES = {0: "ok", 1: "h_min", 2: "max_attempts", 3: "max_subcycles", 4: "newton_fail",
                5: "bad_input", 6: "frozen", 7: "cea_range"}


def _ptr(t):
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _f64(t, shape):
    import torch
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous() and tuple(t.shape) == tuple(shape)):
        raise ValueError("expected a contiguous cuda float64 tensor of shape %s" % (shape,))
    return t


class CellBlockC(ctypes.Structure):
    """gdtk_cell_block of include/gdtk_chem.h."""
    _fields_ = [("ncell", ctypes.c_int), ("first", ctypes.c_int), ("t_interval", ctypes.c_double),
                ("rho", ctypes.c_void_p), ("u", ctypes.c_void_p), ("T", ctypes.c_void_p), ("p", ctypes.c_void_p),
                ("massf", ctypes.c_void_p), ("dt_chem", ctypes.c_void_p), ("status", ctypes.c_void_p)]


class ReactorCells:
    """A gas model + mechanism pair with batch entry points (chem_reactor_update_cells etc.)."""

    def __init__(self, gas_file, chem_file):
        self.gmodel = GasModel(gas_file)
        self.reactor = ThermochemicalReactor(self.gmodel, chem_file)
        nsp, nr, method, tight = (ctypes.c_int() for _ in range(4))
        check(lib().chem_reactor_info(self.reactor.id, ctypes.byref(nsp), ctypes.byref(nr), ctypes.byref(method),
                                      ctypes.byref(tight)), "chem_reactor_info")
        self.nsp, self.nr = nsp.value, nr.value
        self.method = "rkf" if method.value == 0 else "alpha-qss"
        self.tight = bool(tight.value)
        self.species_names = self.gmodel.species_names
        self.mol_masses = np.array(self.gmodel.mol_masses)

    def thermo_from_pT(self, p, T, massf, status=None):
        import torch
        n = p.shape[0]
        rho = torch.empty_like(p)
        u = torch.empty_like(p)
        check(lib().gas_model_update_thermo_from_pT_cells(self.gmodel.id, n, _ptr(_f64(p, (n,))), _ptr(_f64(T, (n,))),
                                                          _ptr(_f64(massf, (self.nsp, n))), _ptr(rho), _ptr(u),
                                                          _ptr(status), _stream()), "update_thermo_from_pT_cells")
        return rho, u

    def thermo_from_rhou(self, rho, u, massf, T, p, status=None):
        """Updates T (in: guess) and p in place."""
        n = rho.shape[0]
        check(lib().gas_model_update_thermo_from_rhou_cells(self.gmodel.id, n, _ptr(_f64(rho, (n,))),
                                                            _ptr(_f64(u, (n,))), _ptr(_f64(massf, (self.nsp, n))),
                                                            _ptr(_f64(T, (n,))), _ptr(_f64(p, (n,))), _ptr(status),
                                                            _stream()), "update_thermo_from_rhou_cells")

    def update(self, rho, u, T, p, massf, dt_chem, t_interval, status=None, T_frozen=0.0,
               flags=UPDATE_THERMO | RETRY, cell_counters=None, totals=None):
        """One chemistry increment per cell, in place (chem_reactor_update_cells_ex)."""
        n = rho.shape[0]
        for t in (rho, u, T, p, dt_chem):
            _f64(t, (n,))
        _f64(massf, (self.nsp, n))
        check(lib().chem_reactor_update_cells_ex(self.reactor.id, n, _ptr(rho), _ptr(u), _ptr(T), _ptr(p),
                                                 _ptr(massf), _ptr(dt_chem), _ptr(status), float(t_interval),
                                                 float(T_frozen), int(flags), _stream(), _ptr(cell_counters),
                                                 _ptr(totals)), "chem_reactor_update_cells")

    def block_table(self, blocks):
        """ctypes array of gdtk_cell_block for a list of dicts with keys rho, u, T, p, massf,
        dt_chem, t_interval and optionally status (cuda tensors)."""
        table = (CellBlockC * len(blocks))()
        for k, b in enumerate(blocks):
            n = b["rho"].shape[0]
            for key in ("rho", "u", "T", "p", "dt_chem"):
                _f64(b[key], (n,))
            _f64(b["massf"], (self.nsp, n))
            st = b.get("status")
            table[k] = CellBlockC(n, 0, float(b["t_interval"]), b["rho"].data_ptr(), b["u"].data_ptr(),
                                  b["T"].data_ptr(), b["p"].data_ptr(), b["massf"].data_ptr(), b["dt_chem"].data_ptr(),
                                  st.data_ptr() if st is not None else None)
        return table

    def update_blocks(self, blocks, T_frozen=0.0, flags=UPDATE_THERMO | RETRY, cell_counters=None, totals=None,
                      table=None):
        """All blocks in one persistent launch (chem_reactor_update_blocks); in place."""
        if table is None:
            table = self.block_table(blocks)
        check(lib().chem_reactor_update_blocks(self.reactor.id, len(table), table, float(T_frozen), int(flags),
                                               _stream(), _ptr(cell_counters), _ptr(totals)),
              "chem_reactor_update_blocks")

    def update_host(self, rho, u, T, p, massf, dt_chem, t_interval, status=None, T_frozen=0.0,
                    flags=UPDATE_THERMO | RETRY):
        """Host-array form (numpy, float64, massf (nsp, n)); returns the number of failed cells."""
        n = rho.shape[0]
        arrs = [rho, u, T, p, massf, dt_chem]
        for a in arrs:
            if a.dtype != np.float64 or not a.flags['C_CONTIGUOUS']:
                raise ValueError("expected C-contiguous float64 arrays")
        st = status if status is not None else np.empty(n, np.int32)
        vp = lambda a: ctypes.c_void_p(a.ctypes.data)
        return check(lib().chem_reactor_update_cells_host(self.reactor.id, n, vp(rho), vp(u), vp(T), vp(p), vp(massf),
                                                          vp(dt_chem), vp(st), float(t_interval), float(T_frozen),
                                                          int(flags)), "chem_reactor_update_cells_host")

    def source_terms(self, rho, T, massf, status=None):
        import torch
        n = rho.shape[0]
        out = torch.empty((self.nsp, n), dtype=torch.float64, device=rho.device)
        check(lib().chem_reactor_source_terms_cells(self.reactor.id, n, _ptr(_f64(rho, (n,))), _ptr(_f64(T, (n,))),
                                                    _ptr(_f64(massf, (self.nsp, n))), _ptr(out), _ptr(status),
                                                    _stream()), "chem_reactor_source_terms_cells")
        return out

    def flop_model(self):
        """[F_kc, F_rhs, F_step, F_corr, F_newton]: reference-algorithm FP64 operations per unit."""
        out = (ctypes.c_double * 5)()
        check(lib().chem_reactor_flop_model(self.reactor.id, out), "chem_reactor_flop_model")
        return [out[i] for i in range(5)]

    def algorithmic_flops(self, totals, n_cells_counted=None):
        """FLOPs of a batch from its work counters [steps, rhs, kc, newton, rejects, estimates]."""
        F = self.flop_model()
        steps, rhs, kc, newton, _, est = [float(x) for x in totals]
        corr = max(rhs - steps - est, 0.0) if self.method == "alpha-qss" else 0.0
        return F[0] * kc + F[1] * rhs + F[2] * steps + F[3] * corr + F[4] * newton

    def set_lane_stats(self, stats):
        """Diagnostics (chem_reactor_set_lane_stats): a cuda int64 tensor of 24 slots that later fast-kernel
        launches add to -- per phase k, warp executions [2k], active lanes [2k + 1], and with a kernel
        generated under GDTK_PHASE_CLOCKS=1 the SM cycles [16 + k].  None turns it off."""
        if stats is not None:
            import torch
            if not (stats.is_cuda and stats.dtype == torch.int64 and stats.numel() >= 24 and stats.is_contiguous()):
                raise ValueError("expected a contiguous cuda int64 tensor of at least 24 slots")
        check(lib().chem_reactor_set_lane_stats(self.reactor.id, _ptr(stats)), "chem_reactor_set_lane_stats")

    def last_launch(self):
        v = [ctypes.c_int() for _ in range(4)]
        check(lib().chem_reactor_last_launch(self.reactor.id, *[ctypes.byref(x) for x in v]), "last_launch")
        return dict(grid=v[0].value, block=v[1].value, smem=v[2].value, blocks_per_sm=v[3].value)


def measure_fp64_peak():
    v = ctypes.c_double()
    check(lib().gdtk_measure_fp64_peak(ctypes.byref(v)), "gdtk_measure_fp64_peak")
    return v.value


class ReactorCells2T:
    """A two-temperature gas with its multi-temperature reactor (chem_reactor2t_* of include/gdtk_chem.h):
    cells are SoA FP64 cuda tensors, mass fractions (nsp, n); launches go on torch's current stream."""

    def __init__(self, gas_file, chem_file, eem_file):
        self.id = check(lib().chem_reactor2t_new(gas_file.encode(), chem_file.encode(), eem_file.encode()),
                        "chem_reactor2t_new")
        nsp, nr, neem = (ctypes.c_int() for _ in range(3))
        check(lib().chem_reactor2t_info(self.id, ctypes.byref(nsp), ctypes.byref(nr), ctypes.byref(neem)),
              "chem_reactor2t_info")
        self.nsp, self.nr, self.neem = nsp.value, nr.value, neem.value

    def thermo_from_pT(self, p, T, T_ve, massf):
        """(rho, u, u_ve) of cells given p, T, T_ve and mass fractions."""
        import torch
        n = p.shape[0]
        for t in (p, T, T_ve):
            _f64(t, (n,))
        _f64(massf, (self.nsp, n))
        rho, u, u_ve = (torch.empty_like(p) for _ in range(3))
        check(lib().chem_reactor2t_thermo_from_pT_cells(self.id, n, _ptr(p), _ptr(T), _ptr(T_ve), _ptr(massf),
                                                        _ptr(rho), _ptr(u), _ptr(u_ve), _stream()),
              "chem_reactor2t_thermo_from_pT_cells")
        return rho, u, u_ve

    def update(self, rho, T, T_ve, p, massf, dt_chem, t_interval, status=None, u=None, u_ve=None, steps=None):
        """One update of every cell over t_interval, in place (T, T_ve, p, massf, dt_chem; u, u_ve out)."""
        n = rho.shape[0]
        for t in (rho, T, T_ve, p, dt_chem):
            _f64(t, (n,))
        _f64(massf, (self.nsp, n))
        check(lib().chem_reactor2t_update_cells(self.id, n, _ptr(rho), _ptr(T), _ptr(T_ve), _ptr(p), _ptr(massf),
                                                _ptr(u), _ptr(u_ve), _ptr(dt_chem), _ptr(status), float(t_interval),
                                                _ptr(steps), _stream()), "chem_reactor2t_update_cells")
