"""Throughput benchmark of the operator-split chemistry update (one JSON line on stdout).

Workload (default): 1,048,576 independent cells of 13-species H2-air (Jachimowski 1992,
33 reactions, alpha-QSS with tight temperature coupling, as its mechanism file says), half
cold (300-600 K) and half igniting (1100-2800 K), p = 10^U[log10 2e4, log10 5e5] Pa, one
chemistry update of dt = 1e-6 s per cell from a fresh step size (dt_chem = -1), followed
by update_thermo_from_rhou, i.e. one thermochemical_increment per cell.  A step is that
update over all cells; before each step the seeded initial state is restored on the device
(the restore copy is inside the timed region; it is < 0.1% of a step).  The cell arrays
(~150 MB) exceed the 129 MB L2, so no separate L2 flush is done.

--impl gdtk (default): the CUDA engine (gdtk_gb300).  `value` = cells/s with inputs resident in
HBM; `e2e` = the same through the host-pointer C-ABI entry point
(chem_reactor_update_cells_host) from page-locked host arrays, copies included.
--impl reference: the reference algorithm on the host CPU cores (oracle/, a C++ restatement of
the reference's CPU chemistry update, OpenMP over cells), on a bounded sample of the same cells.

Multi-GPU (torchrun): each rank integrates its own replica of the cells (cells are
independent; there is no data exchange), `value` = all ranks' cells / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
MECH = os.path.join(ROOT, "tests", "golden", "mech")
METRIC = "cell chem updates/s: plain FP64 vs surrogate+fallback at ≤1e-4 ΔY, 1 GB300"

WORKLOADS = {
    "h2air-1M": dict(gas="j92-gas.lua", chem="j92-chem.lua", n=1048576, dt=1.0e-6, kind="h2air", seed=1),
    "air5-4096": dict(gas="park5-gas.lua", chem="park5-chem.lua", n=4096, dt=1.0e-6, kind="air5", seed=0),
    # 64 uneven blocks (log-uniform 2,048..524,288 cells), own T/p ranges and dt in {1e-7, 1e-6, 1e-5} s,
    # 20 split steps with dt_chem carried, each split step one CUDA-graph replay of one launch
    "h2air-blocks64": dict(gas="j92-gas.lua", chem="j92-chem.lua", n=0, dt=0.0, kind="blocks", seed=2,
                           nblocks=64, split_steps=20),
    # in-loop drop-in: a 2048 x 1024 mixing-layer block, 100 split steps of 5e-7 s through the
    # thermochemical_increment contract (T_frozen = 300 K, dt_chem carried, retry, rhou update)
    "h2air-mixing-layer": dict(gas="j92-gas.lua", chem="j92-chem.lua", n=2048 * 1024, dt=5.0e-7, kind="layer",
                               seed=4, nx=2048, ny=1024, split_steps=100, T_frozen=300.0),
    # learned surrogate: 4x256 GELU MLP trained on 16,777,216 samples of the FP64 update (cells of the
    # h2air-1M distribution, dt log-uniform in [0.5, 2] us, 5% held out); inference + gate + FP64
    # fallback on 4,194,304 fresh cells at dt = 1e-6 s, against the plain FP64 update of the same cells
    # two-temperature reactor: Park's 5-species 2-T air (examples/lmr/3D/cylinder-larc inputs), Landau-Teller
    # exchange and Marrone-Treanor coupling, non-equilibrium post-shock cells, dt = 1e-6 s
    "air2t-262144": dict(gas="park2t-gas.lua", chem="park2t-chem.lua", eem="park2t-eem.lua", n=262144, dt=1.0e-6,
                         kind="air2t", seed=7),
    # large mechanism: the reference's 75-species, 474-reaction C2H2/C2H4 model (alpha-QSS, one warp per
    # cell) on shock-tube ignition states of its acetylene example, dt = 1e-6 s
    "c2h2-262144": dict(gas="c2h2-gas.lua", chem="c2h2-chem.lua", n=262144, dt=1.0e-6, kind="c2h2", seed=5),
    # the surrogate network's forward layer alone: D = GELU(A W^T + b) over 1,048,576 rows, K = N = 256, BF16
    # in and out, tcgen05 (TMEM) kernel against the mma.sync kernel on the same operands
    "mlp-gemm-1M": dict(gas="j92-gas.lua", chem="j92-chem.lua", n=1048576, dt=0.0, kind="gemm", seed=6, K=256, N=256),
    "h2air-surrogate": dict(gas="j92-gas.lua", chem="j92-chem.lua", n=4194304, dt=1.0e-6, kind="surrogate",
                            seed=3, train_samples=16777216, epochs=30, batch=8192, error_epochs=8),
}


def make_cells(w, names=None, M=None, n=None):
    from gdtk_gb300.workloads import acetylene_cells, air5_cells, h2air_cells
    n = n or w["n"]
    if w["kind"] == "air5":
        return air5_cells(n, seed=w["seed"])
    if w["kind"] == "c2h2":
        return acetylene_cells(names, M, n, seed=w["seed"])
    return h2air_cells(names, M, n, seed=w["seed"], gas_file=os.path.join(MECH, w["gas"]))


# Environment switches read when the mechanism kernel is generated (alternate code forms, phase clocks).
CODEGEN_ENV = ("GDTK_KB_EXP", "GDTK_KC_UNROLLED", "GDTK_KC_UNROLL", "GDTK_G_UNROLL", "GDTK_RHS_FENCE",
               "GDTK_PHASE_CLOCKS", "GDTK_CHEM_REFERENCE_ORDER")


def codegen_env():
    """The kernel-generation switches set in this process's environment (recorded in the line's config)."""
    return {k: os.environ[k] for k in CODEGEN_ENV if os.environ.get(k)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, device="cpu"):
    """The largest of each rank's x (a float) over the default process group; x itself without one.
    device: where the reduction tensor lives ("cpu" for gloo, the rank's cuda device for nccl)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


PHASES = ["iteration", "rate constants", "right-hand side", "step control", "Newton iteration", "cell completion",
          "refill", "alpha-QSS update"]


def lane_stats_summary(s):
    """Per phase of the fast kernel (chem_reactor_set_lane_stats slots): warp executions, mean active
    lanes, and the share of all warps' SM cycles when the kernel counted them (GDTK_PHASE_CLOCKS=1)."""
    s = np.asarray(s, dtype=np.float64)
    cyc = s[16:24]
    out = {}
    for k, name in enumerate(PHASES):
        d = {"warp_executions": int(s[2 * k]), "active_lanes": float(s[2 * k + 1] / s[2 * k]) if s[2 * k] else 0.0}
        if cyc.sum() > 0:
            d["time_share"] = float(cyc[k] / cyc.sum())
        out[name] = d
    return out


def replica_throughput(cells_per_rank, world_size, steps, max_ms):
    """Whole-job cell-updates/s of `world_size` replicas that each updated `cells_per_rank` cells
    `steps` times, timed by the slowest rank (max_ms for all the steps)."""
    return cells_per_rank * world_size * steps / (max_ms * 1e-3)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace('.', '', 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace('.', '', 1).isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, name in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def profile_record(name, workload):
    """The entry for `workload` in profiles/<name> (summaries of committed ncu captures), or None."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f).get(workload)


def roofline_fp64(issued, n, kernel_ms, peak, ref_flops, traffic, work_per_cell):
    """The FP64 roofline object of a chemistry-update line.

    achieved / frac: FP64 FLOP the kernel issues (2 DFMA + DADD + DMUL thread instructions, per cell
    from the committed ncu capture of the same workload in profiles/fp64_issued.json, times the cells
    of one launch) over the CUDA-event launch time, against the DFMA probe's peak.  The reference-
    operation figure (the reference's add/mul/div = 1, exp/log = 20, pow = 40 per unit of work, with
    the kernel's own work counters) is reported beside it under its own name."""
    kernel_s = kernel_ms * 1e-3
    ref = None
    if ref_flops is not None:
        ref = {"achieved": ref_flops / kernel_s / 1e12, "frac": ref_flops / kernel_s / 1e12 / peak,
               "flops_per_launch": ref_flops, "work_per_cell": list(map(float, work_per_cell)),
               "convention": "reference operations per unit of work: add/sub/mul/div 1, exp/log 20, pow 40"}
    out = {"bound": "fp64", "achieved": None, "peak": peak, "unit": "TFLOP/s", "frac": None, "traffic": traffic,
           "basis": "issued FP64 FLOP: 2 x DFMA + DADD + DMUL thread instructions",
           "peak_source": "measured: gdtk_measure_fp64_peak DFMA probe on this GPU (no FP64 entry in "
                          "MEASURED_PEAKS.json)",
           "kernel_ms": kernel_ms, "reference_operation_count": ref}
    if issued:
        f = issued["flop_per_cell"] * n
        out.update(achieved=f / kernel_s / 1e12, frac=f / kernel_s / 1e12 / peak, issued_flops_per_launch=f,
                   issued_source="profiles/fp64_issued.json (%d-cell ncu capture: %s)" %
                                 (issued["cells"], issued["command"]))
        # FP64 pipe issue: thread-level DFMA + DADD + DMUL instructions per second against the probe's
        # FMA instruction rate (peak / 2); a kernel whose every FP64 slot held an FMA on an active lane
        # would reach 1 on both bases, one whose slots held adds and multiplies reaches 1 here only
        inst = (issued["dfma"] + issued["dadd"] + issued["dmul"]) / issued["cells"] * n
        out["fp64_issue"] = {"thread_instructions_per_launch": inst,
                             "frac": inst / kernel_s / (peak * 1e12 / 2.0),
                             "basis": "DFMA + DADD + DMUL thread instructions (same capture) per second, "
                                      "over the DFMA probe's instruction rate"}
    return out


def roofline_fp64_estimated(ref_flops, total_s, peak, extra=None):
    """FP64 roofline of a workload of the H2-air mechanism without its own issued-FLOP capture: the
    reference-operation count of its work counters, and from it the issued FLOP estimated with the
    issued / reference ratio of the h2air-1M capture (same mechanism and kernel; the ratio depends on
    the mix of rate-constant, right-hand-side and Newton work, so the figure is an estimate)."""
    rec = profile_record("fp64_issued.json", "h2air-1M")
    ref = {"achieved": ref_flops / total_s / 1e12, "frac": ref_flops / total_s / 1e12 / peak,
           "flops": ref_flops,
           "convention": "reference operations per unit of work: add/sub/mul/div 1, exp/log 20, pow 40"}
    out = {"bound": "fp64", "achieved": None, "peak": peak, "unit": "TFLOP/s", "frac": None, "traffic": None,
           "reference_operation_count": ref}
    if rec and rec.get("reference_flop_per_cell"):
        ratio = rec["flop_per_cell"] / rec["reference_flop_per_cell"]
        out.update(achieved=ref["achieved"] * ratio, frac=ref["frac"] * ratio,
                   basis="issued FP64 FLOP (2 x DFMA + DADD + DMUL), estimated as the reference-operation "
                         "count x %.4f, the issued / reference ratio of the h2air-1M capture "
                         "(profiles/fp64_issued.json)" % ratio)
    if extra:
        out.update(extra)
    return out


def fp64_peak_reference():
    """The FP64 roofline denominator: measured on this GPU by the library's DFMA probe."""
    from gdtk_gb300.cells import measure_fp64_peak
    return max(measure_fp64_peak() for _ in range(3))


def cpu_reference_run(w, T, p, Y, rho, u, max_seconds, nthreads=0):
    """Times the oracle (reference algorithm, C++ restatement) on a bounded sample of cells."""
    import oracle
    orc = oracle.Oracle(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    n_total = T.shape[0]
    threads = nthreads if nthreads > 0 else oracle.max_threads()

    def run(idx):
        t0 = time.perf_counter()
        out = orc.chem_update(rho[idx], u[idx], T[idx], p[idx], Y[:, idx].T, np.full(len(idx), -1.0), w["dt"],
                              nthreads=threads)
        return time.perf_counter() - t0, out

    # probe with a small strided sample, then size the sample to about max_seconds
    probe = np.arange(0, n_total, max(n_total // 256, 1))[:256]
    dt_probe, _ = run(probe)
    per_cell = dt_probe / len(probe)
    m = int(min(n_total, max(len(probe), max_seconds / max(per_cell, 1e-9))))
    idx = np.linspace(0, n_total - 1, m).astype(np.int64)
    secs, out = run(idx)
    return dict(value=m / secs, cells=m, seconds=secs, threads=threads, out=out, idx=idx)


def run_blocks(args, w, tune=True, cpu=True):
    """Uneven multi-block batch: one graph replay per split step (returns the JSON line).  tune=False
    takes the default launch shape (256 threads, longest-first); cpu=False leaves out the CPU sample."""
    import torch
    import gdtk_gb300
    from gdtk_gb300 import autotune
    from gdtk_gb300.cells import ReactorCells, UPDATE_THERMO, RETRY
    from gdtk_gb300.workloads import h2air_blocks, h2air_cells
    rc = ReactorCells(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    dev = torch.device("cuda", 0)
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    choice, oflag = {}, 0
    if tune:   # launch-shape autotuning on a sample of the same mixture (cached per mechanism and device)
        sT, sp, sY = h2air_cells(rc.species_names, rc.mol_masses, 262144, seed=77, gas_file=rc.gmodel.file_name)
        dT, dp, dY = t64(sT), t64(sp), t64(sY)
        srho, su = rc.thermo_from_pT(dp, dT, dY)
        sample = dict(rho=srho, u=su, T=dT, p=dp, massf=dY, dt_chem=torch.full((262144,), -1.0,
                                                                             dtype=torch.float64, device=dev))
        choice, oflag, _ = autotune.tune(rc, sample, 1.0e-6, tag="h2air-262144", allow_warp=False)
    flags = UPDATE_THERMO | RETRY | oflag
    spec = h2air_blocks(rc.species_names, rc.mol_masses, nblocks=w["nblocks"], seed=w["seed"],
                        gas_file=rc.gmodel.file_name)
    blocks, init = [], []
    for b in spec:
        n = b["T"].shape[0]
        T, p, Y = t64(b["T"]), t64(b["p"]), t64(b["Y"])
        rho, u = rc.thermo_from_pT(p, T, Y)
        d = dict(rho=rho, u=u, T=T, p=p, massf=Y, dt_chem=torch.full((n,), -1.0, dtype=torch.float64, device=dev),
                 status=torch.zeros(n, dtype=torch.int32, device=dev), t_interval=b["dt"])
        blocks.append(d)
        init.append({k: (v.clone() if torch.is_tensor(v) else v) for k, v in d.items()})
    ncell = sum(b["rho"].shape[0] for b in blocks)
    table = rc.block_table(blocks)
    totals = torch.zeros(6, dtype=torch.int64, device=dev)
    # warm-up: one uncaptured split step on a copy (sizes the scratch, loads the kernel)
    scratch = [{k: (v.clone() if torch.is_tensor(v) else v) for k, v in b.items()} for b in blocks]
    rc.update_blocks(scratch, flags=flags)
    torch.cuda.synchronize()
    del scratch
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            rc.update_blocks(blocks, flags=flags, totals=totals, table=table)
    torch.cuda.synchronize()
    for b, i in zip(blocks, init):   # capture does not run; make sure the state is the initial one
        for k in ("T", "p", "massf", "dt_chem"):
            b[k].copy_(i[k])
    totals.zero_()
    torch.cuda.synchronize()
    nsteps = w["split_steps"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    clocks.start()
    with torch.cuda.stream(stream):
        for k in range(nsteps):
            ev[k][0].record(stream)
            graph.replay()
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    lat = np.array([a.elapsed_time(b) for a, b in ev])
    total_ms = float(lat.sum())
    tot = totals.cpu().numpy().astype(np.float64)
    flops = rc.algorithmic_flops(tot)
    peak = fp64_peak_reference()
    failed = int(sum(int(((b["status"] != 0) & (b["status"] != 6)).sum()) for b in blocks))
    by_status = {}
    for b in blocks:
        v, c = np.unique(b["status"].cpu().numpy(), return_counts=True)
        for vv, cc in zip(v, c):
            by_status[int(vv)] = by_status.get(int(vv), 0) + int(cc)
    # CPU baseline: the oracle over the same 20 split steps on a strided sample of every block
    cpu_cells, cpu_secs = 0, 0.0
    if cpu:
        import oracle
        orc = oracle.Oracle(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    for b, i in zip(blocks, init) if cpu else ():
        n = b["rho"].shape[0]
        idx = np.arange(0, n, max(n // 32, 1))[:32]
        rho, u = i["rho"].cpu().numpy()[idx], i["u"].cpu().numpy()[idx]
        T, p = i["T"].cpu().numpy()[idx], i["p"].cpu().numpy()[idx]
        Y = i["massf"].cpu().numpy()[:, idx].T
        dtc = np.full(len(idx), -1.0)
        t0 = time.perf_counter()
        for _ in range(nsteps):
            o = orc.chem_update(rho, u, T, p, Y, dtc, b["t_interval"])
            T, p, Y, dtc = o["T"], o["p"], o["massf"], o["dt_chem"]
        cpu_secs += time.perf_counter() - t0
        cpu_cells += len(idx) * nsteps
    return {
        "metric": METRIC, "value": ncell * nsteps / (total_ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1,
        "steps": nsteps, "warmup": 1, "ms_per_step": total_ms / nsteps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "h2air-blocks64", "blocks": len(blocks), "cells": ncell,
                   "dt_per_block": [b["t_interval"] for b in blocks], "graph": "one CUDA-graph replay per split step",
                   "launch_shape": {k: choice.get(k) for k in ("block", "min_blocks", "order", "refill_chunk",
                                                                 "cells_per_warp")},
                   "tuning_ms": {"%d/%d/%s/%d/%d" % (r["block"], r["min_blocks"], r["order"], r["refill_chunk"],
                                                     r["cells_per_warp"]): round(r["ms"], 1)
                                 for r in choice.get("results", [])},
                   "cells_failed": failed,
                   "cells_by_status_last_step": by_status,
                   "l2": "inputs larger than L2 (no flush)"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "per_step": [round(float(x), 3) for x in lat]},
        "roofline": roofline_fp64_estimated(flops, total_ms * 1e-3, peak,
                                            {"work_per_cell_update": (tot / (ncell * nsteps)).tolist()}),
        "cpu_baseline": {"value": cpu_cells / cpu_secs, "unit": "cell-updates/s", "cores": oracle.max_threads(),
                         "kind": "port", "sample": "32 strided cells of each block over the 20 split steps"}
                        if cpu else None,
        "e2e": None, "clocks": clk, "gpu_launches": nsteps * 5,
    }


def run_layer(args, w):
    """In-loop drop-in on a mixing-layer block: split steps as graph replays, final fields
    compared with the CPU reference algorithm on sampled columns (returns the JSON line)."""
    import torch
    import oracle
    from gdtk_gb300.cells import ReactorCells, UPDATE_THERMO, RETRY
    from gdtk_gb300.workloads import h2air_mixing_layer
    rc = ReactorCells(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    dev = torch.device("cuda", 0)
    nx, ny = w["nx"], w["ny"]
    if args.cells:
        nx = max(1, args.cells // ny)
    n = nx * ny
    T0, p0, Y0 = h2air_mixing_layer(rc.species_names, rc.mol_masses, nx=nx, ny=ny, seed=w["seed"])
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    T, p, Y = t64(T0), t64(p0), t64(Y0)
    rho, u = rc.thermo_from_pT(p, T, Y)
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    totals = torch.zeros(6, dtype=torch.int64, device=dev)
    flags = UPDATE_THERMO | RETRY
    init = (T.clone(), p.clone(), Y.clone(), dtc.clone())
    rc.update(rho, u, T, p, Y, dtc, w["dt"], status=st, T_frozen=w["T_frozen"], flags=flags)   # warm-up
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            rc.update(rho, u, T, p, Y, dtc, w["dt"], status=st, T_frozen=w["T_frozen"], flags=flags, totals=totals)
    for a, b in zip((T, p, Y, dtc), init):
        a.copy_(b)
    totals.zero_()
    torch.cuda.synchronize()
    nsteps = w["split_steps"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    clocks.start()
    with torch.cuda.stream(stream):
        for k in range(nsteps):
            ev[k][0].record(stream)
            graph.replay()
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    lat = np.array([a.elapsed_time(b) for a, b in ev])
    total_ms = float(lat.sum())
    tot = totals.cpu().numpy().astype(np.float64)
    flops = rc.algorithmic_flops(tot)
    peak = fp64_peak_reference()
    # the reference algorithm on the CPU over the same 100 split steps, on sampled columns
    orc = oracle.Oracle(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    cols = np.linspace(0, nx - 1, min(4, nx)).astype(np.int64)
    idx = np.concatenate([c + nx * np.arange(ny) for c in cols])
    cT, cp, cY, cdt = T0[idx].copy(), p0[idx].copy(), Y0[:, idx].T.copy(), np.full(len(idx), -1.0)
    crho, cu = rho.cpu().numpy()[idx], u.cpu().numpy()[idx]
    t0 = time.perf_counter()
    for _ in range(nsteps):
        o = orc.chem_update(crho, cu, cT, cp, cY, cdt, w["dt"], T_frozen=w["T_frozen"])
        cT, cp, cY, cdt = o["T"], o["p"], o["massf"], o["dt_chem"]
    cpu_secs = time.perf_counter() - t0
    gT, gY = T.cpu().numpy()[idx], Y.cpu().numpy()[:, idx].T
    dY = float(np.abs(gY - cY).max())
    relT = float((np.abs(gT - cT) / cT).max())
    # both against a tight (Radau, rtol 1e-10) integration of the coupled ODE over the same
    # interval, on cells through the mixing zone of the first sampled column
    from oracle.tight import integrate_cell
    zone = np.arange(ny // 2 - 30, ny // 2 + 30, 6)
    tg = {"gpu_dY": 0.0, "gpu_dT": 0.0, "cpu_dY": 0.0, "cpu_dT": 0.0, "cells": int(len(zone))}
    tight_ref = []
    for j in zone:
        mf, Tt = integrate_cell(orc, crho[j], cu[j], T0[idx][j], Y0[:, idx][:, j], nsteps * w["dt"], rtol=1e-10,
                                tight=True)
        tight_ref.append((j, mf, Tt))
        tg["gpu_dY"] = max(tg["gpu_dY"], float(np.abs(gY[j] - mf).max()))
        tg["gpu_dT"] = max(tg["gpu_dT"], float(abs(gT[j] - Tt) / Tt))
        tg["cpu_dY"] = max(tg["cpu_dY"], float(np.abs(cY[j] - mf).max()))
        tg["cpu_dT"] = max(tg["cpu_dT"], float(abs(cT[j] - Tt) / Tt))
    status = st.cpu().numpy()
    sur = None
    if not args.no_surrogate:
        sur = layer_surrogate_leg(rc, w, rho, u, init, (T, Y), nsteps, total_ms, idx, (cT, cY), tight_ref, flags)
    line = {
        "metric": METRIC, "value": n * nsteps / (total_ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1,
        "steps": nsteps, "warmup": 1, "ms_per_step": total_ms / nsteps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "h2air-mixing-layer", "nx": nx, "ny": ny, "cells": n, "dt": w["dt"],
                   "T_frozen": w["T_frozen"], "graph": "one CUDA-graph replay per split step",
                   "cells_frozen_last_step": int((status == 6).sum()),
                   "cells_failed_last_step": int(((status != 0) & (status != 6)).sum())},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "first": float(lat[0]), "last": float(lat[-1])},
        "accuracy_vs_cpu_reference": {"columns": cols.tolist(), "cells": int(len(idx)), "max_abs_dY": dY,
                                      "max_rel_dT": relT},
        "accuracy_vs_tight_integration": tg,
        "roofline": roofline_fp64_estimated(flops, total_ms * 1e-3, peak),
        "cpu_baseline": {"value": len(idx) * nsteps / cpu_secs, "unit": "cell-updates/s",
                         "cores": oracle.max_threads(), "kind": "port",
                         "sample": "%d full columns (%d cells) over the %d split steps" % (len(cols), len(idx), nsteps)},
        "e2e": None, "clocks": clk, "gpu_launches": nsteps * 5,
    }
    if sur is not None:
        line["surrogate"] = sur
    return line


def layer_surrogate_leg(rc, w, rho, u, init, plain, nsteps, plain_ms, idx, cpu_final, tight_ref, flags):
    """Surrogate + FP64 fallback over the mixing layer's split steps, against the plain GPU update, the
    CPU reference on the sampled columns and the tight integrations (the surrogate half of the in-loop
    comparison).  The network is trained on samples of the layer's own states: every 10th split step of
    an untimed plain run, up to 200,000 unfrozen cells each, advanced by the FP64 update over dt drawn
    log-uniform in [dt/2, 2 dt] (8,388,608 samples, 5% held out); its error gate is calibrated on 262,144
    fresh draws from the same states (split-conformal, half the target bars, as in the default line)."""
    import torch
    from gdtk_gb300.surrogate import calibrate_error_gate
    dev = rho.device
    sync = torch.cuda.synchronize
    dt, Tf = w["dt"], w["T_frozen"]
    n = rho.shape[0]
    t0 = time.perf_counter()
    T, p, Y, dtc = (x.clone() for x in init)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    pool = []
    for k in range(nsteps):
        if k % 10 == 0:
            live = torch.nonzero(T > Tf).flatten()
            if live.numel():
                sel = live[torch.randperm(live.numel(), generator=g, device=dev)[:200000]]
                pool.append((T[sel].cpu().numpy(), p[sel].cpu().numpy(), Y[:, sel].cpu().numpy()))
        rc.update(rho, u, T, p, Y, dtc, dt, status=st, T_frozen=Tf, flags=flags)
    sync()
    PT = np.concatenate([a[0] for a in pool])
    Pp = np.concatenate([a[1] for a in pool])
    PY = np.concatenate([a[2] for a in pool], axis=1)

    def cells(m, seed):
        r = np.random.Generator(np.random.PCG64(seed)).integers(0, PT.shape[0], m)
        return PT[r].copy(), Pp[r].copy(), np.ascontiguousarray(PY[:, r])

    sg, X, Yt, train, hold, tr = train_surrogate(rc, 8388608, 30, 8, 8192, seed=13, cells=cells,
                                                 dt_range=(0.5 * dt, 2.0 * dt))
    del X, Yt, train, hold
    torch.cuda.empty_cache()
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    cT, cp, cY = cells(262144, 977)
    sg.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=2e-4, max_dY=0.0)
    cal = calibrate_error_gate(rc, sg, t64(cT), t64(cp), t64(cY), dt)
    t_setup = time.perf_counter() - t0
    # the split steps from the initial state, surrogate + fallback (wall clock, device synchronised: the gate
    # reads its rejected count on the host)
    T, p, Y, dtc = (x.clone() for x in init)
    gate = torch.empty(n, dtype=torch.int32, device=dev)
    lat, acc_frac = [], []
    for k in range(nsteps):
        live = T > Tf
        sync()
        t1 = time.perf_counter()
        sg.update(rho, u, T, p, Y, dtc, dt, status=st, T_frozen=Tf, flags=flags, gate=gate)
        sync()
        lat.append((time.perf_counter() - t1) * 1e3)
        acc_frac.append(float(((gate == 0) & (st == 0) & live).sum()) / max(int(live.sum()), 1))
    lat = np.array(lat)
    pT, pY = plain
    unfrozen = (init[0] > Tf)
    eY = (Y - pY).abs().amax(dim=0)[unfrozen]
    eT = ((T - pT).abs() / pT)[unfrozen]
    gT, gY = T.cpu().numpy()[idx], Y.cpu().numpy()[:, idx].T
    cT_, cY_ = cpu_final
    tight = {"cells": len(tight_ref), "max_dY": 0.0, "max_rel_dT": 0.0}
    for j, mf, Tt in tight_ref:
        tight["max_dY"] = max(tight["max_dY"], float(np.abs(gY[j] - mf).max()))
        tight["max_rel_dT"] = max(tight["max_rel_dT"], float(abs(gT[j] - Tt) / Tt))
    total = float(lat.sum())
    return {
        "cell_updates_per_s": n * nsteps / (total * 1e-3), "speedup_vs_plain": plain_ms / total,
        "ms_per_split_step": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                              "first": float(lat[0]), "last": float(lat[-1])},
        "accepted_fraction_of_unfrozen_cells": {"mean": float(np.mean(acc_frac)), "first_step": acc_frac[0],
                                                "last_step": acc_frac[-1]},
        "final_fields_vs_plain_gpu": {"cells": int(unfrozen.sum()), "max_abs_dY": float(eY.max()),
                                      "max_rel_dT": float(eT.max())},
        "final_fields_vs_cpu_reference": {"cells": int(len(idx)), "max_abs_dY": float(np.abs(gY - cY_).max()),
                                          "max_rel_dT": float((np.abs(gT - cT_) / cT_).max())},
        "final_fields_vs_tight_integration": tight,
        "calibration": cal,
        "training": {"samples": tr["samples"], "heldout": tr["heldout"], "epochs": 30,
                     "state_pool": int(PT.shape[0]), "sample_generation_s": tr["sample_generation_s"],
                     "train_s": tr["train_s"], "setup_s_total": t_setup,
                     "heldout_median_max_dY": float(np.median(tr["eY"])),
                     "heldout_p99_max_dY": float(np.percentile(tr["eY"], 99))},
        "timing": "wall clock around each split step with the device synchronised, against the plain line's "
                  "CUDA-graph replay time",
    }


def train_surrogate(rc, n_train, epochs, error_epochs, batch, seed=7, cells=None, dt_range=(0.5e-6, 2.0e-6)):
    """The surrogate of `rc` trained on n_train samples that the FP64 update generates (5% held out),
    with its error model; `cells` and `dt_range` as for generate_samples (default: the H2-air cells).
    Returns (sg, X, Y, train rows, held-out rows, info)."""
    import torch
    from gdtk_gb300.surrogate import ChemSurrogate, generate_samples
    dev = torch.device("cuda", 0)
    sync = torch.cuda.synchronize
    sg = ChemSurrogate(rc, width=256, depth=4, seed=0)
    X, Yt, valid, t_gen = generate_samples(rc, sg, n_train, seed=seed, cells=cells, dt_range=dt_range)
    rows = torch.nonzero(valid).flatten().to(torch.int32)
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    perm = rows[torch.randperm(rows.shape[0], generator=g, device=dev)]
    hold = perm[: rows.shape[0] // 20].contiguous()
    train = perm[rows.shape[0] // 20:].contiguous()
    sg.fit_normalisation(X, Yt, train)
    sync()
    t1 = time.perf_counter()
    hist = sg.train(X, Yt, train, epochs=epochs, batch=batch, lr=2e-3)
    sync()
    t_train = time.perf_counter() - t1
    # error model: the 0.9 quantile of log10 of the network's own |dY| error, on the same samples
    sg.add_error_model(width=128, depth=2, seed=1)
    sync()
    t1 = time.perf_counter()
    ehist = sg.train_error_model(X, Yt, train, epochs=error_epochs, batch=batch, quantile=0.9)
    sync()
    t_err = time.perf_counter() - t1
    eY, eT = sg.heldout_error(X, Yt, hold)
    est = sg.predict_error(X[hold.long()].contiguous()).cpu().numpy()
    le = np.log10(np.maximum(eY, 0.1 * eT) + 1e-12)   # the error the error model estimates
    err_model_stats = {"epochs": error_epochs, "train_s": t_err, "quantile": 0.9,
                       "heldout_fraction_below_estimate": float((le <= est).mean()),
                       "heldout_rank_correlation": float(np.corrcoef(np.argsort(np.argsort(est)),
                                                                     np.argsort(np.argsort(le)))[0, 1]),
                       "loss_first_epoch": ehist[0], "loss_last_epoch": ehist[-1]}
    info = dict(sample_generation_s=t_gen, train_s=t_train, hist=hist, eY=eY, eT=eT, error_model=err_model_stats,
                samples=int(rows.shape[0]), heldout=int(hold.shape[0]))
    return sg, X, Yt, train, hold, info


def surrogate_leg(rc, srho, su, sT, sp, sY, dt, plain_ms, plain_T, plain_Y, plain_st, reps=3):
    """The surrogate + FP64 fallback form of the same update, for the default line.

    The network (16-256x4-14, BF16) is trained on 16,777,216 samples of the FP64 update (cells of
    this workload's distribution, dt log-uniform in [0.5, 2] us, 5% held out), its error gate is
    calibrated on 262,144 fresh cells (split-conformal: every accepted calibration cell within
    5e-5 in Y and 5e-4 relative in T, half the target bars), and then it updates the benchmark's own
    cells.  Errors of the accepted cells are against the plain FP64 update of those cells and, on a
    sample, against a tight Radau integration of the same ODE (the oracle, as the checker)."""
    import torch
    import oracle
    from oracle.tight import integrate_cell
    from gdtk_gb300.cells import UPDATE_THERMO, RETRY
    from gdtk_gb300.surrogate import calibrate_error_gate
    from gdtk_gb300.workloads import h2air_cells
    dev = sT.device
    sync = torch.cuda.synchronize
    t0 = time.perf_counter()
    sg, X, Yt, train, hold, tr = train_surrogate(rc, 16777216, 30, 8, 8192)
    del X, Yt, train, hold
    torch.cuda.empty_cache()
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    cT, cp, cY = h2air_cells(rc.species_names, rc.mol_masses, 262144, seed=91, gas_file=rc.gmodel.file_name)
    # energy check at 2e-4: the T from (rho, u, Y_new) agrees with T + the predicted dT to 2e-4, whose own
    # error the error model bounds, so the final T is within the calibrated bound
    sg.set_gate(elem_tol=1e-4, neg_tol=1e-5, T_tol=2e-4, max_dY=0.0)
    cal = calibrate_error_gate(rc, sg, t64(cT), t64(cp), t64(cY), dt)
    t_setup = time.perf_counter() - t0
    n = sT.shape[0]
    T, p, Y = sT.clone(), sp.clone(), sY.clone()
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    gate = torch.empty(n, dtype=torch.int32, device=dev)
    times = []
    for k in range(reps + 1):
        T.copy_(sT); p.copy_(sp); Y.copy_(sY); dtc.fill_(-1.0)
        sync()
        t1 = time.perf_counter()
        res = sg.update(srho, su, T, p, Y, dtc, dt, status=st, flags=UPDATE_THERMO | RETRY, gate=gate)
        sync()
        if k:
            times.append(time.perf_counter() - t1)
    secs = float(np.mean(times))
    acc = (gate == 0) & (plain_st == 0)
    eY = (Y - plain_Y).abs().amax(dim=0)
    eT = (T - plain_T).abs() / plain_T
    # against a tight integration of the coupled ODE: accepted cells, hot and cold, and the plain result
    orc = oracle.Oracle(rc.gmodel.file_name, rc.reactor.filename1)
    ai = torch.nonzero(acc).flatten().cpu().numpy()
    hot = ai[sT.cpu().numpy()[ai] > 1000.0]
    cold = ai[sT.cpu().numpy()[ai] <= 1000.0]
    pick = np.concatenate([hot[np.linspace(0, len(hot) - 1, min(len(hot), 12)).astype(np.int64)] if len(hot) else hot,
                           cold[np.linspace(0, len(cold) - 1, min(len(cold), 4)).astype(np.int64)] if len(cold) else cold])
    hr, hu, hT0, hY0 = srho.cpu().numpy(), su.cpu().numpy(), sT.cpu().numpy(), sY.cpu().numpy()
    gY, gT, pY, pT = Y.cpu().numpy(), T.cpu().numpy(), plain_Y.cpu().numpy(), plain_T.cpu().numpy()
    tight = {"cells": int(len(pick)), "surrogate_max_dY": 0.0, "surrogate_max_rel_dT": 0.0, "plain_max_dY": 0.0,
             "plain_max_rel_dT": 0.0}
    for c in pick:
        mf, Tt = integrate_cell(orc, hr[c], hu[c], hT0[c], hY0[:, c], dt, rtol=1e-10, tight=True)
        tight["surrogate_max_dY"] = max(tight["surrogate_max_dY"], float(np.abs(gY[:, c] - mf).max()))
        tight["surrogate_max_rel_dT"] = max(tight["surrogate_max_rel_dT"], float(abs(gT[c] - Tt) / Tt))
        tight["plain_max_dY"] = max(tight["plain_max_dY"], float(np.abs(pY[:, c] - mf).max()))
        tight["plain_max_rel_dT"] = max(tight["plain_max_rel_dT"], float(abs(pT[c] - Tt) / Tt))
    return {
        "cell_updates_per_s": n / secs, "ms_per_update": secs * 1e3, "speedup_vs_plain": plain_ms / (secs * 1e3),
        "accepted_fraction": float(acc.float().mean()), "fallback_cells": int(res["fallback"]),
        "gate_counts": res["gate"],
        "error_vs_fp64_update": {"cells": int(acc.sum()), "max_dY": float(eY[acc].max()) if bool(acc.any()) else 0.0,
                                 "max_rel_dT": float(eT[acc].max()) if bool(acc.any()) else 0.0},
        "error_vs_tight_oracle": tight,
        "target": {"max_dY": 1e-4, "max_rel_dT": 1e-3, "speedup": 5.0},
        "calibration": cal,
        "network": "MLP 16-256x4-14 GELU, BF16 weights/activations, FP32 accumulation; error model 32-128x2-1",
        "training": {"samples": tr["samples"], "heldout": tr["heldout"], "epochs": 30,
                     "sample_generation_s": tr["sample_generation_s"], "train_s": tr["train_s"],
                     "setup_s_total": t_setup, "heldout_median_max_dY": float(np.median(tr["eY"])),
                     "heldout_p99_max_dY": float(np.percentile(tr["eY"], 99))},
        "timing": "wall clock around each call with the device synchronised (the gate reads the rejected count "
                  "on the host); speed-up against the plain line's ms_per_step",
    }


def cpu_two_temperature_run(w, T, Tve, p, Y, rho, max_seconds, nthreads=0):
    """Times the compiled two-temperature restatement (oracle/twotemp_oracle.cpp) on a bounded, evenly
    strided sample of the cells, all host threads."""
    import oracle
    from oracle.two_temperature_reactor import TwoTemperatureReactor, CompiledTwoTemperatureReactor
    r = TwoTemperatureReactor(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]), os.path.join(MECH, w["eem"]))
    c = CompiledTwoTemperatureReactor(r)
    threads = nthreads if nthreads > 0 else oracle.max_threads()
    n_total = T.shape[0]

    def run(idx):
        t0 = time.perf_counter()
        c.update_cells(rho[idx], T[idx], Tve[idx], p[idx], Y[:, idx].T, w["dt"], nthreads=threads)
        return time.perf_counter() - t0

    probe = np.arange(0, n_total, max(n_total // 512, 1))[:512]
    per_cell = run(probe) / len(probe)
    m = int(min(n_total, max(len(probe), max_seconds / max(per_cell, 1e-9))))
    idx = np.linspace(0, n_total - 1, m).astype(np.int64)
    secs = run(idx)
    return dict(value=m / secs, cells=m, seconds=secs, threads=threads)


def run_two_temperature_reference(args, w):
    """Reference arm of the two-temperature workload: the compiled restatement on the host cores."""
    from oracle.two_temperature import TwoTemperatureGas
    from gdtk_gb300.workloads import air2t_cells
    gas = TwoTemperatureGas(os.path.join(MECH, w["gas"]))
    T, Tve, p, Y = air2t_cells(w["n"], seed=w["seed"])
    Tk = np.where(np.arange(gas.nsp)[:, None] == gas.electron, Tve[None, :], T[None, :])
    rho = p / (Y * gas.R[:, None] * Tk).sum(axis=0)   # update_from_pT's density (two_temperature_gas.d:84-92)
    steps = []
    for s in range(args.warmup + args.steps):
        r = cpu_two_temperature_run(w, T, Tve, p, Y, rho, max_seconds=min(args.cpu_seconds, 20.0))
        if s >= args.warmup:
            steps.append(r)
    v = float(np.mean([r["value"] for r in steps]))
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean([r["seconds"] for r in steps]) * 1e3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "cells": w["n"], "dt": w["dt"], "mechanism": w["chem"],
                   "sample_cells_per_step": steps[0]["cells"]},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": steps[0]["threads"], "kind": "port",
                         "sample": "%d of the %d cells (evenly strided) per step, compiled two-temperature "
                                   "restatement, all host threads" % (steps[0]["cells"], w["n"])},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_two_temperature(args, w):
    """The two-temperature reactor over a batch of non-equilibrium air cells (chem_reactor2t_update_cells)."""
    import torch
    import gdtk_gb300
    from gdtk_gb300.cells import ReactorCells2T
    from gdtk_gb300.workloads import air2t_cells
    gdtk_gb300.lib()
    rc = ReactorCells2T(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]), os.path.join(MECH, w["eem"]))
    n = w["n"]
    dev = torch.device("cuda", 0)
    T0, Tve0, p0, Y0 = air2t_cells(n, seed=w["seed"])
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    sT, sTve, sp, sY = t64(T0), t64(Tve0), t64(p0), t64(Y0)
    rho, _, _ = rc.thermo_from_pT(sp, sT, sTve, sY)
    T, Tve, p, Y = sT.clone(), sTve.clone(), sp.clone(), sY.clone()
    dtc = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    u, uve = torch.empty_like(rho), torch.empty_like(rho)
    steps = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()

    def reset():
        T.copy_(sT); Tve.copy_(sTve); p.copy_(sp); Y.copy_(sY); dtc.fill_(-1.0)

    for _ in range(args.warmup):
        reset()
        rc.update(rho, T, Tve, p, Y, dtc, w["dt"], status=st, u=u, u_ve=uve)
    torch.cuda.synchronize()
    peak = fp64_peak_reference()
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    clocks.start()
    steps.zero_()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for s in range(args.steps):
        reset()
        ev[s][0].record(stream)
        rc.update(rho, T, Tve, p, Y, dtc, w["dt"], status=st, u=u, u_ve=uve, steps=steps)
        ev[s][1].record(stream)
    k1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = k0.elapsed_time(k1)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    ok = int((st == 0).sum())
    # end to end: pinned host arrays in, the update, results out, every step
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hrho, hT, hTve, hp, hY = pin(rho.cpu().numpy()), pin(T0), pin(Tve0), pin(p0), pin(Y0)
    oT, oTve, op, oY = (torch.empty_like(x).pin_memory() for x in (hT, hTve, hp, hY))
    e2e_times = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        drho, dT_, dTve_, dp_, dY_ = (x.to(dev, non_blocking=True) for x in (hrho, hT, hTve, hp, hY))
        ddt = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
        rc.update(drho, dT_, dTve_, dp_, dY_, ddt, w["dt"], status=st, u=u, u_ve=uve)
        for h, d in ((oT, dT_), (oTve, dTve_), (op, dp_), (oY, dY_)):
            h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    issued = profile_record("fp64_issued.json", args.workload)
    attempts = float(steps.item()) / args.steps / n
    cpu = None
    if not args.no_cpu_baseline:
        r = cpu_two_temperature_run(w, T0, Tve0, p0, Y0, rho.cpu().numpy(), max_seconds=args.cpu_seconds)
        cpu = {"value": r["value"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
               "sample": "%d of the %d cells (evenly strided), %.1f s on %d threads, compiled two-temperature "
                         "restatement (oracle/twotemp_oracle.cpp)" % (r["cells"], n, r["seconds"], r["threads"])}
    return {
        "metric": METRIC, "value": n * args.steps / (total_ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "cells": n, "mechanism": w["chem"], "energy_exchange": w["eem"],
                   "dt": w["dt"], "method": "rkf (multi-temperature reactor)", "cells_ok": ok,
                   "rkf_attempts_per_cell": attempts, "l2": "inputs larger than L2 (no flush): %.0f MB of cell "
                   "state" % (n * 8 * (6 + rc.nsp) / 1e6)},
        "roofline": roofline_fp64(issued, n, kernel_ms, peak, None, None, None),
        "cpu_baseline": cpu,
        "e2e": {"value": n / float(np.mean(e2e_times)), "unit": "cell-updates/s",
                "h2d_bytes_per_step": n * 8 * (4 + rc.nsp), "d2h_bytes_per_step": n * 8 * (3 + rc.nsp)},
        "clocks": clk, "gpu_launches": args.steps,
    }


def run_gemm(args, w):
    """The surrogate's forward layer on the tensor cores: tcgen05 kernel and mma.sync kernel, CUDA-event
    timed over `steps` launches each (inputs and outputs 512 MB each, larger than L2)."""
    import ctypes
    import torch
    import gdtk_gb300
    from gdtk_gb300 import lib, check
    gdtk_gb300.lib()
    M, N, K = w["n"], w["N"], w["K"]
    g = torch.Generator(device="cuda")
    g.manual_seed(w["seed"])
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    W = (torch.randn((N, K), generator=g, device="cuda") / 16.0).to(torch.bfloat16)
    b = torch.randn(N, generator=g, device="cuda")
    Dh = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
    stream = torch.cuda.current_stream()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())

    def launch():
        check(lib().gdtk_mlp_gemm(M, N, K, ptr(A), K, 0, ptr(W), K, 1, ptr(b), 1, None, None, ptr(Dh), N, 1,
                                  ctypes.c_void_p(stream.cuda_stream)), "gdtk_mlp_gemm")

    reps = 100   # launches per step: one launch is a fraction of a millisecond

    def timed(tc):
        lib().gdtk_mlp_tcgen05(1 if tc else 0, None, None)
        for _ in range(args.warmup):
            launch()
        torch.cuda.synchronize()
        n0 = ctypes.c_ulonglong()
        lib().gdtk_mlp_tcgen05(-1, ctypes.byref(n0), None)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps * reps):
            launch()
        e1.record(stream)
        torch.cuda.synchronize()
        n1, err = ctypes.c_ulonglong(), ctypes.c_int()
        lib().gdtk_mlp_tcgen05(-1, ctypes.byref(n1), ctypes.byref(err))
        if err.value:
            raise RuntimeError("a tcgen05 wait gave up (%d)" % err.value)
        return e0.elapsed_time(e1) / (args.steps * reps), n1.value - n0.value, Dh.clone()

    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    clocks.start()
    ms_tc, n_tc, out_tc = timed(True)
    clk = clocks.stop()
    ms_ms, n_ms, out_ms = timed(False)
    lib().gdtk_mlp_tcgen05(1, None, None)
    if n_tc != args.steps * reps or n_ms != 0:
        raise RuntimeError("unexpected kernel path (%d tcgen05 launches of %d)" % (n_tc, args.steps * reps))
    diff = (out_tc.float() - out_ms.float()).abs().max().item()
    flops = 2.0 * M * N * K
    traffic = float(M * K * 2 + N * K * 2 + M * N * 2)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peaks = json.load(f)
    tf_peak = peaks.get("bf16_tflops", 1900.0)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    tf = flops / (ms_tc * 1e-3) / 1e12
    gbs = traffic / (ms_tc * 1e-3) / 1e9
    return {
        "metric": "BF16 GEMM + bias + GELU TFLOP/s (surrogate forward layer), 1 GB300", "value": tf,
        "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_tc * reps,
        "ms_per_launch": ms_tc, "launches_per_step": reps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": args.workload, "M": M, "N": N, "K": K, "act": "gelu", "out": "bf16",
                   "l2": "inputs and outputs larger than L2 (512 MB each, no flush)",
                   "kernel": "gemm_tc_kernel: TMA loads, tcgen05.mma M=128 into TMEM, tcgen05.ld epilogue"},
        # K = N = 256 puts the layer below the ridge point (128 FLOP per byte): HBM bounds it
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                     "traffic": None, "algorithmic_bytes_per_launch": traffic,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                     "tensor": {"achieved": tf, "peak": tf_peak, "unit": "TFLOP/s", "frac": tf / tf_peak,
                                "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured, burst)"}},
        "mma_sync": {"value": flops / (ms_ms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_launch": ms_ms,
                     "speedup_of_tcgen05": ms_ms / ms_tc, "max_abs_diff_bf16_out": diff},
        "cpu_baseline": None, "e2e": None, "clocks": clk, "gpu_launches": args.steps * reps,
    }


def run_surrogate(args, w):
    """Surrogate + FP64 fallback against the plain FP64 update on fresh cells (returns the JSON line)."""
    import torch
    import oracle
    from gdtk_gb300.cells import ReactorCells, UPDATE_THERMO, RETRY
    from gdtk_gb300.workloads import h2air_cells
    rc = ReactorCells(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    dev = torch.device("cuda", 0)
    n = args.cells or w["n"]
    n_train = w["train_samples"] if not args.cells else max(65536, 4 * args.cells)
    sync = torch.cuda.synchronize
    epochs = args.epochs or w["epochs"]
    sg, X, Yt, train, hold, tr = train_surrogate(rc, n_train, epochs, w["error_epochs"], w["batch"])
    t_gen, t_train, hist = tr["sample_generation_s"], tr["train_s"], tr["hist"]
    eY, eT = tr["eY"], tr["eT"]
    err_model_stats = tr["error_model"]
    steps_per_epoch = train.shape[0] // w["batch"]
    train_flop = 3 * 2 * sum(a * b for a, b in zip(sg.layer_dims()[:-1], sg.layer_dims()[1:])) * \
        steps_per_epoch * w["batch"] * epochs
    del X, Yt, hold, train
    torch.cuda.empty_cache()

    # ---- fresh cells
    T0, p0, Y0 = h2air_cells(rc.species_names, rc.mol_masses, n, seed=w["seed"] * 1000 + 17,
                             gas_file=rc.gmodel.file_name)
    t64 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    sT, sp, sY = t64(T0), t64(p0), t64(Y0)
    srho, su = rc.thermo_from_pT(sp, sT, sY)
    sdt = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    T, p, Y, dtc = sT.clone(), sp.clone(), sY.clone(), sdt.clone()
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    flags = UPDATE_THERMO | RETRY

    def restore():
        T.copy_(sT); p.copy_(sp); Y.copy_(sY); dtc.copy_(sdt)
        sync()

    # plain FP64 update of the same cells (the baseline and the error reference)
    peak = fp64_peak_reference()
    totals = torch.zeros(6, dtype=torch.int64, device=dev)
    plain_s = []
    for k in range(1 + args.steps):
        restore()
        totals.zero_()
        t1 = time.perf_counter()
        rc.update(srho, su, T, p, Y, dtc, w["dt"], status=st, flags=flags, totals=totals)
        sync()
        if k:
            plain_s.append(time.perf_counter() - t1)
    plain_T, plain_Y, plain_st = T.clone(), Y.clone(), st.clone()
    plain_flops = rc.algorithmic_flops(totals.cpu().numpy().astype(np.float64))
    plain_time = float(np.mean(plain_s))

    # surrogate + fallback at a sweep of gate settings; the first is the default (reported value)
    checks = dict(elem_tol=1e-4, neg_tol=1e-5, T_tol=1e-3)
    settings = [("error model 1e-4", dict(checks, max_dY=0.0), 1e-4),
                ("error model 3e-4", dict(checks, max_dY=0.0), 3e-4),
                ("error model 1e-3", dict(checks, max_dY=0.0), 1e-3),
                ("magnitude cap 5e-4", dict(checks, max_dY=5e-4), 0.0),
                ("magnitude cap 2e-3", dict(checks, max_dY=2e-3), 0.0),
                ("checks only", dict(checks, max_dY=0.0), 0.0)]
    gate = torch.empty(n, dtype=torch.int32, device=dev)
    sweep = []
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    for si, (name, gs, etol) in enumerate(settings):
        sg.set_gate(**gs)
        sg.set_error_gate(etol)
        reps = (1 + args.steps) if si == 0 else 1
        times = []
        if si == 0:
            clocks.start()
        for k in range(reps):
            restore()
            t1 = time.perf_counter()
            res = sg.update(srho, su, T, p, Y, dtc, w["dt"], status=st, flags=flags, gate=gate,
                            monitor_stride=1024)
            sync()
            times.append(time.perf_counter() - t1)
        if si == 0:
            clk = clocks.stop()
            first_T, first_Y, first_gate = T.clone(), Y.clone(), gate.clone()
        secs = float(np.mean(times[1:] if reps > 1 else times))
        acc = (gate == 0) & (plain_st == 0)
        e = (Y[:, acc] - plain_Y[:, acc]).abs().amax(dim=0).double()
        et = ((T[acc] - plain_T[acc]).abs() / plain_T[acc]).double()
        q = lambda v, x: float(torch.quantile(v[:min(v.shape[0], 1 << 24)], x)) if v.numel() else 0.0
        sweep.append({"gate": name, **gs, "error_model_tol": etol, "seconds": secs, "cell_updates_per_s": n / secs,
                      "speedup_vs_plain": plain_time / secs, "accepted_fraction": float(acc.float().mean()),
                      "rejected_fraction": res["fallback"] / n, "gate_counts": res["gate"],
                      "fallback_failed": res["fallback_failed"],
                      "error_vs_fp64": {"cells": int(acc.sum()), "max_dY": float(e.max()) if e.numel() else 0.0,
                                        "p999_dY": q(e, 0.999), "p99_dY": q(e, 0.99), "median_dY": q(e, 0.5),
                                        "max_rel_dT": float(et.max()) if et.numel() else 0.0,
                                        "p999_rel_dT": q(et, 0.999)},
                      "monitor": res["monitor"]})
    # surrogate results of the default gate against the CPU reference algorithm on a strided sample
    acc0 = ((first_gate == 0) & (plain_st == 0)).cpu().numpy()
    idx = np.flatnonzero(acc0)
    idx = idx[np.linspace(0, len(idx) - 1, min(len(idx), 2000)).astype(np.int64)] if len(idx) else idx
    orc = oracle.Oracle(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    cpu_err = None
    if len(idx):
        o = orc.chem_update(srho.cpu().numpy()[idx], su.cpu().numpy()[idx], T0[idx], p0[idx], Y0[:, idx].T,
                            np.full(len(idx), -1.0), w["dt"])
        okc = o["status"] == 0
        sY_ = first_Y.cpu().numpy()[:, idx].T
        sT_ = first_T.cpu().numpy()[idx]
        pY_ = plain_Y.cpu().numpy()[:, idx].T
        cpu_err = {"cells": int(okc.sum()),
                   "surrogate_max_dY": float(np.abs(sY_[okc] - o["massf"][okc]).max()),
                   "surrogate_max_rel_dT": float((np.abs(sT_[okc] - o["T"][okc]) / o["T"][okc]).max()),
                   "plain_gpu_max_dY": float(np.abs(pY_[okc] - o["massf"][okc]).max())}
    cpu = None
    if not args.no_cpu_baseline:
        r = cpu_reference_run(w, T0, p0, Y0, srho.cpu().numpy(), su.cpu().numpy(), max_seconds=args.cpu_seconds)
        cpu = {"value": r["value"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
               "sample": "%d of the %d cells (evenly strided), %.1f s on %d threads" %
                         (r["cells"], n, r["seconds"], r["threads"])}
    d = sweep[0]
    achieved = plain_flops / plain_time / 1e12
    return {
        "metric": METRIC, "value": d["cell_updates_per_s"], "unit": "cell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": 1, "ms_per_step": d["seconds"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+bf16", "data": "synthetic",
        "config": {"workload": "h2air-surrogate", "cells": n, "dt": w["dt"], "dt_chem_in": -1.0,
                   "network": "MLP 16-256x4-14 GELU, BF16 weights/activations, FP32 accumulation",
                   "train_samples": int(n_train), "heldout_fraction": 0.05, "epochs": epochs,
                   "batch": w["batch"], "l2": "inputs larger than L2 (no flush)"},
        "plain_fp64": {"cell_updates_per_s": n / plain_time, "seconds": plain_time,
                       "reference_operation_frac": achieved / peak,
                       "cells_failed": int(((plain_st != 0) & (plain_st != 6)).sum().item())},
        "surrogate_speedup_vs_plain": d["speedup_vs_plain"],
        "sweep": sweep,
        "accuracy_vs_cpu_reference": cpu_err,
        "training": {"sample_generation_s": t_gen, "train_s": t_train, "samples_per_s":
                     steps_per_epoch * w["batch"] * epochs / t_train, "tflops": train_flop / t_train / 1e12,
                     "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1]},
        "error_model": err_model_stats,
        "heldout": {"rows": int(len(eY)), "median_max_dY": float(np.median(eY)),
                    "p99_max_dY": float(np.percentile(eY, 99)), "max_dY": float(eY.max()),
                    "median_rel_dT": float(np.median(eT)), "p99_rel_dT": float(np.percentile(eT, 99))},
        "roofline": roofline_fp64_estimated(plain_flops, plain_time, peak,
                                            {"kernel": "plain FP64 update of the same cells (the fallback's kernel)"}),
        "cpu_baseline": cpu, "e2e": None, "clocks": clk,
        # per 1M-cell chunk: features, 5 GEMMs, gate; fallback: gather, cost + 3 ordering kernels,
        # chemistry, scatter; monitor: repack, cost + 3 ordering kernels, chemistry, compare
        "gpu_launches": ((n + (1 << 20) - 1) >> 20) * 7 + 7 + 7,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gdtk", "reference"], default="gdtk")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="h2air-1M")
    ap.add_argument("--cells", type=int, default=0, help="override the cell count (parity/debug runs)")
    ap.add_argument("--epochs", type=int, default=0, help="surrogate mode: override the training epochs")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true", help="leave out the surrogate + fallback object")
    ap.add_argument("--no-blocks", action="store_true", help="leave out the 64-block batch object")
    ap.add_argument("--lane-stats", action="store_true",
                    help="after the timed region, one more update with the kernel's lane statistics attached; "
                         "with GDTK_PHASE_CLOCKS=1 in the environment the line also gets each phase's share of "
                         "warp time")
    args = ap.parse_args()
    # the timed kernel is never the phase-clock build: that one is generated only for the untimed
    # lane-statistics update below
    phase_clocks = os.environ.pop("GDTK_PHASE_CLOCKS", "") == "1"
    w = dict(WORKLOADS[args.workload])
    if args.cells:
        w["n"] = args.cells
    ws, rank, local = dist_env()

    if w["kind"] == "layer":
        if args.impl == "reference" or rank != 0:
            if args.impl == "reference" and rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the mixing-layer mode reports its CPU "
                                  "baseline inside the gdtk line"}))
            return 0
        print(json.dumps(run_layer(args, w)))
        return 0

    if w["kind"] == "air2t":
        if rank != 0:
            return 0
        print(json.dumps(run_two_temperature_reference(args, w) if args.impl == "reference"
                         else run_two_temperature(args, w)))
        return 0

    if w["kind"] == "gemm":
        if args.impl == "reference" or rank != 0:
            if args.impl == "reference" and rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the surrogate network has no counterpart "
                                  "in the reference"}))
            return 0
        print(json.dumps(run_gemm(args, w)))
        return 0

    if w["kind"] == "surrogate":
        if args.impl == "reference" or rank != 0:
            if args.impl == "reference" and rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the surrogate mode reports its CPU "
                                  "baseline inside the gdtk line"}))
            return 0
        print(json.dumps(run_surrogate(args, w)))
        return 0

    if w["kind"] == "blocks":
        if args.impl == "reference" or rank != 0:
            if args.impl == "reference" and rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the multi-block mode reports its CPU "
                                  "baseline inside the gdtk line"}))
            return 0
        print(json.dumps(run_blocks(args, w)))
        return 0

    if args.impl == "reference":
        if rank != 0:
            return 0
        from gdtk_gb300.gas import GasModel
        # gas-state setup (rho, u from p, T) uses the same CPU oracle as the timed run
        import oracle
        orc = oracle.Oracle(os.path.join(MECH, w["gas"]))
        gm_names = orc.names
        T, p, Y = make_cells(w, gm_names, orc.M)
        rho, u = orc.update_thermo_from_pT(p, T, Y.T)
        steps = []
        for s in range(args.warmup + args.steps):
            r = cpu_reference_run(w, T, p, Y, rho, u, max_seconds=min(args.cpu_seconds, 20.0))
            if s >= args.warmup:
                steps.append(r)
        v = float(np.mean([r["value"] for r in steps]))
        line = {
            "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean([r["seconds"] for r in steps]) * 1e3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "cells": w["n"], "dt": w["dt"], "mechanism": w["chem"],
                       "sample_cells_per_step": steps[0]["cells"]},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": steps[0]["threads"], "kind": "port",
                             "sample": "%d of the %d cells (evenly strided) per step, all host threads" %
                                       (steps[0]["cells"], w["n"])},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    import torch
    import gdtk_gb300
    if not os.path.exists(gdtk_gb300.LIB_PATH):
        gdtk_gb300.build()
    gdtk_gb300.lib()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from gdtk_gb300.cells import ReactorCells, UPDATE_THERMO, RETRY
    dev = torch.device("cuda", local if ws > 1 else 0)
    rc = ReactorCells(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
    n = w["n"]
    T0, p0, Y0 = make_cells(w, rc.species_names, rc.mol_masses)
    flags = UPDATE_THERMO | RETRY

    def t64(a):
        return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)

    sT, sp, sY = t64(T0), t64(p0), t64(Y0)
    srho, su = rc.thermo_from_pT(sp, sT, sY)
    sdt = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
    T, p, Y, dtc = sT.clone(), sp.clone(), sY.clone(), sdt.clone()
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    totals = torch.zeros(6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    tuned = None
    if n <= 16384 and not (rc.nsp > 32 or rc.nr > 128):
        # a small batch at one thread per cell fills a fraction of the GPU's lanes: the autotuner also tries
        # one warp per cell and the launch shapes, on this workload's own cells (before the timed region)
        from gdtk_gb300 import autotune
        sample = dict(rho=srho, u=su, T=sT, p=sp, massf=sY, dt_chem=sdt)
        choice, oflag, _ = autotune.tune(rc, sample, w["dt"], tag=args.workload, use_cache=False)
        flags |= oflag
        tuned = {k: choice.get(k) for k in ("block", "min_blocks", "order", "refill_chunk", "cells_per_warp", "ms")}

    def step(tot=None):
        T.copy_(sT); p.copy_(sp); Y.copy_(sY); dtc.copy_(sdt)
        rc.update(srho, su, T, p, Y, dtc, w["dt"], status=st, flags=flags, totals=tot)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    peak = fp64_peak_reference()

    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local if ws > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    clocks.start()
    totals.zero_()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for s in range(args.steps):
        T.copy_(sT); p.copy_(sp); Y.copy_(sY); dtc.copy_(sdt)
        ev[s][0].record(stream)
        rc.update(srho, su, T, p, Y, dtc, w["dt"], status=st, flags=flags, totals=totals)
        ev[s][1].record(stream)
    k1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    total_ms = k0.elapsed_time(k1)
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = replica_throughput(n, ws, args.steps, total_ms)
    status = st.cpu().numpy()
    tot = totals.cpu().numpy().astype(np.float64)
    flops = rc.algorithmic_flops(tot / args.steps)
    kernel_ms = float(np.mean(launch_ms))
    achieved = flops / (kernel_ms * 1e-3) / 1e12

    # ---- end to end through the host-pointer C ABI (page-locked host arrays)
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        hrho, hu = pin(srho.cpu().numpy()), pin(su.cpu().numpy())
        hT, hp, hY, hdt = pin(T0), pin(p0), pin(Y0), pin(np.full(n, -1.0))
        hst = pin(np.zeros(n, np.int32))
        rc.update_host(hrho, hu, hT.copy(), hp.copy(), hY.copy(), hdt.copy(), w["dt"], status=hst, flags=flags)
        e2e_steps = max(1, min(args.steps, 3))
        times = []
        for _ in range(e2e_steps):
            hT[:] = T0; hp[:] = p0; hY[:] = Y0; hdt[:] = -1.0
            t0 = time.perf_counter()
            rc.update_host(hrho, hu, hT, hp, hY, hdt, w["dt"], status=hst, flags=flags)
            times.append(time.perf_counter() - t0)
        nsp = rc.nsp
        e2e_s = max_over_ranks(float(np.mean(times)), dev)
        e2e = {"value": replica_throughput(n, ws, 1, e2e_s * 1e3), "unit": "cell-updates/s",
               "h2d_bytes_per_step": n * 8 * (5 + nsp), "d2h_bytes_per_step": n * (8 * (3 + nsp) + 4),
               "steps": e2e_steps}

    # ---- diagnostics: lane occupancy and (with GDTK_PHASE_CLOCKS=1) time per phase, on an untimed update
    lanes = None
    if args.lane_stats:
        drc = rc
        if phase_clocks:   # a separately generated, instrumented kernel for this diagnostic update only
            os.environ["GDTK_PHASE_CLOCKS"] = "1"
            drc = ReactorCells(os.path.join(MECH, w["gas"]), os.path.join(MECH, w["chem"]))
        stats = torch.zeros(24, dtype=torch.int64, device=dev)
        drc.set_lane_stats(stats)
        T.copy_(sT); p.copy_(sp); Y.copy_(sY); dtc.copy_(sdt)
        drc.update(srho, su, T, p, Y, dtc, w["dt"], status=st, flags=flags)
        torch.cuda.synchronize()
        drc.set_lane_stats(None)
        if phase_clocks:
            os.environ.pop("GDTK_PHASE_CLOCKS", None)
        lanes = lane_stats_summary(stats.cpu().numpy())

    # ---- CPU baseline (reference algorithm on the host cores), rank 0 at N=1 only
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        r = cpu_reference_run(w, T0, p0, Y0, srho.cpu().numpy(), su.cpu().numpy(), max_seconds=args.cpu_seconds)
        cpu = {"value": r["value"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
               "sample": "%d of the %d cells (evenly strided), %.1f s on %d threads" %
                         (r["cells"], n, r["seconds"], r["threads"])}

    # ---- the surrogate + FP64 fallback form of the same update (the second half of the metric)
    sur = None
    if rank == 0 and ws == 1 and args.workload == "h2air-1M" and not args.no_surrogate:
        plain_T, plain_Y, plain_st = T.clone(), Y.clone(), st.clone()   # the last timed step's plain result
        sur = surrogate_leg(rc, srho, su, sT, sp, sY, w["dt"], ms_per_step, plain_T, plain_Y, plain_st)

    # ---- the uneven multi-block batch (config of 64 blocks, per-split-step latency), default shape
    blk = None
    if rank == 0 and ws == 1 and args.workload == "h2air-1M" and not args.no_blocks:
        b = run_blocks(args, WORKLOADS["h2air-blocks64"], tune=False, cpu=False)
        lat = b["latency_ms"]
        blk = {"workload": "h2air-blocks64", "cell_updates_per_s": b["value"], "cells": b["config"]["cells"],
               "blocks": b["config"]["blocks"], "split_steps": b["steps"],
               "ms_per_split_step": {"mean": b["ms_per_step"], "p50": lat["p50"], "p99": lat["p99"],
                                     "p99_over_p50": lat["p99"] / lat["p50"]},
               "per_split_step_ms": lat["per_step"], "cells_failed_last_step": b["config"]["cells_failed"],
               "launch_shape": "default (256 threads x 1 block per SM, longest-first), no tuning",
               "roofline_frac": b["roofline"]["frac"], "roofline_basis": b["roofline"].get("basis"),
               "timing": "CUDA events around each graph replay of one split step, after one untimed split step",
               "clocks": b["clocks"]}

    if rank == 0:
        traffic = None
        tj = profile_record("traffic.json", args.workload)
        if tj:
            traffic = tj["bytes_per_cell"] * n
        issued = profile_record("fp64_issued.json", args.workload)
        ok = int((status == 0).sum())
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "cells_per_gpu": n, "mechanism": w["chem"], "dt": w["dt"],
                       "method": rc.method, "tight_coupling": rc.tight, "dt_chem_in": -1.0,
                       "l2": "inputs larger than L2 (no flush): %.0f MB of cell state" % (n * 8 * (5 + rc.nsp) / 1e6),
                       "parallelism": "replicas x%d" % ws,
                       "cells_ok": ok, "cells_failed": int(n - ok), "codegen_env": codegen_env(),
                       "autotuned": tuned},
            "roofline": roofline_fp64(issued, n, kernel_ms, peak, flops, traffic, tot / args.steps / n),
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            # thread per cell: cost pre-pass, 3 ordering kernels, chemistry; one warp per cell: chemistry
            "gpu_launches": args.steps * (1 if (rc.nsp > 32 or rc.nr > 128 or flags & 16) else 5),
        }
        if sur is not None:
            line["surrogate"] = sur
        if blk is not None:
            line["blocks64"] = blk
        if lanes is not None:
            line["lane_stats"] = lanes
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
