"""Launch-shape autotuner for the mechanism-specialised chemistry kernel.

The kernel's throughput depends on how many threads each SM keeps resident and on how the
register file and shared memory are split between them (each thread holds its kf/kb and
method vectors in shared memory), on the order in which the persistent work queue hands out
cells and how many it hands out per atomic (the refill chunk), and on how many cells a warp
integrates at once (32, one per thread; or 1, with species and reactions over the lanes).  The
tuner times a sample of the caller's own cells under
  (threads per block, blocks per SM) x (longest-first | index order), then refill chunks on
  the best of those, then one warp per cell,
keeps the fastest, and records the choice in a versioned JSON file keyed by mechanism, device
and workload tag, so later runs reuse it without timing.
"""
import hashlib
import json
import os
import time

from . import lib, check

CACHE_VERSION = 2
SHAPES = [(256, 1), (224, 1), (192, 1), (160, 1), (128, 1), (128, 2), (96, 2), (64, 2), (64, 3)]
ORDERS = {"longest-first": 0, "index": 8}
CHUNKS = [128, 1024]          # refill chunks tried on the best shape (0: exactly the lanes that need a cell)
WARP_PER_CELL = 16            # GDTK_CHEM_WARP_PER_CELL
THREAD_LIMITS = (32, 128)     # species and reactions of the thread-per-cell kernel


def cache_path():
    d = os.environ.get("GDTK_JIT_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "gdtk_gb300")
    return os.path.join(d, "tune.json")


def _key(rc, tag):
    import torch
    h = hashlib.sha1()
    for f in (rc.gmodel.file_name, rc.reactor.filename1):
        with open(f, "rb") as fh:
            h.update(fh.read())
    return "%s|%s|%s|v%d" % (h.hexdigest()[:16], torch.cuda.get_device_name(), tag, CACHE_VERSION)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(table):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".%d.tmp" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def set_refill_chunk(rc, cells):
    check(lib().chem_reactor_set_refill_chunk(rc.reactor.id, int(cells)), "chem_reactor_set_refill_chunk")


def apply(rc, choice):
    """Loads the chosen variant into `rc`; returns the flags the caller adds to its updates."""
    if choice.get("cells_per_warp", 32) == 1:
        return WARP_PER_CELL
    check(lib().chem_reactor_configure(rc.reactor.id, int(choice["block"]), int(choice["min_blocks"])),
          "chem_reactor_configure")
    set_refill_chunk(rc, choice.get("refill_chunk", 0))
    return ORDERS[choice["order"]]


def _time(rc, sample, t_interval, flags, repeats):
    """Fastest of `repeats` updates of a copy of `sample` (after one untimed run), in ms."""
    import torch
    best = None
    for _ in range(repeats + 1):   # first run compiles / warms up
        T, p, Y, dt = (sample["T"].clone(), sample["p"].clone(), sample["massf"].clone(), sample["dt_chem"].clone())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc.update(sample["rho"], sample["u"], T, p, Y, dt, t_interval, flags=flags)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return best


def tune(rc, sample, t_interval, tag="default", repeats=1, use_cache=True, flags=3, allow_warp=True):
    """Picks the chemistry kernel variant for `rc` on `sample` (dict of cuda tensors rho, u, T, p,
    massf, dt_chem; left unchanged).  Dimensions, searched in turn:
      cells per warp 32 (one thread per cell): (threads per block, blocks per SM) x visit order, then
        the refill chunk on the best of those;
      cells per warp 1 (one warp per cell; the only variant for mechanisms beyond 32 species or 128
        reactions), unless allow_warp is False (the block-batch entry point takes thread-per-cell only).
    Returns (choice, extra_flags, results)."""
    key = _key(rc, tag) + ("" if allow_warp else "|thread-per-cell")
    table = _load() if use_cache else {}
    if use_cache and key in table:
        choice = table[key]
        return choice, apply(rc, choice), choice.get("results", [])
    large = rc.nsp > THREAD_LIMITS[0] or rc.nr > THREAD_LIMITS[1]
    results = []
    if not large:
        set_refill_chunk(rc, 0)
        for block, mb in SHAPES:
            if check_shape(rc, block, mb) is False:
                continue
            for oname, oflag in ORDERS.items():
                ms = _time(rc, sample, t_interval, flags | oflag, repeats)
                results.append(dict(block=block, min_blocks=mb, order=oname, refill_chunk=0, cells_per_warp=32,
                                    ms=ms))
        if results:
            best = min(results, key=lambda r: r["ms"])
            check_shape(rc, best["block"], best["min_blocks"])
            for cells in CHUNKS:
                set_refill_chunk(rc, cells)
                ms = _time(rc, sample, t_interval, flags | ORDERS[best["order"]], repeats)
                results.append(dict(best, refill_chunk=cells, ms=ms))
            set_refill_chunk(rc, 0)
    if allow_warp or large:
        ms = _time(rc, sample, t_interval, flags | WARP_PER_CELL, repeats)
        results.append(dict(block=0, min_blocks=0, order="index", refill_chunk=0, cells_per_warp=1, ms=ms))
    if not results:
        raise RuntimeError("no kernel variant fits this mechanism")
    choice = dict(min(results, key=lambda r: r["ms"]))
    choice["results"] = results
    choice["when"] = time.strftime("%Y-%m-%dT%H:%M:%S")
    if use_cache:
        table[key] = choice
        _save(table)
    return choice, apply(rc, choice), results


def check_shape(rc, block, min_blocks):
    """True if the shape compiles and fits; False otherwise (the variant stays loaded if True)."""
    rcode = lib().chem_reactor_configure(rc.reactor.id, block, min_blocks)
    return rcode == 0
