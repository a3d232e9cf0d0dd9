"""Launch-shape autotuner for the mechanism-specialised chemistry kernel.

The kernel's throughput depends on how many threads each SM keeps resident and on how the
register file and shared memory are split between them (each thread holds its kf/kb and
method vectors in shared memory), and on the order in which the persistent work queue hands
out cells.  The tuner times a sample of the caller's own cells under each candidate
  (threads per block, blocks per SM) x (longest-first | index order)
that fits the shared-memory budget, keeps the fastest, and records the choice in a versioned
JSON file keyed by mechanism, device and workload tag, so later runs reuse it without timing.
"""
import hashlib
import json
import os
import time

from . import lib, check

CACHE_VERSION = 1
SHAPES = [(256, 1), (224, 1), (192, 1), (160, 1), (128, 1), (128, 2), (96, 2), (64, 2), (64, 3)]
ORDERS = {"longest-first": 0, "index": 8}


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


def apply(rc, choice):
    check(lib().chem_reactor_configure(rc.reactor.id, int(choice["block"]), int(choice["min_blocks"])),
          "chem_reactor_configure")
    return ORDERS[choice["order"]]


def tune(rc, sample, t_interval, tag="default", repeats=1, use_cache=True, flags=3):
    """Picks the launch shape for `rc` on `sample` (dict of cuda tensors rho, u, T, p, massf,
    dt_chem; left unchanged).  Returns (choice, extra_flags, results)."""
    import torch
    key = _key(rc, tag)
    table = _load() if use_cache else {}
    if use_cache and key in table:
        choice = table[key]
        return choice, apply(rc, choice), choice.get("results", [])
    results = []
    for block, mb in SHAPES:
        if check_shape(rc, block, mb) is False:
            continue
        for oname, oflag in ORDERS.items():
            best = None
            for _ in range(repeats + 1):   # first run compiles / warms up
                T, p, Y, dt = (sample["T"].clone(), sample["p"].clone(), sample["massf"].clone(),
                               sample["dt_chem"].clone())
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                rc.update(sample["rho"], sample["u"], T, p, Y, dt, t_interval, flags=flags | oflag)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            results.append(dict(block=block, min_blocks=mb, order=oname, ms=best))
    if not results:
        raise RuntimeError("no launch shape fits this mechanism")
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
