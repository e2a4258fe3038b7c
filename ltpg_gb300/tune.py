"""Autotuner for the tuned kernels' launch shape.

Searches block size, ops per thread, blocks per SM, the slot-read filter, the
warp dedupe, the staging ways and (YCSB) where the rows are read (at execute,
after the check for committed transactions only, or write-first) on the
batches already uploaded to an engine, times each candidate with CUDA events
on the engine's stream, and keeps the fastest.  Every candidate's commit
bitmaps are compared with the plain path's on the same batch before it may
win: a launch shape can change speed, never a commit decision.  The reference
fixes its block and grid sizes at compile time (TF/Predefine.h:36-46) and
sweeps them by rewriting that file (TF/tpcc_script.py:18-44).

Results are cached per (GPU, workload).  Lookups read the caller's cache file
first (cache_path, else $LTPG_TUNE_CACHE, else
~/.cache/ltpg_gb300/tuned_launch.json), then the shapes shipped with the
package (ltpg_gb300/tuned_launch.json, read-only); new results are written to
the caller's file only (`bench.py --retune --tune-cache FILE` tunes a
benchmark workload and writes its entry there).
"""
import itertools
import json
import os

import numpy as np

from . import abi

SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned_launch.json")
BLOCKS = (128, 256, 512)


def user_cache_path():
    """The caller-writable cache file: $LTPG_TUNE_CACHE, else under ~/.cache."""
    env = os.environ.get("LTPG_TUNE_CACHE")
    if env:
        return env
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "ltpg_gb300", "tuned_launch.json")


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _key(workload_key):
    return f"{_gpu_name()}|{workload_key}"


def _read(path):
    try:
        return json.load(open(path))
    except (OSError, ValueError):
        return {}


def load_cached(workload_key, cache_path=None):
    """The cached shape of this GPU and workload: the caller's cache file
    first, then the shipped shapes; None when neither has one."""
    for path in (cache_path or user_cache_path(), SHIPPED):
        cfg = _read(path).get(_key(workload_key))
        if cfg:
            return cfg
    return None


def save_cached(workload_key, cfg, cache_path=None):
    """Adds this GPU's and workload's shape to the caller's cache file."""
    path = cache_path or user_cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    data = _read(path)
    data[_key(workload_key)] = cfg
    with open(path + ".tmp", "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(path + ".tmp", path)


def candidates(workload, staging=False, blocks=BLOCKS):
    """Launch shapes to try.  blocks_per_sm caps are in units of 256-thread
    blocks' worth of warps, so every block size is tried at the same
    resident-warp caps."""
    def cap(b, bs):
        return 0 if b == 0 else max(1, b * 256 // bs)

    if workload == "ycsb":
        out = []
        for bs in blocks:
            grid = itertools.product([1, 2, 4], [0, 2, 4], [0, 1], [0, 1], [2, 4] if staging else [4])
            out += [dict(block_threads=bs, ops_per_thread=o, blocks_per_sm=cap(b, bs), filter=f, dedupe=d,
                         stage_ways=w, late_reads=0) for o, b, f, d, w in grid]
            # late reads (in the check kernel, or a kernel of their own) run the
            # one-op-per-lane registration kernel whatever ops_per_thread says
            grid = itertools.product([1, 2], [0, 2, 4], [0, 1], [0, 1], [2, 4] if staging else [4])
            out += [dict(block_threads=bs, ops_per_thread=1, blocks_per_sm=cap(b, bs), filter=f, dedupe=d,
                         stage_ways=w, late_reads=r) for r, b, f, d, w in grid]
            # write-first registration: no warp dedupe; the filter applies to the updates
            out += [dict(block_threads=bs, ops_per_thread=1, blocks_per_sm=cap(b, bs), filter=f, dedupe=0,
                         stage_ways=4, late_reads=3) for b, f in itertools.product([0, 2, 4], [0, 1])]
        return out
    # TPC-C: blocks of 2P threads on tiles of P transactions
    return [dict(block_threads=bs, ops_per_thread=4, blocks_per_sm=cap(b, bs), filter=f, dedupe=d, stage_ways=4,
                 late_reads=0)
            for bs in blocks for b, f, d in itertools.product([0, 2, 4, 6], [0, 1], [0, 1])]


def _time_batches(eng, slots, reps, mode, torch):
    stream = torch.cuda.ExternalStream(eng.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    eng.sync()
    ev0.record(stream)
    for _ in range(reps):
        for s in slots:
            eng.run_batch(s, mode)
    ev1.record(stream)
    eng.sync()
    return ev0.elapsed_time(ev1) / (reps * len(slots))


def autotune(eng, workload, slots, reload, mode="fused", reps=3, staging=False, verify_slot=None, log=None,
             cands=None):
    """Times every candidate launch shape (cands, default candidates()) on the
    uploaded batches in `slots`.

    reload(): restores the table image (used before each verification run so
    plain and tuned start from the same state).  Returns (best_cfg, table)."""
    import torch
    wl = "ycsb" if workload == "ycsb" else "tpcc"
    vslot = slots[0] if verify_slot is None else verify_slot
    n = None
    # reference bitmap of the plain path
    reload()
    eng.run_batch(vslot, "plain")
    eng.sync()
    st = eng.stats(vslot)
    n = int(st["n_txn"])
    want = eng.commit_bitmap(vslot, n)
    table = []
    best = None
    for cfg in (cands if cands is not None else candidates(wl, staging)):
        try:
            eng.set_launch(wl, **cfg)
        except Exception as e:  # an invalid shape for this GPU
            table.append((cfg, None, str(e)))
            continue
        reload()
        eng.run_batch(vslot, mode)
        eng.sync()
        ok = np.array_equal(eng.commit_bitmap(vslot, n), want)
        if not ok:
            table.append((cfg, None, "bitmap differs from the plain path"))
            continue
        _time_batches(eng, slots, 1, mode, torch)  # warm
        ms = _time_batches(eng, slots, reps, mode, torch)
        table.append((cfg, ms, "ok"))
        if log:
            log(f"{cfg} {ms:.4f} ms/batch")
        if best is None or ms < best[1]:
            best = (cfg, ms)
    if best is None:
        raise RuntimeError("no launch shape reproduced the plain path's commit bitmap")
    eng.set_launch(wl, **best[0])
    return dict(best[0], ms_per_batch=best[1]), table


def apply_cached_or_tune(eng, workload, workload_key, slots, reload, cache_path=None, retune=False, **kw):
    """Uses the cached launch shape for this GPU and workload (unless retune),
    else tunes and adds the result to the caller's cache file."""
    wl = "ycsb" if workload == "ycsb" else "tpcc"
    cfg = None if retune else load_cached(workload_key, cache_path)
    if cfg:
        eng.set_launch(wl, **{k: v for k, v in cfg.items() if k in dict(abi.LaunchC._fields_)})
        return cfg, "cache"
    best, _ = autotune(eng, workload, slots, reload, **kw)
    save_cached(workload_key, best, cache_path)
    return best, "tuned"
