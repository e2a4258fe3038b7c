"""Benchmark: committed transactions per second of the GB300 engine.

Default workload: YCSB high contention (10,000,000 records of 10 x uint64,
batches of 1,048,576 transactions x 16 operations, 95% read / 5% update, Zipf
theta 0.99, hot set re-permuted every 8 batches, 32 distinct batches resident
in HBM).  A step is one batch through the tuned path (two fused kernels per
batch, the whole run captured as CUDA graphs).  The plain three-kernel path is
timed on the same batches, and both are checked to give bit-identical commit
bitmaps and table images.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload ycsb_hc|ycsb_small|tpcc|...] [--theta T] [--no-sweep] [--no-tpcc]
                  [--no-small]

The default line also carries the TPC-C W=64 NewOrder+Payment workload (key
"tpcc": tuned and plain, bit-exactness, end to end, HBM and atomic
rooflines, CPU baseline), the YCSB theta sweep 0 / 0.6 / 0.8 / 0.99 (key
"theta_sweep", tuned against plain) and the small-batch YCSB workload (key
"small_batches": 65,536 transactions x 10 ops on 1 M records, tuned against
plain).

--impl reference times the reference protocol's CPU replay (the oracle port,
all host threads) on the same workload; the reference has no CPU implementation
of its own.  Under torchrun each rank runs an independent replica (the path
does not shard here), rank 0 prints one JSON line.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "ycsb_hc": dict(kind="ycsb", n_records=10_000_000, n_txn=1 << 20, ops=16, update_pct=5, theta=0.99,
                    rotate_every=8, n_batches=32,
                    name="YCSB high contention: 10M x 10 uint64, 1,048,576 txn x 16 ops, 95/5, "
                         "Zipf theta=0.99, hot set rotating every 8 batches, 32 batches"),
    "ycsb_hc_prof": dict(kind="ycsb", n_records=10_000_000, n_txn=1 << 18, ops=16, update_pct=5, theta=0.99,
                         rotate_every=8, n_batches=4,
                         name="YCSB high contention, profiling size: 10M x 10 uint64, 262,144 txn x 16 ops, "
                              "95/5, Zipf theta=0.99, 4 batches"),
    "ycsb_scan": dict(kind="ycsb", n_records=10_000_000, n_txn=1 << 18, ops=10, update_pct=5, theta=0.99,
                      rotate_every=8, n_batches=16, scan_len=10,
                      name="YCSB range scans: 10M x 10 uint64, 262,144 txn x 10 ops, 95/5, every read scans "
                           "10 keys, Zipf theta=0.99"),
    "ycsb_small": dict(kind="ycsb", n_records=1_000_000, n_txn=65536, ops=10, update_pct=50, theta=0.6,
                       rotate_every=0, n_batches=32,
                       name="YCSB small: 1M x 10 uint64, 65,536 txn x 10 ops, 50/50, Zipf theta=0.6"),
    "tpcc": dict(kind="tpcc", warehouses=64, n_txn=1 << 20, n_batches=8,
                 name="TPC-C NewOrder+Payment 50/50, W=64, 1,048,576 txn per batch"),
    "tpcc_mix": dict(kind="tpcc", warehouses=64, n_txn=1 << 20, n_batches=8,
                     mix=dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4, by_name_pct=60),
                     name="TPC-C five-transaction mix 45/43/4/4/4 (customers by last name 60 %), W=64, "
                          "1,048,576 txn per batch"),
    "tpcc_prof": dict(kind="tpcc", warehouses=16, n_txn=1 << 18, n_batches=4,
                      name="TPC-C NewOrder+Payment 50/50, profiling size: W=16, 262,144 txn per batch"),
    "tpcc_mix_prof": dict(kind="tpcc", warehouses=16, n_txn=1 << 18, n_batches=4,
                          mix=dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4,
                                   by_name_pct=60),
                          name="TPC-C five-transaction mix, profiling size: W=16, 262,144 txn per batch"),
}
SEED = 20261203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1024)
    ap.add_argument("--warmup", type=int, default=32)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ycsb_hc", choices=sorted(WORKLOADS))
    ap.add_argument("--theta", type=float, default=None)
    ap.add_argument("--mode", default="graph", choices=["fused", "graph", "persistent"])
    ap.add_argument("--no-small", action="store_true", help="skip the small-batch (65,536 txn) record")
    ap.add_argument("--no-sweep", action="store_true", help="skip the theta 0/0.6/0.8/0.99 sweep (YCSB)")
    ap.add_argument("--no-tpcc", action="store_true", help="skip the TPC-C W=64 record of the YCSB line")
    ap.add_argument("--cpu-batches-tpcc", type=int, default=3,
                    help="whole TPC-C batches replayed by the single-threaded CPU baseline")
    ap.add_argument("--ref-scale-iters", type=int, default=10,
                    help="timed batches of the reference's kernels at the headline scale")
    ap.add_argument("--cpu-batches", type=int, default=12,
                    help="batches in the CPU-baseline sample (about 10 s of oracle replay at the default sizes)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=64,
                    help="steps of the end-to-end leg (host wall clock; long enough to average out host stalls)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop section")
    ap.add_argument("--no-device-gen", action="store_true", help="skip the device-generator section")
    ap.add_argument("--late-reads", type=int, choices=[0, 1, 2, 3], default=None,
                    help="YCSB: override the launch setting late_reads (0 rows read at execute, 1 after the check "
                         "in the check kernel, 2 in a kernel of their own, 3 write-first registration)")
    ap.add_argument("--retune", action="store_true",
                    help="tune the launch shape even when one is cached, and cache the result")
    ap.add_argument("--tune-cache", default=None,
                    help="cache file the autotuner reads first and writes (default: ltpg_gb300.tune.user_cache_path())")
    ap.add_argument("--no-tune", action="store_true",
                    help="the engine's default launch shape, no autotuning (profiling runs)")
    ap.add_argument("--no-predictor", action="store_true", help="skip the predictor section")
    ap.add_argument("--serve-seconds", type=float, default=0.25)
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the reference's own kernels / the engine on the reference's compiled shapes")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        # one process per GPU over NCCL; gloo where there is no GPU (the
        # reference arm's CPU replay, and the multi-rank tests)
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return ws, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def _reduce_device(dist):
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        import select
        self.first = ""
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            # the first sample is taken before the region opens, so a region
            # shorter than the sampling period still has the state at its start
            if select.select([self.p.stdout], [], [], 5.0)[0]:
                self.first = self.p.stdout.readline()
        except OSError:
            self.p = None
        self.t0 = time.time()
        return self

    def __exit__(self, *exc):
        self.t1 = time.time()
        self.rows = []
        if self.p is None:
            return
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        for line in (self.first + out).strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 8:
                self.rows.append(f)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---- byte model (algorithmic bytes, logical, no sector rounding) --------------------
def ycsb_bytes_per_txn(k, u, commit_rate, scan=1, late=False):
    """Per transaction: op words 4k, value offset 4, update values 8uk, registration
    (8-byte slot word read+written) 16 per update and 16 per key a read covers,
    check loads 8 per key a read covers / 16 per update, row reads 80 per key a
    read covers, committed update stores 8 per update of a committed
    transaction, result 8, flags 1+1, bitmap 1/8.  A read covers `scan` keys
    (1: point reads).  Returns bytes of (execute, check + write-back, 0, 0).

    late (1: reads in the check kernel, 2: a read kernel of their own):
    execute registers only; the check reads op words, slots and writes flags
    and bitmap; the reads read the committed transactions' op words (4k times
    the commit rate) and rows (80 per covered key of a read times the commit
    rate) and write the result 8 (late 2 also reads the flag 1); the
    write-back reads the flag 1 and, for a committed transaction, its value
    offset 4, op words 4k and update values 8uk, and stores 8uk.  Returns
    bytes of (execute, check + reads, 0, write-back) for late 1 and
    (execute, check, reads, write-back) for late 2.

    late 3 (write-first registration): "execute" is the write registration
    (op words 4k, slot RMW 16 per update) and the read registration (op words
    4k, one 16-byte slot load per covered key of a read, which also carries
    the conditional registration, RAW flag 1); the check reads op words 4k and
    16 per update and ORs the flag 1; the reads as above; the write-back also
    reads and writes the flag (1 + 1) and writes the bitmap 1/8."""
    if not late:
        exec_b = 4 * k + 16 * u * k + (16 + 80) * (1 - u) * k * scan + 8
        check_b = (4 * k + 4 + 8 * (1 - u) * k * scan + 16 * u * k + 8 * u * k + 8 * u * k * commit_rate + 1
                   + 1 / 8)
        return exec_b, check_b, 0.0, 0.0
    exec_b = 4 * k + 16 * u * k + 16 * (1 - u) * k * scan
    check_b = 4 * k + 8 * (1 - u) * k * scan + 16 * u * k + 1 + 1 / 8
    read_b = commit_rate * (4 * k + 80 * (1 - u) * k * scan) + 8
    wb_b = 1 + commit_rate * (4 + 4 * k + 16 * u * k)
    if late == 1:
        return exec_b, check_b + read_b, 0.0, wb_b
    if late == 3:
        return (8 * k + 16 * u * k + 16 * (1 - u) * k * scan + 1, 4 * k + 16 * u * k + 1, read_b + 1,
                wb_b + 1 + 1 / 8)
    return exec_b, check_b, read_b + 1, wb_b


def profile_traffic(workload, kernel):
    """DRAM bytes per transaction measured by ncu, from profiles/<kernel>_<workload>.md
    (or the profiling-size variant of the workload, whose traffic per transaction
    is the same: it grows in proportion to the batch)."""
    for wl in (workload, workload + "_prof"):
        path = os.path.join(ROOT, "profiles", f"{kernel}_{wl}.md")
        if os.path.exists(path):
            m = re.search(r"dram_bytes_per_txn:\s*([0-9.]+)", open(path).read())
            if m:
                return float(m.group(1))
    return None


def ycsb_exec_kernel_name(launch, stride):
    """Name of the execute kernel the tuned path launches for this shape."""
    opt = (launch or {}).get("ops_per_thread", 1)
    if (opt == 1 or (launch or {}).get("late_reads")) and stride <= 32:
        return "ycsb_exec_coop"
    if opt in (2, 4) and stride % opt == 0 and ((stride // opt) & (stride // opt - 1)) == 0:
        return "ycsb_exec_fast"
    return "ycsb_exec_tuned"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path)), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


# ---- YCSB ---------------------------------------------------------------------------
def make_ycsb(w, theta):
    from ltpg_gb300 import YcsbGenerator
    g = YcsbGenerator(SEED, w["n_records"], w["n_txn"], w["ops"], w["update_pct"], theta, w["rotate_every"],
                      w.get("scan_len", 0))
    return [g.batch(i) for i in range(w["n_batches"])]


def step_chunks(n_slots, steps, start=0):
    """The (first slot, count) calls that run `steps` batches from slot `start`."""
    out, i = [], 0
    while i < steps:
        s = (start + i) % n_slots
        cnt = min(steps - i, n_slots - s)
        out.append((s, cnt))
        i += cnt
    return out


def run_steps(eng, n_slots, steps, mode, start=0):
    """Runs `steps` batches, batch i in slot (start + i) % n_slots, as few calls as possible."""
    for s, cnt in step_chunks(n_slots, steps, start):
        if mode == "graph":
            eng.run_batches(s, cnt, "graph")
        else:
            for j in range(cnt):
                eng.run_batch(s + j, mode)
    return (start + steps) % n_slots


def prepare_graphs(eng, n_slots, steps, mode, start):
    """Graph mode: runs each distinct call of a timed run of `steps` batches
    from `start` once, untimed, so that its graph is captured and
    instantiated before the timed region, which then only replays graphs.
    Extra untimed batches change no commit decision (a batch's outcome depends
    on its operations alone)."""
    if mode != "graph":
        return
    for s, cnt in sorted(set(step_chunks(n_slots, steps, start))):
        eng.run_batches(s, cnt, "graph")
    eng.sync()


def timed(eng, torch, n_slots, steps, mode, start, dist):
    stream = torch.cuda.ExternalStream(eng.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    prepare_graphs(eng, n_slots, steps, mode, start)
    eng.sync()
    barrier(dist)
    torch.cuda.synchronize()
    c0, l0 = eng.counters()
    ev0.record(stream)
    nxt = run_steps(eng, n_slots, steps, mode, start)
    ev1.record(stream)
    eng.sync()
    torch.cuda.synchronize()
    barrier(dist)
    c1, l1 = eng.counters()
    return ev0.elapsed_time(ev1) / 1e3, c1 - c0, l1 - l0, nxt


def kernel_split(eng, n_slots, mode, start):
    """Per-kernel times of one more pass over the slots, after the timed region:
    the events that split a batch into its kernels are recorded only here, so
    the timed region carries no instrumentation (on 40-us batches it cost a
    quarter of the time).  Rows: slots; columns: execute, check, reads,
    write-back (a phase inside another kernel reads 0: the tuned check kernel
    also writes back unless YCSB reads late)."""
    eng.set_profiling(True)
    run_steps(eng, n_slots, n_slots, mode, start)
    eng.sync()
    kt = np.array([eng.kernel_times(s) for s in range(n_slots)])
    eng.set_profiling(False)
    return kt


def modes_run(eng, torch, n_slots, steps, reload):
    """The same resident batches through each execution mode of the tuned
    path: fused (two kernels per batch), graph (one CUDA graph over the
    slots), persistent (one cooperative kernel per batch, grid barrier between
    the phases).  Committed txn/s and ms per batch."""
    out = {}
    for m in ["fused", "graph", "persistent"]:
        reload()
        eng.sync()
        nxt = run_steps(eng, n_slots, 4, m)
        secs, commits, launches, _ = timed(eng, torch, n_slots, steps, m, nxt, None)
        out[m] = {"value": commits / secs, "ms_per_batch": secs * 1e3 / steps, "launches_per_batch": launches / steps}
    return out


def h2d_link_gbs(nbytes, reps=4):
    """Host-to-device copy rate of this machine (one pinned buffer of the batch's
    size, one cudaMemcpyAsync, CUDA events): the bound of the end-to-end rate
    when a batch's copy takes longer than its kernels."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d.copy_(h, non_blocking=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        d.copy_(h, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    return nbytes * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9


def e2e_run(eng, pinned, mode, steps, n_slots, n_txn, dist, depth=3):
    """End to end through the pipelined host-buffer calls (ltpg_submit_*_host /
    ltpg_host_wait): every step copies its pinned host batch to the device,
    runs it and copies its commit bitmap back to pinned host memory; up to
    `depth` steps are in flight, so one batch's copy overlaps the previous
    one's kernels.  Host wall time from the first submit to the last bitmap."""
    import ltpg_gb300 as L
    depth = max(1, min(depth, n_slots))
    words = (n_txn + 31) // 32
    bits = [L.pinned_empty(words) for _ in range(depth)]

    def go(count):
        for i in range(count):
            s = i % depth
            if i >= depth:
                eng.host_wait(s)
            eng.submit_host(s, pinned[i % len(pinned)], mode, bits[s])
        for i in range(max(0, count - depth), count):
            eng.host_wait(i % depth)

    go(depth + 2)
    c0, _ = eng.counters()
    barrier(dist)
    t0 = time.perf_counter()
    go(steps)
    t1 = time.perf_counter()
    c1, _ = eng.counters()
    return dict(secs=t1 - t0, commits=c1 - c0, steps=steps, depth=depth, link_GBs=h2d_link_gbs(pinned[0].nbytes()),
                h2d=int(np.mean([p.nbytes() for p in pinned])), d2h=words * 4)


def ycsb_bench(args, w, theta, dist, want_extras=True):
    import torch
    import ltpg_gb300 as L
    batches = make_ycsb(w, theta)
    n_slots = len(batches)
    eng = L.Engine(device=0, n_slots=n_slots, max_txn=w["n_txn"], max_ops_per_txn=w["ops"])
    res = {}
    try:
        eng.load_ycsb(SEED, w["n_records"])
        for i, b in enumerate(batches):
            eng.upload(i, b)
        for mode in ["plain", args.mode]:
            if mode != "plain" and args.no_tune:
                res["launch"] = dict(eng.get_launch("ycsb"), source="default")
            elif mode != "plain":
                from ltpg_gb300 import tune
                wkey = f"{w['key']}|theta={theta}"
                cfg, how = tune.apply_cached_or_tune(eng, "ycsb", wkey, list(range(min(8, n_slots))),
                                                     lambda: eng.load_ycsb(SEED, w["n_records"]),
                                                     cache_path=args.tune_cache, retune=args.retune)
                res["launch"] = dict(cfg, source=how)
            if mode != "plain" and args.late_reads is not None:
                eng.set_launch("ycsb", late_reads=args.late_reads)
                res["launch"] = dict(res["launch"], late_reads=args.late_reads, source=res["launch"]["source"] +
                                     " + --late-reads")
            eng.load_ycsb(SEED, w["n_records"])
            eng.sync()
            nxt = run_steps(eng, n_slots, args.warmup, mode)
            with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
                secs, commits, launches, nxt = timed(eng, torch, n_slots, args.steps, mode, nxt, dist)
            kt = kernel_split(eng, n_slots, mode, nxt) if mode != "plain" and want_extras else None
            res[mode] = dict(secs=secs, commits=commits, launches=launches, clocks=clk.summary(), kt=kt)
        if want_extras:
            res["modes"] = modes_run(eng, torch, n_slots, min(args.steps, 64),
                                     lambda: eng.load_ycsb(SEED, w["n_records"]))
        # access-pattern ceilings of this GPU (the practical rooflines of the kernels' parts)
        if want_extras:
            res["ceilings"] = {
                "copy_GBs": eng.microbench("copy", 1 << 27) / 1e9,
                "row_gather_5lane_GBs": eng.microbench("gather_coop", 16_000_000) / 1e9,
                "row_gather_1thread_GBs": eng.microbench("gather_thread", 16_000_000) / 1e9,
                "slot_load_G_per_s": eng.microbench("slot_load", 16_000_000) / 1e9,
                "red_min_random_G_per_s": eng.microbench("red_random", 16_000_000) / 1e9,
                "red_min_one_slot_G_per_s": eng.microbench("red_hot", 1_000_000) / 1e9,
            }
        # bit-exactness of the tuned path against the plain path on the first
        # batches (four with the extras, two for the sweep and the small batches)
        ref = {}
        for mode in ["plain", args.mode]:
            eng.load_ycsb(SEED, w["n_records"])
            outs = []
            for i in range(min(len(batches), 4 if want_extras else 2)):
                eng.upload(0, batches[i])
                eng.run_batch(0, mode if mode != "graph" else "graph")
                eng.sync()
                outs.append(eng.commit_bitmap(0, w["n_txn"]))
                # results of the committed transactions (with late reads an
                # aborted transaction's result is 0 by definition)
                com = (eng.txn_flags(0, w["n_txn"]) & L.FLAG_COMMIT) != 0
                outs.append(eng.txn_results(0, w["n_txn"])[com])
            img = eng.download_table(L.TABLE_YCSB)
            ref[mode] = (outs, int(np.bitwise_xor.reduce(img)), int(img.sum()))
        a, b = ref["plain"], ref[args.mode]
        exact = all(np.array_equal(x, y) for x, y in zip(a[0], b[0])) and a[1:] == b[1:]
        # end to end through the host-buffer C-ABI call (pinned host batch, H2D + run + bitmap D2H)
        e2e = None
        if want_extras:
            eng.load_ycsb(SEED, w["n_records"])
            pinned = [L.pinned_copy(b) for b in batches[:min(len(batches), 8)]]
            e2e = e2e_run(eng, pinned, args.mode, args.e2e_steps, n_slots, w["n_txn"], dist)
    finally:
        eng.close()
    return res, exact, e2e, batches


def cpu_baseline_ycsb(w, batches, n_batches, threads=1):
    import oracle
    o = oracle.YcsbOracle(SEED, w["n_records"])
    commits, secs = 0, 0.0
    for b in batches[:n_batches]:
        t0 = time.perf_counter()
        _, _, _, c = o.run(b, threads=threads)
        secs += time.perf_counter() - t0
        commits += c
    return commits / secs, secs, commits


# ---- TPC-C --------------------------------------------------------------------------
def tpcc_bench(args, w, dist, want_extras=True):
    import torch
    import ltpg_gb300 as L
    g = L.TpccGenerator(SEED, w["warehouses"], w["n_txn"], **w.get("mix", {}))
    batches = [g.next() for _ in range(w["n_batches"])]
    n_slots = len(batches)
    max_lines = max(b.n_lines for b in batches)
    eng = L.Engine(device=0, n_slots=n_slots, max_txn=w["n_txn"], max_ops_per_txn=16, max_lines=max_lines)
    res = {}
    try:
        eng.load_tpcc(SEED, w["warehouses"])
        for i, b in enumerate(batches):
            eng.upload(i, b)
        for mode in ["plain", args.mode]:
            if mode != "plain" and args.no_tune:
                res["launch"] = dict(eng.get_launch("tpcc"), source="default")
            elif mode != "plain":
                from ltpg_gb300 import tune
                cfg, how = tune.apply_cached_or_tune(eng, "tpcc", w["key"], list(range(min(4, n_slots))),
                                                     lambda: eng.load_tpcc(SEED, w["warehouses"]),
                                                     cache_path=args.tune_cache, retune=args.retune)
                res["launch"] = dict(cfg, source=how)
            eng.load_tpcc(SEED, w["warehouses"])
            eng.sync()
            nxt = run_steps(eng, n_slots, args.warmup, mode)
            with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
                secs, commits, launches, nxt = timed(eng, torch, n_slots, args.steps, mode, nxt, dist)
            kt = kernel_split(eng, n_slots, mode, nxt) if mode != "plain" else None
            res[mode] = dict(secs=secs, commits=commits, launches=launches, clocks=clk.summary(), kt=kt)
        if want_extras:
            res["modes"] = modes_run(eng, torch, n_slots, min(args.steps, 64),
                                     lambda: eng.load_tpcc(SEED, w["warehouses"]))
        ref = {}
        for mode in ["plain", args.mode]:
            eng.load_tpcc(SEED, w["warehouses"])
            outs = []
            for i in range(2):
                eng.upload(0, batches[i])
                eng.run_batch(0, mode)
                eng.sync()
                outs.append(eng.commit_bitmap(0, w["n_txn"]))
            ref[mode] = (outs, [int(np.bitwise_xor.reduce(eng.download_table(t))) for t in range(9)])
        a, b = ref["plain"], ref[args.mode]
        exact = all(np.array_equal(x, y) for x, y in zip(a[0], b[0])) and a[1] == b[1]
        eng.load_tpcc(SEED, w["warehouses"])
        # order lines in the 4-byte packed form, unpacked on the device
        pinned = [L.pinned_copy(b.with_packed_lines()) for b in batches[:4]]
        e2e = e2e_run(eng, pinned, args.mode, args.e2e_steps, n_slots, w["n_txn"], dist)
    finally:
        eng.close()
    return res, exact, e2e, batches


def cpu_baseline_tpcc(w, batches, n_batches):
    import oracle
    o = oracle.TpccOracle(SEED, w["warehouses"])
    commits, secs = 0, 0.0
    for b in batches[:n_batches]:
        t0 = time.perf_counter()
        _, _, _, c = o.run(b)
        secs += time.perf_counter() - t0
        commits += c
    return commits / secs, secs, commits


# ---- the reference's compiled batch shapes -------------------------------------------
# LTPG/YCSB/1 is compiled for 10,000 transactions x (9 reads + 1 write) over
# 1,000,000 records; LTPG/TPCC-allopt-final for 65,536 Payments over 64
# warehouses.  Both arms build the same batches here: the reference arm times
# the reference's own kernels on them, our arm times the engine.
REF_Y1 = dict(n_records=1_000_000, n_txn=10_000, theta=0.99)
REF_TF = dict(warehouses=64, n_txn=65_536)


def ref_shape_batches():
    from ltpg_gb300 import TpccGenerator, YcsbBatch, YcsbGenerator, abi
    B, n = REF_Y1["n_txn"], REF_Y1["n_records"]
    g = YcsbGenerator(SEED, n - 1, B, 10, 0, REF_Y1["theta"])
    b = g.batch(0)
    # keys 1 .. n-1: the reference routes key 0 around registration in its Zipf mode
    keys = (b.ops.reshape(B, b.op_stride)[:, :10] & ((1 << abi.YCSB_KEY_BITS) - 1)).astype(np.uint32) + 1
    ops = np.full((B, 12), abi.YCSB_OP_PAD, dtype=np.uint32)
    ops[:, :9] = keys[:, :9]
    ops[:, 9] = np.uint32(0x80000000) | keys[:, 9]
    yb = YcsbBatch(ops.ravel(), np.arange(B + 1, dtype=np.uint32), np.arange(B, dtype=np.uint64) + 7, B, 10)
    tb = TpccGenerator(SEED, REF_TF["warehouses"], REF_TF["n_txn"], neworder_pct=0).next()
    mb = mixed_tpcc_batch(TpccGenerator(SEED, REF_TF["warehouses"], 70000, neworder_pct=50), REF_TF["n_txn"] // 2,
                          REF_TF["n_txn"] // 2)
    return keys, yb, tb, mb


def mixed_tpcc_batch(g, nc, pc):
    """The first nc NewOrders and pc Payments of the generator's next batch, in
    their order (TID = position), order lines repacked: the reference's TF
    build with NEWORDER_PERCENT = 50 takes exactly that many of each."""
    from ltpg_gb300 import TpccBatch, abi
    b = g.next()
    kind = b.txns["kind_info"] & 0xFF
    no, pay = kind == abi.TPCC_NEWORDER, kind == abi.TPCC_PAYMENT
    sel = (no & (np.cumsum(no) <= nc)) | (pay & (np.cumsum(pay) <= pc))
    x = b.txns[sel].copy()
    cnt = np.where((x["kind_info"] & 0xFF) == abi.TPCC_NEWORDER, (x["kind_info"] >> 8) & 0xFF, 0).astype(np.int64)
    new_off = np.cumsum(cnt) - cnt
    src = np.repeat(x["line_off"].astype(np.int64), cnt) + (np.arange(int(cnt.sum())) - np.repeat(new_off, cnt))
    x["line_off"] = new_off.astype(np.uint32)
    return TpccBatch(x, b.lines[src])


# The same sources compiled at the headline scale (oracle/ref_build.py y1_c2,
# tf_c3): 1,048,576 YCSB transactions x (15 reads + 1 write) over 10,000,000
# records at theta 0.99 (uniform mode: every key registers), and 1,048,576
# TPC-C transactions, 524,288 NewOrders + 524,288 Payments, W = 64.
REF_Y1_C2 = dict(n_records=10_000_000, n_txn=1 << 20, ops=16, theta=0.99)
REF_TF_C3 = dict(warehouses=64, n_txn=1 << 20)


def ref_scale_batches():
    from ltpg_gb300 import TpccGenerator, YcsbBatch, YcsbGenerator, abi
    B, n, k = REF_Y1_C2["n_txn"], REF_Y1_C2["n_records"], REF_Y1_C2["ops"]
    g = YcsbGenerator(SEED, n, B, k, 0, REF_Y1_C2["theta"], 8)
    keys = (g.batch(0).ops.reshape(B, k) & ((1 << abi.YCSB_KEY_BITS) - 1)).astype(np.uint32)
    ops = keys.copy()
    ops[:, k - 1] |= np.uint32(0x80000000)  # reads first, then the one write
    yb = YcsbBatch(ops.ravel(), np.arange(B + 1, dtype=np.uint32), np.arange(B, dtype=np.uint64) + 7, B, k)
    half = REF_TF_C3["n_txn"] // 2
    mb = mixed_tpcc_batch(TpccGenerator(SEED, REF_TF_C3["warehouses"], 1_100_000, neworder_pct=50), half, half)
    return keys, yb, mb


def reference_gpu(iters, scale_iters=10):
    """The reference's own three kernels (LTPG/YCSB/1, LTPG/TPCC-allopt-final,
    compiled for sm_103a) on its compiled shapes and at the headline scale,
    CUDA events around each kernel, its per-batch clears outside the timed
    span."""
    from oracle import reference
    if not reference.available():
        return {"unavailable": "reference cubins not built (oracle/_ref is made where the reference sources are)"}
    keys, _, tb, mb = ref_shape_batches()
    out = {}
    r = reference.RefY1()
    flags, mark, ms = r.run(keys[:, :9], keys[:, 9], iters=iters)
    commits = int((flags[:r.covered] & 8 != 0).sum())
    out["ycsb_10k_x10"] = {"batch_txn": r.B, "covered_txn": r.covered, "ms_per_batch": sum(ms),
                           "kernel_ms": ms, "commits": commits, "committed_per_s": commits / (sum(ms) * 1e-3),
                           "theta": REF_Y1["theta"], "iters": iters}
    t = reference.RefTF()
    flags, ms = t.run(tb.txns, iters=iters)
    commits = int((flags & 8 != 0).sum())
    out["payment_65536"] = {"batch_txn": t.B, "ms_per_batch": sum(ms), "kernel_ms": ms, "commits": commits,
                            "committed_per_s": commits / (sum(ms) * 1e-3), "iters": iters}
    if reference.available("tf50"):  # the same sources with NEWORDER_PERCENT = 50
        t = reference.RefTF("tf50")
        flags, ms = t.run(mb.txns, mb.lines, iters=iters)
        commits = int((flags & 8 != 0).sum())
        out["neworder_payment_65536"] = {"batch_txn": t.B, "ms_per_batch": sum(ms), "kernel_ms": ms,
                                         "commits": commits, "committed_per_s": commits / (sum(ms) * 1e-3),
                                         "iters": iters}
    if scale_iters and reference.available("y1_c2") and reference.available("tf_c3"):
        keys, _, mb = ref_scale_batches()
        r = reference.RefY1("y1_c2")
        flags, mark, ms = r.run(keys[:, :-1], keys[:, -1], iters=scale_iters)
        commits = int((flags[:r.covered] & 8 != 0).sum())
        out["ycsb_1m_x16"] = {"batch_txn": r.B, "covered_txn": r.covered, "ms_per_batch": sum(ms),
                              "kernel_ms": ms, "commits": commits, "committed_per_s": commits / (sum(ms) * 1e-3),
                              "theta": REF_Y1_C2["theta"], "iters": scale_iters}
        t = reference.RefTF("tf_c3")
        flags, ms = t.run(mb.txns, mb.lines, iters=scale_iters)
        commits = int((flags & 8 != 0).sum())
        out["neworder_payment_1m"] = {"batch_txn": t.B, "ms_per_batch": sum(ms), "kernel_ms": ms,
                                      "commits": commits, "committed_per_s": commits / (sum(ms) * 1e-3),
                                      "iters": scale_iters}
    return out


def engine_on_ref_shapes(iters, scale_iters=10):
    """The engine on the batches reference_gpu() times, in each launch mode
    (plain, fused, persistent, graph), the same batch in every slot, CUDA
    events around `iters` batches (at the headline scale: max(8, scale_iters)
    batches, with the tuned launch shape of the high-contention YCSB
    workload; the reference's 10,000-transaction YCSB batch with its own
    tuned shape); `best_mode` names the fastest."""
    import torch

    import ltpg_gb300 as L
    from ltpg_gb300 import tune
    _, yb, tb, mb = ref_shape_batches()
    small = tune.load_cached("ycsb_ref_10k|theta=0.99")

    def load_small(e):
        e.load_ycsb(SEED, REF_Y1["n_records"])
        if small:
            e.set_launch("ycsb", **{k: v for k, v in small.items() if k in dict(L.abi.LaunchC._fields_)})

    shapes = [("ycsb_10k_x10", load_small, yb, dict(max_ops_per_txn=10), iters),
              ("payment_65536", lambda e: e.load_tpcc(SEED, REF_TF["warehouses"]), tb,
               dict(max_ops_per_txn=16, max_lines=16), iters),
              ("neworder_payment_65536", lambda e: e.load_tpcc(SEED, REF_TF["warehouses"]), mb,
               dict(max_ops_per_txn=16, max_lines=max(16, mb.n_lines)), iters)]
    if scale_iters:
        _, yb2, mb2 = ref_scale_batches()
        hc = tune.load_cached("ycsb_hc|theta=0.99")

        def load_y(e):
            e.load_ycsb(SEED, REF_Y1_C2["n_records"])
            if hc:
                e.set_launch("ycsb", **{k: v for k, v in hc.items() if k in dict(L.abi.LaunchC._fields_)})

        big = max(8, scale_iters)
        shapes += [("ycsb_1m_x16", load_y, yb2, dict(max_ops_per_txn=16), big),
                   ("neworder_payment_1m", lambda e: e.load_tpcc(SEED, REF_TF_C3["warehouses"]), mb2,
                    dict(max_ops_per_txn=16, max_lines=mb2.n_lines), big)]
    out = {}
    for name, load, b, kw, n_it in shapes:
        n_slots = 8 if b.n_txn <= 65536 else 2
        e = L.Engine(device=0, n_slots=n_slots, max_txn=b.n_txn, **kw)
        try:
            load(e)
            for s in range(n_slots):
                e.upload(s, b)
            res = {}
            for mode in ["plain", "fused", "persistent", "graph"]:
                nxt = run_steps(e, n_slots, 16 if n_slots == 8 else 2, mode)
                secs, commits, launches, _ = timed(e, torch, n_slots, n_it, mode, nxt, None)
                res[mode] = {"ms_per_batch": secs * 1e3 / n_it, "committed_per_s": commits / secs,
                             "launches_per_batch": launches / n_it}
            res["best_mode"] = min(("plain", "fused", "persistent", "graph"), key=lambda m: res[m]["ms_per_batch"])
            res["commits"] = commits // n_it
            res["batch_txn"] = b.n_txn
            out[name] = res
        finally:
            e.close()
    return out


# ---- reference arm: the protocol's CPU replay on all host threads ------------------
def reference_arm(args, w, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t_start = time.perf_counter()
    theta = None
    if w["kind"] == "ycsb":
        import oracle
        from ltpg_gb300 import YcsbGenerator
        theta = args.theta if args.theta is not None else w["theta"]
        g = YcsbGenerator(SEED, w["n_records"], w["n_txn"], w["ops"], w["update_pct"], theta, w["rotate_every"],
                          w.get("scan_len", 0))
        nb = min(w["n_batches"], 8)
        batches = [g.batch(i) for i in range(nb)]
        o = oracle.YcsbOracle(SEED, w["n_records"])
        # each step: one whole batch replayed with all host threads
        for i in range(args.warmup):
            o.run(batches[i % nb], threads=threads)
        commits, t0 = 0, time.perf_counter()
        for i in range(args.steps):
            commits += o.run(batches[(args.warmup + i) % nb], threads=threads)[3]
        secs = time.perf_counter() - t0
        sample = f"{args.steps} whole batches of {w['n_txn']} txn, {nb} distinct, multi-threaded replay"
        kind = "port"
    else:
        import oracle
        from ltpg_gb300 import TpccGenerator
        g = TpccGenerator(SEED, w["warehouses"], w["n_txn"], **w.get("mix", {}))
        nb = 4
        batches = [g.next() for _ in range(nb)]
        o = oracle.TpccOracle(SEED, w["warehouses"])
        # each step: one whole batch replayed with all host threads, the
        # generator's batches in a cycle over the advancing image
        for i in range(args.warmup):
            o.run(batches[i % nb], threads=threads)
        commits, t0 = 0, time.perf_counter()
        for i in range(args.steps):
            commits += o.run(batches[(args.warmup + i) % nb], threads=threads)[3]
        secs = time.perf_counter() - t0
        sample = f"{args.steps} whole batches of {w['n_txn']} txn, {nb} distinct, multi-threaded replay"
        kind = "port"
    v = commits / secs
    line = {"impl": "reference", "metric": "committed txns/s", "value": v, "unit": "txn/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": secs * 1e3 / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": bench_config(w, theta),
            "cpu_baseline": {"value": v, "unit": "txn/s", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "txn/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_start}
    if not args.no_reference_gpu:
        try:
            line["reference_gpu"] = reference_gpu(200, args.ref_scale_iters)
        except Exception as exc:  # the CPU arm's line stands on its own
            line["reference_gpu"] = {"unavailable": f"{type(exc).__name__}: {exc}"[:200]}
    print(json.dumps(line), flush=True)


def bench_config(w, theta):
    """The workload as both arms name it: the same dict in both JSON lines."""
    cfg = {"workload": w["name"], "batch_txn": w["n_txn"],
           "l2": "inputs larger than L2 (table, registration slots and batch exceed 129 MB)"}
    if w["kind"] == "ycsb":
        cfg["theta"] = theta
    return cfg


def tpcc_registrations_per_txn(batches):
    """Registration atomics per transaction that the tuned TPC-C execute
    kernel issues before its slot filter: NewOrder 3 header ops + 2 per order
    line (stock write, ORDER-LINE insert), Payment 3 (customer read and write,
    HISTORY insert); reads of WAREHOUSE / DISTRICT / ITEM do not register."""
    from ltpg_gb300 import abi
    total, n = 0, 0
    for b in batches:
        kind = b.txns["kind_info"] & 0xFF
        cnt = (b.txns["kind_info"] >> 8) & 0xFF
        no = kind == abi.TPCC_NEWORDER
        total += int((3 + 2 * cnt[no].astype(np.int64)).sum()) + 3 * int((kind == abi.TPCC_PAYMENT).sum())
        n += len(kind)
    return total / n


def workload_record(args, w, theta, dist, res, exact, e2e, batches, peaks, peak_kind):
    """One workload's figures (after the reductions over ranks): tuned value,
    plain path, bit-exactness, roofline of the dominant kernel, end to end."""
    tuned, plain = res[args.mode], res["plain"]
    launch = res.get("launch")
    ceilings = res.get("ceilings")
    secs = reduce_max(dist, tuned["secs"])
    value = reduce_sum(dist, tuned["commits"]) / secs
    p_secs = reduce_max(dist, plain["secs"])
    p_value = reduce_sum(dist, plain["commits"]) / p_secs
    e2e_value = reduce_sum(dist, e2e["commits"]) / reduce_max(dist, e2e["secs"])
    B = w["n_txn"]
    commit_rate = tuned["commits"] / (args.steps * B)
    kt = tuned["kt"]
    exec_ms, cwb_ms, read_ms, wb_ms = (float(np.mean(kt[:, i])) for i in range(4))
    late = int((launch or {}).get("late_reads") or 0) if w["kind"] == "ycsb" and ((w["ops"] + 3) & ~3) <= 32 else 0
    if late == 3:
        kernel_ms = {"registration": exec_ms, "check": cwb_ms, "reads": read_ms, "decide_write_back": wb_ms}
    elif late == 2:
        kernel_ms = {"execute": exec_ms, "check": cwb_ms, "reads": read_ms, "write_back": wb_ms}
    elif late == 1:
        kernel_ms = {"execute": exec_ms, "check_reads": cwb_ms, "write_back": wb_ms}
    else:
        kernel_ms = {"execute": exec_ms, "check_writeback": cwb_ms}
    prof_kernel = None
    if w["kind"] == "ycsb":
        eb, cb, rb, wb = ycsb_bytes_per_txn(w["ops"], w["update_pct"] / 100, commit_rate,
                                            max(1, w.get("scan_len", 0)), late)
        ek = ycsb_exec_kernel_name(launch, (w["ops"] + 3) & ~3)
        ck = "ycsb_checkwb_tuned"
        wk = "ycsb_writeback_late"
        if late == 3:  # the registration interval is two kernels; the reads' dominates
            ek, ck, wk = "ycsb_wf_reads_list", "ycsb_wf_check_list", "ycsb_writeback_list"
        cands = [(ek, eb, exec_ms), (ck, cb, cwb_ms)]
        if late:
            cands += [("ycsb_read_late", rb, read_ms), (wk, wb, wb_ms)]
        kernel, kbytes, kms = max(cands, key=lambda c: c[2])
        # the late-read variants of the execute and check kernels have profile
        # summaries of their own (one execute kernel for both; two check kernels)
        prof_kernel = kernel
        if late in (1, 2) and kernel == ek:
            prof_kernel = kernel + "_late"
        elif late in (1, 2) and kernel == ck:
            prof_kernel = kernel + f"_late{late}"
    else:
        # NewOrder avg 10 lines, Payment; per-op byte model in tpcc_bytes_per_txn
        eb, cb = tpcc_bytes_per_txn(w.get("mix"), commit_rate)
        kernel, kbytes, kms = ("tpcc_exec_tuned", eb, exec_ms) if exec_ms >= cwb_ms else \
            ("tpcc_checkwb_tuned", cb, cwb_ms)
    achieved = kbytes * B / (kms / 1e3) / 1e9 if kms > 0 else None
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = profile_traffic(w["key"], prof_kernel or kernel)
    roof = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
            "algorithmic_bytes_per_txn": kbytes,
            "traffic": traffic * B if traffic else None,
            "traffic_note": "ncu dram bytes per transaction of a 262,144-transaction capture "
                            "scaled to the batch" if traffic else None,
            "kernel_ms": kernel_ms,
            "pattern_ceilings": ceilings,
            # the dominant kernel against the measured ceiling of its own
            # access pattern (random 80-byte rows read by 5-lane groups),
            # where that is the binding pattern
            "pattern": ({"ceiling": "row_gather_5lane_GBs", "GBs": ceilings["row_gather_5lane_GBs"],
                         "frac": achieved / ceilings["row_gather_5lane_GBs"]}
                        if ceilings and achieved and kernel in ("ycsb_read_late", "ycsb_exec_coop") else None)}
    if w["kind"] == "tpcc" and not w.get("mix") and kernel == "tpcc_exec_tuned" and kms > 0:
        # the execute kernel is issue- and atomic-bound: its registration
        # reductions against the measured random red.min rate of this GPU
        regs = tpcc_registrations_per_txn(batches)
        rate = regs * B / (kms / 1e3) / 1e9
        ceil = (ceilings or {}).get("red_min_random_G_per_s")
        roof["atomics"] = {"registrations_per_txn": regs, "G_per_s": rate, "ceiling": "red_min_random_G_per_s",
                           "ceiling_G_per_s": ceil, "frac": rate / ceil if ceil else None}
    return {
        "value": value, "ms_per_step": secs * 1e3 / args.steps,
        "plain": {"value": p_value, "ms_per_step": p_secs * 1e3 / args.steps,
                  "speedup_tuned_over_plain": value / p_value if p_value else None},
        "bit_exact_tuned_vs_plain": bool(exact),
        "commit_rate": commit_rate,
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "txn/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"], "steps": e2e["steps"], "in_flight": e2e["depth"],
                "api": "ltpg_submit_*_host / ltpg_host_wait (pinned host buffers)",
                "inputs": ("op words, value offsets and values" if w["kind"] == "ycsb"
                           else "transaction records and order lines packed in 4 bytes"),
                # the copy of a step's batch at the measured host-to-device rate:
                # the end-to-end rate cannot pass commits per step / this time
                "h2d_link_GBs": e2e["link_GBs"],
                "link_bound_value": (e2e["commits"] / e2e["steps"]) / (e2e["h2d"] / (e2e["link_GBs"] * 1e9))},
        "gpu_launches": int(tuned["launches"]),
        "launch": launch,
        "clocks": tuned["clocks"],
        "modes": res.get("modes"),
    }


def main():
    args = parse()
    ws, rank, local, dist = dist_setup()
    w = dict(WORKLOADS[args.workload], key=args.workload)
    if args.impl == "reference":
        reference_arm(args, w, rank)
        return
    import __graft_entry__
    __graft_entry__.build()
    import torch
    torch.cuda.set_device(local)
    peaks, peak_kind = measured_peaks()
    if w["kind"] == "ycsb":
        theta = args.theta if args.theta is not None else w["theta"]
        res, exact, e2e, batches = ycsb_bench(args, w, theta, dist)
    else:
        theta = None
        res, exact, e2e, batches = tpcc_bench(args, w, dist)
    rec = workload_record(args, w, theta, dist, res, exact, e2e, batches, peaks, peak_kind)
    # the TPC-C headline workload beside the YCSB one, with the YCSB run's
    # access-pattern ceilings for its atomic roofline
    tp = None
    if args.workload == "ycsb_hc" and not args.no_tpcc:
        wt = dict(WORKLOADS["tpcc"], key="tpcc")
        r2, ex2, e2e2, b2 = tpcc_bench(args, wt, dist)
        r2["ceilings"] = res.get("ceilings")
        tp = workload_record(args, wt, None, dist, r2, ex2, e2e2, b2, peaks, peak_kind)
        tp["config"] = bench_config(wt, None)
        if rank == 0 and not args.no_cpu_baseline:
            v, s_, c = cpu_baseline_tpcc(wt, b2, args.cpu_batches_tpcc)
            tp["cpu_baseline"] = {"value": v, "unit": "txn/s", "cores": 1, "kind": "port",
                                  "sample": f"{min(args.cpu_batches_tpcc, len(b2))} whole batches of "
                                            f"{wt['n_txn']} txn in order, single-threaded oracle replay, {s_:.1f} s"}
    sweep = None
    if args.workload == "ycsb_hc" and not args.no_sweep:
        sweep = {}
        ws_ = dict(w, n_batches=min(w["n_batches"], 8))
        for th in [0.0, 0.6, 0.8, 0.99]:
            r, ex, _, _ = ycsb_bench(args, ws_, th, dist, want_extras=False)
            t_v = reduce_sum(dist, r[args.mode]["commits"]) / reduce_max(dist, r[args.mode]["secs"])
            p_v = reduce_sum(dist, r["plain"]["commits"]) / reduce_max(dist, r["plain"]["secs"])
            sweep[str(th)] = {"tuned": t_v, "plain": p_v, "speedup": t_v / p_v if p_v else None,
                              "bit_exact_tuned_vs_plain": bool(ex), "launch": r.get("launch")}
    # small batches (65,536 transactions on a 1 M-record table): the
    # latency-bound shape, more steps so that the timed region is not a few
    # launches long
    small = None
    if args.workload == "ycsb_hc" and not args.no_small:
        wsm = dict(WORKLOADS["ycsb_small"], key="ycsb_small")
        a2 = argparse.Namespace(**vars(args))
        a2.steps, a2.warmup = max(args.steps, 320), max(args.warmup, 32)
        r, ex, _, _ = ycsb_bench(a2, wsm, wsm["theta"], dist, want_extras=False)
        t_s, p_s = reduce_max(dist, r[args.mode]["secs"]), reduce_max(dist, r["plain"]["secs"])
        t_v = reduce_sum(dist, r[args.mode]["commits"]) / t_s
        p_v = reduce_sum(dist, r["plain"]["commits"]) / p_s
        small = {"workload": wsm["name"], "tuned": t_v, "plain": p_v, "speedup": t_v / p_v if p_v else None,
                 "ms_per_batch_tuned": t_s * 1e3 / a2.steps, "ms_per_batch_plain": p_s * 1e3 / a2.steps,
                 "steps": a2.steps, "warmup": a2.warmup, "bit_exact_tuned_vs_plain": bool(ex),
                 "launch": r.get("launch")}
    if rank != 0:
        return
    B = w["n_txn"]
    line = {
        "metric": "committed txns/s", "value": rec["value"], "unit": "txn/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": bench_config(w, theta),
        "mode": args.mode, "parallelism": "replicas" if ws > 1 else "single GPU",
        "plain": rec["plain"],
        "bit_exact_tuned_vs_plain": rec["bit_exact_tuned_vs_plain"],
        "commit_rate": rec["commit_rate"],
        "roofline": rec["roofline"],
        "e2e": rec["e2e"],
        "gpu_launches": rec["gpu_launches"],
        "launch": rec["launch"],
        "clocks": rec["clocks"],
    }
    if rec.get("modes"):
        line["modes"] = rec["modes"]
    if not args.no_cpu_baseline:
        if w["kind"] == "ycsb":
            v, s, c = cpu_baseline_ycsb(w, batches, args.cpu_batches)
        else:
            v, s, c = cpu_baseline_tpcc(w, batches, args.cpu_batches)
        line["cpu_baseline"] = {"value": v, "unit": "txn/s", "cores": 1, "kind": "port",
                                "sample": f"{min(args.cpu_batches, len(batches))} whole batches of {B} txn in order, "
                                          f"single-threaded oracle replay, {s:.1f} s"}
    if tp is not None:
        line["tpcc"] = tp
    if sweep is not None:
        line["theta_sweep"] = sweep
    if small is not None:
        line["small_batches"] = small
    if not args.no_predictor and w["kind"] == "ycsb" and w["n_txn"] >= (1 << 18):
        line["predictor"] = predictor_section(w, batches)
    if not args.no_reference_gpu and args.workload == "ycsb_hc":
        line["reference_shapes"] = engine_on_ref_shapes(200, args.ref_scale_iters)
    if not args.no_serving and args.workload == "ycsb_hc":
        line["serving"] = serving_section(args)
    if not args.no_device_gen and args.workload in ("ycsb_hc", "tpcc", "tpcc_mix"):
        line["device_generator"] = device_gen_section(w)
    print(json.dumps(line), flush=True)


def device_gen_section(w, reps=8):
    """Batches of this workload generated on the GPU (ltpg_gen_*_batch_device,
    byte-identical to the host generator): ms per batch on the device (CUDA
    events) and on the host (one call, all host threads for YCSB, one for the
    sequential TPC-C loop), and committed txn/s of steps that generate their
    batch on the device and run it (graph mode)."""
    import torch
    import ltpg_gb300 as L
    B = w["n_txn"]
    if w["kind"] == "ycsb":
        e = L.Engine(device=0, n_slots=2, max_txn=B, max_ops_per_txn=w["ops"])
        e.load_ycsb(SEED, w["n_records"])
        g = L.YcsbGenerator(SEED, w["n_records"], B, w["ops"], w["update_pct"], w["theta"], w["rotate_every"],
                            w.get("scan_len", 0))
        gen = lambda slot, i: e.generate(slot, g, 100 + i)  # noqa: E731
        t0 = time.time()
        g.batch(99)
        host_ms = (time.time() - t0) * 1e3
    else:
        e = L.Engine(device=0, n_slots=2, max_txn=B, max_ops_per_txn=16, max_lines=15 * B)
        e.load_tpcc(SEED, w["warehouses"])
        gh = L.TpccGenerator(SEED + 1, w["warehouses"], B, **w.get("mix", {}))
        t0 = time.time()
        gh.next()
        host_ms = (time.time() - t0) * 1e3
        g = L.TpccGenerator(SEED + 1, w["warehouses"], B, **w.get("mix", {}))
        gen = lambda slot, i: e.generate(slot, g)  # noqa: E731
    try:
        stream = torch.cuda.ExternalStream(e.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        for i in range(3):
            gen(i % 2, i)
            e.run_batch(i % 2, "graph")
        e.sync()
        ev[0].record(stream)
        for i in range(reps):
            gen(i % 2, 3 + i)
        ev[1].record(stream)
        c0 = e.counters()[0]
        ev[2].record(stream)
        for i in range(reps):
            gen(i % 2, 3 + reps + i)
            e.run_batch(i % 2, "graph")
        ev[3].record(stream)
        e.sync()
        commits = e.counters()[0] - c0
        gen_ms = ev[0].elapsed_time(ev[1]) / reps
        step_ms = ev[2].elapsed_time(ev[3]) / reps
        # pipelined: batch i+1 generated on the copy stream while batch i runs,
        # bitmaps to pinned host memory; host wall time
        bits = [L.pinned_empty((B + 31) // 32) for _ in range(2)]
        sub = ((lambda i: e.submit_generated(i % 2, g, "graph", bits[i % 2], batch_id=1000 + i))
               if w["kind"] == "ycsb" else (lambda i: e.submit_generated(i % 2, g, "graph", bits[i % 2])))
        for i in range(2):
            sub(i)
        for i in range(2):
            e.host_wait(i)
        c1 = e.counters()[0]
        t0 = time.time()
        for i in range(2, 2 + reps):
            if i >= 4:
                e.host_wait(i % 2)
            sub(i)
        for i in range(reps, reps + 2):
            e.host_wait(i % 2)
        wall = time.time() - t0
        p_commits = e.counters()[0] - c1
    finally:
        e.close()
    return {"device_ms_per_batch": gen_ms, "host_ms_per_batch": host_ms,
            "host_threads": os.cpu_count() if w["kind"] == "ycsb" else 1,
            "generate_and_run": {"value": commits / (step_ms * reps / 1e3), "unit": "txn/s",
                                 "ms_per_step": step_ms},
            "generate_and_run_pipelined": {"value": p_commits / wall, "unit": "txn/s",
                                           "ms_per_step": wall * 1e3 / reps,
                                           "api": "ltpg_submit_generated / ltpg_host_wait, 2 in flight"}}


def serving_section(args):
    """Serving loop: Poisson arrivals at 1M / 5M / 20M txn/s, 70 % TPC-C
    (W = 64) and 30 % YCSB (1M records, 10 ops, 50/50, theta 0.9), batches
    closing at 262,144 requests or 2 ms, 40 GB device budget; plain (three
    kernels per part) vs tuned (fused kernels with the autotuned launch shapes
    of the TPC-C W=64 and small-YCSB workloads).  The tuned arm is not run as
    CUDA graphs: a graph is captured for one batch size, and served batches
    differ in size."""
    import ltpg_gb300 as L
    from ltpg_gb300 import tune

    def shape(key):
        cfg = tune.load_cached(key, args.tune_cache) or {}
        return {k: v for k, v in cfg.items() if k in dict(L.abi.LaunchC._fields_)}
    tp = dict(seed=SEED, warehouses=64, n_txn=262144)
    yp = dict(seed=SEED + 1, n_records=1_000_000, n_txn=262144, ops_per_txn=10, update_pct=50, theta=0.9)
    c = L.Engine(device=0, n_slots=4, max_txn=262144, max_ops_per_txn=16, max_lines=15 * 262144)
    y = L.Engine(device=0, n_slots=4, max_txn=262144, max_ops_per_txn=10)
    out = {}
    try:
        for rate in [1e6, 5e6, 2e7]:
            for mode in ["plain", "fused"]:
                c.load_tpcc(tp["seed"], tp["warehouses"])
                y.load_ycsb(yp["seed"], yp["n_records"])
                if mode == "fused":
                    c.set_launch("tpcc", **shape("tpcc"))
                    y.set_launch("ycsb", **shape("ycsb_small|theta=0.6"))
                st = L.serve(c, y, rate=rate, duration_s=args.serve_seconds, tpcc_params=tp, ycsb_params=yp,
                             deadline_ms=2.0, max_batch=262144, tpcc_pct=70, mode=mode, budget_bytes=40 << 30,
                             slots=4)
                out[f"{rate / 1e6:g}M/s {'tuned' if mode != 'plain' else 'plain'}"] = {
                    "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "p999_ms": st["p999_ms"],
                    "close_wait_ms": st["wait_ms"], "launch_ms_per_batch": st["launch_ms"],
                    "device_ms_per_batch": st["device_ms"],
                    "committed_per_s": st["throughput"], "submitted": st["submitted"],
                    "commit_rate": st["committed"] / max(1, st["submitted"]), "batches": st["batches"],
                    "mean_batch": st["mean_batch"], "slot_waits": st["waited_for_slot"]}
    finally:
        c.close()
        y.close()
    return out


def predictor_section(w, batches):
    """Predictor-guided staging on the benchmark stream: staging hit rate,
    execute-kernel time and whole batches (the predictor's own step included:
    device time per batch and committed txn/s), trained vs untrained vs no
    staging, with the slot filter off (the warp-aggregated path the predictor
    complements) and on.  Every variant's commit bitmaps and final table are
    compared with the no-staging run of the same filter setting."""
    import torch
    import ltpg_gb300 as L
    out = {}
    n_slots = 8
    for filt in [0, 1]:
        ref = None
        for name, kw in [("no_staging", None), ("trained", dict(train=True, stage=True)),
                         ("untrained", dict(train=False, stage=True))]:
            e = L.Engine(device=0, n_slots=n_slots, max_txn=w["n_txn"], max_ops_per_txn=w["ops"])
            try:
                e.load_ycsb(SEED, w["n_records"])
                e.set_launch("ycsb", ops_per_thread=1, filter=filt, dedupe=1, stage_ways=1, blocks_per_sm=0)
                if kw:
                    e.predictor(enable=True, seed=7, **kw)
                e.set_profiling(True)
                stream = torch.cuda.ExternalStream(e.stream())
                hits, ms, batch_ms, commits, bits = [], [], [], 0, []
                for i, b in enumerate(batches[:24]):
                    e.upload(i % n_slots, b)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    e.run_batch(i % n_slots, "fused")
                    e1.record(stream)
                    e.sync()
                    torch.cuda.synchronize()
                    bits.append(e.commit_bitmap(i % n_slots, b.n_txn))
                    if i >= 8:
                        st = e.stats(i % n_slots)
                        hits.append(st["staged_ops"] / (b.n_txn * w["ops"]))
                        ms.append(e.kernel_times(i % n_slots)[0])
                        batch_ms.append(e0.elapsed_time(e1))
                        commits += int(st["commits"])
                img = e.download_table(L.TABLE_YCSB)
                got = (bits, int(np.bitwise_xor.reduce(img)), int(img.sum()))
                if ref is None:
                    ref = got
                rec = {"staging_hit_rate": float(np.mean(hits)), "execute_ms": float(np.mean(ms)),
                       "batch_ms": float(np.mean(batch_ms)),
                       "committed_per_s": commits / (float(np.sum(batch_ms)) * 1e-3),
                       "bit_exact_vs_no_staging": bool(all(np.array_equal(x, y) for x, y in zip(got[0], ref[0]))
                                                       and got[1:] == ref[1:])}
                if kw and kw["train"]:
                    rec["loss"] = e.predictor_stats()["loss"]
                out[f"filter{filt}_{name}"] = rec
            finally:
                e.close()
    return out


def tpcc_bytes_per_txn(mix=None, commit_rate=1.0):
    """Algorithmic bytes per TPC-C transaction (10 lines per NewOrder on
    average), weighted by the workload's mix (default 50/50 NewOrder/Payment).
    Only ops that can conflict register and check: no transaction writes a
    WAREHOUSE, DISTRICT or ITEM row through registration, so NewOrder has 3 + 2
    per line (customer read, NEW-ORDER and ORDER inserts, stock write,
    ORDER-LINE insert), Payment 3 (customer read and write, HISTORY insert),
    OrderStatus 3 reads, Delivery 4 (two of them read and write their row),
    StockLevel 1.  Execute: 32 B record + 8 B per line, 16 B registration per
    op (Delivery's read-and-write rows: 32), reads W/D tax, C discount, item
    price, balance, OL_AMOUNT, S_QUANTITY (8 B each).  Check+write-back: record
    and lines again, 16 B slot load per op, flag and bitmap bytes, and the
    writes of committed transactions, weighted by the measured commit rate
    (NewOrder: ORDER 64, NEW-ORDER 24, per line stock 4x8 read+write, ORDER-LINE
    80 + price and dist reads 16; Payment: 2 hot adds 16, customer 3x8
    read+write, HISTORY 64; Delivery: NEW-ORDER 24, carrier 8, delivery date 8,
    customer 2x8 read+write)."""
    mix = mix or {}
    no = mix.get("neworder_pct", 50)
    os_, dl, sl = mix.get("orderstatus_pct", 0), mix.get("delivery_pct", 0), mix.get("stocklevel_pct", 0)
    pay = 100 - no - os_ - dl - sl
    ex = {"no": 32 + 80 + 16 * 23 + 24 + 8 * 10 + 8, "pay": 32 + 16 * 3 + 8 + 8, "os": 32 + 16 * 3 + 8,
          "dl": 32 + 16 * 6 + 8, "sl": 32 + 16 + 8}
    ck = {"no": 32 + 80 + 16 * 23 + 2, "pay": 32 + 16 * 3 + 2, "os": 32 + 16 * 3 + 2, "dl": 32 + 16 * 4 + 2,
          "sl": 32 + 16 + 2}
    wr = {"no": 64 + 24 + 10 * (64 + 80 + 16), "pay": 16 + 48 + 64, "os": 0, "dl": 24 + 8 + 8 + 32, "sl": 0}
    share = {"no": no, "pay": pay, "os": os_, "dl": dl, "sl": sl}
    return (sum(ex[k] * share[k] for k in ex) / 100.0,
            sum((ck[k] + commit_rate * wr[k]) * share[k] for k in ck) / 100.0)


if __name__ == "__main__":
    main()
