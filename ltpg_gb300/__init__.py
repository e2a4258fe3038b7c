"""ltpg_gb300 — GB300 engine for LTPG's deterministic batch concurrency control.

Python host mirror of the engine's C ABI (include/ltpg.h), in the roles of the
reference's host classes:
  Engine            Database + Query device buffers and the three kernels
                    (TF/Database.h:13-348, TF/Query.h:297-639, TF/tp.cu:11-117)
  YcsbGenerator     MakeYCSB / YCSBQuery::initial_ycsb_a_query (Y1/Query.h:18-188)
  TpccGenerator     MakeNeworder / MakePayment / Query::initial_* (TF/Query.h:16-212,478-525)
All device work runs in libltpg.so; there is no CPU fallback: importing this
package on a machine without the built library raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (FLAG_COMMIT, FLAG_RAW, FLAG_WAR, FLAG_WAW, MODES, MODE_FUSED, MODE_GRAPH,  # noqa: F401
                  MODE_PERSISTENT, MODE_PLAIN, TABLE_YCSB, TPCC_COLS)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libltpg.so")
_lib = None


class LtpgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ltpg error {code}: {msg}")
        self.code = code


def lib():
    """The loaded engine library (build it with ltpg_gb300.build.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m ltpg_gb300.build` first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in abi.SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


BENCH_LIB_PATH = os.path.join(HERE, "libltpg_bench.so")
_bench_lib = None


def bench_lib():
    """The measurement-only library (access-pattern ceilings), built beside libltpg.so."""
    global _bench_lib
    if _bench_lib is None:
        if not os.path.exists(BENCH_LIB_PATH):
            raise ImportError(f"{BENCH_LIB_PATH} is missing: run `python -m ltpg_gb300.build` first")
        L = C.CDLL(BENCH_LIB_PATH)
        for name, (res, args) in abi.BENCH_SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bench_lib = L
    return _bench_lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def key_bucket(keys):
    """Key-hash bucket of each key (the staging / predictor granularity)."""
    k = np.asarray(keys, dtype=np.uint64)
    return (((k * np.uint64(0x9E3779B1)) & np.uint64(0xFFFFFFFF)) >> np.uint64(16)).astype(np.uint32)


class YcsbBatch:
    """A YCSB batch in the engine's format (see include/ltpg.h)."""

    def __init__(self, ops, val_off, vals, n_txn, ops_per_txn):
        """val_off None: the batch carries no value offsets, the engine makes
        them on the device from the op words (n_updates = len(vals))."""
        self.ops = np.ascontiguousarray(ops, dtype=np.uint32)
        self.val_off = None if val_off is None else np.ascontiguousarray(val_off, dtype=np.uint32)
        self.vals = np.ascontiguousarray(vals, dtype=np.uint64)
        self.n_txn = int(n_txn)
        self.ops_per_txn = int(ops_per_txn)
        self.op_stride = (self.ops_per_txn + 3) & ~3
        self.n_updates = len(self.vals) if self.val_off is None else int(self.val_off[self.n_txn])

    def as_c(self):
        return abi.YcsbBatchC(self.n_txn, self.ops_per_txn, self.op_stride, self.n_updates,
                              self.ops.ctypes.data, None if self.val_off is None else self.val_off.ctypes.data,
                              self.vals.ctypes.data if len(self.vals) else None)

    def without_offsets(self):
        """The same batch without its value offsets (the engine makes them)."""
        return YcsbBatch(self.ops, None, self.vals[:self.n_updates], self.n_txn, self.ops_per_txn)

    def nbytes(self):
        offs = 0 if self.val_off is None else (self.n_txn + 1) * 4
        return self.n_txn * self.op_stride * 4 + offs + self.n_updates * 8

    @staticmethod
    def from_ops(op_lists, values):
        """Builds a batch from per-transaction lists of (key, is_update, field) and
        per-transaction lists of update values (hand-written test batches)."""
        B = len(op_lists)
        k = max(len(o) for o in op_lists)
        stride = (k + 3) & ~3
        ops = np.full(B * stride, abi.YCSB_OP_PAD, dtype=np.uint32)
        val_off = np.zeros(B + 1, dtype=np.uint32)
        vals = []
        for t, lst in enumerate(op_lists):
            nu = 0
            for j, (key, upd, field) in enumerate(lst):
                ops[t * stride + j] = (0x80000000 if upd else 0) | ((field & 0xF) << 27) | key
                nu += bool(upd)
            assert nu == len(values[t])
            vals.extend(values[t])
            val_off[t + 1] = val_off[t] + nu
        return YcsbBatch(ops, val_off, np.array(vals, dtype=np.uint64), B, k)


class TpccBatch:
    TXN_DTYPE = np.dtype([("kind_info", "<u4"), ("w", "<u4"), ("c_w", "<u4"), ("c_id", "<u4"), ("a", "<u4"),
                          ("b", "<u4"), ("c", "<u4"), ("line_off", "<u4")])
    LINE_DTYPE = np.dtype([("i_id", "<u4"), ("supply_w", "<u2"), ("qty", "<u2")])

    def __init__(self, txns, lines, txn_base=0, packed=None):
        """packed (with lines None): the order lines in the 4-byte form of
        ltpg_tpcc_pack_lines, unpacked on the device by the packed calls."""
        self.txns = np.ascontiguousarray(txns, dtype=self.TXN_DTYPE)
        self.packed = None if packed is None else np.ascontiguousarray(packed, dtype=np.uint32)
        self.lines = np.ascontiguousarray(np.empty(0, dtype=self.LINE_DTYPE) if lines is None else lines,
                                          dtype=self.LINE_DTYPE)
        self.n_txn = len(self.txns)
        self.n_lines = len(self.packed) if lines is None and self.packed is not None else len(self.lines)
        self.txn_base = int(txn_base)

    def as_c(self):
        return abi.TpccBatchC(self.n_txn, self.n_lines, self.txn_base, self.txns.ctypes.data,
                              self.lines.ctypes.data if len(self.lines) else None)

    def with_packed_lines(self):
        """The same batch with its order lines packed in 4 bytes (ltpg_tpcc_pack_lines)."""
        p = np.empty(max(self.n_lines, 1), dtype=np.uint32)
        r = lib().ltpg_tpcc_pack_lines(self.lines.ctypes.data if self.n_lines else None, self.n_lines, _p(p))
        if r:
            raise LtpgError(r, "an order line does not fit the packed form")
        return TpccBatch(self.txns, None, self.txn_base, packed=p[:self.n_lines])

    def nbytes(self):
        return self.n_txn * 32 + self.n_lines * (4 if self.packed is not None else 8)


def pinned_copy(batch):
    """Copy of a batch whose arrays live in pinned host memory (ltpg_host_alloc),
    so host<->device copies run at full link speed.  Keep the returned object
    alive while the engine uses it."""
    def pin(a):
        n = max(a.nbytes, 16)
        ptr = lib().ltpg_host_alloc(n)
        if not ptr:
            raise MemoryError("ltpg_host_alloc failed")
        buf = (C.c_char * n).from_address(ptr)
        out = np.frombuffer(buf, dtype=a.dtype, count=a.size)
        out[:] = a
        _PINNED[id(out)] = ptr
        return out

    if isinstance(batch, YcsbBatch):
        return YcsbBatch(pin(batch.ops), None if batch.val_off is None else pin(batch.val_off), pin(batch.vals),
                         batch.n_txn, batch.ops_per_txn)
    if batch.packed is not None:
        return TpccBatch(pin(batch.txns), None, batch.txn_base, packed=pin(batch.packed))
    return TpccBatch(pin(batch.txns), pin(batch.lines), batch.txn_base)


_PINNED = {}


def pinned_empty(n, dtype=np.uint32):
    """Uninitialised array of n elements in pinned host memory (for bitmaps of
    pipelined host calls); keep it alive while the engine writes it."""
    dtype = np.dtype(dtype)
    nbytes = max(int(n) * dtype.itemsize, 16)
    ptr = lib().ltpg_host_alloc(nbytes)
    if not ptr:
        raise MemoryError("ltpg_host_alloc failed")
    out = np.frombuffer((C.c_char * nbytes).from_address(ptr), dtype=dtype, count=int(n))
    _PINNED[id(out)] = ptr
    return out


def _check(code, ctx=None):
    if code != abi.OK:
        msg = lib().ltpg_last_error(ctx).decode() if ctx else "invalid argument"
        raise LtpgError(code, msg)


class YcsbGenerator:
    """Deterministic YCSB batches (Zipf by Gray et al., splitmix64 streams)."""

    def __init__(self, seed, n_records, n_txn, ops_per_txn=10, update_pct=50, theta=0.6, rotate_every=0,
                 scan_len=0):
        """scan_len >= 2: every read is a range scan of scan_len keys."""
        self.params = abi.YcsbParamsC(seed, n_records, n_txn, ops_per_txn, update_pct, rotate_every, theta, scan_len,
                                      0)
        h = C.c_void_p()
        _check(lib().ltpg_gen_create_ycsb(C.byref(self.params), C.byref(h)))
        self._h = h
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib().ltpg_gen_capacity(h, C.byref(a), C.byref(b)))
        self.cap_ops, self.cap_vals = a.value, b.value

    def batch(self, batch_id):
        p = self.params
        ops = np.empty(self.cap_ops, dtype=np.uint32)
        val_off = np.empty(p.n_txn + 1, dtype=np.uint32)
        vals = np.empty(self.cap_vals, dtype=np.uint64)
        out = abi.YcsbBatchC()
        _check(lib().ltpg_gen_ycsb_batch(self._h, batch_id, _p(ops), _p(val_off), _p(vals), C.byref(out)))
        return YcsbBatch(ops, val_off, vals[:out.n_updates].copy(), p.n_txn, p.ops_per_txn)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ltpg_gen_destroy(self._h)
            self._h = None


class TpccGenerator:
    """Deterministic, stateful TPC-C NewOrder/Payment batches (draw in order)."""

    def __init__(self, seed, warehouses, n_txn, neworder_pct=50, remote_line_pct=1, remote_pay_pct=15,
                 by_name_pct=0, table_seed=None, orderstatus_pct=0, delivery_pct=0, stocklevel_pct=0):
        """by_name_pct: share of Payments / OrderStatus that name their customer
        by last name; table_seed: seed the tables were loaded with (default:
        seed); orderstatus / delivery / stocklevel_pct: shares of the other three
        TPC-C transactions, taken from Payment's."""
        self.params = abi.TpccParamsC(seed, warehouses, n_txn, neworder_pct, remote_line_pct, remote_pay_pct,
                                      by_name_pct, seed if table_seed is None else table_seed, orderstatus_pct,
                                      delivery_pct, stocklevel_pct, 0)
        h = C.c_void_p()
        _check(lib().ltpg_gen_create_tpcc(C.byref(self.params), C.byref(h)))
        self._h = h
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib().ltpg_gen_capacity(h, C.byref(a), C.byref(b)))
        self.cap_txn, self.cap_lines = a.value, b.value
        self.next_id = 0

    def next(self):
        txns = np.empty(self.cap_txn, dtype=TpccBatch.TXN_DTYPE)
        lines = np.empty(self.cap_lines, dtype=TpccBatch.LINE_DTYPE)
        out = abi.TpccBatchC()
        _check(lib().ltpg_gen_tpcc_batch(self._h, self.next_id, _p(txns), _p(lines), C.byref(out)))
        self.next_id += 1
        return TpccBatch(txns[:out.n_txn].copy(), lines[:out.n_lines].copy(), out.txn_base)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ltpg_gen_destroy(self._h)
            self._h = None


class Engine:
    """One GPU context: tables, batch slots, phases, results."""

    def __init__(self, device=0, n_slots=2, max_txn=1 << 16, max_ops_per_txn=16, max_lines=0,
                 strict_insert=False, ref_name_lookup=False):
        cfg = abi.ConfigC(device, n_slots, max_txn, max_ops_per_txn, max_lines,
                          (abi.CFG_STRICT_INSERT if strict_insert else 0) |
                          (abi.CFG_REF_NAME_LOOKUP if ref_name_lookup else 0))
        h = C.c_void_p()
        code = lib().ltpg_create(C.byref(cfg), C.byref(h))
        if code != abi.OK:
            raise LtpgError(code, "ltpg_create failed")
        self._h = h
        self.device = device
        self.n_slots = n_slots
        self.max_txn = max_txn

    def _ck(self, code):
        _check(code, self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().ltpg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # stream / sync
    def set_stream(self, stream_ptr):
        self._ck(lib().ltpg_set_stream(self._h, C.c_void_p(stream_ptr)))

    def stream(self):
        return lib().ltpg_get_stream(self._h)

    def sync(self):
        self._ck(lib().ltpg_sync(self._h))

    # tables
    def load_ycsb(self, seed, n_records):
        self._ck(lib().ltpg_db_load_ycsb(self._h, seed, n_records))

    def load_tpcc(self, seed, warehouses):
        self._ck(lib().ltpg_db_load_tpcc(self._h, seed, warehouses))

    def table_shape(self, table):
        r, c = C.c_uint64(), C.c_uint32()
        self._ck(lib().ltpg_db_table_shape(self._h, table, C.byref(r), C.byref(c)))
        return r.value, c.value

    def download_table(self, table):
        rows, cols = self.table_shape(table)
        a = np.empty(rows * cols, dtype=np.uint64)
        self._ck(lib().ltpg_db_download(self._h, table, _p(a), a.nbytes))
        return a

    def upload_table(self, table, a):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        self._ck(lib().ltpg_db_upload(self._h, table, _p(a), a.nbytes))

    # batches
    def upload(self, slot, batch):
        cb = batch.as_c()
        if isinstance(batch, YcsbBatch):
            self._ck(lib().ltpg_batch_upload_ycsb(self._h, slot, C.byref(cb)))
        elif batch.packed is not None:
            self._ck(lib().ltpg_batch_upload_tpcc_packed(self._h, slot, C.byref(cb), _p(batch.packed)))
        else:
            self._ck(lib().ltpg_batch_upload_tpcc(self._h, slot, C.byref(cb)))

    def generate(self, slot, gen, batch_id=None):
        """Makes a generator's batch on the GPU, directly in `slot` (asynchronous
        on the engine's stream): byte-identical to gen.batch(batch_id) /
        gen.next().  A TPC-C generator continues in order from gen.next_id and
        keeps its state on the GPU from then on (its host batches are refused)."""
        if isinstance(gen, YcsbGenerator):
            if batch_id is None:
                raise ValueError("a YCSB batch needs its batch_id")
            self._ck(lib().ltpg_gen_ycsb_batch_device(self._h, gen._h, batch_id, slot))
        else:
            self._ck(lib().ltpg_gen_tpcc_batch_device(self._h, gen._h, gen.next_id, slot))
            gen.next_id += 1

    def submit_generated(self, slot, gen, mode, bitmap, batch_id=None):
        """Pipelined device generation: gen's batch is made on the GPU in `slot`
        on the copy stream (overlapping earlier batches' kernels), run in `mode`,
        and its commit bitmap copied to `bitmap` (pinned, from pinned_empty);
        host_wait(slot) returns when it is there.  TPC-C: the next batch in
        order (batch_id ignored)."""
        m = MODES[mode] if isinstance(mode, str) else mode
        if isinstance(gen, YcsbGenerator):
            if batch_id is None:
                raise ValueError("a YCSB batch needs its batch_id")
            bid = batch_id
        else:
            bid = gen.next_id
        self._ck(lib().ltpg_submit_generated(self._h, gen._h, bid, slot, m, _p(bitmap) if bitmap is not None else None))
        if not isinstance(gen, YcsbGenerator):
            gen.next_id += 1

    def download_batch(self, slot):
        """The batch held by `slot` (uploaded or generated on the GPU)."""
        bi = abi.BatchInfoC()
        self._ck(lib().ltpg_batch_info_get(self._h, slot, C.byref(bi)))

        def part(i, dtype, count):
            a = np.empty(count, dtype=dtype)
            self._ck(lib().ltpg_batch_download(self._h, slot, i, _p(a) if count else None, a.nbytes))
            return a

        if bi.workload == abi.WORKLOAD_YCSB:
            return YcsbBatch(part(0, np.uint32, bi.n_op_words), part(1, np.uint32, bi.n_txn + 1),
                             part(2, np.uint64, bi.n_updates), bi.n_txn, bi.ops_per_txn)
        return TpccBatch(part(0, TpccBatch.TXN_DTYPE, bi.n_txn), part(1, TpccBatch.LINE_DTYPE, bi.n_lines),
                         bi.txn_base)

    def execute_register(self, slot):
        self._ck(lib().ltpg_execute_register(self._h, slot))

    def check_conflict(self, slot):
        self._ck(lib().ltpg_check_conflict(self._h, slot))

    def write_back(self, slot):
        self._ck(lib().ltpg_write_back(self._h, slot))

    def run_batch(self, slot, mode="plain"):
        self._ck(lib().ltpg_run_batch(self._h, slot, MODES[mode] if isinstance(mode, str) else mode))

    def run_batches(self, first, count, mode="graph"):
        self._ck(lib().ltpg_run_batches(self._h, first, count, MODES[mode] if isinstance(mode, str) else mode))

    def run_host(self, slot, batch, mode="plain", bitmap=None):
        """Upload + run + bitmap download, synchronised (host-buffer call)."""
        words = (batch.n_txn + 31) // 32
        out = bitmap if bitmap is not None else np.empty(words, dtype=np.uint32)
        cb = batch.as_c()
        m = MODES[mode] if isinstance(mode, str) else mode
        if isinstance(batch, YcsbBatch):
            self._ck(lib().ltpg_run_ycsb_host(self._h, slot, C.byref(cb), m, _p(out)))
        else:
            self._ck(lib().ltpg_run_tpcc_host(self._h, slot, C.byref(cb), m, _p(out)))
        return out

    def submit_host(self, slot, batch, mode, bitmap):
        """Pipelined host-buffer call (ltpg_submit_*_host): returns once the copy,
        run and bitmap download are enqueued; `bitmap` (pinned_empty) holds the
        result after host_wait(slot).  Keep `batch` and `bitmap` alive and
        unchanged until then."""
        cb = batch.as_c()
        m = MODES[mode] if isinstance(mode, str) else mode
        if isinstance(batch, YcsbBatch):
            self._ck(lib().ltpg_submit_ycsb_host(self._h, slot, C.byref(cb), m, _p(bitmap)))
        elif batch.packed is not None:
            self._ck(lib().ltpg_submit_tpcc_packed_host(self._h, slot, C.byref(cb), _p(batch.packed), m, _p(bitmap)))
        else:
            self._ck(lib().ltpg_submit_tpcc_host(self._h, slot, C.byref(cb), m, _p(bitmap)))

    def host_wait(self, slot):
        self._ck(lib().ltpg_host_wait(self._h, slot))

    # results
    def commit_bitmap(self, slot, n_txn):
        out = np.empty((n_txn + 31) // 32, dtype=np.uint32)
        self._ck(lib().ltpg_commit_bitmap(self._h, slot, _p(out), len(out)))
        return out

    def txn_flags(self, slot, n_txn):
        out = np.empty(n_txn, dtype=np.uint8)
        self._ck(lib().ltpg_txn_flags(self._h, slot, _p(out), n_txn))
        return out

    def txn_results(self, slot, n_txn):
        out = np.empty(n_txn, dtype=np.int64)
        self._ck(lib().ltpg_txn_results(self._h, slot, _p(out), n_txn))
        return out

    def stats(self, slot):
        s = abi.StatsC()
        self._ck(lib().ltpg_batch_stats_get(self._h, slot, C.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.StatsC._fields_}

    def set_launch(self, workload, **kw):
        """Sets fields of the tuned launch shape (block_threads, ops_per_thread,
        blocks_per_sm, stage_ways, filter, dedupe, late_reads) of workload
        'ycsb' or 'tpcc'.  late_reads = 1: YCSB rows are read after the check,
        by committed transactions only (an aborted transaction's result is 0)."""
        wl = abi.WORKLOAD_YCSB if workload == "ycsb" else abi.WORKLOAD_TPCC
        cur = abi.LaunchC()
        self._ck(lib().ltpg_get_launch(self._h, wl, C.byref(cur)))
        for k, v in kw.items():
            setattr(cur, k, v)
        self._ck(lib().ltpg_set_launch(self._h, wl, C.byref(cur)))

    def get_launch(self, workload):
        wl = abi.WORKLOAD_YCSB if workload == "ycsb" else abi.WORKLOAD_TPCC
        cur = abi.LaunchC()
        self._ck(lib().ltpg_get_launch(self._h, wl, C.byref(cur)))
        return {k: getattr(cur, k) for k, _ in abi.LaunchC._fields_}

    def stage_set(self, buckets):
        """Stages the given key-hash buckets in shared memory (empty list: off)."""
        arr = np.ascontiguousarray(buckets, dtype=np.uint32)
        self._ck(lib().ltpg_stage_set(self._h, _p(arr) if len(arr) else None, len(arr)))

    def bucket_counts(self, reset=False):
        out = np.empty(abi.STAGE_BUCKETS, dtype=np.uint32)
        self._ck(lib().ltpg_bucket_counts(self._h, _p(out), int(bool(reset))))
        return out

    def predictor(self, enable=True, train=True, stage=True, lr=3e-3, seed=1):
        """Turns the contention predictor on (it then runs after every tuned YCSB batch)."""
        cfg = abi.PredictorC(int(enable), int(train), int(stage), 1, lr, 0, seed)
        self._ck(lib().ltpg_predictor_enable(self._h, C.byref(cfg)))

    def predictor_stats(self):
        loss, steps = C.c_float(), C.c_uint64()
        self._ck(lib().ltpg_predictor_stats(self._h, C.byref(loss), C.byref(steps)))
        return {"loss": loss.value, "train_steps": steps.value}

    def predictor_params(self, values=None):
        if values is None:
            out = np.empty(abi.PRED_PARAMS, dtype=np.float32)
            self._ck(lib().ltpg_predictor_get_params(self._h, _p(out), len(out)))
            return out
        v = np.ascontiguousarray(values, dtype=np.float32)
        self._ck(lib().ltpg_predictor_set_params(self._h, _p(v), len(v)))

    def predictor_forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty(len(x), dtype=np.float32)
        self._ck(lib().ltpg_predictor_forward(self._h, _p(x), len(x), _p(out)))
        return out

    def predictor_gradients(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        out = np.empty(abi.PRED_PARAMS, dtype=np.float32)
        self._ck(lib().ltpg_predictor_gradients(self._h, _p(x), _p(t), len(x), _p(out)))
        return out

    def counters(self):
        """(transactions committed, kernels launched) since the engine was created."""
        a, b = C.c_uint64(), C.c_uint64()
        self._ck(lib().ltpg_counters(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    MICROBENCH = {"copy": 0, "gather_thread": 1, "gather_coop": 2, "slot_load": 3, "red_random": 4,
                  "red_hot": 5, "h2d_kernel": 6, "h2d_copy": 7}

    def microbench(self, kind, n_items, iters=5):
        """Rate of one access pattern alone on this engine's device and stream
        (ltpg_microbench in include/ltpg_bench.h, from libltpg_bench.so)."""
        out = C.c_double()
        code = bench_lib().ltpg_microbench(self.device, self.stream(), self.MICROBENCH[kind], n_items, iters,
                                           C.byref(out))
        if code:
            raise LtpgError(code, f"microbench {kind} failed")
        return out.value

    def set_profiling(self, on=True):
        self._ck(lib().ltpg_set_profiling(self._h, int(bool(on))))

    def kernel_times(self, slot):
        """[execute, check, reads, write-back] ms of the slot's last run (profiling on)."""
        out = (C.c_float * 4)()
        self._ck(lib().ltpg_kernel_times(self._h, slot, out))
        return list(out)

    # test hooks (ltpg_debug_* in include/ltpg.h)
    def debug_set_epoch(self, epoch):
        """Makes the next batch run at batch epoch `epoch` (1 .. 2^32 - 1)."""
        self._ck(lib().ltpg_debug_set_epoch(self._h, epoch))

    def debug_epoch(self):
        """The device's current batch epoch."""
        out = C.c_uint32()
        self._ck(lib().ltpg_debug_get_epoch(self._h, C.byref(out)))
        return out.value

    def debug_barrier(self, limit_ns=0, skip_block=None):
        """Bounds the persistent kernels' grid-barrier waits by limit_ns (0: default)
        and makes block `skip_block` never arrive (None: every block arrives)."""
        self._ck(lib().ltpg_debug_barrier(self._h, limit_ns, 0xFFFFFFFF if skip_block is None else skip_block))


class Server:
    """Continuous batching of caller-owned transactions over a TPC-C engine and
    a YCSB engine (ltpg_server_open / ltpg_serve_submit / ltpg_serve_poll in
    include/ltpg.h).  Requests are ("tpcc", txn_record, lines) or ("ycsb",
    op_words, update_values); ids count from 0 in submission order."""

    def __init__(self, tpcc_engine, ycsb_engine, max_batch=262144, deadline_ms=2.0, mode="fused", slots=4,
                 budget_bytes=0, ycsb_ops=16):
        cfg = abi.ServerCfgC(deadline_ms, budget_bytes, max_batch, MODES[mode] if isinstance(mode, str) else mode,
                             slots, ycsb_ops)
        h = C.c_void_p()
        _check(lib().ltpg_server_open(tpcc_engine._h, ycsb_engine._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self._engines = (tpcc_engine, ycsb_engine)

    def submit(self, requests):
        """Admits the requests; returns the id of the first."""
        n = len(requests)
        arr = (abi.RequestC * max(1, n))()
        keep = []
        for i, r in enumerate(requests):
            if r[0] == "tpcc":
                txn = np.ascontiguousarray(np.asarray(r[1]).reshape(1), dtype=TpccBatch.TXN_DTYPE)
                lines = np.ascontiguousarray(r[2], dtype=TpccBatch.LINE_DTYPE)
                keep += [txn, lines]
                arr[i] = abi.RequestC(abi.WORKLOAD_TPCC, len(lines), txn.ctypes.data,
                                      lines.ctypes.data if len(lines) else None, None, None)
            else:
                ops = np.ascontiguousarray(r[1], dtype=np.uint32)
                vals = np.ascontiguousarray(r[2], dtype=np.uint64)
                keep += [ops, vals]
                arr[i] = abi.RequestC(abi.WORKLOAD_YCSB, len(ops), None, None, ops.ctypes.data,
                                      vals.ctypes.data if len(vals) else None)
        first = C.c_uint64()
        code = lib().ltpg_serve_submit(self._h, arr, n, C.byref(first))
        if code:
            raise LtpgError(code, "ltpg_serve_submit failed")
        return first.value

    def poll(self, first_id, n):
        """(flags, results) of the finished requests first_id, first_id + 1, ... (at most n)."""
        flags = np.zeros(n, dtype=np.uint8)
        res = np.zeros(n, dtype=np.int64)
        done = C.c_uint32()
        code = lib().ltpg_serve_poll(self._h, first_id, n, _p(flags), _p(res), C.byref(done))
        if code:
            raise LtpgError(code, "ltpg_serve_poll failed")
        return flags[:done.value], res[:done.value]

    def flush(self):
        code = lib().ltpg_serve_flush(self._h)
        if code:
            raise LtpgError(code, "ltpg_serve_flush failed")

    def batch_log(self):
        """[(first id, request count)] of the batches closed so far."""
        n = C.c_size_t()
        lib().ltpg_serve_batch_log(self._h, None, None, 0, C.byref(n))
        first = np.zeros(n.value, dtype=np.uint64)
        cnt = np.zeros(n.value, dtype=np.uint32)
        lib().ltpg_serve_batch_log(self._h, _p(first), _p(cnt), n.value, C.byref(n))
        return list(zip(first.tolist(), cnt.tolist()))

    def close(self):
        """Flushes and frees the server; returns its stats dict."""
        st = abi.ServeStatsC()
        code = lib().ltpg_server_close(self._h, C.byref(st))
        self._h = None
        if code:
            raise LtpgError(code, "ltpg_server_close failed")
        return {k: getattr(st, k) for k, _ in abi.ServeStatsC._fields_}


def serve(tpcc_engine, ycsb_engine, rate, duration_s, tpcc_params, ycsb_params, deadline_ms=2.0,
          max_batch=262144, tpcc_pct=70, mode="fused", budget_bytes=40 << 30, slots=4, seed=1, record=False):
    """Runs the continuous-batching request loop (see ltpg_serve_run in include/ltpg.h).

    tpcc_params / ycsb_params: dicts of TpccGenerator / YcsbGenerator arguments
    (seed, warehouses, n_txn, ...) describing the request pools.  Returns the
    stats dict, and with record=True also the replay record."""
    cfg = abi.ServeCfgC(rate, duration_s, deadline_ms, budget_bytes, seed, max_batch, tpcc_pct,
                        MODES[mode] if isinstance(mode, str) else mode, slots)
    tp = abi.TpccParamsC(tpcc_params["seed"], tpcc_params["warehouses"], tpcc_params.get("n_txn", 262144),
                         tpcc_params.get("neworder_pct", 50), tpcc_params.get("remote_line_pct", 1),
                         tpcc_params.get("remote_pay_pct", 15), tpcc_params.get("by_name_pct", 0),
                         tpcc_params.get("table_seed", tpcc_params["seed"]), tpcc_params.get("orderstatus_pct", 0),
                         tpcc_params.get("delivery_pct", 0), tpcc_params.get("stocklevel_pct", 0), 0)
    yp = abi.YcsbParamsC(ycsb_params["seed"], ycsb_params["n_records"], ycsb_params.get("n_txn", 262144),
                         ycsb_params.get("ops_per_txn", 10), ycsb_params.get("update_pct", 50),
                         ycsb_params.get("rotate_every", 0), ycsb_params.get("theta", 0.9))
    st = abi.ServeStatsC()
    rec = C.c_void_p()
    code = lib().ltpg_serve_run(tpcc_engine._h, ycsb_engine._h, C.byref(cfg), C.byref(tp), C.byref(yp),
                                C.byref(st), C.byref(rec) if record else None)
    _check(code, tpcc_engine._h)
    stats = {k: getattr(st, k) for k, _ in abi.ServeStatsC._fields_}
    if not record:
        return stats
    nb, nc, ny = C.c_uint64(), C.c_uint64(), C.c_uint64()
    lib().ltpg_serve_record_sizes(rec, C.byref(nb), C.byref(nc), C.byref(ny))
    out = {"batches": np.zeros((nb.value, 4), dtype=np.uint64),
           "tpcc_flags": np.zeros(nc.value, dtype=np.uint8), "tpcc_results": np.zeros(nc.value, dtype=np.int64),
           "ycsb_flags": np.zeros(ny.value, dtype=np.uint8), "ycsb_results": np.zeros(ny.value, dtype=np.int64)}
    lib().ltpg_serve_record_get(rec, _p(out["batches"]), _p(out["tpcc_flags"]), _p(out["tpcc_results"]),
                                _p(out["ycsb_flags"]), _p(out["ycsb_results"]))
    lib().ltpg_serve_record_free(rec)
    return stats, out
