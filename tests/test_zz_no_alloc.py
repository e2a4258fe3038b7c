"""The no-allocation entry point (ltpg_ycsb_batch_noalloc) against the regular one.

Some callers cannot allocate device memory: a host runtime that owns all GPU
memory through its own pool, or a latency-critical thread, where cudaMalloc /
cudaFree can block or synchronise the device.  ltpg_ycsb_batch_noalloc takes
their device buffers and keeps its own scratch in static device memory.  This
test runs two batches in a row through it and through the regular engine
(ltpg_create / upload / run_batch) and requires identical outputs, bit for bit.
It sits in its own file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import ltpg_gb300
from ltpg_gb300 import Engine, YcsbGenerator, abi

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point(gpu):
    import torch
    n, B, k, seed = 200_000, 50_000, 10, 77
    g = YcsbGenerator(seed, n, B, k, 50, 0.9)
    batches = [g.batch(0), g.batch(1)]
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=k)
    try:
        eng.load_ycsb(seed, n)
        rows0 = eng.download_table(abi.TABLE_YCSB)
        want = []
        for b in batches:
            eng.upload(0, b)
            eng.run_batch(0, "plain")
            eng.sync()
            want.append((eng.txn_flags(0, B), eng.commit_bitmap(0, B), eng.txn_results(0, B),
                         eng.download_table(abi.TABLE_YCSB)))
    finally:
        eng.close()

    dev = torch.device("cuda", 0)
    rows = torch.from_numpy(rows0.view(np.int64)).to(dev)
    flags = torch.empty(B, dtype=torch.uint8, device=dev)
    bitmap = torch.empty((B + 31) // 32, dtype=torch.int32, device=dev)
    results = torch.empty(B, dtype=torch.int64, device=dev)
    L = ltpg_gb300.lib()
    for b, (wf, wb, wr, wrows) in zip(batches, want):
        ops = torch.from_numpy(b.ops.view(np.int32)).to(dev)
        val_off = torch.from_numpy(b.val_off.view(np.int32)).to(dev)
        vals = torch.from_numpy(b.vals.view(np.int64)).to(dev)
        torch.cuda.synchronize()
        rc = L.ltpg_ycsb_batch_noalloc(0, C.c_void_p(rows.data_ptr()), n, C.c_void_p(ops.data_ptr()),
                                       C.c_void_p(val_off.data_ptr()), C.c_void_p(vals.data_ptr()), B, k,
                                       C.c_void_p(flags.data_ptr()), C.c_void_p(bitmap.data_ptr()),
                                       C.c_void_p(results.data_ptr()), None)
        assert rc == abi.OK
        assert np.array_equal(flags.cpu().numpy(), wf)
        assert np.array_equal(bitmap.cpu().numpy().view(np.uint32), wb)
        assert np.array_equal(results.cpu().numpy(), wr)
        assert np.array_equal(rows.cpu().numpy().view(np.uint64), wrows)


def _run_both(n, seed, batches, k):
    """Runs the batches in order through the regular engine (plain mode) and
    through ltpg_ycsb_batch_noalloc on a copy of the same table, and returns
    per batch (regular status, no-allocation status, regular outputs,
    no-allocation outputs); outputs = (flags, bitmap, results, table)."""
    import torch
    B = max(b.n_txn for b in batches)
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=k)
    want = []
    try:
        eng.load_ycsb(seed, n)
        rows0 = eng.download_table(abi.TABLE_YCSB)
        for b in batches:
            eng.upload(0, b)
            eng.run_batch(0, "plain")
            code = abi.OK
            try:
                eng.sync()
            except ltpg_gb300.LtpgError as e:
                code = e.code
            want.append((code, (eng.txn_flags(0, b.n_txn), eng.commit_bitmap(0, b.n_txn),
                                eng.txn_results(0, b.n_txn), eng.download_table(abi.TABLE_YCSB))))
    finally:
        eng.close()
    dev = torch.device("cuda", 0)
    rows = torch.from_numpy(rows0.view(np.int64)).to(dev)
    L = ltpg_gb300.lib()
    out = []
    for b, (wcode, wout) in zip(batches, want):
        flags = torch.empty(b.n_txn, dtype=torch.uint8, device=dev)
        bitmap = torch.empty((b.n_txn + 31) // 32, dtype=torch.int32, device=dev)
        results = torch.empty(b.n_txn, dtype=torch.int64, device=dev)
        ops = torch.from_numpy(b.ops.view(np.int32)).to(dev)
        val_off = torch.from_numpy(b.val_off.view(np.int32)).to(dev)
        vals = torch.from_numpy(np.concatenate([b.vals, np.zeros(1, np.uint64)]).view(np.int64)).to(dev)
        torch.cuda.synchronize()
        rc = L.ltpg_ycsb_batch_noalloc(0, C.c_void_p(rows.data_ptr()), n, C.c_void_p(ops.data_ptr()),
                                       C.c_void_p(val_off.data_ptr()), C.c_void_p(vals.data_ptr()), b.n_txn,
                                       b.ops_per_txn, C.c_void_p(flags.data_ptr()), C.c_void_p(bitmap.data_ptr()),
                                       C.c_void_p(results.data_ptr()), None)
        got = (flags.cpu().numpy(), bitmap.cpu().numpy().view(np.uint32), results.cpu().numpy(),
               rows.cpu().numpy().view(np.uint64))
        out.append((wcode, rc, wout, got))
    return out


def _assert_same(wout, got):
    for name, w, g in zip(("flags", "bitmap", "results", "table"), wout, got):
        assert np.array_equal(w, g), f"{name} differ"


def test_noalloc_out_of_range_key_then_clean_batch(gpu):
    """A key past the table's end gives LTPG_ERR_BOUNDS (the call clears the
    shared error word); the next call on the same scratch is exact."""
    from ltpg_gb300 import YcsbBatch
    n, k = 5000, 4
    bad = YcsbBatch.from_ops([[(3, 1, 2), (n, 0, 0)], [(3, 0, 0), (7, 1, 1)]], [[11], [12]])
    g = YcsbGenerator(5, n, 4000, k, 50, 0.9)
    res = _run_both(n, 5, [bad, g.batch(0), g.batch(1)], k)
    assert res[0][0] == abi.ERR_BOUNDS and res[0][1] == abi.ERR_BOUNDS
    for wcode, rc, wout, got in res:
        assert rc == wcode
        _assert_same(wout, got)


def test_noalloc_smaller_table_after_larger(gpu):
    big = _run_both(300_000, 6, [YcsbGenerator(6, 300_000, 20000, 10, 50, 0.9).batch(0)], 10)
    small = _run_both(1000, 7, [YcsbGenerator(7, 1000, 3000, 10, 50, 0.9).batch(i) for i in range(2)], 10)
    for wcode, rc, wout, got in big + small:
        assert rc == wcode == abi.OK
        _assert_same(wout, got)


def test_noalloc_across_the_last_epoch(gpu):
    """The shared scratch is epoch-tagged; four calls that start two epochs
    short of the last one cross it (the call that would pass it first sets
    the scratch back to its cleared state) and stay exact."""
    L = ltpg_gb300.lib()
    n, k = 20000, 16
    g = YcsbGenerator(8, n, 8192, k, 20, 0.99)
    assert L.ltpg_debug_noalloc_set_epoch(0, 0xFFFFFFFE) == abi.OK
    res = _run_both(n, 8, [g.batch(i) for i in range(4)], k)
    for wcode, rc, wout, got in res:
        assert rc == wcode == abi.OK
        _assert_same(wout, got)
    ep = C.c_uint32()
    assert L.ltpg_debug_noalloc_get_epoch(0, C.byref(ep)) == abi.OK
    assert ep.value == 3  # ...FE, ...FF, then 1, 2


def test_noalloc_rejects_tables_beyond_its_scratch(gpu):
    L = ltpg_gb300.lib()
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ltpg_ycsb_batch_noalloc(0, one, abi.NOALLOC_MAX_RECORDS + 1, one, one, one, 1, 1, one, one, one, None)
    assert rc == abi.ERR_INVALID
