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


def test_noalloc_rejects_tables_beyond_its_scratch(gpu):
    L = ltpg_gb300.lib()
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ltpg_ycsb_batch_noalloc(0, one, abi.NOALLOC_MAX_RECORDS + 1, one, one, one, 1, 1, one, one, one, None)
    assert rc == abi.ERR_INVALID
