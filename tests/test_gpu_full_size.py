"""Parity at the benchmark sizes: the tuned engine against the oracle on
full batches — YCSB high contention (10M records, 1,048,576 transactions x 16
ops, 95/5, theta = 0.99, hot set rotating every 8 batches, across a rotation;
rows read at execute, and write-first registration with late reads),
and TPC-C at W = 64 with 1,048,576 transactions (NewOrder / Payment 50/50 and
the five-kind mix with names).  Every flag, bitmap word, result and table row
bit-exact; plus the size-independent properties: commit bits = commit flags,
the stats' counters = counts over the flags, tuned = plain."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, TpccGenerator, YcsbGenerator, abi

pytestmark = pytest.mark.gpu
B = 1 << 20


def _properties(e, slot, flags, bitmap):
    com = (flags & abi.FLAG_COMMIT) != 0
    bits = np.unpackbits(bitmap.view(np.uint8), bitorder="little")[: len(flags)].astype(bool)
    assert np.array_equal(bits, com)
    st = e.stats(slot)
    assert st["commits"] == int(com.sum())
    assert st["raw"] == int(((flags & abi.FLAG_RAW) != 0).sum())
    assert st["war"] == int(((flags & abi.FLAG_WAR) != 0).sum())
    assert st["waw"] == int(((flags & abi.FLAG_WAW) != 0).sum())


@pytest.mark.parametrize("late", [0, 3], ids=["reads-at-execute", "write-first"])
def test_ycsb_high_contention_full_size(gpu, late):
    """late = 3 is the benchmark's launch setting (write-first registration,
    rows read by committed transactions only: an aborted one's result is 0)."""
    n = 10_000_000
    g = YcsbGenerator(20261203, n, B, 16, 5, 0.99, 8)
    o = oracle.YcsbOracle(20261203, n)
    e = Engine(device=0, n_slots=2, max_txn=B, max_ops_per_txn=16)
    try:
        e.set_launch("ycsb", late_reads=late)
        e.load_ycsb(20261203, n)
        for i, (bid, mode) in enumerate([(6, "graph"), (7, "fused"), (8, "graph"), (9, "persistent")]):
            b = g.batch(bid)
            e.upload(i % 2, b)
            e.run_batch(i % 2, mode)
            e.sync()
            flags, bitmap, results, commits = o.run(b)
            got = e.txn_flags(i % 2, B)
            assert np.array_equal(got, flags), np.nonzero(got != flags)[0][:10]
            assert np.array_equal(e.commit_bitmap(i % 2, B), bitmap)
            res = e.txn_results(i % 2, B)
            com = (flags & abi.FLAG_COMMIT) != 0
            assert np.array_equal(res, results if late == 0 else np.where(com, results, 0))
            _properties(e, i % 2, got, e.commit_bitmap(i % 2, B))
            assert 0.2 < commits / B < 0.9
        assert np.array_equal(e.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        e.close()


@pytest.mark.parametrize("mix", [{}, dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4,
                                          by_name_pct=60)], ids=["50-50", "mix"])
def test_tpcc_w64_full_size(gpu, mix):
    W = 64
    g = TpccGenerator(20261203, W, B, **mix)
    batches = [g.next() for _ in range(2)]
    o = oracle.TpccOracle(20261203, W)
    e = Engine(device=0, n_slots=2, max_txn=B, max_ops_per_txn=16, max_lines=max(b.n_lines for b in batches))
    p = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=16, max_lines=max(b.n_lines for b in batches))
    try:
        e.load_tpcc(20261203, W)
        p.load_tpcc(20261203, W)
        for i, (b, mode) in enumerate(zip(batches, ["graph", "persistent"])):
            e.upload(i, b)
            e.run_batch(i, mode)
            p.upload(0, b)
            p.run_batch(0, "plain")
            e.sync()
            p.sync()
            flags, bitmap, results, _ = o.run(b)
            got = e.txn_flags(i, B)
            assert np.array_equal(got, flags), np.nonzero(got != flags)[0][:10]
            assert np.array_equal(e.commit_bitmap(i, B), bitmap)
            assert np.array_equal(e.txn_results(i, B), results)
            assert np.array_equal(p.txn_flags(0, B), flags)
            _properties(e, i, got, e.commit_bitmap(i, B))
        for t in range(abi.TPCC_TABLES):
            assert np.array_equal(e.download_table(t), o.tables[t]), t
            assert np.array_equal(p.download_table(t), o.tables[t]), t
    finally:
        e.close()
        p.close()
