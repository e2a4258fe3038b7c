"""Batches made on the GPU (ltpg_gen_*_batch_device): byte-identical to the
host generator's batch after batch — YCSB at every Zipf setting, rotation,
scans and a tiny table; TPC-C with its per-warehouse counters, order memory,
O_ID wrap-around inside one batch and Delivery's 30,000-order clamp — and run
by the engine exactly like uploaded batches."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, LtpgError, TpccGenerator, YcsbGenerator, abi

pytestmark = pytest.mark.gpu
MIX = dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4)


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=2, max_txn=1 << 17, max_ops_per_txn=16, max_lines=15 << 17)
    yield e
    e.close()


def _same_ycsb(got, want):
    assert got.n_txn == want.n_txn and got.ops_per_txn == want.ops_per_txn
    n = want.n_txn * want.op_stride
    assert np.array_equal(got.ops[:n], want.ops[:n]), np.nonzero(got.ops[:n] != want.ops[:n])[0][:10]
    assert np.array_equal(got.val_off, want.val_off[: want.n_txn + 1])
    assert np.array_equal(got.vals, want.vals)


@pytest.mark.parametrize("case", [
    dict(n=100_000, B=20000, k=10, upd=50, theta=0.6, rot=0, scan=0),
    dict(n=1_000_000, B=30000, k=16, upd=5, theta=0.99, rot=8, scan=0),
    dict(n=50_000, B=10000, k=7, upd=30, theta=0.0, rot=0, scan=0),
    dict(n=200_000, B=10000, k=10, upd=5, theta=0.99, rot=0, scan=10),
    dict(n=20, B=3000, k=16, upd=50, theta=0.9, rot=4, scan=0),  # resampling and the free-key walk
])
def test_ycsb_device_batches_equal_host(eng, case):
    eng.load_ycsb(5, case["n"])
    g = YcsbGenerator(5, case["n"], case["B"], case["k"], case["upd"], case["theta"], case["rot"], case["scan"])
    for bid in [0, 1, 9, 17]:
        eng.generate(bid % 2, g, bid)
        _same_ycsb(eng.download_batch(bid % 2), g.batch(bid))


def _same_tpcc(got, want):
    assert got.txn_base == want.txn_base
    bad = np.nonzero(got.txns != want.txns)[0]
    assert len(bad) == 0, (bad[:10], got.txns[bad[:3]], want.txns[bad[:3]])
    assert np.array_equal(got.lines, want.lines)


@pytest.mark.parametrize("W,B,kw", [
    (4, 20000, {}),                                       # NewOrder / Payment 50/50 by id
    (2, 20000, dict(MIX, by_name_pct=60)),                # the five-kind mix, names
    (1, 80000, MIX),                                      # O_IDs wrap inside a batch; Delivery's clamp
    (3, 30000, dict(neworder_pct=10, orderstatus_pct=30, delivery_pct=30, stocklevel_pct=10, by_name_pct=100)),
])
def test_tpcc_device_batches_equal_host(eng, W, B, kw):
    eng.load_tpcc(7, W)
    gd, gh = TpccGenerator(7, W, B, **kw), TpccGenerator(7, W, B, **kw)
    for _ in range(2):  # host batches first: the state moves to the GPU at the first device batch
        _same_tpcc(gd.next(), gh.next())
    for i in range(4):
        eng.generate(i % 2, gd)
        _same_tpcc(eng.download_batch(i % 2), gh.next())
    with pytest.raises(LtpgError) as ei:
        gd.next()
    assert ei.value.code == abi.ERR_STATE


def test_engine_runs_device_batches(eng):
    W = 2
    eng.load_tpcc(11, W)
    o = oracle.TpccOracle(11, W)
    gd, gh = TpccGenerator(11, W, 20000, by_name_pct=60, **MIX), TpccGenerator(11, W, 20000, by_name_pct=60, **MIX)
    for i, mode in enumerate(["plain", "graph", "fused", "graph"]):
        eng.generate(i % 2, gd)
        eng.run_batch(i % 2, mode)
        eng.sync()
        b = gh.next()
        flags, bitmap, results, _ = o.run(b)
        assert np.array_equal(eng.txn_flags(i % 2, b.n_txn), flags)
        assert np.array_equal(eng.commit_bitmap(i % 2, b.n_txn), bitmap)
        assert np.array_equal(eng.txn_results(i % 2, b.n_txn), results)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), t

    n = 200_000
    eng.load_ycsb(13, n)
    yo = oracle.YcsbOracle(13, n)
    g = YcsbGenerator(13, n, 30000, 16, 5, 0.99, 8)
    for bid, mode in enumerate(["plain", "graph", "graph"]):
        eng.generate(0, g, bid)
        eng.run_batch(0, mode)
        eng.sync()
        flags, bitmap, results, _ = yo.run(g.batch(bid))
        assert np.array_equal(eng.txn_flags(0, 30000), flags)
        assert np.array_equal(eng.txn_results(0, 30000), results)
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), yo.rows)


def test_device_generation_checks(eng):
    eng.load_tpcc(3, 2)
    with pytest.raises(LtpgError):
        eng.generate(0, TpccGenerator(3, 4, 1000))  # more warehouses than loaded
    small = Engine(device=0, n_slots=1, max_txn=1 << 12, max_ops_per_txn=16, max_lines=1 << 12)
    try:
        small.load_tpcc(3, 1)
        with pytest.raises(LtpgError) as ei:
            small.generate(0, TpccGenerator(3, 1, 1 << 12))  # lines beyond max_lines
        assert ei.value.code == abi.ERR_INVALID
    finally:
        small.close()


def test_pipelined_device_generation(eng):
    """ltpg_submit_generated: each batch generated on the copy stream while the
    one before it runs, two slots in flight; bitmaps, flags and the final image
    equal the oracle's run of the host generator's batches."""
    from ltpg_gb300 import pinned_empty
    depth = 2
    n, B = 200_000, 20000
    eng.load_ycsb(17, n)
    yo = oracle.YcsbOracle(17, n)
    g = YcsbGenerator(17, n, B, 16, 5, 0.99, 4)
    want = [yo.run(g.batch(i))[1] for i in range(6)]
    bits = [pinned_empty((B + 31) // 32) for _ in range(depth)]
    for i in range(6):
        if i >= depth:
            eng.host_wait(i % depth)
            assert np.array_equal(bits[i % depth], want[i - depth]), i - depth
        eng.submit_generated(i % depth, g, "graph", bits[i % depth], batch_id=i)
    for i in range(6 - depth, 6):
        eng.host_wait(i % depth)
        assert np.array_equal(bits[i % depth], want[i]), i
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), yo.rows)

    W = 2
    eng.load_tpcc(19, W)
    to = oracle.TpccOracle(19, W)
    gd, gh = TpccGenerator(19, W, B, by_name_pct=60, **MIX), TpccGenerator(19, W, B, by_name_pct=60, **MIX)
    want = [to.run(gh.next()) for _ in range(6)]
    for i in range(6):
        if i >= depth:
            eng.host_wait(i % depth)
            assert np.array_equal(bits[i % depth], want[i - depth][1]), i - depth
        eng.submit_generated(i % depth, gd, "fused", bits[i % depth])
    for i in range(6 - depth, 6):
        eng.host_wait(i % depth)
        assert np.array_equal(bits[i % depth], want[i][1]), i
        assert np.array_equal(eng.txn_flags(i % depth, B), want[i][0])
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), to.tables[t]), t
