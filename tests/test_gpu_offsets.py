"""YCSB batches uploaded without value offsets (val_off = NULL): the engine
makes them on the device from the op words (a scan of each transaction's
update count).  The offsets equal the host's, every mode and late-read
setting gives the oracle's flags, bitmap, results and table, the pipelined
host calls too, and a batch whose values do not match its update ops is
reported as LTPG_ERR_BOUNDS without a fault."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, LtpgError, YcsbBatch, YcsbGenerator, abi, pinned_copy, pinned_empty

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=4, max_txn=1 << 14, max_ops_per_txn=32)
    yield e
    e.close()


@pytest.mark.parametrize("k,upd,B", [(16, 5, 10000), (10, 50, 3000), (3, 30, 1), (32, 20, 2049), (7, 0, 5000)])
def test_device_offsets_equal_the_host_offsets(eng, k, upd, B):
    eng.load_ycsb(61, 5000)
    b = YcsbGenerator(61, 5000, B, k, upd, 0.9).batch(0)
    eng.upload(0, b.without_offsets())
    eng.sync()
    got = eng.download_batch(0)
    assert np.array_equal(got.val_off[: B + 1], b.val_off[: B + 1])
    assert np.array_equal(got.vals[: b.n_updates], b.vals[: b.n_updates])


@pytest.mark.parametrize("mode", ["plain", "fused", "persistent", "graph"])
@pytest.mark.parametrize("late", [0, 3])
def test_batches_without_offsets_match_oracle(eng, mode, late):
    n = 20000
    eng.load_ycsb(62, n)
    eng.set_launch("ycsb", late_reads=late)
    o = oracle.YcsbOracle(62, n)
    g = YcsbGenerator(62, n, 8192, 16, 10, 0.99)
    try:
        for bid in range(4):
            b = g.batch(bid)
            eng.upload(bid % 2, b.without_offsets())
            eng.run_batch(bid % 2, mode)
            eng.sync()
            wf, wb, wr = o.run(b)[:3]
            assert np.array_equal(eng.txn_flags(bid % 2, b.n_txn), wf)
            assert np.array_equal(eng.commit_bitmap(bid % 2, b.n_txn), wb)
            got = eng.txn_results(bid % 2, b.n_txn)
            if late and mode != "plain":  # late reads: an aborted transaction's result is 0
                wr = np.where((wf & abi.FLAG_COMMIT) != 0, wr, 0)
            assert np.array_equal(got, wr)
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        eng.set_launch("ycsb", late_reads=0)


def test_pipelined_host_calls_without_offsets(eng):
    """ltpg_submit_ycsb_host / ltpg_host_wait with pinned batches that carry no
    offsets: the offsets are made on the copy stream behind the op words."""
    n = 20000
    eng.load_ycsb(63, n)
    o = oracle.YcsbOracle(63, n)
    g = YcsbGenerator(63, n, 8192, 16, 10, 0.99)
    batches = [g.batch(i) for i in range(6)]
    pinned = [pinned_copy(b.without_offsets()) for b in batches]
    words = (8192 + 31) // 32
    bits = [pinned_empty(words) for _ in range(3)]
    for i, p in enumerate(pinned):
        s = i % 3
        if i >= 3:
            eng.host_wait(s)
            assert np.array_equal(bits[s], o.run(batches[i - 3])[1])
        eng.submit_host(s, p, "graph", bits[s])
    for i in range(3, 6):
        eng.host_wait(i % 3)
        assert np.array_equal(bits[i % 3], o.run(batches[i])[1])
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)


@pytest.mark.parametrize("mode", ["plain", "graph"])
def test_values_that_do_not_match_the_update_ops_report_error(eng, mode):
    n = 1000
    eng.load_ycsb(64, n)
    b = YcsbBatch.from_ops([[(5, True, 1), (6, True, 2), (7, False, 0)], [(8, True, 3)]], [[41, 42], [43]])
    short = YcsbBatch(b.ops, None, b.vals[:2], b.n_txn, b.ops_per_txn)  # three update ops, two values
    eng.upload(0, short)
    eng.run_batch(0, mode)
    with pytest.raises(LtpgError) as ei:
        eng.sync()
    assert ei.value.code == abi.ERR_BOUNDS
    # the context stays usable
    eng.load_ycsb(64, n)
    o = oracle.YcsbOracle(64, n)
    eng.upload(0, b.without_offsets())
    eng.run_batch(0, mode)
    eng.sync()
    assert np.array_equal(eng.commit_bitmap(0, b.n_txn), o.run(b)[1])
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
