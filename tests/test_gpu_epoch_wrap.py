"""Batch epochs across their last value, and grid-barrier waits that run out.

Registration slots carry a batch tag (0xFFFFFFFF - epoch), so the tables are
never cleared between batches.  The epoch is a 32-bit word: before a launch
would run a batch past epoch 0xFFFFFFFF, the engine sets every slot back to
the cleared state and the epoch to 1.  These tests start four batches short of
that point (ltpg_debug_set_epoch) and run eight batches across it, in every
run mode, with the flags, bitmap, results and table image bit-exact against
the oracle.

The persistent kernels' grid barriers are bounded waits.  A test hook makes
one block never arrive and shortens the bound to 1 ms: the launch must end
with LTPG_ERR_TIMEOUT, leave the table untouched, and the next batch on the
same context must be bit-exact against the oracle (the reference's epoch loop
only prints and stops, TF/tp.cu:159-164).
"""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, LtpgError, TpccGenerator, YcsbGenerator, abi

pytestmark = pytest.mark.gpu
NEAR_END = 0xFFFFFFFF - 3  # batches at ...FC, FD, FE, FF, then the reset to 1


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=8, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15)
    yield e
    e.close()


def check_slot(e, slot, b, want, late):
    wf, wb, wr = want[:3]
    flags = e.txn_flags(slot, b.n_txn)
    assert np.array_equal(flags, wf), f"flags differ at {np.nonzero(flags != wf)[0][:10]}"
    assert np.array_equal(e.commit_bitmap(slot, b.n_txn), wb)
    got = e.txn_results(slot, b.n_txn)
    if late:  # late reads: an aborted transaction's result is 0
        wr = np.where((wf & abi.FLAG_COMMIT) != 0, wr, 0)
    assert np.array_equal(got, wr)


YCSB_SHAPES = [("plain", 0), ("fused", 0), ("graph", 0), ("persistent", 0), ("graph", 3), ("persistent", 3)]


@pytest.mark.parametrize("mode,late", YCSB_SHAPES)
def test_ycsb_across_the_last_epoch(eng, mode, late):
    n = 20000
    eng.set_launch("ycsb", late_reads=late)
    eng.load_ycsb(41, n)
    o = oracle.YcsbOracle(41, n)
    g = YcsbGenerator(41, n, 8192, 16, 20, 0.99)  # hot keys repeat across the batches
    eng.debug_set_epoch(NEAR_END)
    for bid in range(8):
        b = g.batch(bid)
        eng.upload(bid % 2, b)
        eng.run_batch(bid % 2, mode)
        eng.sync()
        check_slot(eng, bid % 2, b, o.run(b), late)
    assert eng.debug_epoch() == 5
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    eng.set_launch("ycsb", late_reads=0)


def test_ycsb_graph_of_four_batches_across_the_last_epoch(eng):
    """A 4-batch graph ends exactly on the last epoch; its next replay starts
    after the reset."""
    n = 20000
    eng.set_launch("ycsb", late_reads=3)
    eng.load_ycsb(43, n)
    o = oracle.YcsbOracle(43, n)
    g = YcsbGenerator(43, n, 8192, 16, 20, 0.99)
    eng.debug_set_epoch(NEAR_END)
    for rep in range(2):
        batches = [g.batch(4 * rep + i) for i in range(4)]
        for i, b in enumerate(batches):
            eng.upload(i, b)
        eng.run_batches(0, 4, "graph")
        eng.sync()
        for i, b in enumerate(batches):
            check_slot(eng, i, b, o.run(b), True)
        assert eng.debug_epoch() == (0 if rep == 0 else 5)  # 0: wrapped on the device, reset before the next
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    eng.set_launch("ycsb", late_reads=0)


@pytest.mark.parametrize("mode", ["plain", "fused", "graph", "persistent"])
def test_tpcc_across_the_last_epoch(eng, mode):
    eng.load_tpcc(9, 2)
    o = oracle.TpccOracle(9, 2)
    g = TpccGenerator(9, 2, 4096)
    eng.debug_set_epoch(NEAR_END)
    for bid in range(8):
        b = g.next()
        eng.upload(bid % 2, b)
        eng.run_batch(bid % 2, mode)
        eng.sync()
        check_slot(eng, bid % 2, b, o.run(b), False)
    assert eng.debug_epoch() == 5
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), f"table {t} differs"


@pytest.mark.parametrize("late", [0, 2, 3])
def test_ycsb_persistent_barrier_timeout_then_next_batch_exact(eng, late):
    n = 50000
    eng.set_launch("ycsb", late_reads=late)
    eng.load_ycsb(45, n)
    o = oracle.YcsbOracle(45, n)
    g = YcsbGenerator(45, n, 1 << 15, 16, 10, 0.9)
    b = g.batch(0)
    eng.upload(0, b)
    eng.debug_barrier(limit_ns=1_000_000, skip_block=0)
    try:
        eng.run_batch(0, "persistent")
        with pytest.raises(LtpgError) as ei:
            eng.sync()
        assert ei.value.code == abi.ERR_TIMEOUT
    finally:
        eng.debug_barrier(0, None)
    # no phase after the failed barrier ran: the table is the loaded image
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    for bid, mode in enumerate(["persistent", "graph"]):
        b = g.batch(bid)
        eng.upload(0, b)
        eng.run_batch(0, mode)
        eng.sync()
        check_slot(eng, 0, b, o.run(b), late != 0)
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    eng.set_launch("ycsb", late_reads=0)


def test_tpcc_persistent_barrier_timeout_then_next_batch_exact(eng):
    eng.load_tpcc(11, 2)
    o = oracle.TpccOracle(11, 2)
    g = TpccGenerator(11, 2, 1 << 14)
    b = g.next()
    eng.upload(0, b)
    eng.debug_barrier(limit_ns=1_000_000, skip_block=0)
    try:
        eng.run_batch(0, "persistent")
        with pytest.raises(LtpgError) as ei:
            eng.sync()
        assert ei.value.code == abi.ERR_TIMEOUT
    finally:
        eng.debug_barrier(0, None)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), f"table {t} written by the failed launch"
    # the generator's counters moved on: the same batch runs again, then the next
    for mode in ["persistent", "fused"]:
        eng.upload(0, b)
        eng.run_batch(0, mode)
        eng.sync()
        check_slot(eng, 0, b, o.run(b), False)
        b = g.next()
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), f"table {t} differs"
