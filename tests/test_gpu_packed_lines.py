"""TPC-C batches whose order lines cross the host link packed in 4 bytes and
are unpacked on the device: the same flags, bitmap, results and tables as the
unpacked upload (against the oracle), in every mode, through the pipelined
host calls too, and for a batch without order lines."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, TpccGenerator, abi, pinned_copy, pinned_empty

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=4, max_txn=1 << 14, max_ops_per_txn=16, max_lines=15 << 14)
    yield e
    e.close()


def _same(e, o, b, slot):
    wf, wb, wr = o.run(b)[:3]
    assert np.array_equal(e.txn_flags(slot, b.n_txn), wf)
    assert np.array_equal(e.commit_bitmap(slot, b.n_txn), wb)
    assert np.array_equal(e.txn_results(slot, b.n_txn), wr)


@pytest.mark.parametrize("mode", ["plain", "fused", "persistent", "graph"])
def test_packed_upload_matches_oracle(eng, mode):
    eng.load_tpcc(21, 4)
    o = oracle.TpccOracle(21, 4)
    g = TpccGenerator(21, 4, 6000)
    for bid in range(3):
        b = g.next()
        eng.upload(bid % 2, b.with_packed_lines())
        eng.run_batch(bid % 2, mode)
        eng.sync()
        _same(eng, o, b, bid % 2)
        got = eng.download_batch(bid % 2)
        assert np.array_equal(got.lines, b.lines)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t])


def test_packed_batch_without_lines(eng):
    eng.load_tpcc(22, 2)
    o = oracle.TpccOracle(22, 2)
    g = TpccGenerator(22, 2, 2000, neworder_pct=0)  # Payments only: no order lines
    b = g.next()
    assert b.n_lines == 0
    eng.upload(0, b.with_packed_lines())
    eng.run_batch(0, "graph")
    eng.sync()
    _same(eng, o, b, 0)


def test_pipelined_packed_host_calls(eng):
    eng.load_tpcc(23, 8)
    o = oracle.TpccOracle(23, 8)
    g = TpccGenerator(23, 8, 4096)
    batches = [g.next() for _ in range(6)]
    pinned = [pinned_copy(b.with_packed_lines()) for b in batches]
    bits = [pinned_empty((4096 + 31) // 32) for _ in range(3)]
    for i, p in enumerate(pinned):
        s = i % 3
        if i >= 3:
            eng.host_wait(s)
            assert np.array_equal(bits[s], o.run(batches[i - 3])[1])
        eng.submit_host(s, p, "graph", bits[s])
    for i in range(3, 6):
        eng.host_wait(i % 3)
        assert np.array_equal(bits[i % 3], o.run(batches[i])[1])
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t])


def test_packed_upload_five_kind_mix(eng):
    """The five-transaction mix (customers by last name too) with packed lines,
    fused and graph, against the oracle."""
    eng.load_tpcc(24, 4)
    o = oracle.TpccOracle(24, 4)
    g = TpccGenerator(24, 4, 6000, neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4,
                      by_name_pct=60)
    for bid, mode in enumerate(["fused", "graph", "persistent"]):
        b = g.next()
        eng.upload(bid % 2, b.with_packed_lines())
        eng.run_batch(bid % 2, mode)
        eng.sync()
        _same(eng, o, b, bid % 2)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t])
