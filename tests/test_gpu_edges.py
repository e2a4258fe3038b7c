"""Edge cases of caller-made batches, bit-exact against the oracle in every
mode: ragged transactions (0 .. k ops, all-pad transactions), the same key
read and updated, the same field updated twice in one transaction (the later
update wins, as in op order), NewOrders listing one item twice (two stock
updates in line order), NewOrders of 1 and 15 lines, keys at the table's end,
and an empty batch rejected."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, LtpgError, TpccBatch, YcsbBatch, abi

pytestmark = pytest.mark.gpu
MODES = ["plain", "fused", "persistent", "graph"]


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=2, max_txn=1 << 15, max_ops_per_txn=32, max_lines=15 << 15)
    yield e
    e.close()


def _same(e, o, b, slot, mode):
    e.upload(slot, b)
    e.run_batch(slot, mode)
    e.sync()
    want = o.run(b)
    got = (e.txn_flags(slot, b.n_txn), e.commit_bitmap(slot, b.n_txn), e.txn_results(slot, b.n_txn))
    for g, w, what in zip(got, want[:3], ["flags", "bitmap", "results"]):
        assert np.array_equal(g, w), (what, np.nonzero(g != w)[0][:10])


def _ycsb_ragged_dups(rng, n, B, k):
    """Ragged transactions with repeated keys: some update one field twice."""
    ops, vals = [], []
    for t in range(B):
        m = int(rng.integers(0, k + 1))
        lst, vs = [], []
        for j in range(m):
            if j > 0 and rng.random() < 0.3:  # repeat an earlier key of this transaction
                key = lst[int(rng.integers(0, j))][0]
            else:
                key = int(rng.integers(0, n))
            upd = bool(rng.random() < 0.5)
            field = int(rng.integers(0, 2)) if upd else 0  # two fields: repeated updates often hit the same one
            lst.append((key, upd, field))
            if upd:
                vs.append(int(rng.integers(0, 2**63)))
        ops.append(lst)
        vals.append(vs)
    ops[0], vals[0] = [], []  # an all-pad transaction
    return YcsbBatch.from_ops(ops, vals)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("k", [7, 16, 32])
def test_ycsb_ragged_and_repeated_keys(eng, mode, k):
    n = 5000
    eng.load_ycsb(3, n)
    o = oracle.YcsbOracle(3, n)
    rng = np.random.default_rng(k)
    for i in range(2):
        _same(eng, o, _ycsb_ragged_dups(rng, n, 3000, k), i % 2, mode)
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)


@pytest.mark.parametrize("mode", MODES)
def test_ycsb_keys_at_table_end(eng, mode):
    n = 1000
    eng.load_ycsb(4, n)
    o = oracle.YcsbOracle(4, n)
    ops = [[(n - 1, True, 9), (n - 2, False, 0)], [(n - 1, False, 0)], [(0, True, 0), (n - 1, True, 3)]]
    vals = [[11], [], [12, 13]]
    _same(eng, o, YcsbBatch.from_ops(ops, vals), 0, mode)
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)


def _no(w, d, c_id, o_id, ol_id, items, line_off):
    ki = abi.TPCC_NEWORDER | (len(items) << 8) | (d << 16)
    return (ki, w, w, c_id, o_id, o_id, ol_id, line_off)


@pytest.mark.parametrize("mode", MODES)
def test_tpcc_repeated_items_and_line_counts(eng, mode):
    """NewOrders listing one item twice (both stock updates apply, as in line
    order), of 0, 1 and 15 lines, and NewOrders sharing stock rows."""
    W = 2
    eng.load_tpcc(5, W)
    o = oracle.TpccOracle(5, W)
    txns, lines = [], []
    rng = np.random.default_rng(9)
    for t in range(400):
        cnt = [1, 15, 5, 3, 0][t % 5]
        items = [int(rng.integers(0, 40)) for _ in range(cnt)]  # 40 items: repeats within and across orders
        txns.append(_no(t % W, t % 10, t % 3000, t % 30000, (15 * t) % 450000, items, len(lines)))
        for it in items:
            lines.append((it, t % W, int(rng.integers(1, 11))))
    b = TpccBatch(np.array(txns, dtype=TpccBatch.TXN_DTYPE), np.array(lines, dtype=TpccBatch.LINE_DTYPE), 100)
    _same(eng, o, b, 0, mode)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), t


def test_empty_batch_is_rejected(eng):
    eng.load_ycsb(6, 100)
    empty = YcsbBatch(np.zeros(0, np.uint32), np.zeros(1, np.uint32), np.zeros(0, np.uint64), 0, 4)
    with pytest.raises(LtpgError) as ei:
        eng.upload(0, empty)
    assert ei.value.code == abi.ERR_INVALID
    o = oracle.YcsbOracle(6, 100)  # the engine is still usable
    _same(eng, o, YcsbBatch.from_ops([[(1, True, 2)], [(1, False, 0)]], [[5], []]), 0, "graph")
