"""OrderStatus, Delivery and StockLevel (the reference's all-transaction
variant, TA/Execute.h:1592-2231): known answers worked out from the protocol's
rules, the generator's mix, and stream stability.  CPU only."""
import numpy as np

import oracle
from ltpg_gb300 import TpccBatch, TpccGenerator, abi

NO, PAY, OS, DL, SL = 0, 1, 2, 3, 4
C_COLS = abi.TPCC_COLS


def txn(kind, w=0, d=0, c_w=0, c_d=0, c_id=0, a=0, b=0, c=0, line_off=0, hi=0):
    """One record; hi = kind_info bits 8..15 (line count / carrier / threshold)."""
    return (kind | (hi << 8) | (d << 16) | (c_d << 24), w, c_w, c_id, a, b, c, line_off)


def batch(rows, lines=(), base=1000):
    t = np.array(rows, dtype=TpccBatch.TXN_DTYPE)
    ln = np.array(lines, dtype=TpccBatch.LINE_DTYPE) if lines else np.zeros(0, dtype=TpccBatch.LINE_DTYPE)
    return TpccBatch(t, ln, base)


def row(o, table, r):
    return o.tables[table].reshape(-1, C_COLS[table])[r].copy()


def test_delivery_alone_applies_its_writes():
    o = oracle.TpccOracle(2, 1)
    ol_amount = int(row(o, abi.T_ORDERLINE, 77)[8])
    cust0 = row(o, abi.T_CUSTOMER, 3000 * 4 + 9)
    b = batch([txn(DL, w=0, d=4, c_id=9, a=120, b=120, c=77, hi=7)])
    flags, bitmap, results, commits = o.run(b)
    assert flags[0] == abi.FLAG_COMMIT and commits == 1
    assert results[0] == ol_amount
    assert (row(o, abi.T_NEWORDER, 120) == np.uint64(2**64 - 1)).all()  # deleted
    assert row(o, abi.T_ORDER, 120)[5] == 7                            # O_CARRIER_ID
    assert row(o, abi.T_ORDERLINE, 77)[6] == 1000                      # OL_DELIVERY_D = txn_base + TID
    cust = row(o, abi.T_CUSTOMER, 3000 * 4 + 9)
    assert int(cust[5].astype(np.int64)) == int(cust0[5].astype(np.int64)) + ol_amount
    assert cust[8] == cust0[8] + 1


def test_delivery_after_neworder_of_the_same_order_aborts():
    """NewOrder (TID 0) inserts ORDER row 5 and ORDER-LINE row 40; Delivery
    (TID 1) reads and updates both: RAW and WAW -> abort.  The NewOrder
    commits."""
    o = oracle.TpccOracle(2, 1)
    lines = [(11, 0, 3)]
    b = batch([txn(NO, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=1, line_off=0),
               txn(DL, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=3)], lines)
    flags = o.run(b)[0]
    assert flags[0] == abi.FLAG_COMMIT
    assert flags[1] == abi.FLAG_RAW | abi.FLAG_WAR | abi.FLAG_WAW


def test_neworder_after_delivery_of_the_same_order_aborts():
    """Delivery (TID 0) registers ORDER row 5 for read and write; the NewOrder
    (TID 1) inserting it sees WAR and WAW -> abort; the Delivery commits."""
    o = oracle.TpccOracle(2, 1)
    lines = [(11, 0, 3)]
    b = batch([txn(DL, w=0, d=1, c_id=2, a=5, b=6, c=41, hi=3),
               txn(NO, w=0, d=1, c_id=3, a=5, b=5, c=40, hi=1, line_off=0)], lines)
    flags = o.run(b)[0]
    assert flags[0] == abi.FLAG_COMMIT
    assert flags[1] & abi.FLAG_WAW and not flags[1] & abi.FLAG_COMMIT


def test_read_only_kinds_commit_with_raw():
    """StockLevel and OrderStatus after writers of their rows: RAW only, and
    a transaction without WAR commits (TF/Execute_neworder.h:692)."""
    o = oracle.TpccOracle(2, 1)
    lines = [(11, 0, 3)]
    q0 = int(row(o, abi.T_STOCK, 11)[2])
    b = batch([txn(NO, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=1, line_off=0),
               txn(SL, w=0, d=1, a=11, hi=15),
               txn(OS, w=0, d=1, c_w=0, c_d=1, c_id=2, a=5, b=40)], lines)
    flags, _, results, _ = o.run(b)
    assert flags[1] == abi.FLAG_RAW | abi.FLAG_COMMIT
    assert flags[2] == abi.FLAG_RAW | abi.FLAG_COMMIT
    assert results[1] == q0  # batch-start S_QUANTITY
    assert results[2] == int(row(o, abi.T_CUSTOMER, 3000 + 2)[5].astype(np.int64))  # C_BALANCE


def test_mix_generator_shares_and_stream_stability():
    """The three extra kinds take their shares from Payment's; with the shares
    at zero the generator's stream is unchanged."""
    base = TpccGenerator(4, 3, 20000).next()
    again = TpccGenerator(4, 3, 20000, orderstatus_pct=0, delivery_pct=0, stocklevel_pct=0).next()
    assert np.array_equal(base.txns, again.txns) and np.array_equal(base.lines, again.lines)
    g = TpccGenerator(4, 3, 40000, neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4)
    g.next()
    b = g.next()
    share = np.bincount(b.txns["kind_info"] & 0xFF, minlength=5) / b.n_txn
    assert abs(share[NO] - 0.45) < 0.02 and abs(share[PAY] - 0.43) < 0.02
    assert all(abs(share[k] - 0.04) < 0.01 for k in (OS, DL, SL))
    # Delivery takes the oldest undelivered orders: NEW-ORDER row = ORDER row
    dl = b.txns[(b.txns["kind_info"] & 0xFF) == DL]
    assert np.array_equal(dl["a"], dl["b"])
    carrier = (dl["kind_info"] >> 8) & 0xFF
    assert carrier.min() >= 1 and carrier.max() <= 10


def test_multithreaded_replay_equals_single_threaded():
    """The oracle's pthreads replay (the reference arm's CPU baseline) gives the
    single-threaded replay's flags, bitmap, results and image, batch after
    batch, with names, all five kinds and hot YTD adds."""
    W, B = 2, 20000
    kw = dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4, by_name_pct=60)
    o1, o8 = oracle.TpccOracle(41, W), oracle.TpccOracle(41, W)
    g = TpccGenerator(41, W, B, **kw)
    for _ in range(3):
        b = g.next()
        a, m = o1.run(b), o8.run(b, threads=8)
        for x, y in zip(a, m):
            assert np.array_equal(x, y)
    for t1, t8 in zip(o1.tables, o8.tables):
        assert np.array_equal(t1, t8)
