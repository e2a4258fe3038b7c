"""The full TPC-C mix on the GPU (NewOrder / Payment / OrderStatus / Delivery /
StockLevel, 45/43/4/4/4, customers by name 60 %): flags, bitmap, results and
every table bit-exact against the oracle, in every mode."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, TpccGenerator, abi
from test_tpcc_mix import DL, NO, OS, SL, batch, txn

pytestmark = pytest.mark.gpu
MIX = dict(neworder_pct=45, orderstatus_pct=4, delivery_pct=4, stocklevel_pct=4, by_name_pct=60)


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=4, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15)
    yield e
    e.close()


@pytest.fixture(scope="module")
def eng_strict(gpu):
    e = Engine(device=0, n_slots=2, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15, strict_insert=True)
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
    return want[0]


def _tables(e, o):
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(e.download_table(t), o.tables[t]), f"table {t}"


@pytest.mark.parametrize("W,mode", [(1, "plain"), (3, "plain"), (2, "fused"), (3, "persistent"), (2, "graph")])
def test_mix_matches_oracle(eng, W, mode):
    eng.load_tpcc(31, W)
    o = oracle.TpccOracle(31, W)
    g = TpccGenerator(31, W, 20000, **MIX)
    kinds_seen = set()
    for i in range(4):
        b = g.next()
        flags = _same(eng, o, b, i % 2, mode)
        k = b.txns["kind_info"] & 0xFF
        kinds_seen |= set(np.unique(k[(flags & abi.FLAG_COMMIT) != 0]).tolist())
    assert kinds_seen == {0, 1, 2, 3, 4}
    _tables(eng, o)


def test_mix_strict_insert(eng_strict):
    W = 2
    eng_strict.load_tpcc(33, W)
    o = oracle.TpccOracle(33, W, strict=True)
    g = TpccGenerator(33, W, 12000, **MIX)
    for i, mode in enumerate(["plain", "fused", "graph"]):
        _same(eng_strict, o, g.next(), i % 2, mode)
    _tables(eng_strict, o)


@pytest.mark.parametrize("mode", ["plain", "fused", "persistent"])
def test_mix_known_answers(eng, mode):
    """The CPU known-answer batches of test_tpcc_mix on the engine."""
    cases = [
        ([txn(DL, w=0, d=4, c_id=9, a=120, b=120, c=77, hi=7)], ()),
        ([txn(NO, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=1), txn(DL, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=3)],
         [(11, 0, 3)]),
        ([txn(DL, w=0, d=1, c_id=2, a=5, b=6, c=41, hi=3), txn(NO, w=0, d=1, c_id=3, a=5, b=5, c=40, hi=1)],
         [(11, 0, 3)]),
        ([txn(NO, w=0, d=1, c_id=2, a=5, b=5, c=40, hi=1), txn(SL, w=0, d=1, a=11, hi=15),
          txn(OS, w=0, d=1, c_w=0, c_d=1, c_id=2, a=5, b=40)], [(11, 0, 3)]),
    ]
    for rows, lines in cases:
        eng.load_tpcc(2, 1)
        o = oracle.TpccOracle(2, 1)
        _same(eng, o, batch(rows, list(lines)), 0, mode)
        _tables(eng, o)


@pytest.mark.parametrize("filt,dedupe,bps", [(0, 0, 0), (1, 0, 2), (0, 1, 6), (1, 1, 0)])
def test_launch_shapes_do_not_change_outcomes(eng, filt, dedupe, bps):
    """Every TPC-C launch shape the autotuner can pick (slot filter, warp
    dedupe of header registrations, blocks per SM) gives the oracle's outcome."""
    W = 3
    eng.load_tpcc(37, W)
    o = oracle.TpccOracle(37, W)
    g = TpccGenerator(37, W, 30000, **MIX)
    try:
        eng.set_launch("tpcc", filter=filt, dedupe=dedupe, blocks_per_sm=bps)
        for i, mode in enumerate(["fused", "persistent", "graph"]):
            _same(eng, o, g.next(), i % 2, mode)
        _tables(eng, o)
    finally:
        eng.set_launch("tpcc", filter=0, dedupe=0, blocks_per_sm=0)
