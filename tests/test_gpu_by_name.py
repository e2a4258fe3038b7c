"""Payment by customer last name on the GPU: the sorted per-district name
index and its binary-search lookup, the reference-arithmetic mode, not-found
Payments — bit-exact against the oracle."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, TpccBatch, TpccGenerator, abi

pytestmark = pytest.mark.gpu
C_ID_COL, C_LAST_COL = 0, 13


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=4, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15)
    yield e
    e.close()


@pytest.fixture(scope="module")
def eng_ref(gpu):
    e = Engine(device=0, n_slots=2, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15, ref_name_lookup=True)
    yield e
    e.close()


def _run(e, slot, b, mode):
    e.upload(slot, b)
    e.run_batch(slot, mode)
    e.sync()
    return e.txn_flags(slot, b.n_txn), e.commit_bitmap(slot, b.n_txn), e.txn_results(slot, b.n_txn)


def _same(e, o, b, slot, mode):
    got = _run(e, slot, b, mode)
    want = o.run(b)
    for g, w, what in zip(got, want[:3], ["flags", "bitmap", "results"]):
        assert np.array_equal(g, w), (what, np.nonzero(g != w)[0][:10])
    return want[0]


def _tables_equal(e, o):
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(e.download_table(t), o.tables[t]), f"table {t}"


@pytest.mark.parametrize("W,mode", [(1, "plain"), (2, "fused"), (3, "persistent"), (2, "graph")])
def test_by_name_mix_matches_oracle(eng, W, mode):
    eng.load_tpcc(13, W)
    o = oracle.TpccOracle(13, W)
    g = TpccGenerator(13, W, 20000, by_name_pct=60)
    for i in range(3):
        flags = _same(eng, o, g.next(), i % 2, mode)
        assert not (flags & abi.FLAG_NOT_FOUND).any()
    _tables_equal(eng, o)


def test_not_found_payments(eng):
    W, B = 2, 8000
    eng.load_tpcc(17, W)
    o = oracle.TpccOracle(17, W)
    b = TpccGenerator(17, W, B, neworder_pct=40, by_name_pct=100).next()
    txns = b.txns.copy()
    by_name = ((txns["kind_info"] & 0xFF) == abi.TPCC_PAYMENT) & ((txns["kind_info"] & abi.PAY_BY_NAME) != 0)
    idx = np.nonzero(by_name)[0]
    miss = idx[::5]
    txns["c_id"][miss] = (txns["c_id"][miss] & ~np.uint32(0xFF)) | np.uint32(200)
    txns["c_id"][idx[1]] = (777777 << 8) | 0  # no such name
    mb = TpccBatch(txns, b.lines, b.txn_base)
    for slot, mode in enumerate(["plain", "graph"]):
        flags = _same(eng, o, mb, slot, mode)
        assert (flags[miss] == abi.FLAG_NOT_FOUND).all() and flags[idx[1]] == abi.FLAG_NOT_FOUND
    _tables_equal(eng, o)


def test_name_index_follows_uploaded_customers(eng):
    """The index is rebuilt when the customer table is uploaded: with the
    reference's names (C_LAST = row % 20) the old queries resolve differently
    (or not at all), the same way in the engine and the oracle."""
    W = 1
    eng.load_tpcc(19, W)
    o = oracle.TpccOracle(19, W)
    cust = o.tables[abi.T_CUSTOMER].reshape(-1, abi.TPCC_COLS[abi.T_CUSTOMER])
    cust[:, C_LAST_COL] = np.arange(len(cust)) % 20
    eng.upload_table(abi.T_CUSTOMER, o.tables[abi.T_CUSTOMER])
    txns = TpccGenerator(19, W, 6000, neworder_pct=0, by_name_pct=100).next().txns.copy()
    names = (txns["c_id"] >> 8) % 20
    txns["c_id"] = (names << 8) | (txns["c_id"] & 0xFF)
    b = TpccBatch(txns, np.zeros(0, dtype=TpccBatch.LINE_DTYPE))
    cid, found = o.resolve(b)
    assert found.all()  # 150 holders per name, nth < 150
    _same(eng, o, b, 0, "fused")
    _tables_equal(eng, o)


@pytest.mark.parametrize("data", ["generated", "reference"])
def test_reference_lookup_mode_matches_oracle(eng_ref, data):
    W = 2
    eng_ref.load_tpcc(23, W)
    o = oracle.TpccOracle(23, W, ref_name_lookup=True)
    cust = o.tables[abi.T_CUSTOMER].reshape(-1, abi.TPCC_COLS[abi.T_CUSTOMER])
    if data == "reference":
        cust[:, C_LAST_COL] = np.arange(len(cust)) % 20
        eng_ref.upload_table(abi.T_CUSTOMER, o.tables[abi.T_CUSTOMER])
    rng = np.random.default_rng(2)
    g = TpccGenerator(23, W, 12000, neworder_pct=30, by_name_pct=100)
    for i, mode in enumerate(["plain", "persistent", "graph"]):
        b0 = g.next()
        txns = b0.txns.copy()
        by_name = ((txns["kind_info"] & 0xFF) == abi.TPCC_PAYMENT) & ((txns["kind_info"] & abi.PAY_BY_NAME) != 0)
        names = txns["c_id"] >> 8
        if data == "reference":
            names = names % 20
        nth = rng.integers(0, 160, len(txns)).astype(np.uint32)
        txns["c_id"] = np.where(by_name, (names << 8) | nth, txns["c_id"])
        b = TpccBatch(txns, b0.lines, b0.txn_base)
        flags = _same(eng_ref, o, b, i % 2, mode)
        assert not (flags & abi.FLAG_NOT_FOUND).any()  # the reference rule always yields a C_ID
    _tables_equal(eng_ref, o)

