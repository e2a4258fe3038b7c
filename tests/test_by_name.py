"""Payment by customer last name (the reference's KERNEL_CID path,
TF/tp.cu:11-23, TF/Execute_payment.h:13-36, TF/Genericfunction.h:29-77): the
generator, the oracle's two lookup rules, known answers.  CPU only."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import TpccBatch, TpccGenerator, abi

C_ID_COL, C_LAST_COL = 0, 13


def _customers(o):
    return o.tables[abi.T_CUSTOMER].reshape(-1, abi.TPCC_COLS[abi.T_CUSTOMER])


def _by_name(txns):
    return ((txns["kind_info"] & 0xFF) == abi.TPCC_PAYMENT) & ((txns["kind_info"] & abi.PAY_BY_NAME) != 0)


def test_generator_by_name_names_the_by_id_customer():
    """Same seed, by_name_pct 100 vs 0: every Payment of the first names the
    customer that the second picks by id (the name draw comes last)."""
    W, B = 3, 6000
    g1 = TpccGenerator(21, W, B, neworder_pct=30, by_name_pct=100)
    g0 = TpccGenerator(21, W, B, neworder_pct=30, by_name_pct=0)
    o = oracle.TpccOracle(21, W)
    for _ in range(2):
        b1, b0 = g1.next(), g0.next()
        bn = _by_name(b1.txns)
        pay = (b1.txns["kind_info"] & 0xFF) == abi.TPCC_PAYMENT
        assert bn.sum() == pay.sum() > 0
        for f in ["w", "c_w", "a", "b", "c", "line_off"]:
            assert np.array_equal(b1.txns[f], b0.txns[f])
        ki = b1.txns["kind_info"].copy()
        ki[bn] &= ~np.uint32(abi.PAY_BY_NAME)
        assert np.array_equal(ki, b0.txns["kind_info"])
        assert np.array_equal(b1.lines, b0.lines)
        cid, found = o.resolve(b1)
        assert found.all()
        assert np.array_equal(cid, b0.txns["c_id"])
        # the query word is (name << 8) | nth with name = the customer's C_LAST
        cust = _customers(o)
        x = b1.txns[bn]
        rows = 30000 * x["c_w"].astype(np.int64) + 3000 * (x["kind_info"] >> 24).astype(np.int64) + cid[bn]
        assert np.array_equal(x["c_id"] >> 8, cust[rows, C_LAST_COL])


def test_by_name_batches_replay_like_by_id():
    W, B = 2, 5000
    g1 = TpccGenerator(5, W, B, by_name_pct=60)
    g0 = TpccGenerator(5, W, B, by_name_pct=0)
    o1, o0 = oracle.TpccOracle(5, W), oracle.TpccOracle(5, W)
    for _ in range(3):
        b1, b0 = g1.next(), g0.next()
        assert 0.2 < _by_name(b1.txns).mean() < 0.4  # 50 % Payment x 60 %
        r1, r0 = o1.run(b1), o0.run(b0)
        for a, b in zip(r1[:3], r0[:3]):
            assert np.array_equal(a, b)
    for t1, t0 in zip(o1.tables, o0.tables):
        assert np.array_equal(t1, t0)


def test_not_found_payment_neither_registers_nor_commits():
    W, B = 1, 3000
    o = oracle.TpccOracle(8, W)
    b = TpccGenerator(8, W, B, neworder_pct=0, by_name_pct=100).next()
    txns = b.txns.copy()
    miss = np.arange(0, B, 7)
    txns["c_id"][miss] = (txns["c_id"][miss] & ~np.uint32(0xFF)) | np.uint32(250)  # no name has 251 holders
    # a name no customer has (C_LAST < 1000 in the generated image)
    txns["c_id"][5] = (5000 << 8) | 0
    miss = np.union1d(miss, [5])
    mb = TpccBatch(txns, b.lines, b.txn_base)
    cid, found = o.resolve(mb)
    assert not found[miss].any() and found.sum() == B - len(miss)
    hist0 = o.tables[abi.T_HISTORY].copy()
    flags, bitmap, results, commits = o.run(mb)
    assert (flags[miss] == abi.FLAG_NOT_FOUND).all()
    assert (results[miss] == 0).all()
    keep = np.setdiff1d(np.arange(B), miss)
    assert not (flags[keep] & abi.FLAG_NOT_FOUND).any()
    assert commits == int(((flags & abi.FLAG_COMMIT) != 0).sum()) > 0
    # a not-found Payment writes no HISTORY row
    hist = o.tables[abi.T_HISTORY].reshape(-1, abi.TPCC_COLS[abi.T_HISTORY])
    h0 = hist0.reshape(hist.shape)
    rows = txns["a"][miss].astype(np.int64)  # W = 1: HISTORY row = H_ID
    assert np.array_equal(hist[rows], h0[rows])


def _ref_warp_lookup(index, dist, c_last):
    """A literal emulation of __FIND_CID_INDEX's warp (TF/Genericfunction.h:29-77):
    32 lanes in lockstep; __shfl_sync(.., tmp, i) reads lane i % 32's tmp.  A
    lane leaves the loop when its own sum reaches c_last_id; a lane that has
    left contributes nothing to later shuffles (they read the caller's own
    lane only, so this never matters).  Returns lane 0's C_ID row, or None."""
    name, nth = c_last >> 8, c_last & 0xFF
    active = [True] * 32
    cum, flag = [0] * 32, [0] * 32
    it = 0
    while any(active):
        tmp = [0] * 32
        for lane in range(32):
            i = lane + 32 * it
            if active[lane] and i >= 3000:
                active[lane] = False
            if active[lane]:
                tmp[lane] = int(index(dist + i) == name)
        for lane in range(32):
            if not active[lane]:
                continue
            i = lane + 32 * it
            cnt = sum(tmp[i % 32] for _ in range(32))
            cum[lane] += cnt
            flag[lane] += 32
            if cum[lane] >= nth:
                active[lane] = False
        it += 1
    c = cum[0]
    if c < nth:
        return None
    for i in range(flag[0] - 1, 0, -1):
        if index(dist + i) == name:
            if c == nth:
                return dist + i
            c -= 1
    return 0


@pytest.mark.parametrize("data", ["reference", "generated"])
def test_reference_lookup_restatement(data):
    """LTPG_CFG_REF_NAME_LOOKUP in the oracle vs the literal warp emulation, on
    the reference's own customer data (C_LAST = row % 20, TF/Database.h:180) and
    on the generated image; nth = 0 on the reference data has known answers."""
    W = 2
    o = oracle.TpccOracle(3, W, ref_name_lookup=True)
    cust = _customers(o)
    if data == "reference":
        cust[:, C_LAST_COL] = np.arange(len(cust)) % 20
    rng = np.random.default_rng(4)
    n = 400
    txns = np.zeros(n, dtype=TpccBatch.TXN_DTYPE)
    c_w = rng.integers(0, W, n)
    c_d = rng.integers(0, 10, n)
    if data == "reference":
        names = rng.integers(0, 20, n)
        nth = rng.integers(0, 150, n)
        names[:20], nth[:20], c_w[:20], c_d[:20] = np.arange(20), 0, 0, 0
    else:
        rows = 30000 * c_w + 3000 * c_d + rng.integers(0, 3000, n)
        names = cust[rows, C_LAST_COL].astype(np.int64)
        nth = rng.integers(0, 8, n)
    c_w[-1], c_d[-1] = W - 1, 9  # the last district: the walk may pass the table's end
    txns["kind_info"] = abi.TPCC_PAYMENT | abi.PAY_BY_NAME | (c_d.astype(np.uint32) << 24)
    txns["c_w"] = c_w
    txns["c_id"] = (names.astype(np.uint32) << 8) | nth.astype(np.uint32)
    b = TpccBatch(txns, np.zeros(0, dtype=TpccBatch.LINE_DTYPE))
    cid, found = o.resolve(b)
    assert found.all()
    rows_total = len(cust)

    def index(r):
        return int(cust[r, C_LAST_COL]) if r < rows_total else -1

    for t in range(n):
        row = _ref_warp_lookup(index, 30000 * int(c_w[t]) + 3000 * int(c_d[t]), int(txns["c_id"][t]))
        want = 0 if row is None else int(cust[row, C_ID_COL])
        assert cid[t] == want, (t, int(names[t]), int(nth[t]))
    if data == "reference":
        # nth = 0: the walk covers positions 31 .. 1, so names 1..11 land on
        # their second holder (20 + name), name 0 on nothing (position 0 is
        # skipped, position 20 is passed with the sum still at 32 > 0)
        assert list(cid[:20]) == [0] + list(range(21, 32)) + list(range(12, 20))
