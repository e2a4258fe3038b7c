"""The reference's own CUDA kernels on our batches: the parity pin.

The reference ships no tests and no golden vectors, so its kernels themselves
are the pin.  oracle/ref_build.py compiles LTPG/YCSB/1 and
LTPG/TPCC-allopt-final as shipped (sm_103a cubins plus struct layouts from
their own headers); oracle/reference.py feeds them our batches.  Their
per-transaction conflict flags must equal the oracle's and the engine's.
"""
import numpy as np
import pytest

import oracle
from oracle import reference
from ltpg_gb300 import Engine, TpccBatch, TpccGenerator, YcsbBatch, YcsbGenerator, abi

pytestmark = pytest.mark.gpu
KEY_MASK = (1 << abi.YCSB_KEY_BITS) - 1


@pytest.fixture(scope="module")
def ref(gpu):
    if not reference.available():
        pytest.skip("reference kernels not built: oracle/_ref is made by oracle/ref_build.py where the "
                    "reference sources are")
    return True


def _ycsb_batch(read_keys, write_keys, values):
    B = len(write_keys)
    ops = np.full((B, 12), abi.YCSB_OP_PAD, dtype=np.uint32)
    ops[:, :9] = read_keys
    ops[:, 9] = np.uint32(0x80000000) | write_keys.astype(np.uint32)
    val_off = np.arange(B + 1, dtype=np.uint32)
    return YcsbBatch(ops.ravel(), val_off, values, B, 10)


@pytest.mark.parametrize("theta", [0.0, 0.6, 0.99])
def test_reference_ycsb_flags_match(ref, theta):
    r = reference.RefY1()
    B, n = r.B, r.n
    assert (B, n, r.reads) == (10000, 1000000, 9)
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=10)
    try:
        eng.load_ycsb(5, n)
        o = oracle.YcsbOracle(5, n)
        g = YcsbGenerator(5, n - 1, B, 10, 0, theta)  # keys 0 .. n-2, shifted to 1 .. n-1 below
        for bid in range(2):
            b = g.batch(bid)
            keys = (b.ops.reshape(B, b.op_stride)[:, :10] & KEY_MASK).astype(np.uint32) + 1
            ref_flags, mark = r.run(keys[:, :9], keys[:, 9])
            ours = _ycsb_batch(keys[:, :9], keys[:, 9], np.arange(B, dtype=np.uint64) + 7)
            want = o.run(ours)[0]
            # the reference's grids reach every op of the first 9,984 transactions
            # only (covered_txns); the last 16 lose their write registration and
            # checks.  Missing registrations of larger TIDs cannot change the
            # flags of smaller ones, so the covered prefix is exact.
            c = r.covered
            assert c == 9984
            assert np.array_equal(ref_flags[:c], want[:c]), np.nonzero(ref_flags[:c] != want[:c])[0][:10]
            assert np.array_equal(mark[:c].astype(bool), (want[:c] & abi.FLAG_COMMIT) != 0)
            for mode in ["plain", "graph"]:
                eng.upload(0, ours)
                eng.run_batch(0, mode)
                eng.sync()
            # the engine ran the batch twice (plain, graph) on an evolving image;
            # flags depend only on the keys, not on the values
            assert np.array_equal(eng.txn_flags(0, B), want)
            assert 0 < int((want & abi.FLAG_COMMIT != 0).sum()) <= B
    finally:
        eng.close()


def test_reference_payment_flags_match(ref):
    r = reference.RefTF()
    B, W = r.B, r.W
    assert (B, W) == (65536, 64)
    g = TpccGenerator(9, W, B, neworder_pct=0)
    o = oracle.TpccOracle(9, W)
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=16, max_lines=16)
    try:
        eng.load_tpcc(9, W)
        for _ in range(2):
            b = g.next()
            ref_flags = r.run(b.txns)
            want = o.run(b)[0]
            assert r.covered == B  # TF's grids reach every Payment op
            assert np.array_equal(ref_flags, want), np.nonzero(ref_flags != want)[0][:10]
            eng.upload(0, b)
            eng.run_batch(0, "graph")
            eng.sync()
            assert np.array_equal(eng.txn_flags(0, B), want)
            assert (want & abi.FLAG_WAW).any() and (want & abi.FLAG_COMMIT).any()
    finally:
        eng.close()


def _mixed_batch(g, nc, pc):
    """The first nc NewOrders and pc Payments of the generator's next batch, in
    their order (TID = position), order lines repacked."""
    from ltpg_gb300 import TpccBatch
    b = g.next()
    kind = b.txns["kind_info"] & 0xFF
    no, pay = kind == abi.TPCC_NEWORDER, kind == abi.TPCC_PAYMENT
    sel = (no & (np.cumsum(no) <= nc)) | (pay & (np.cumsum(pay) <= pc))
    assert no[sel].sum() == nc and pay[sel].sum() == pc
    x = b.txns[sel].copy()
    cnt = np.where((x["kind_info"] & 0xFF) == abi.TPCC_NEWORDER, (x["kind_info"] >> 8) & 0xFF, 0).astype(np.int64)
    new_off = np.cumsum(cnt) - cnt
    total = int(cnt.sum())
    src = np.repeat(x["line_off"].astype(np.int64), cnt) + (np.arange(total) - np.repeat(new_off, cnt))
    lines = b.lines[src]
    x["line_off"] = new_off.astype(np.uint32)
    return TpccBatch(x, lines)


def test_reference_neworder_flags_match(ref):
    """NewOrders and Payments together, pinned by the reference's own TF
    kernels compiled with NEWORDER_PERCENT = 50: per-transaction RAW / WAR /
    WAW and commit equal the oracle's (default insert mode, which follows the
    reference's NEW-ORDER registration) and the engine's."""
    if not reference.available("tf50"):
        pytest.skip("tf50 not built (oracle/ref_build.py where the reference sources are)")
    r = reference.RefTF("tf50")
    nc, pc, W = r.L["neworder_cnt"], r.L["payment_cnt"], r.W
    assert (nc, pc, W) == (32768, 32768, 64)
    g = TpccGenerator(13, W, 70000, neworder_pct=50)  # about 35,000 of each kind per batch
    o = oracle.TpccOracle(13, W)
    eng = Engine(device=0, n_slots=1, max_txn=nc + pc, max_ops_per_txn=16, max_lines=15 * nc)
    try:
        eng.load_tpcc(13, W)
        for _ in range(2):
            b = _mixed_batch(g, nc, pc)
            assert b.txns["c"].max() + 15 < 450000  # ORDER-LINE keys stay inside each warehouse's range
            ref_flags = r.run(b.txns, b.lines)
            want = o.run(b)[0]
            assert r.covered >= max(nc, pc)
            bad = np.nonzero(ref_flags != want)[0]
            assert len(bad) == 0, (bad[:10], ref_flags[bad[:5]], want[bad[:5]], b.txns["kind_info"][bad[:5]] & 0xFF)
            eng.upload(0, b)
            eng.run_batch(0, "graph")
            eng.sync()
            assert np.array_equal(eng.txn_flags(0, b.n_txn), want)
            no = (b.txns["kind_info"] & 0xFF) == abi.TPCC_NEWORDER
            assert (want[no] & abi.FLAG_COMMIT).any() and (want[no] & abi.FLAG_WAW).any()
    finally:
        eng.close()


@pytest.mark.parametrize("data", ["generated", "reference"])
def test_reference_name_lookup_matches(ref, data):
    """The reference's KERNEL_CID (TF/tp.cu:11-23) on our Payments by last name
    (nth = 0, where its warp stays converged) writes the C_IDs that the
    oracle's LTPG_CFG_REF_NAME_LOOKUP rule computes, and the engine in that
    mode gives the oracle's flags — on the generated names and on the
    reference's own (C_LAST = row % 20, TF/Database.h:180)."""
    r = reference.RefTF()
    B, W = r.B, r.W
    o = oracle.TpccOracle(9, W, ref_name_lookup=True)
    cust = o.tables[abi.T_CUSTOMER].reshape(-1, abi.TPCC_COLS[abi.T_CUSTOMER])
    if data == "reference":
        cust[:, 13] = np.arange(len(cust)) % 20
    b = TpccGenerator(9, W, B, neworder_pct=0, by_name_pct=60).next()
    txns = b.txns.copy()
    by_name = ((txns["kind_info"] & 0xFF) == abi.TPCC_PAYMENT) & ((txns["kind_info"] & abi.PAY_BY_NAME) != 0)
    names = txns["c_id"] >> 8
    if data == "reference":
        names = names % 20
    txns["c_id"] = np.where(by_name, names << 8, txns["c_id"])  # nth = 0
    mb = TpccBatch(txns, b.lines, b.txn_base)
    ref_cid = r.cid(txns, cust[:, 13], cust[:, 0])
    want, found = o.resolve(mb)
    assert found.all()
    assert np.array_equal(ref_cid[by_name], want[by_name]), np.nonzero(ref_cid[by_name] != want[by_name])[0][:10]
    assert np.array_equal(ref_cid[~by_name], txns["c_id"][~by_name])
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=16, max_lines=16, ref_name_lookup=True)
    try:
        eng.load_tpcc(9, W)
        if data == "reference":
            eng.upload_table(abi.T_CUSTOMER, o.tables[abi.T_CUSTOMER])
        eng.upload(0, mb)
        eng.run_batch(0, "graph")
        eng.sync()
        assert np.array_equal(eng.txn_flags(0, B), o.run(mb)[0])
    finally:
        eng.close()


def _ycsb_write_last_batch(keys):
    """One batch of len(keys) transactions whose last key is an update and the
    others reads (the reference's fixed shape: reads first, then the write)."""
    B, k = keys.shape
    stride = (k + 3) & ~3
    ops = np.full((B, stride), abi.YCSB_OP_PAD, dtype=np.uint32)
    ops[:, :k - 1] = keys[:, :k - 1]
    ops[:, k - 1] = np.uint32(0x80000000) | keys[:, k - 1]
    return YcsbBatch(ops.ravel(), np.arange(B + 1, dtype=np.uint32), np.arange(B, dtype=np.uint64) + 7, B, k)


def test_reference_ycsb_flags_match_at_headline_scale(ref):
    """YCSB/1 compiled at the high-contention scale (1,048,576 transactions x
    (15 reads + 1 write), 10,000,000 records, uniform mode so that every key
    registers): its flags on a theta = 0.99 batch equal the oracle's and the
    engine's for every transaction."""
    if not reference.available("y1_c2"):
        pytest.skip("y1_c2 not built (oracle/ref_build.py where the reference sources are)")
    r = reference.RefY1("y1_c2")
    B, n = r.B, r.n
    assert (B, n, r.reads) == (1 << 20, 10_000_000, 15) and r.covered == B
    g = YcsbGenerator(21, n, B, 16, 0, 0.99, 8)
    keys = (g.batch(0).ops.reshape(B, 16) & KEY_MASK).astype(np.uint32)
    ref_flags, mark = r.run(keys[:, :15], keys[:, 15])
    b = _ycsb_write_last_batch(keys)
    want = oracle.YcsbOracle(21, n).run(b, threads=8)[0]
    assert np.array_equal(ref_flags, want), np.nonzero(ref_flags != want)[0][:10]
    assert np.array_equal(mark.astype(bool), (want & abi.FLAG_COMMIT) != 0)
    assert (want & abi.FLAG_RAW).any() and (want & abi.FLAG_WAW).any()
    eng = Engine(device=0, n_slots=1, max_txn=B, max_ops_per_txn=16)
    try:
        eng.load_ycsb(21, n)
        eng.set_launch("ycsb", late_reads=3)
        eng.upload(0, b)
        eng.run_batch(0, "graph")
        eng.sync()
        assert np.array_equal(eng.txn_flags(0, B), want)
    finally:
        eng.close()


def test_reference_neworder_payment_flags_match_at_headline_scale(ref):
    """TPCC-allopt-final compiled for the TPC-C headline batch (1,048,576
    transactions, 524,288 NewOrders + 524,288 Payments, W = 64): its flags
    equal the oracle's and the engine's for every transaction."""
    if not reference.available("tf_c3"):
        pytest.skip("tf_c3 not built (oracle/ref_build.py where the reference sources are)")
    r = reference.RefTF("tf_c3")
    nc, pc, W = r.L["neworder_cnt"], r.L["payment_cnt"], r.W
    assert (nc, pc, W) == (1 << 19, 1 << 19, 64) and r.covered >= max(nc, pc)
    g = TpccGenerator(23, W, 1_100_000, neworder_pct=50)
    b = _mixed_batch(g, nc, pc)
    # the first batch's order-line ids stay far from each warehouse's end, so
    # the reference's unwrapped ORDER-LINE keys (W * 450000 + OL_ID + i) are in range
    assert b.txns["c"].max() + 15 < 450000
    ref_flags = r.run(b.txns, b.lines)
    want = oracle.TpccOracle(23, W).run(b, threads=8)[0]
    bad = np.nonzero(ref_flags != want)[0]
    assert len(bad) == 0, (bad[:10], ref_flags[bad[:5]], want[bad[:5]])
    eng = Engine(device=0, n_slots=1, max_txn=b.n_txn, max_ops_per_txn=16, max_lines=b.n_lines)
    try:
        eng.load_tpcc(23, W)
        eng.upload(0, b)
        eng.run_batch(0, "graph")
        eng.sync()
        assert np.array_equal(eng.txn_flags(0, b.n_txn), want)
    finally:
        eng.close()
