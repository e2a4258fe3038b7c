"""GPU engine vs the oracle, bit-exact, through the C ABI (libltpg.so)."""
import os

import numpy as np
import pytest

import oracle
from kat import GOLDEN, load, mask_rows, tpcc_apply_expected, tpcc_batch, ycsb_batch, ycsb_expected_digest
from ltpg_gb300 import Engine, LtpgError, TpccBatch, TpccGenerator, YcsbBatch, YcsbGenerator, abi

pytestmark = pytest.mark.gpu
MODES = ["plain", "fused", "persistent", "graph"]
KY = load("kat_ycsb.json")
KT = load("kat_tpcc.json")


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=8, max_txn=1 << 17, max_ops_per_txn=32, max_lines=15 << 17)
    yield e
    e.close()


def run_and_fetch(e, slot, batch, mode):
    e.upload(slot, batch)
    e.run_batch(slot, mode)
    e.sync()
    return (e.txn_flags(slot, batch.n_txn), e.commit_bitmap(slot, batch.n_txn), e.txn_results(slot, batch.n_txn))


def assert_same(got, want):
    gf, gb, gr = got
    wf, wb, wr = want[:3]
    assert np.array_equal(gf, wf), f"flags differ at {np.nonzero(gf != wf)[0][:10]}"
    assert np.array_equal(gb, wb)
    assert np.array_equal(gr, wr), f"results differ at {np.nonzero(gr != wr)[0][:10]}"


# ---- YCSB -----------------------------------------------------------------------
@pytest.mark.parametrize("mode", MODES)
def test_ycsb_known_answers(eng, mode):
    for case in KY["cases"]:
        eng.load_ycsb(KY["seed"], KY["n_records"])
        o = oracle.YcsbOracle(KY["seed"], KY["n_records"])
        rows0 = o.rows.copy()
        got = run_and_fetch(eng, 0, ycsb_batch(case), mode)
        assert got[0].tolist() == case["flags"], case["name"]
        assert np.array_equal(got[2], ycsb_expected_digest(rows0, case))
        o.run(ycsb_batch(case))
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows), case["name"]


@pytest.mark.parametrize("B,k,upd,theta", [(1, 10, 50, 0.6), (31, 10, 50, 0.6), (32, 16, 50, 0.6),
                                           (33, 16, 50, 0.9), (1000, 1, 50, 0.99), (1000, 32, 30, 0.99),
                                           (4099, 7, 50, 0.0), (65536, 10, 50, 0.6)])
@pytest.mark.parametrize("mode", MODES)
def test_ycsb_vs_oracle(eng, B, k, upd, theta, mode):
    n = 50000
    eng.load_ycsb(17, n)
    o = oracle.YcsbOracle(17, n)
    g = YcsbGenerator(17, n, B, k, upd, theta)
    for bid in range(3):  # several batches: epoch tags, image carried over
        b = g.batch(bid)
        got = run_and_fetch(eng, bid % 2, b, mode)
        assert_same(got, o.run(b))
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)


def test_ycsb_golden_fixture(eng):
    z = np.load(os.path.join(GOLDEN, "gen_ycsb.npz"))
    p = z["params"]
    n, B, k = int(p[1]), int(p[2]), int(p[3])
    eng.load_ycsb(int(p[0]), n)
    for bid in range(int(z["n_batches"])):
        b = YcsbBatch(z[f"ops{bid}"], z[f"val_off{bid}"], z[f"vals{bid}"], B, k)
        got = run_and_fetch(eng, 0, b, "plain")
        assert_same(got, (z[f"flags{bid}"], z[f"bitmap{bid}"], z[f"results{bid}"]))
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), z["rows_final"])


def test_ycsb_graph_over_many_slots(eng):
    """One CUDA graph over 6 batches in 6 slots, replayed twice; equals the
    sequential replay of the 12 batches."""
    n = 30000
    eng.load_ycsb(5, n)
    o = oracle.YcsbOracle(5, n)
    g = YcsbGenerator(5, n, 20000, 16, 10, 0.99)
    batches = [g.batch(i) for i in range(6)]
    for rep in range(2):
        for i, b in enumerate(batches):
            eng.upload(i, b)
        eng.run_batches(0, 6, "graph")
        eng.sync()
        for i, b in enumerate(batches):
            want = o.run(b)
            assert np.array_equal(eng.txn_flags(i, b.n_txn), want[0]), (rep, i)
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)


def test_ycsb_out_of_range_key_reports_error(eng):
    eng.load_ycsb(1, 100)
    bad = YcsbBatch.from_ops([[(3, 0, 0)], [(100, 1, 0)]], [[], [7]])
    eng.upload(0, bad)
    eng.run_batch(0, "plain")
    with pytest.raises(LtpgError) as ei:
        eng.sync()
    assert ei.value.code == abi.ERR_BOUNDS
    # the context stays usable and the table was not touched out of range
    o = oracle.YcsbOracle(1, 100)
    ok = YcsbBatch.from_ops([[(3, 1, 2)], [(4, 0, 0)]], [[9], []])
    assert_same(run_and_fetch(eng, 0, ok, "plain"), o.run(ok))


def test_ycsb_host_call_end_to_end(eng):
    n = 20000
    eng.load_ycsb(8, n)
    o = oracle.YcsbOracle(8, n)
    g = YcsbGenerator(8, n, 10000, 10, 50, 0.8)
    for bid, mode in enumerate(MODES):
        b = g.batch(bid)
        bits = eng.run_host(1, b, mode)
        assert np.array_equal(bits, o.run(b)[1])


@pytest.mark.parametrize("mode", ["plain", "fused", "graph"])
def test_pipelined_host_calls(eng, mode):
    """ltpg_submit_*_host / ltpg_host_wait with three batches in flight: every
    bitmap equals the oracle's, for YCSB and TPC-C, and a bad batch's error
    comes back from its wait."""
    from ltpg_gb300 import pinned_copy, pinned_empty
    n, B, depth = 30000, 8000, 3
    eng.load_ycsb(12, n)
    o = oracle.YcsbOracle(12, n)
    g = YcsbGenerator(12, n, B, 16, 5, 0.99, rotate_every=2)
    batches = [pinned_copy(g.batch(i)) for i in range(7)]
    bits = [pinned_empty((B + 31) // 32) for _ in range(depth)]
    want = [o.run(b) for b in batches]
    for i, b in enumerate(batches):
        if i >= depth:
            eng.host_wait(i % depth)
            assert np.array_equal(bits[i % depth], want[i - depth][1]), i - depth
        eng.submit_host(i % depth, b, mode, bits[i % depth])
    for i in range(len(batches) - depth, len(batches)):
        eng.host_wait(i % depth)
        assert np.array_equal(bits[i % depth], want[i][1]), i
        assert np.array_equal(eng.txn_flags(i % depth, B), want[i][0])
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    # an out-of-range key: the error is reported by the wait
    bad = g.batch(9)
    ops = bad.ops.copy()
    ops[0] = (ops[0] & ~np.uint32((1 << abi.YCSB_KEY_BITS) - 1)) | np.uint32(n + 5)
    badb = pinned_copy(YcsbBatch(ops, bad.val_off, bad.vals, bad.n_txn, bad.ops_per_txn))
    eng.submit_host(0, badb, mode, bits[0])
    with pytest.raises(LtpgError) as ei:
        eng.host_wait(0)
    assert ei.value.code == abi.ERR_BOUNDS
    eng.load_ycsb(12, n)  # the failed batch may have left partial state

    W = 2
    eng.load_tpcc(14, W)
    to = oracle.TpccOracle(14, W)
    tg = TpccGenerator(14, W, B, by_name_pct=60)
    tb = [pinned_copy(tg.next()) for _ in range(5)]
    twant = [to.run(b) for b in tb]
    for i, b in enumerate(tb):
        if i >= depth:
            eng.host_wait(i % depth)
            assert np.array_equal(bits[i % depth], twant[i - depth][1]), i - depth
        eng.submit_host(i % depth, b, mode, bits[i % depth])
    for i in range(len(tb) - depth, len(tb)):
        eng.host_wait(i % depth)
        assert np.array_equal(bits[i % depth], twant[i][1]), i
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), to.tables[t]), t


# ---- TPC-C --------------------------------------------------------------------------
@pytest.fixture(scope="module")
def eng_strict(gpu):
    e = Engine(device=0, n_slots=2, max_txn=1 << 15, max_ops_per_txn=16, max_lines=15 << 15, strict_insert=True)
    yield e
    e.close()


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("mode", MODES)
def test_tpcc_known_answers(eng, eng_strict, strict, mode):
    e = eng_strict if strict else eng
    for case in KT["cases"]:
        e.load_tpcc(KT["seed"], KT["warehouses"])
        init = [e.download_table(t) for t in range(abi.TPCC_TABLES)]
        flags = run_and_fetch(e, 0, tpcc_batch(case), mode)[0]
        assert flags.tolist() == (case["strict_flags"] if strict else case["flags"]), case["name"]
        want = tpcc_apply_expected(init, case, flags)
        skip = case.get("unspecified_rows", [])
        got = mask_rows([e.download_table(t) for t in range(abi.TPCC_TABLES)], skip)
        want = mask_rows(want, skip)
        for t in range(abi.TPCC_TABLES):
            assert np.array_equal(got[t], want[t]), (case["name"], t)


@pytest.mark.parametrize("W,B,no_pct", [(1, 1, 50), (1, 33, 50), (1, 4096, 50), (2, 20000, 50), (3, 9000, 100),
                                        (2, 7000, 0)])
@pytest.mark.parametrize("mode", MODES)
def test_tpcc_vs_oracle(eng, W, B, no_pct, mode):
    eng.load_tpcc(23, W)
    o = oracle.TpccOracle(23, W)
    g = TpccGenerator(23, W, B, neworder_pct=no_pct)
    for bid in range(3):
        b = g.next()
        got = run_and_fetch(eng, bid % 2, b, mode)
        assert_same(got, o.run(b))
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), t


def test_tpcc_golden_fixture(eng):
    z = np.load(os.path.join(GOLDEN, "gen_tpcc.npz"))
    p = z["params"]
    eng.load_tpcc(int(p[0]), int(p[1]))
    for bid in range(int(z["n_batches"])):
        b = TpccBatch(z[f"txns{bid}"].view(TpccBatch.TXN_DTYPE), z[f"lines{bid}"].view(TpccBatch.LINE_DTYPE),
                      int(z[f"txn_base{bid}"]))
        got = run_and_fetch(eng, 0, b, "plain")
        assert_same(got, (z[f"flags{bid}"], z[f"bitmap{bid}"], z[f"results{bid}"]))
    for t in range(abi.TPCC_TABLES):
        assert int(np.bitwise_xor.reduce(eng.download_table(t))) == int(z["xor"][t])


def test_tpcc_invalid_record_reports_error(eng):
    eng.load_tpcc(1, 1)
    case = {"txns": [{"kind": "PAY", "w": 0, "d": 0, "c_w": 0, "c_d": 0, "c_id": 0, "a": 0, "amount": 5},
                     {"kind": "PAY", "w": 3, "d": 0, "c_w": 0, "c_d": 0, "c_id": 0, "a": 0, "amount": 5}]}
    eng.upload(0, tpcc_batch(case))
    eng.run_batch(0, "plain")
    with pytest.raises(LtpgError) as ei:
        eng.sync()
    assert ei.value.code == abi.ERR_BOUNDS


# ---- tuning never changes outcomes ------------------------------------------------------
@pytest.mark.parametrize("opt,filt,dd,bps", [(1, 0, 0, 0), (1, 1, 1, 2), (2, 0, 1, 1), (4, 1, 0, 0), (8, 1, 1, 0),
                                             (4, 0, 0, 3)])
@pytest.mark.parametrize("k", [3, 4, 7, 10, 16, 20, 32])
def test_launch_shapes_do_not_change_outcomes(eng, opt, filt, dd, bps, k):
    """Every launch shape gives the oracle's results; strides that are not a
    power of two (k = 10 -> 12, 20) run the one-op-per-lane kernel with padded
    lanes."""
    n = 40000
    eng.load_ycsb(31, n)
    o = oracle.YcsbOracle(31, n)
    g = YcsbGenerator(31, n, 9000, k, 10, 0.99)
    saved = eng.get_launch("ycsb")
    try:
        eng.set_launch("ycsb", ops_per_thread=opt, filter=filt, dedupe=dd, blocks_per_sm=bps)
        for bid, mode in enumerate(["fused", "persistent", "graph"]):
            b = g.batch(bid)
            assert_same(run_and_fetch(eng, bid % 2, b, mode), o.run(b))
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        eng.set_launch("ycsb", **saved)


@pytest.mark.parametrize("ways,k,opt", [(1, 16, None), (2, 16, None), (4, 16, None), (4, 10, 1), (2, 20, 1)])
def test_staging_does_not_change_outcomes(eng, ways, k, opt):
    """Stage the hottest buckets (and, in a second round, every bucket, so that
    most keys collide and fall back to the global path): results stay bit-exact
    and the staged registrations are counted."""
    from ltpg_gb300 import key_bucket
    n = 100000
    eng.load_ycsb(41, n)
    o = oracle.YcsbOracle(41, n)
    g = YcsbGenerator(41, n, 30000, k, 5, 0.99, rotate_every=2)
    saved = eng.get_launch("ycsb")
    try:
        eng.set_launch("ycsb", stage_ways=ways, **({} if opt is None else {"ops_per_thread": opt}))
        for bid in range(6):
            b = g.batch(bid)
            keys = (b.ops.reshape(b.n_txn, -1)[:, :k] & ((1 << 27) - 1)).ravel()
            cnt = np.bincount(key_bucket(keys), minlength=abi.STAGE_BUCKETS)
            staged = np.argsort(-cnt, kind="stable")[:abi.STAGE_ENTRIES // ways] if bid < 3 else \
                np.arange(abi.STAGE_BUCKETS)
            eng.stage_set(staged)
            mode = ["fused", "persistent", "graph"][bid % 3]
            assert_same(run_and_fetch(eng, bid % 2, b, mode), o.run(b))
            st = eng.stats(bid % 2)
            assert st["staged_ops"] > 0
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
        counts = eng.bucket_counts(reset=True)
        assert counts.sum() > 0
    finally:
        eng.stage_set([])
        eng.set_launch("ycsb", **saved)


def test_graph_replay_after_reupload(eng):
    """A graph captured for a slot stays correct when a different batch (other
    line count, other transaction numbers) is uploaded into that slot."""
    eng.load_tpcc(61, 2)
    o = oracle.TpccOracle(61, 2)
    g = TpccGenerator(61, 2, 6000)
    batches = [g.next() for _ in range(4)]
    for b in batches[:2]:                # both slots in use before any capture
        eng.upload(batches.index(b), b)
    for i, b in enumerate(batches):
        eng.upload(i % 2, b)
        eng.run_batch(i % 2, "graph")
        eng.sync()
        assert_same((eng.txn_flags(i % 2, b.n_txn), eng.commit_bitmap(i % 2, b.n_txn),
                     eng.txn_results(i % 2, b.n_txn)), o.run(b))
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(eng.download_table(t), o.tables[t]), t
    n = 20000
    eng.load_ycsb(62, n)
    yo = oracle.YcsbOracle(62, n)
    yg = YcsbGenerator(62, n, 5000, 16, 20, 0.9)
    yb = [yg.batch(i) for i in range(4)]
    eng.upload(0, yb[0])
    eng.upload(1, yb[1])
    for i, b in enumerate(yb):
        eng.upload(i % 2, b)
        eng.run_batch(i % 2, "graph")
        eng.sync()
        assert np.array_equal(eng.txn_flags(i % 2, b.n_txn), yo.run(b)[0])
    assert np.array_equal(eng.download_table(abi.TABLE_YCSB), yo.rows)
