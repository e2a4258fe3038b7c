"""The oracle (CPU replay) against the hand-derived known answers and the committed golden batches."""
import os

import numpy as np
import pytest

import oracle
from kat import (GOLDEN, load, mask_rows, tpcc_apply_expected, tpcc_batch, ycsb_batch, ycsb_expected_digest,
                 ycsb_expected_image)
from ltpg_gb300 import TpccGenerator, YcsbBatch, YcsbGenerator, abi

KY = load("kat_ycsb.json")
KT = load("kat_tpcc.json")


@pytest.mark.parametrize("case", KY["cases"], ids=[c["name"] for c in KY["cases"]])
def test_ycsb_known_answers(built_lib, case):
    o = oracle.YcsbOracle(KY["seed"], KY["n_records"])
    rows0 = o.rows.copy()
    flags, bitmap, results, commits = o.run(ycsb_batch(case))
    assert flags.tolist() == case["flags"]
    assert commits == sum(f & 8 != 0 for f in case["flags"])
    assert np.array_equal(bitmap, oracle.pack_bits(np.array(case["flags"]) & 8 != 0))
    assert np.array_equal(o.rows, ycsb_expected_image(KY["n_records"], KY["seed"], case))
    assert np.array_equal(results, ycsb_expected_digest(rows0, case))


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("case", KT["cases"], ids=[c["name"] for c in KT["cases"]])
def test_tpcc_known_answers(built_lib, case, strict):
    o = oracle.TpccOracle(KT["seed"], KT["warehouses"], strict=strict)
    init = [a.copy() for a in o.tables]
    flags, _, _, _ = o.run(tpcc_batch(case))
    expect = case["strict_flags"] if strict else case["flags"]
    assert flags.tolist() == expect
    want = tpcc_apply_expected(init, case, flags)
    skip = case.get("unspecified_rows", [])
    got, want = mask_rows(o.tables, skip), mask_rows(want, skip)
    for t in range(abi.TPCC_TABLES):
        assert np.array_equal(got[t], want[t]), f"table {t}"


def test_tpcc_results_known_answer(built_lib):
    """NewOrder total and Payment balance of one hand-checked pair."""
    o = oracle.TpccOracle(KT["seed"], KT["warehouses"])
    case = KT["cases"][1]  # neworder_then_payment_same_customer
    T = o.tables
    no = case["txns"][0]
    price = {i: int(T[abi.T_ITEM][i * 5 + 2]) for i, _, _ in no["lines"]}
    total = sum(q * price[i] for i, _, q in no["lines"])
    disc = int(T[abi.T_CUSTOMER][(0 * 30000 + 1 * 3000 + 5) * 21 + 4])
    wtax = int(T[abi.T_WAREHOUSE][0 * 9 + 1])
    dtax = int(T[abi.T_DISTRICT][(0 * 10 + 1) * 11 + 2])
    bal = int(np.int64(T[abi.T_CUSTOMER][(0 * 30000 + 1 * 3000 + 5) * 21 + 5].view(np.int64)))
    _, _, results, _ = o.run(tpcc_batch(case))
    assert results[0] == total * (10000 - disc) * (10000 + wtax + dtax) // 10 ** 8
    assert results[1] == bal - 500


def test_multithreaded_replay_matches(built_lib):
    g = YcsbGenerator(21, 20000, 30000, 16, 20, 0.9)
    for bid in range(3):
        b = g.batch(bid)
        o1, o2 = oracle.YcsbOracle(21, 20000), oracle.YcsbOracle(21, 20000)
        r1, r2 = o1.run(b), o2.run(b, threads=6)
        for x, y in zip(r1, r2):
            assert np.array_equal(np.asarray(x), np.asarray(y))
        assert np.array_equal(o1.rows, o2.rows)


def test_out_of_range_key_rejected(built_lib):
    o = oracle.YcsbOracle(1, 10)
    b = YcsbBatch.from_ops([[(3, 0, 0)], [(10, 1, 0)]], [[], [5]])
    with pytest.raises(ValueError):
        o.run(b)


def test_invalid_tpcc_record_rejected(built_lib):
    o = oracle.TpccOracle(1, 1)
    case = {"txns": [{"kind": "PAY", "w": 1, "d": 0, "c_w": 0, "c_d": 0, "c_id": 0, "a": 0, "amount": 5}]}
    with pytest.raises(ValueError):
        o.run(tpcc_batch(case))


def _golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip(f"{name} missing: run tests/golden/make_golden.py")
    return np.load(path)


def test_golden_ycsb_generator_and_replay(built_lib):
    """Regenerates the committed YCSB batches and replays them: the generator's
    bytes and the oracle's outputs must not drift."""
    z = _golden("gen_ycsb.npz")
    p = z["params"]
    g = YcsbGenerator(int(p[0]), int(p[1]), int(p[2]), int(p[3]), int(p[4]), float(z["theta"]), int(p[5]))
    o = oracle.YcsbOracle(int(p[0]), int(p[1]))
    for bid in range(int(z["n_batches"])):
        b = g.batch(bid)
        assert np.array_equal(b.ops, z[f"ops{bid}"]) and np.array_equal(b.vals, z[f"vals{bid}"])
        flags, bitmap, results, _ = o.run(b)
        assert np.array_equal(flags, z[f"flags{bid}"]) and np.array_equal(results, z[f"results{bid}"])
    assert oracle.lib().oracle_splitmix64(0) == int(z["sm0"])
    assert np.array_equal(o.rows[:4096], z["rows_head"])
    assert int(np.bitwise_xor.reduce(o.rows)) == int(z["rows_xor"])


def test_golden_tpcc_generator_and_replay(built_lib):
    z = _golden("gen_tpcc.npz")
    p = z["params"]
    g = TpccGenerator(int(p[0]), int(p[1]), int(p[2]))
    o = oracle.TpccOracle(int(p[0]), int(p[1]))
    for bid in range(int(z["n_batches"])):
        b = g.next()
        assert np.array_equal(b.txns.view(np.uint32), z[f"txns{bid}"])
        assert np.array_equal(b.lines.view(np.uint32), z[f"lines{bid}"])
        flags, _, results, _ = o.run(b)
        assert np.array_equal(flags, z[f"flags{bid}"]) and np.array_equal(results, z[f"results{bid}"])
    for t in range(abi.TPCC_TABLES):
        assert int(np.bitwise_xor.reduce(o.tables[t])) == int(z["xor"][t])


def test_ycsb_range_scans_known_answers():
    """Range-scan reads (span in a read's field bits; every read of the
    reference's YCSB/2 scans 10 keys, Y2/Execute.h:24-32): every covered key
    is registered and checked, keys past the table's end are left out, and the
    result xors every covered row."""
    n = 20
    o = oracle.YcsbOracle(6, n)
    rows0 = o.rows.reshape(n, 10).copy()
    upd = lambda key, field: np.uint32(0x80000000 | (field << 27) | key)
    scan = lambda key, span: np.uint32((span << 27) | key)
    pad = np.uint32(0xFFFFFFFF)
    ops = np.array([[upd(5, 2), pad, pad, pad],          # t0: writes key 5
                    [scan(3, 3), pad, pad, pad],         # t1: reads keys 3..6 -> RAW (key 5), commits
                    [upd(4, 0), pad, pad, pad],          # t2: writes key 4, read by t1 -> WAR, commits
                    [scan(18, 5), upd(9, 1), pad, pad],  # t3: reads 18..19 (clamped), writes 9
                    [scan(8, 1), pad, pad, pad]],        # t4: reads 8..9 -> RAW (key 9 by t3)
                   dtype=np.uint32)
    val_off = np.array([0, 1, 1, 2, 3, 3], dtype=np.uint32)
    vals = np.array([111, 222, 333], dtype=np.uint64)
    b = YcsbBatch(ops.ravel(), val_off, vals, 5, 1)
    b.ops_per_txn, b.op_stride = 2, 4
    flags, bitmap, results, commits = o.run(b)
    assert flags[0] == abi.FLAG_COMMIT
    assert flags[1] == abi.FLAG_RAW | abi.FLAG_COMMIT
    assert flags[2] == abi.FLAG_WAR | abi.FLAG_COMMIT
    assert flags[3] == abi.FLAG_COMMIT
    assert flags[4] == abi.FLAG_RAW | abi.FLAG_COMMIT
    x = lambda keys: int(np.bitwise_xor.reduce(rows0[keys].ravel()))
    u64 = lambda v: int(v) & (2**64 - 1)  # results are int64 (mod 2^64)
    assert u64(results[1]) == x([3, 4, 5, 6])
    assert u64(results[3]) == x([18, 19])
    assert u64(results[4]) == x([8, 9])
    rows = o.rows.reshape(n, 10)
    assert rows[5, 2] == 111 and rows[4, 0] == 222 and rows[9, 1] == 333


def test_ycsb_generator_scans():
    g = YcsbGenerator(3, 5000, 2000, 8, 20, 0.6, scan_len=10)
    b = g.batch(0)
    w = b.ops.reshape(b.n_txn, b.op_stride)[:, :8]
    reads = (w >> 31) == 0
    assert ((w[reads] >> 27) & 0xF == 9).all()  # span 9: 10 keys
    assert g.batch(0).ops.tobytes() == b.ops.tobytes()
    flags = oracle.YcsbOracle(3, 5000).run(b)[0]
    assert ((flags & abi.FLAG_COMMIT) != 0).any()
