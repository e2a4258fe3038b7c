"""The autotuner end to end on a GPU: it searches block size with the other
launch settings, every winner reproduces the plain path's commit bitmap, and
the result lands in the caller's cache file (not the package)."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, TpccGenerator, YcsbGenerator, abi, tune

pytestmark = pytest.mark.gpu


def _check_cached(tmp_path, key, best):
    path = str(tmp_path / "tuned.json")
    tune.save_cached(key, best, path)
    assert tune.load_cached(key, path) == best
    assert tune.load_cached(key + "|absent", path) is None


def test_autotune_ycsb_small(gpu, tmp_path):
    n, B, k = 200_000, 16384, 10
    g = YcsbGenerator(31, n, B, k, 50, 0.6)
    batches = [g.batch(i) for i in range(5)]
    eng = Engine(device=0, n_slots=4, max_txn=B, max_ops_per_txn=k)
    try:
        eng.load_ycsb(31, n)
        for i in range(4):
            eng.upload(i, batches[i])
        best, table = tune.autotune(eng, "ycsb", [0, 1, 2, 3], lambda: eng.load_ycsb(31, n), mode="graph")
        ok = [c for c, ms, st in table if st == "ok"]
        assert {c["block_threads"] for c in ok} == set(tune.BLOCKS)
        assert {c["late_reads"] for c in ok} == {0, 1, 2, 3}
        assert len(ok) == len(table), [t for t in table if t[2] != "ok"][:3]
        assert best["block_threads"] in tune.BLOCKS and best["ms_per_batch"] > 0
        # the winner on a batch it was not tuned on, against the oracle
        eng.load_ycsb(31, n)
        o = oracle.YcsbOracle(31, n)
        b = batches[4]
        eng.upload(0, b)
        eng.run_batch(0, "graph")
        eng.sync()
        wf, wb, wr, _ = o.run(b)
        assert np.array_equal(eng.txn_flags(0, B), wf)
        assert np.array_equal(eng.commit_bitmap(0, B), wb)
        com = (wf & abi.FLAG_COMMIT) != 0
        assert np.array_equal(eng.txn_results(0, B)[com], wr[com])
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        eng.close()
    _check_cached(tmp_path, "test_ycsb_small", best)


def test_autotune_tpcc(gpu, tmp_path):
    W, B = 4, 16384
    g = TpccGenerator(33, W, B)
    batches = [g.next() for _ in range(5)]
    eng = Engine(device=0, n_slots=4, max_txn=B, max_ops_per_txn=16, max_lines=max(b.n_lines for b in batches))
    try:
        eng.load_tpcc(33, W)
        for i in range(4):
            eng.upload(i, batches[i])
        best, table = tune.autotune(eng, "tpcc", [0, 1, 2, 3], lambda: eng.load_tpcc(33, W), mode="graph")
        ok = [c for c, ms, st in table if st == "ok"]
        assert len(ok) == len(table) and {c["block_threads"] for c in ok} == set(tune.BLOCKS)
        # every block size, one batch after another on the same image, against the oracle
        eng.load_tpcc(33, W)
        o = oracle.TpccOracle(33, W)
        for b, bs in zip(batches, [128, 256, 512, best["block_threads"], 512]):
            eng.set_launch("tpcc", **{k: v for k, v in dict(best, block_threads=bs).items()
                                      if k in dict(abi.LaunchC._fields_)})
            eng.upload(0, b)
            eng.run_batch(0, "graph")
            eng.sync()
            wf, wb, wr, _ = o.run(b)
            assert np.array_equal(eng.txn_flags(0, B), wf), bs
            assert np.array_equal(eng.txn_results(0, B), wr), bs
        for t in range(abi.TPCC_TABLES):
            assert np.array_equal(eng.download_table(t), o.tables[t]), t
    finally:
        eng.close()
    _check_cached(tmp_path, "test_tpcc", best)
