"""YCSB range scans on the GPU (a read's field bits name its span; the
reference's YCSB/2 scans 10 keys per read, Y2/Execute.h:24-32): every launch
shape and mode, with and without shared-memory staging, bit-exact against the
oracle — flags, bitmap, results and the table image."""
import numpy as np
import pytest

import oracle
from ltpg_gb300 import Engine, YcsbGenerator, abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=4, max_txn=1 << 15, max_ops_per_txn=16)
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


@pytest.mark.parametrize("opt", [1, 2, 4, 8])
@pytest.mark.parametrize("k,scan", [(4, 10), (10, 3), (16, 16)])
def test_scans_match_oracle(eng, opt, k, scan):
    n = 30000
    eng.load_ycsb(41, n)
    o = oracle.YcsbOracle(41, n)
    g = YcsbGenerator(41, n, 6000, k, 20, 0.9, scan_len=scan)
    saved = eng.get_launch("ycsb")
    try:
        eng.set_launch("ycsb", ops_per_thread=opt)
        for i, mode in enumerate(["plain", "fused", "persistent", "graph"]):
            flags = _same(eng, o, g.batch(i), i % 2, mode)
            assert (flags & abi.FLAG_RAW).any() and (flags & abi.FLAG_COMMIT).any()
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        eng.set_launch("ycsb", **saved)


def test_scans_with_staging_and_table_end(eng):
    """Staged hot buckets (the scan's first key may be staged, the rest take the
    global path), and scans that run past the last key."""
    from ltpg_gb300 import key_bucket
    n = 2000
    eng.load_ycsb(43, n)
    o = oracle.YcsbOracle(43, n)
    g = YcsbGenerator(43, n, 4000, 8, 10, 0.99, scan_len=12)
    saved = eng.get_launch("ycsb")
    try:
        eng.set_launch("ycsb", ops_per_thread=1, stage_ways=4)
        for i, mode in enumerate(["fused", "persistent", "graph"]):
            b = g.batch(i)
            keys = (b.ops.reshape(b.n_txn, -1)[:, :8] & ((1 << 27) - 1)).ravel()
            cnt = np.bincount(key_bucket(keys), minlength=abi.STAGE_BUCKETS)
            eng.stage_set(np.argsort(-cnt, kind="stable")[:abi.STAGE_ENTRIES // 4])
            _same(eng, o, b, i % 2, mode)
        assert np.array_equal(eng.download_table(abi.TABLE_YCSB), o.rows)
    finally:
        eng.stage_set([])
        eng.set_launch("ycsb", **saved)
