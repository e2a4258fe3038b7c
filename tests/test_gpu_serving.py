"""Serving loop: continuous batching of a TPC-C + YCSB request mix.

Each request's outcome depends on the batch it lands in (the protocol orders
by position in the batch), so "the same alone and in the mix" is checked per
batch placement: the loop records where every request went; replaying each
recorded batch alone, in order, through the plain three-kernel path on fresh
engines must give the same flags and results (exact) and the same tables.
"""
import numpy as np
import pytest

import ltpg_gb300 as L
from ltpg_gb300 import Engine, TpccBatch, TpccGenerator, YcsbBatch, YcsbGenerator, abi

pytestmark = pytest.mark.gpu

TP = dict(seed=31, warehouses=2, n_txn=20000)
YP = dict(seed=32, n_records=100000, n_txn=20000, ops_per_txn=10, update_pct=50, theta=0.9)


def _engines():
    c = Engine(device=0, n_slots=4, max_txn=1 << 16, max_ops_per_txn=16, max_lines=15 << 16)
    y = Engine(device=0, n_slots=4, max_txn=1 << 16, max_ops_per_txn=10)
    c.load_tpcc(TP["seed"], TP["warehouses"])
    y.load_ycsb(YP["seed"], YP["n_records"])
    return c, y


def _tpcc_pool(n):
    g = TpccGenerator(TP["seed"], TP["warehouses"], min(TP["n_txn"], max(n, 1)))
    txns, lines, have = [], [], 0
    while have < n:
        b = g.next()
        take = min(b.n_txn, n - have)
        t = b.txns[:take].copy()
        cnt = (t["kind_info"] >> 8) & 0xFF
        cnt[(t["kind_info"] & 0xFF) != abi.TPCC_NEWORDER] = 0
        l_end = int(t["line_off"][-1] + cnt[-1]) if take else 0
        lines.append(b.lines[:l_end])
        txns.append(t)
        have += take
    txns = np.concatenate(txns)
    cnt = (txns["kind_info"] >> 8) & 0xFF
    cnt[(txns["kind_info"] & 0xFF) != abi.TPCC_NEWORDER] = 0
    off = np.concatenate([[0], np.cumsum(cnt.astype(np.int64))])
    return txns, np.concatenate(lines), off


def _ycsb_pool(n):
    g = YcsbGenerator(YP["seed"], YP["n_records"], min(YP["n_txn"], max(n, 1)), YP["ops_per_txn"],
                      YP["update_pct"], YP["theta"])
    ops, vals, voff, have, bid = [], [], [0], 0, 0
    while have < n:
        b = g.batch(bid)
        bid += 1
        take = min(b.n_txn, n - have)
        ops.append(b.ops[:take * b.op_stride])
        vals.append(b.vals[:b.val_off[take]])
        voff.extend((voff[-1] + b.val_off[1:take + 1]).tolist())
        have += take
    return np.concatenate(ops), np.concatenate(vals), np.array(voff, dtype=np.int64)


def test_results_same_alone_and_in_the_mix():
    c, y = _engines()
    try:
        stats, rec = L.serve(c, y, rate=2e6, duration_s=0.03, tpcc_params=TP, ycsb_params=YP, deadline_ms=0.5,
                             max_batch=1 << 16, mode="fused", slots=4, record=True)
        mix_tables = [c.download_table(t) for t in range(abi.TPCC_TABLES)]
        mix_ycsb = y.download_table(abi.TABLE_YCSB)
    finally:
        c.close()
        y.close()
    assert stats["submitted"] > 20000 and stats["batches"] > 10
    assert 0 < stats["p50_ms"] <= stats["p99_ms"] <= stats["p999_ms"]
    nc, ny = len(rec["tpcc_flags"]), len(rec["ycsb_flags"])
    assert nc + ny == stats["submitted"]
    ctx, clines, coff = _tpcc_pool(nc)
    yops, yvals, yoff = _ycsb_pool(ny)
    stride = (YP["ops_per_txn"] + 3) & ~3
    c, y = _engines()
    try:
        for b0, bn, y0, yn in rec["batches"].astype(np.int64):
            if bn:
                t = ctx[b0:b0 + bn].copy()
                t["line_off"] = (coff[b0:b0 + bn] - coff[b0]).astype(np.uint32)
                batch = TpccBatch(t, clines[coff[b0]:coff[b0 + bn]], txn_base=b0)
                c.upload(0, batch)
                c.run_batch(0, "plain")
                c.sync()
                assert np.array_equal(c.txn_flags(0, bn), rec["tpcc_flags"][b0:b0 + bn])
                assert np.array_equal(c.txn_results(0, bn), rec["tpcc_results"][b0:b0 + bn])
            if yn:
                batch = YcsbBatch(yops[y0 * stride:(y0 + yn) * stride], (yoff[y0:y0 + yn + 1] - yoff[y0]),
                                  yvals[yoff[y0]:yoff[y0 + yn]], yn, YP["ops_per_txn"])
                y.upload(0, batch)
                y.run_batch(0, "plain")
                y.sync()
                assert np.array_equal(y.txn_flags(0, yn), rec["ycsb_flags"][y0:y0 + yn])
                assert np.array_equal(y.txn_results(0, yn), rec["ycsb_results"][y0:y0 + yn])
        for t in range(abi.TPCC_TABLES):
            assert np.array_equal(c.download_table(t), mix_tables[t]), t
        assert np.array_equal(y.download_table(abi.TABLE_YCSB), mix_ycsb)
    finally:
        c.close()
        y.close()


def test_admission_by_memory_budget():
    c, y = _engines()
    try:
        with pytest.raises(L.LtpgError) as ei:  # budget below the resident registration tables
            L.serve(c, y, rate=1e5, duration_s=0.01, tpcc_params=TP, ycsb_params=YP, max_batch=1 << 16,
                    budget_bytes=1 << 20)
        assert ei.value.code == abi.ERR_NOMEM
        one_slot = 54 << 20  # registration tables (25 MB here) + one 65,536-request slot (20 MB), not two
        stats = L.serve(c, y, rate=2e6, duration_s=0.02, tpcc_params=TP, ycsb_params=YP, max_batch=1 << 16,
                        budget_bytes=one_slot, slots=4)
        assert stats["slots"] == 1 and stats["committed"] > 0
    finally:
        c.close()
        y.close()


@pytest.mark.parametrize("ycsb_late,mode", [(0, "fused"), (3, "graph")])
def test_caller_requests_same_alone_and_in_the_mix(ycsb_late, mode):
    """Caller-owned requests through ltpg_serve_submit / ltpg_serve_poll: two
    request sources (a TPC-C client and a YCSB client, interleaved by one
    driving thread) submit in chunks of varying size with polls in between;
    results come back by id.  Replaying each logged batch alone, in order, on
    fresh engines gives every request's flags and result, and the tables.
    Also with the YCSB engine on write-first registration (late_reads 3, the
    update list) in graph mode, where every batch size is a new graph; there
    an aborted YCSB request's result is 0."""
    rng = np.random.default_rng(5)
    nc, ny = 12000, 15000
    ctx, clines, coff = _tpcc_pool(nc)
    yops, yvals, yoff = _ycsb_pool(ny)
    stride = (YP["ops_per_txn"] + 3) & ~3
    # the two sources' arrival order, interleaved at random
    order = np.array([0] * nc + [1] * ny)
    rng.shuffle(order)
    reqs, kind_idx = [], []
    ic = iy = 0
    for o in order:
        if o == 0:
            reqs.append(("tpcc", ctx[ic], clines[coff[ic]:coff[ic + 1]]))
            kind_idx.append((0, ic))
            ic += 1
        else:
            ops = yops[iy * stride:iy * stride + YP["ops_per_txn"]]
            reqs.append(("ycsb", ops, yvals[yoff[iy]:yoff[iy + 1]]))
            kind_idx.append((1, iy))
            iy += 1
    c, y = _engines()
    y.set_launch("ycsb", late_reads=ycsb_late)
    flags = np.zeros(len(reqs), dtype=np.uint8)
    results = np.zeros(len(reqs), dtype=np.int64)
    try:
        srv = L.Server(c, y, max_batch=3000, deadline_ms=0.3, mode=mode, slots=3, ycsb_ops=YP["ops_per_txn"])
        pos, got = 0, 0
        while pos < len(reqs):
            k = int(rng.integers(1, 700))
            first = srv.submit(reqs[pos:pos + k])
            assert first == pos
            pos += k
            f, r = srv.poll(got, len(reqs) - got)  # finished requests come back as a prefix of the ids
            flags[got:got + len(f)] = f
            results[got:got + len(f)] = r
            got += len(f)
        srv.flush()
        f, r = srv.poll(got, len(reqs) - got)
        flags[got:got + len(f)] = f
        results[got:got + len(f)] = r
        got += len(f)
        assert got == len(reqs)
        with pytest.raises(L.LtpgError):  # results already returned are forgotten
            srv.poll(0, 1)
        log = srv.batch_log()
        stats = srv.close()
        mix_tables = [c.download_table(t) for t in range(abi.TPCC_TABLES)]
        mix_ycsb = y.download_table(abi.TABLE_YCSB)
    finally:
        c.close()
        y.close()
    assert sum(n for _, n in log) == len(reqs) and len(log) > 8
    assert [f for f, _ in log] == list(np.cumsum([0] + [n for _, n in log])[:-1])
    assert stats["submitted"] == len(reqs) and stats["committed"] == int((flags & abi.FLAG_COMMIT != 0).sum())
    assert 0 < stats["p50_ms"] <= stats["p99_ms"]
    c, y = _engines()
    try:
        c_base = 0
        for first, n in log:
            idx = [kind_idx[i] for i in range(first, first + n)]
            ci = [j for k, j in idx if k == 0]
            yi = [j for k, j in idx if k == 1]
            pos_c = [first + t for t, (k, _) in enumerate(idx) if k == 0]
            pos_y = [first + t for t, (k, _) in enumerate(idx) if k == 1]
            if ci:
                t = ctx[ci].copy()
                cnt = (coff[np.array(ci) + 1] - coff[ci]).astype(np.int64)
                t["line_off"] = (np.cumsum(cnt) - cnt).astype(np.uint32)
                lines = np.concatenate([clines[coff[j]:coff[j + 1]] for j in ci])
                c.upload(0, TpccBatch(t, lines, txn_base=c_base))
                c.run_batch(0, "plain")
                c.sync()
                assert np.array_equal(c.txn_flags(0, len(ci)), flags[pos_c])
                assert np.array_equal(c.txn_results(0, len(ci)), results[pos_c])
                c_base += len(ci)
            if yi:
                ops = np.concatenate([yops[j * stride:(j + 1) * stride] for j in yi])
                nv = np.array([yoff[j + 1] - yoff[j] for j in yi], dtype=np.int64)
                voff = np.concatenate([[0], np.cumsum(nv)]).astype(np.uint32)
                vals = np.concatenate([yvals[yoff[j]:yoff[j + 1]] for j in yi] + [np.zeros(0, np.uint64)])
                y.upload(0, YcsbBatch(ops, voff, vals, len(yi), YP["ops_per_txn"]))
                y.run_batch(0, "plain")
                y.sync()
                assert np.array_equal(y.txn_flags(0, len(yi)), flags[pos_y])
                want = y.txn_results(0, len(yi))
                if ycsb_late:
                    want = np.where((flags[pos_y] & abi.FLAG_COMMIT) != 0, want, 0)
                assert np.array_equal(want, results[pos_y])
        for t in range(abi.TPCC_TABLES):
            assert np.array_equal(c.download_table(t), mix_tables[t]), t
        assert np.array_equal(y.download_table(abi.TABLE_YCSB), mix_ycsb)
    finally:
        c.close()
        y.close()
