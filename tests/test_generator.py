"""Deterministic batch generators (the Query.h surface), checked on the CPU."""
import math

import numpy as np
import pytest

from ltpg_gb300 import TpccGenerator, YcsbGenerator, abi

KEY_MASK = (1 << abi.YCSB_KEY_BITS) - 1


def _keys(b):
    ops = b.ops.reshape(b.n_txn, b.op_stride)[:, :b.ops_per_txn]
    return ops & KEY_MASK, (ops >> 31) == 1, (ops >> 27) & 0xF


def test_ycsb_same_seed_same_bytes(built_lib):
    a = YcsbGenerator(9, 5000, 3000, 10, 50, 0.6).batch(4)
    b = YcsbGenerator(9, 5000, 3000, 10, 50, 0.6).batch(4)
    c = YcsbGenerator(10, 5000, 3000, 10, 50, 0.6).batch(4)
    assert np.array_equal(a.ops, b.ops) and np.array_equal(a.vals, b.vals) and np.array_equal(a.val_off, b.val_off)
    assert not np.array_equal(a.ops, c.ops)


def test_ycsb_distinct_keys_padding_and_values(built_lib):
    b = YcsbGenerator(1, 64, 2000, 10, 50, 0.99).batch(0)  # tiny table: many resamples
    keys, upd, field = _keys(b)
    for row in keys:
        assert len(set(row.tolist())) == len(row)
    pad = b.ops.reshape(b.n_txn, b.op_stride)[:, b.ops_per_txn:]
    assert (pad == abi.YCSB_OP_PAD).all()
    assert (keys < 64).all() and (field[upd] < 10).all() and (field[~upd] == 0).all()
    counts = upd.sum(axis=1)
    assert np.array_equal(np.diff(b.val_off.astype(np.int64)), counts)
    assert b.n_updates == counts.sum() == len(b.vals)


@pytest.mark.parametrize("pct", [0, 5, 50, 100])
def test_ycsb_update_share(built_lib, pct):
    b = YcsbGenerator(2, 100000, 20000, 16, pct, 0.0).batch(1)
    _, upd, _ = _keys(b)
    share = upd.mean() * 100
    assert abs(share - pct) < 0.6


@pytest.mark.parametrize("theta", [0.6, 0.8, 0.99])
def test_ycsb_zipf_rank_frequencies(built_lib, theta):
    """Rank frequencies follow 1/r^theta (Gray et al.).  The sampler is exact for
    ranks 0 and 1 and a continuous approximation beyond, so ranks 0-1 are held
    to sampling noise and the log-log slope over ranks 2..2000 to -theta."""
    n = 100000
    b = YcsbGenerator(3, n, 200000, 1, 0, theta).batch(0)  # one op per txn: no resampling
    keys, _, _ = _keys(b)
    cnt = np.bincount(keys.ravel(), minlength=n)
    zeta = np.sum(1.0 / np.arange(1, n + 1) ** theta)
    for r in range(2):
        p = 1.0 / (r + 1) ** theta / zeta
        expect = p * keys.size
        assert abs(cnt[r] - expect) < 5 * math.sqrt(expect) + 5, (r, cnt[r], expect)
    # aggregate in log-spaced rank bands to average out the noise
    edges = np.unique(np.logspace(np.log10(3), np.log10(2000), 12).astype(int))
    mids, dens = [], []
    for lo, hi in zip(edges[:-1], edges[1:]):
        mids.append(np.sqrt(lo * hi))
        dens.append(cnt[lo - 1:hi - 1].mean())
    slope = np.polyfit(np.log(mids), np.log(dens), 1)[0]
    assert abs(slope + theta) < 0.08, slope


def test_ycsb_uniform_when_theta_zero(built_lib):
    n = 1000
    b = YcsbGenerator(4, n, 50000, 1, 0, 0.0).batch(0)
    keys, _, _ = _keys(b)
    cnt = np.bincount(keys.ravel(), minlength=n)
    assert cnt.max() < 50000 / n * 1.6 and cnt.min() > 50000 / n * 0.5


def test_ycsb_hot_set_rotates(built_lib):
    g = YcsbGenerator(5, 200000, 20000, 4, 5, 0.99, rotate_every=8)

    def hottest(bid):
        keys, _, _ = _keys(g.batch(bid))
        return int(np.bincount(keys.ravel()).argmax())

    assert hottest(0) == hottest(7)       # same permutation inside a window of 8
    assert hottest(0) != hottest(8)       # new permutation afterwards
    assert hottest(8) == hottest(15)


def test_tpcc_shapes_and_ranges(built_lib):
    W = 4
    g = TpccGenerator(7, W, 20000)
    b = g.next()
    x = b.txns
    kind = x["kind_info"] & 0xFF
    cnt = (x["kind_info"] >> 8) & 0xFF
    d = (x["kind_info"] >> 16) & 0xFF
    no, pay = kind == abi.TPCC_NEWORDER, kind == abi.TPCC_PAYMENT
    assert (no | pay).all() and abs(no.mean() - 0.5) < 0.02
    assert (cnt[no] >= 5).all() and (cnt[no] <= 15).all() and (cnt[pay] == 0).all()
    assert abs(cnt[no].mean() - 10) < 0.2
    assert (x["w"] < W).all() and (d < 10).all() and (x["c_id"] < 3000).all()
    # segmented line offsets
    assert np.array_equal(x["line_off"][1:], np.cumsum(cnt)[:-1]) and x["line_off"][0] == 0
    assert b.n_lines == cnt.sum()
    ln = b.lines
    assert (ln["i_id"] < 100000).all() and (ln["qty"] >= 1).all() and (ln["qty"] <= 10).all()
    owner_w = np.repeat(x["w"][no], cnt[no])
    remote = ln["supply_w"] != owner_w
    assert 0.005 < remote.mean() < 0.016
    # distinct items per order
    for t in np.nonzero(no)[0][:500]:
        items = ln["i_id"][x["line_off"][t]:x["line_off"][t] + cnt[t]]
        assert len(set(items.tolist())) == len(items)
    # payments: 15% remote customers, amounts 1.00 .. 5000.00
    cw = x["c_w"][pay]
    assert 0.13 < (cw != x["w"][pay]).mean() < 0.17
    amt = x["b"][pay].astype(np.int64) | (x["c"][pay].astype(np.int64) << 32)
    assert amt.min() >= 100 and amt.max() <= 500000
    # NURand(1023, 1, 3000) is skewed: some customers are far more frequent than uniform
    c = np.bincount(x["c_id"], minlength=3000)
    assert c.max() > 4 * len(x) / 3000


def test_tpcc_counters_advance_across_batches(built_lib):
    g = TpccGenerator(8, 1, 3000, neworder_pct=100)
    b0, b1 = g.next(), g.next()
    assert list(b0.txns["a"][:3]) == [0, 1, 2]
    assert b1.txns["a"][0] == 3000 and b1.txn_base == 3000
    ol = b0.txns["c"]
    cnt = (b0.txns["kind_info"] >> 8) & 0xFF
    assert np.array_equal(ol[1:], (np.cumsum(cnt)[:-1]) % 450000)


def test_tpcc_generator_is_deterministic(built_lib):
    a = TpccGenerator(11, 3, 5000).next()
    b = TpccGenerator(11, 3, 5000).next()
    assert np.array_equal(a.txns, b.txns) and np.array_equal(a.lines, b.lines)
