"""Contention predictor on the GPU: forward and gradients against the CPU
oracle, outcomes unchanged with it on, and what it gains.

Tolerances: the GPU rounds W1, W2, the features and the first hidden layer to
BF16 exactly as oracle.predictor_ref does and accumulates in FP32 in another
order, so outputs agree to |dy| <= 2e-3 (1 + |y|) and each gradient tensor to
2e-3 of its largest entry.
"""
import numpy as np
import pytest

import oracle
from oracle import predictor_ref as R
from ltpg_gb300 import Engine, YcsbGenerator, abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(gpu):
    e = Engine(device=0, n_slots=8, max_txn=1 << 18, max_ops_per_txn=16)
    e.load_ycsb(3, 1_000_000)
    e.predictor(enable=True, train=False, stage=False, seed=5)
    yield e
    e.close()


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(R.N_PARAM, dtype=np.float32)
    p[R.W1:R.B1] = rng.normal(0, 0.5, R.B1 - R.W1)
    p[R.B1:R.W2] = rng.normal(0, 0.1, R.H)
    p[R.W2:R.B2] = rng.normal(0, 0.15, R.H * R.H)
    p[R.B2:R.W3] = rng.normal(0, 0.1, R.H)
    p[R.W3:R.B3] = rng.normal(0, 0.2, R.H)
    p[R.B3] = 0.3
    return p


def _features(seed, n):
    rng = np.random.default_rng(seed)
    return np.log1p(rng.integers(0, 1_000_000, (n, R.F)).astype(np.float64) *
                    (rng.random((n, 1)) < 0.3)).astype(np.float32)


@pytest.mark.parametrize("n", [1, 17, 4096])
def test_forward_matches_oracle(eng, n):
    p = _params(n)
    eng.predictor_params(p)
    x = _features(n, n)
    y = eng.predictor_forward(x)
    want, _ = R.forward(p, x)
    assert np.all(np.abs(y - want) <= 2e-3 * (1 + np.abs(want))), np.max(np.abs(y - want))


@pytest.mark.parametrize("n", [64, 4096])
def test_gradients_match_oracle(eng, n):
    p = _params(100 + n)
    eng.predictor_params(p)
    x = _features(200 + n, n)
    t = np.random.default_rng(n).uniform(0, 12, n).astype(np.float32)
    g = eng.predictor_gradients(x, t)
    want = R.gradients(p, x, t)
    for name, lo, hi in [("W1", R.W1, R.B1), ("b1", R.B1, R.W2), ("W2", R.W2, R.B2), ("b2", R.B2, R.W3),
                         ("w3", R.W3, R.B3), ("b3", R.B3, R.N_PARAM)]:
        scale = max(np.max(np.abs(want[lo:hi])), 1e-6)
        assert np.max(np.abs(g[lo:hi] - want[lo:hi])) <= 2e-3 * scale, name


def _stream(n, B, theta, batches, seed=11):
    g = YcsbGenerator(seed, n, B, 16, 5, theta, rotate_every=8)
    return [g.batch(i) for i in range(batches)]


@pytest.mark.parametrize("late", [0, 3])
def test_predictor_never_changes_outcomes(eng, late):
    """With the predictor training and staging after every batch, on the
    default launch and on the benchmark's (write-first registration, slot
    filter on), flags and results equal the oracle's."""
    n, B = 200_000, 20_000
    e = Engine(device=0, n_slots=4, max_txn=B, max_ops_per_txn=16)
    try:
        e.load_ycsb(21, n)
        e.set_launch("ycsb", late_reads=late, filter=1)
        e.predictor(enable=True, train=True, stage=True, seed=3)
        o = oracle.YcsbOracle(21, n)
        for i, b in enumerate(_stream(n, B, 0.99, 12, seed=21)):
            e.upload(i % 4, b)
            e.run_batch(i % 4, ["fused", "graph", "persistent"][i % 3])
            e.sync()
            want = o.run(b)
            assert np.array_equal(e.txn_flags(i % 4, B), want[0]), i
            # with late reads an aborted transaction's result is 0
            wr = np.where((want[0] & abi.FLAG_COMMIT) != 0, want[2], 0) if late else want[2]
            assert np.array_equal(e.txn_results(i % 4, B), wr), i
        assert np.array_equal(e.download_table(abi.TABLE_YCSB), o.rows)
        assert e.predictor_stats()["train_steps"] == 12
    finally:
        e.close()


def _run_stream(e, batches, warm=8):
    """Staging hit rate and mean device time of a whole batch (every kernel of
    the batch and the predictor's step after it) over the batches after `warm`."""
    import torch
    stream = torch.cuda.ExternalStream(e.stream())
    hits, ms = [], []
    for i, b in enumerate(batches):
        e.upload(i % 8, b)
        e.sync()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        e.run_batch(i % 8, "fused")
        ev1.record(stream)
        e.sync()
        if i >= warm:
            st = e.stats(i % 8)
            hits.append(st["staged_ops"] / (b.n_txn * 16))
            ms.append(ev0.elapsed_time(ev1))
    return float(np.mean(hits)), float(np.mean(ms))


def test_predictor_learns_and_gains():
    """On the high-contention stream (10M records, 1,048,576 transactions x 16
    operations, theta = 0.99, hot set re-permuted every 8 batches), on the
    warp-aggregated registration path (slot filter off): the trained network
    stages more of the next batch's registrations than an untrained one, and
    its staging makes whole batches (the predictor's own step included)
    faster than both the untrained network's and no staging.  The training
    loss (MSE of log1p counts) stays bounded; its floor is set by the 1-in-16
    sampled counts of unstaged buckets.  With the slot filter on and
    write-first registration (the autotuned launch), staging does not pay and
    the tuned path runs without it."""
    n, B = 10_000_000, 1 << 20
    batches = _stream(n, B, 0.99, 24)
    out = {}
    for name, kw in [("trained", dict(train=True, stage=True)), ("untrained", dict(train=False, stage=True)),
                     ("off", None)]:
        e = Engine(device=0, n_slots=8, max_txn=B, max_ops_per_txn=16)
        try:
            e.load_ycsb(11, n)
            e.set_launch("ycsb", ops_per_thread=1, filter=0, dedupe=1, stage_ways=1)
            if kw:
                e.predictor(enable=True, seed=7, **kw)
            out[name] = _run_stream(e, batches)
            if name == "trained":
                out["loss"] = e.predictor_stats()["loss"]
        finally:
            e.close()
    print("predictor gain", out)
    hit_t, ms_t = out["trained"]
    hit_u, ms_u = out["untrained"]
    _, ms_off = out["off"]
    assert np.isfinite(out["loss"]) and out["loss"] < 4.0
    assert hit_t > 0.25 and hit_t > 1.3 * hit_u
    assert ms_t < ms_u < ms_off
