"""Writes the generator/replay regression fixtures gen_ycsb.npz and gen_tpcc.npz.

The batches come from the engine's deterministic generators, the expected
outputs from the oracle replay; the known-answer files kat_*.json are
hand-derived and are not produced here.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ltpg_gb300 import TpccGenerator, YcsbGenerator, abi  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def ycsb():
    seed, n, B, k, upd, rot, theta, nb = 1234, 4096, 1024, 10, 50, 0, 0.6, 2
    g = YcsbGenerator(seed, n, B, k, upd, theta, rot)
    o = oracle.YcsbOracle(seed, n)
    out = {"params": np.array([seed, n, B, k, upd, rot], dtype=np.uint64), "theta": np.float64(theta),
           "n_batches": np.int64(nb), "sm0": np.uint64(oracle.lib().oracle_splitmix64(0))}
    for bid in range(nb):
        b = g.batch(bid)
        flags, bitmap, results, _ = o.run(b)
        out[f"ops{bid}"], out[f"vals{bid}"] = b.ops, b.vals
        out[f"val_off{bid}"] = b.val_off
        out[f"flags{bid}"], out[f"bitmap{bid}"], out[f"results{bid}"] = flags, bitmap, results
    out["rows_head"] = o.rows[:4096].copy()
    out["rows_xor"] = np.uint64(np.bitwise_xor.reduce(o.rows))
    out["rows_final"] = o.rows.copy()
    np.savez_compressed(os.path.join(HERE, "gen_ycsb.npz"), **out)


def tpcc():
    seed, W, B, nb = 99, 1, 2048, 2
    g = TpccGenerator(seed, W, B)
    o = oracle.TpccOracle(seed, W)
    out = {"params": np.array([seed, W, B], dtype=np.uint64), "n_batches": np.int64(nb)}
    for bid in range(nb):
        b = g.next()
        flags, bitmap, results, _ = o.run(b)
        out[f"txns{bid}"], out[f"lines{bid}"] = b.txns.view(np.uint32), b.lines.view(np.uint32)
        out[f"txn_base{bid}"] = np.uint64(b.txn_base)
        out[f"flags{bid}"], out[f"bitmap{bid}"], out[f"results{bid}"] = flags, bitmap, results
    out["xor"] = np.array([np.bitwise_xor.reduce(o.tables[t]) for t in range(abi.TPCC_TABLES)], dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "gen_tpcc.npz"), **out)


if __name__ == "__main__":
    ycsb()
    tpcc()
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))
