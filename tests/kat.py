"""Builds the known-answer batches of tests/golden/*.json and their expected images."""
import json
import os

import numpy as np

from ltpg_gb300 import TpccBatch, YcsbBatch, abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def ycsb_batch(case):
    return YcsbBatch.from_ops([[tuple(op) for op in t] for t in case["txns"]], case["values"])


def hash3(seed, a, b):
    M = (1 << 64) - 1

    def sm(x):
        z = (x + 0x9E3779B97F4A7C15) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    return sm(sm(sm(seed) ^ a) ^ b)


def ycsb_expected_image(n, seed, case):
    rows = np.array([hash3(seed, k, f) for k in range(n) for f in range(abi.YCSB_FIELDS)], dtype=np.uint64)
    for key, field, value in case["image"]:
        rows[key * abi.YCSB_FIELDS + field] = value
    return rows


def ycsb_expected_digest(rows0, case):
    out = []
    for t in case["txns"]:
        d = 0
        for j, (key, upd, _) in enumerate(t):
            if not upd:
                x = 0
                for f in range(abi.YCSB_FIELDS):
                    x ^= int(rows0[key * abi.YCSB_FIELDS + f])
                d = (d + x * (2 * j + 1)) & ((1 << 64) - 1)
        out.append(d - (1 << 64) if d >= 1 << 63 else d)
    return np.array(out, dtype=np.int64)


def tpcc_batch(case, txn_base=0):
    txns = np.zeros(len(case["txns"]), dtype=TpccBatch.TXN_DTYPE)
    lines = []
    for i, x in enumerate(case["txns"]):
        rec = txns[i]
        rec["w"] = x["w"]
        rec["c_id"] = x["c_id"]
        rec["line_off"] = len(lines)
        if x["kind"] == "NO":
            rec["kind_info"] = abi.TPCC_NEWORDER | (len(x["lines"]) << 8) | (x["d"] << 16)
            rec["c_w"] = x["w"]
            rec["a"], rec["b"], rec["c"] = x["a"], x["b"], x["c"]
            lines.extend(tuple(ln) for ln in x["lines"])
        else:
            rec["kind_info"] = abi.TPCC_PAYMENT | (x["d"] << 16) | (x["c_d"] << 24)
            rec["c_w"] = x["c_w"]
            rec["a"] = x["a"]
            rec["b"] = x["amount"] & 0xFFFFFFFF
            rec["c"] = x["amount"] >> 32
    ln = np.array(lines, dtype=TpccBatch.LINE_DTYPE) if lines else np.zeros(0, dtype=TpccBatch.LINE_DTYPE)
    return TpccBatch(txns, ln, txn_base)


def tpcc_apply_expected(tables, case, flags, txn_base=0):
    """Applies the committed transactions of a KAT case to copies of the tables
    (a third, plain-Python statement of the write-back)."""
    M = (1 << 64) - 1
    t = [a.copy() for a in tables]

    def row(table, r):
        c = abi.TPCC_COLS[table]
        return t[table][r * c:(r + 1) * c]

    for i, x in enumerate(case["txns"]):
        if not flags[i] & abi.FLAG_COMMIT:
            continue
        date = txn_base + i
        if x["kind"] == "NO":
            w, d = x["w"], x["d"]
            all_local = all(sw == w for _, sw, _ in x["lines"])
            for li, (iid, sw, qty) in enumerate(x["lines"]):
                s = row(abi.T_STOCK, sw * 100000 + iid)
                q = int(s[2])
                s[2] = q - qty if q >= qty + 10 else q - qty + 91
                s[3] += qty
                s[4] += 1
                s[5] += int(sw != w)
                o = row(abi.T_ORDERLINE, w * 450000 + (x["c"] + li) % 450000)
                price = int(row(abi.T_ITEM, iid)[2])
                o[:] = [x["a"], d, w, li + 1, iid, sw, 0, qty, qty * price, int(s[6 + d])]
            row(abi.T_ORDER, w * 30000 + x["a"])[:] = [x["a"], d, w, x["c_id"], date, 0, len(x["lines"]),
                                                        int(all_local)]
            row(abi.T_NEWORDER, w * 30000 + x["b"])[:] = [x["a"], d, w]
        else:
            w, d, amt = x["w"], x["d"], x["amount"]
            wr = row(abi.T_WAREHOUSE, w)
            wr[2] = (int(wr[2]) + amt) & M
            dr = row(abi.T_DISTRICT, w * 10 + d)
            dr[3] = (int(dr[3]) + amt) & M
            c = row(abi.T_CUSTOMER, x["c_w"] * 30000 + x["c_d"] * 3000 + x["c_id"])
            c[5] = (int(c[5]) - amt) & M
            c[6] = (int(c[6]) + amt) & M
            c[7] += 1
            row(abi.T_HISTORY, w * 30000 + x["a"])[:] = [x["c_id"], x["c_d"], x["c_w"], d, w, amt, date, 0]
    return t


def mask_rows(tables, rows):
    """Zeroes rows whose final content the protocol leaves unspecified."""
    out = [a.copy() for a in tables]
    for table, r in rows:
        c = abi.TPCC_COLS[table]
        out[table][r * c:(r + 1) * c] = 0
    return out
