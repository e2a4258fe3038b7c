"""The reference's own kernels, run on our batches (GPU parity pin).

TEST INFRASTRUCTURE ONLY.  Loads the cubins and struct layouts made by
oracle/ref_build.py (oracle/_ref/) and runs them through ref_harness.cu:
  RefY1  LTPG/YCSB/1 as shipped: 10,000 transactions x (9 reads + 1 write)
         over 1,000,000 records (Y1/Predefine.h:8-12).  Its Zipfian mode routes
         key 0 around registration (Y1/Genericfunction.h:163-187), so batches
         for it use keys 1 .. N-1.  RefY1("y1_c2"): the same sources at the
         high-contention scale, 1,048,576 transactions x (15 reads + 1 write)
         over 10,000,000 records, uniform mode (every key registers).
  RefTF  LTPG/TPCC-allopt-final as shipped: 65,536 Payments (NEWORDER_PERCENT
         = 0), 64 warehouses (TF/Predefine.h:8-10), customers by id; and its
         KERNEL_CID by-name lookup (TF/tp.cu:11-23) on its own.  RefTF("tf50"):
         the same sources with NEWORDER_PERCENT = 50 (32,768 NewOrders +
         32,768 Payments); RefTF("tf_c3"): 1,048,576 transactions, half of
         them NewOrders (524,288 of each kind).
Both return per-transaction flags rebuilt from the reference's conflict
counters raw / war / waw (the commit flag from its own rule,
TF/Execute_payment.h:607, Y1/Execute.h:187).
"""
import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
BUILD = os.path.join(HERE, "_build")
HARNESS = os.path.join(BUILD, "libref_harness.so")
_lib = None


def available(prog=None):
    progs = [prog] if prog else ["y1", "tf"]
    return all(os.path.exists(os.path.join(REF, f"{p}{ext}")) for p in progs for ext in [".cubin", "_layout.json"])


def build_harness(force=False):
    src = os.path.join(HERE, "ref_harness.cu")
    if not force and os.path.exists(HARNESS) and os.path.getmtime(HARNESS) >= os.path.getmtime(src):
        return HARNESS
    os.makedirs(BUILD, exist_ok=True)
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    stubs = os.path.join(home, "lib64", "stubs")
    cmd = [os.path.join(home, "bin", "nvcc"), "-shared", "-Xcompiler", "-fPIC", "-O2", src, "-o", HARNESS + ".tmp",
           "-L" + stubs, "-lcuda"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(HARNESS + ".tmp", HARNESS)
    return HARNESS


def _harness():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_harness())
        _lib.ref_launch.restype = C.c_int
        _lib.ref_launch.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_uint),
                                    C.POINTER(C.c_uint), C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_int), C.c_char_p, C.c_int]
        _lib.ref_time.restype = C.c_int
        _lib.ref_time.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_uint),
                                  C.POINTER(C.c_uint), C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_void_p),
                                  C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_uint64), C.POINTER(C.c_ubyte), C.c_int, C.POINTER(C.c_float),
                                  C.c_char_p, C.c_int]
    return _lib


def _launch(prog, layout, bufs, copy_back, resets=None, iters=0, kernels=None):
    """Runs the three kernels (or `kernels` = (names, grids, blocks)) once
    (iters = 0) or times `iters` repetitions, resetting the (buffer, offset,
    length, byte) ranges before each one.  Returns the mean milliseconds of
    each kernel when timing."""
    n = len(bufs)
    kn, kg, kb = kernels or (layout["kernels"], layout["grids"], layout["blocks"])
    nk = len(kn)
    names = (C.c_char_p * nk)(*[k.encode() for k in kn])
    grids = (C.c_uint * nk)(*kg)
    blocks = (C.c_uint * nk)(*kb)
    sizes = (C.c_uint64 * n)(*[b.nbytes for b in bufs])
    ptrs = (C.c_void_p * n)(*[b.ctypes.data for b in bufs])
    cb = (C.c_int * n)(*copy_back)
    err = C.create_string_buffer(256)
    cubin = os.path.join(REF, f"{prog}.cubin").encode()
    if not iters:
        rc = _harness().ref_launch(cubin, nk, names, grids, blocks, n, sizes, ptrs, cb, err, 256)
        ms = None
    else:
        resets = resets or []
        m = len(resets)
        rb = (C.c_int * max(1, m))(*[r[0] for r in resets])
        ro = (C.c_uint64 * max(1, m))(*[r[1] for r in resets])
        rl = (C.c_uint64 * max(1, m))(*[r[2] for r in resets])
        rv = (C.c_ubyte * max(1, m))(*[r[3] for r in resets])
        out = (C.c_float * nk)()
        rc = _harness().ref_time(cubin, nk, names, grids, blocks, n, sizes, ptrs, cb, m, rb, ro, rl, rv, iters, out,
                                 err, 256)
        ms = [float(x) for x in out]
    if rc:
        raise RuntimeError(f"reference kernels failed: {err.value.decode()}")
    return ms


def _flags(raw, war, waw):
    f = (raw > 0).astype(np.uint8) | ((war > 0).astype(np.uint8) << 1) | ((waw > 0).astype(np.uint8) << 2)
    com = (waw == 0) & ((raw == 0) | (war == 0))
    return f | (com.astype(np.uint8) << 3)


def covered_txns(layout, warps_per_group, batch):
    """Transactions whose every op the reference's launch grids reach.  Each
    kernel gives every 32 transactions a group of warps (one per op role); its
    grid, fixed at compile time as roles * B / 512 + 1 blocks, can end inside
    the last group, whose missing warps then never run."""
    full = min((g * b // 32) // w for g, b, w in zip(layout["grids"], layout["blocks"], warps_per_group))
    return min(batch, full * 32)


class RefY1:
    def __init__(self, prog="y1"):
        self.prog = prog
        self.L = json.load(open(os.path.join(REF, f"{prog}_layout.json")))
        self.B = self.L["batch"]
        self.n = self.L["table"]
        self.reads = self.L["reads"]
        writes = self.L["ops"] - self.reads
        # warp roles per 32 transactions: execute 2 per op, check reads + 2 per
        # write, write-back 1 + writes (Y1/Predefine.h:31-35, Y1/Execute.h:79-252)
        self.covered = covered_txns(self.L, [2 * self.L["ops"], self.reads + 2 * writes, 1 + writes], self.B)

    def run(self, read_keys, write_keys, iters=0):
        """read_keys: (B, reads) uint32, write_keys: (B,) uint32, TID = row index.
        Returns the reference's flags and its COMMIT_AND_ABORT marks (and, with
        iters > 0, the mean milliseconds of its three kernels over `iters`
        batches, each after the reference's per-batch clears)."""
        L, B = self.L, self.B
        s, q, lg = L["set"], L["query"], L["log"]
        set_b = np.zeros(s["size"], dtype=np.uint8)
        query = np.zeros(q["size"], dtype=np.uint8)
        qv = query.view(np.uint32)
        # SoA, op-major: LOC_R[op * B + NO] (Y1/Execute.h:20), LOC_W[op * B + NO], TID[NO]
        qv[q["loc_r"] // 4:q["loc_r"] // 4 + self.reads * B] = np.asarray(read_keys, dtype=np.uint32).T.ravel()
        qv[q["loc_w"] // 4:q["loc_w"] // 4 + B] = np.asarray(write_keys, dtype=np.uint32)
        qv[q["tid"] // 4:q["tid"] // 4 + B] = np.arange(B, dtype=np.uint32)
        log = np.zeros(lg["size"], dtype=np.uint8)
        log[:lg["ytd"]] = 0xFF  # registration tables cleared as clear_LOG does (Y1/Database.h:321-326)
        snap = np.zeros(L["snapshot"], dtype=np.uint8)
        index = np.zeros(max(1, L["index"]), dtype=np.uint8)
        # per batch the reference refills its registration tables with 0xFF
        # (clear_LOG) and starts from fresh conflict counters and marks
        resets = [(2, 0, lg["ytd"], 0xFF), (0, s["war"], s["size"] - s["war"], 0)]
        ms = _launch(self.prog, L, [set_b, query, log, snap, index], [1, 0, 0, 0, 0], resets, iters)
        sv = set_b.view(np.uint32)
        raw = sv[s["raw"] // 4:s["raw"] // 4 + B]
        war = sv[s["war"] // 4:s["war"] // 4 + B]
        waw = sv[s["waw"] // 4:s["waw"] // 4 + B]
        mark = sv[s["commit"] // 4:s["commit"] // 4 + B]
        if iters:
            return _flags(raw, war, waw), mark, ms
        return _flags(raw, war, waw), mark


class RefTF:
    """LTPG/TPCC-allopt-final's three kernels: prog "tf" as shipped (65,536
    Payments), or "tf50" (the same sources with NEWORDER_PERCENT = 50:
    32,768 NewOrders + 32,768 Payments per batch)."""

    def __init__(self, prog="tf"):
        self.prog = prog
        self.L = json.load(open(os.path.join(REF, f"{prog}_layout.json")))
        self.B = self.L["batch"]
        self.W = self.L["warehouses"]
        # 147 / 93 / 67 warp roles per 32 transactions (TF/Predefine.h:38-40)
        self.covered = covered_txns(self.L, [147, 93, 67], self.B)

    def run(self, txns, lines=None, iters=0):
        """txns: one batch of NewOrder / Payment records (TpccBatch.TXN_DTYPE),
        TID = index, with exactly the compiled NEWORDER_CNT NewOrders and
        PAYMENT_CNT Payments; lines: the batch's order lines.  Returns the
        flags (and, with iters > 0, the mean milliseconds of the three kernels
        over `iters` batches, each after the per-batch clears)."""
        L = self.L
        NC, PC = L["neworder_cnt"], L["payment_cnt"]
        ps, pq, lg = L["payment_set"], L["payment_query"], L["log"]
        kind = txns["kind_info"] & 0xFF
        no_idx, pay_idx = np.nonzero(kind == 0)[0], np.nonzero(kind == 1)[0]
        assert len(no_idx) == NC and len(pay_idx) == PC and len(txns) == NC + PC
        query = np.zeros(pq["size"], dtype=np.uint8)
        qv = query.view(np.uint32)

        def put(field, values):
            qv[pq[field] // 4:pq[field] // 4 + PC] = np.asarray(values, dtype=np.uint32)

        x = txns[pay_idx]
        ki = x["kind_info"]
        put("W_ID", x["w"])
        put("D_ID", (ki >> 16) & 0xFF)
        put("C_ID", x["c_id"])
        put("C_LAST", np.zeros(PC))
        put("isName", np.zeros(PC))
        put("C_D_ID", ki >> 24)
        put("C_W_ID", x["c_w"])
        put("H_AMOUNT", x["b"])
        put("H_ID", x["a"])
        put("TID", pay_idx)
        pset = np.zeros(ps["size"], dtype=np.uint8)
        nset = np.zeros(max(16, L["neworder_set"]), dtype=np.uint8)
        nquery = np.zeros(max(16, L["neworder_query"]), dtype=np.uint8)
        if NC:
            nf, nv = L["neworder_fields"], nquery.view(np.uint32)
            y = txns[no_idx]
            cnt = (y["kind_info"] >> 8) & 0xFF

            def putn(field, values, at=0, n=NC):
                o = nf[field] // 4 + at
                nv[o:o + n] = np.asarray(values, dtype=np.uint32)

            putn("W_ID", y["w"])
            putn("D_ID", (y["kind_info"] >> 16) & 0xFF)
            putn("C_ID", y["c_id"])
            putn("O_ID", y["a"])
            putn("N_O_ID", y["b"])
            putn("O_OL_CNT", cnt)
            putn("O_OL_ID", y["c"])
            putn("TID", no_idx)
            # line ID of NewOrder j at [NEWORDER_CNT * ID + j] (TF/Execute_neworder.h:177)
            for i in range(15):
                has = cnt > i
                ln = lines[y["line_off"][has] + i]
                for field, col in [("OL_I_ID", "i_id"), ("OL_SUPPLY_W_ID", "supply_w"), ("OL_QUANTITY", "qty")]:
                    v = np.zeros(NC, dtype=np.uint32)
                    v[has] = ln[col]
                    putn(field, v, at=NC * i)
        log = np.zeros(lg["size"], dtype=np.uint8)
        log[:lg["w_ytd"]] = 0xFF  # clear_LOG (TF/Database.h:78-102)
        snap = np.zeros(L["snapshot"], dtype=np.uint8)
        index = np.zeros(max(16, L["index"]), dtype=np.uint8)
        # argument order of KERNEL_EXECUTE / CHECK / WRITEBACK (TF/tp.cu:24-30)
        resets = [(4, 0, lg["w_ytd"], 0xFF), (1, ps["war"], ps["size"] - ps["war"], 0)]
        if NC:
            nc = L["neworder_counters"]
            resets.append((0, nc["war"], L["neworder_set"] - nc["war"], 0))
        ms = _launch(self.prog, L, [nset, pset, nquery, query, log, snap, index], [1 if NC else 0, 1, 0, 0, 0, 0, 0],
                     resets, iters)
        flags = np.zeros(len(txns), dtype=np.uint8)
        sv = pset.view(np.uint32)
        flags[pay_idx] = _flags(sv[ps["raw"] // 4:ps["raw"] // 4 + PC], sv[ps["war"] // 4:ps["war"] // 4 + PC],
                                sv[ps["waw"] // 4:ps["waw"] // 4 + PC])
        if NC:
            nc, nsv = L["neworder_counters"], nset.view(np.uint32)
            flags[no_idx] = _flags(nsv[nc["raw"] // 4:nc["raw"] // 4 + NC], nsv[nc["war"] // 4:nc["war"] // 4 + NC],
                                   nsv[nc["waw"] // 4:nc["waw"] // 4 + NC])
        if iters:
            return flags, ms
        return flags

    def cid(self, txns, c_last, c_id):
        """The reference's KERNEL_CID on one batch of Payments: the C_ID it
        writes for each by-name query (LTPG_PAY_BY_NAME; c_id field =
        (name << 8) | nth).  c_last / c_id: the customer table's C_LAST and C_ID
        columns, loaded into its INDEX and SNAPSHOT as Database.h does
        (TF/Database.h:188-211).

        Only nth = 0 is accepted.  The lookup's lanes leave its shuffle loop at
        different iterations for nth > 0 (a full-mask __shfl_sync after a
        per-lane break, TF/Genericfunction.h:42-57), which is undefined; at
        nth = 0 every lane leaves after the first iteration, together."""
        L, B = self.L, self.B
        assert len(txns) == B
        by_name = ((txns["kind_info"] & 0xFF) == 1) & ((txns["kind_info"] & 0x100) != 0)
        if (txns["c_id"][by_name] & 0xFF).any():
            raise ValueError("KERNEL_CID is run on nth = 0 queries only")
        pq = L["payment_query"]
        query = np.zeros(pq["size"], dtype=np.uint8)
        qv = query.view(np.uint32)

        def put(field, values):
            qv[pq[field] // 4:pq[field] // 4 + B] = np.asarray(values, dtype=np.uint32)

        ki = txns["kind_info"]
        put("W_ID", txns["w"])
        put("D_ID", (ki >> 16) & 0xFF)
        put("C_ID", np.where(by_name, 0, txns["c_id"]))
        put("C_LAST", np.where(by_name, txns["c_id"], 20))
        put("isName", by_name.astype(np.uint32))
        put("C_D_ID", ki >> 24)
        put("C_W_ID", txns["c_w"])
        put("TID", np.arange(B))
        CS = L["customer_size"]
        assert len(c_last) == CS
        snap = np.zeros(L["snapshot"], dtype=np.uint8)
        sv = snap.view(np.uint32)
        o = L["cust_snapshot"] // 4
        sv[o:o + CS] = np.asarray(c_id, dtype=np.uint32)  # customer_snapshot[0 * CUSTOMER_SIZE + row]
        index = np.zeros(L["index"], dtype=np.uint8)
        iv = index.view(np.uint32)
        iv[L["name_index"] // 4:L["name_index"] // 4 + CS] = np.asarray(c_last, dtype=np.uint32)
        pset = np.zeros(L["payment_set"]["size"], dtype=np.uint8)
        log = np.zeros(L["log"]["size"], dtype=np.uint8)
        # KERNEL_CID(PAYMENT_SET*, PAYMENT_QUERY*, LOG*, SNAPSHOT*, INDEX*), <<<GRID_SIZE, BLOCK_SIZE>>> (TF/tp.cu:154)
        _launch("tf", L, [pset, query, log, snap, index], [0, 1, 0, 0, 0],
                kernels=([L["cid_kernel"]], [L["cid_grid"]], [L["cid_block"]]))
        return qv[pq["C_ID"] // 4:pq["C_ID"] // 4 + B].copy()
