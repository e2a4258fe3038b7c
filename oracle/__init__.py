"""CPU replay of the LTPG protocol — the oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
the CPU-baseline leg of bench.py, never by the engine (ltpg_gb300).  The C
sources restate the reference's algorithm (see ltpg_oracle.c for the file:line
anchors) and build into oracle/_build/liboracle.so with gcc.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from ltpg_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "ltpg_oracle.c")
_lib = None


def build(force=False):
    """Compile liboracle.so with gcc (no CUDA needed)."""
    srcs = [SRC, os.path.join(HERE, "..", "include", "ltpg.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-ffp-contract=off", SRC, "-o", tmp]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P, U32, U64, I64 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int64
        _lib.oracle_splitmix64.restype = U64
        _lib.oracle_splitmix64.argtypes = [U64]
        _lib.oracle_hash3.restype = U64
        _lib.oracle_hash3.argtypes = [U64, U64, U64]
        _lib.oracle_ycsb_init.argtypes = [P, U64, U64]
        _lib.oracle_ycsb_batch.restype = I64
        _lib.oracle_ycsb_batch.argtypes = [P, U64, C.POINTER(abi.YcsbBatchC), P, P, P, P, P]
        _lib.oracle_ycsb_batch_mt.restype = I64
        _lib.oracle_ycsb_batch_mt.argtypes = [P, U64, C.POINTER(abi.YcsbBatchC), P, P, P, P, C.c_int]
        _lib.oracle_tpcc_rows.restype = U64
        _lib.oracle_tpcc_rows.argtypes = [U32, U32]
        _lib.oracle_tpcc_slots.restype = U64
        _lib.oracle_tpcc_slots.argtypes = [U32]
        _lib.oracle_tpcc_init_table.argtypes = [P, U32, U32, U64]
        _lib.oracle_tpcc_resolve.restype = None
        _lib.oracle_tpcc_resolve.argtypes = [C.POINTER(P), U32, C.POINTER(abi.TpccBatchC), C.c_int, P, P]
        _lib.oracle_tpcc_batch.restype = I64
        _lib.oracle_tpcc_batch.argtypes = [C.POINTER(P), U32, C.POINTER(abi.TpccBatchC), C.c_int, P, P, P, P, P]
        _lib.oracle_tpcc_batch_mt.restype = I64
        _lib.oracle_tpcc_batch_mt.argtypes = [C.POINTER(P), U32, C.POINTER(abi.TpccBatchC), C.c_int, P, P, P, P, P,
                                              C.c_int]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def pack_bits(b):
    """Bool array -> uint32 words, bit i of word w = element 32 w + i."""
    n = len(b)
    words = (n + 31) // 32
    padded = np.zeros(words * 32, dtype=np.uint64)
    padded[:n] = b
    return (padded.reshape(words, 32) << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)


class YcsbOracle:
    """Single-threaded replay over a host copy of the YCSB table."""

    def __init__(self, seed, n_records):
        self.n = int(n_records)
        self.rows = np.empty(self.n * abi.YCSB_FIELDS, dtype=np.uint64)
        lib().oracle_ycsb_init(_p(self.rows), self.n, seed)
        self.reg_r = np.empty(self.n, dtype=np.uint32)
        self.reg_w = np.empty(self.n, dtype=np.uint32)

    def run(self, batch, threads=1):
        """Replays one batch (a ltpg_gb300.YcsbBatch); returns (flags, bitmap, results, commits)."""
        B = batch.n_txn
        flags = np.zeros(B, dtype=np.uint8)
        bitmap = np.zeros((B + 31) // 32, dtype=np.uint32)
        results = np.zeros(B, dtype=np.int64)
        cb = batch.as_c()
        if threads == 1:
            commits = lib().oracle_ycsb_batch(_p(self.rows), self.n, C.byref(cb), _p(self.reg_r), _p(self.reg_w),
                                              _p(flags), _p(bitmap), _p(results))
        else:
            commits = lib().oracle_ycsb_batch_mt(_p(self.rows), self.n, C.byref(cb), _p(self.reg_r), _p(self.reg_w),
                                                 _p(flags), _p(results), threads)
            bitmap = pack_bits((flags & abi.FLAG_COMMIT) != 0)
        if commits < 0:
            raise ValueError("batch has a key out of range")
        return flags, bitmap, results, int(commits)


class TpccOracle:
    """Replay over host copies of the nine TPC-C tables (one thread, or
    several for the CPU baseline)."""

    def __init__(self, seed, warehouses, strict=False, ref_name_lookup=False):
        self.W = int(warehouses)
        # LTPG_CFG_* word: strict NEW-ORDER insert, reference by-name arithmetic
        self.strict = (abi.CFG_STRICT_INSERT if strict else 0) | (abi.CFG_REF_NAME_LOOKUP if ref_name_lookup else 0)
        L = lib()
        self.tables = []
        for t in range(abi.TPCC_TABLES):
            a = np.empty(L.oracle_tpcc_rows(t, self.W) * abi.TPCC_COLS[t], dtype=np.uint64)
            L.oracle_tpcc_init_table(_p(a), t, self.W, seed)
            self.tables.append(a)
        self._ptrs = (C.c_void_p * abi.TPCC_TABLES)(*[a.ctypes.data for a in self.tables])
        nslots = L.oracle_tpcc_slots(self.W)
        self.reg_r = np.empty(nslots, dtype=np.uint32)
        self.reg_w = np.empty(nslots, dtype=np.uint32)

    def resolve(self, batch):
        """(customer C_ID per transaction after by-name resolution, found flags)."""
        cid = np.zeros(batch.n_txn, dtype=np.uint32)
        found = np.zeros(batch.n_txn, dtype=np.uint8)
        cb = batch.as_c()
        lib().oracle_tpcc_resolve(self._ptrs, self.W, C.byref(cb), self.strict, _p(cid), _p(found))
        return cid, found.astype(bool)

    def run(self, batch, threads=1):
        """Replays one batch; threads > 1: the same phases on that many host
        threads (identical outputs and image)."""
        B = batch.n_txn
        flags = np.zeros(B, dtype=np.uint8)
        bitmap = np.zeros((B + 31) // 32, dtype=np.uint32)
        results = np.zeros(B, dtype=np.int64)
        cb = batch.as_c()
        if threads > 1:
            commits = lib().oracle_tpcc_batch_mt(self._ptrs, self.W, C.byref(cb), self.strict, _p(self.reg_r),
                                                 _p(self.reg_w), _p(flags), _p(bitmap), _p(results), int(threads))
        else:
            commits = lib().oracle_tpcc_batch(self._ptrs, self.W, C.byref(cb), self.strict, _p(self.reg_r),
                                              _p(self.reg_w), _p(flags), _p(bitmap), _p(results))
        if commits < 0:
            raise ValueError("invalid TPC-C batch")
        return flags, bitmap, results, int(commits)
