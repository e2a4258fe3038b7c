"""ctypes mirror of include/ltpg.h (structs, constants, function signatures)."""
import ctypes as C

OK = 0
ERR_INVALID, ERR_CUDA, ERR_STATE, ERR_NOMEM, ERR_TIMEOUT, ERR_BOUNDS = 1, 2, 3, 4, 5, 6
WORKLOAD_YCSB, WORKLOAD_TPCC = 1, 2
MODE_PLAIN, MODE_FUSED, MODE_PERSISTENT, MODE_GRAPH = 0, 1, 2, 3
MODES = {"plain": MODE_PLAIN, "fused": MODE_FUSED, "persistent": MODE_PERSISTENT, "graph": MODE_GRAPH}
FLAG_RAW, FLAG_WAR, FLAG_WAW, FLAG_COMMIT, FLAG_NOT_FOUND = 1, 2, 4, 8, 16
PAY_BY_NAME = 0x100
YCSB_FIELDS = 10
YCSB_OP_PAD = 0xFFFFFFFF
YCSB_KEY_BITS = 27
YCSB_MAX_OPS = 32
TABLE_YCSB = 100
T_WAREHOUSE, T_DISTRICT, T_CUSTOMER, T_HISTORY, T_NEWORDER, T_ORDER, T_ORDERLINE, T_STOCK, T_ITEM = range(9)
TPCC_TABLES = 9
TPCC_COLS = (9, 11, 21, 8, 3, 8, 10, 17, 5)
TPCC_NEWORDER, TPCC_PAYMENT, TPCC_ORDERSTATUS, TPCC_DELIVERY, TPCC_STOCKLEVEL = 0, 1, 2, 3, 4
TPCC_MAX_LINES = 15
CFG_STRICT_INSERT = 1
CFG_REF_NAME_LOOKUP = 2
NOALLOC_MAX_RECORDS = 1 << 20
STAGE_BUCKETS = 65536
STAGE_ENTRIES = 1024
PRED_PARAMS = 4545


class YcsbBatchC(C.Structure):
    _fields_ = [("n_txn", C.c_uint32), ("ops_per_txn", C.c_uint32), ("op_stride", C.c_uint32),
                ("n_updates", C.c_uint32), ("ops", C.c_void_p), ("val_off", C.c_void_p), ("vals", C.c_void_p)]


class YcsbParamsC(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_records", C.c_uint64), ("n_txn", C.c_uint32),
                ("ops_per_txn", C.c_uint32), ("update_pct", C.c_uint32), ("rotate_every", C.c_uint32),
                ("theta", C.c_double), ("scan_len", C.c_uint32), ("pad", C.c_uint32)]


class TpccBatchC(C.Structure):
    _fields_ = [("n_txn", C.c_uint32), ("n_lines", C.c_uint32), ("txn_base", C.c_uint64),
                ("txns", C.c_void_p), ("lines", C.c_void_p)]


class TpccParamsC(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("warehouses", C.c_uint32), ("n_txn", C.c_uint32),
                ("neworder_pct", C.c_uint32), ("remote_line_pct", C.c_uint32), ("remote_pay_pct", C.c_uint32),
                ("by_name_pct", C.c_uint32), ("table_seed", C.c_uint64), ("orderstatus_pct", C.c_uint32),
                ("delivery_pct", C.c_uint32), ("stocklevel_pct", C.c_uint32), ("pad", C.c_uint32)]


class ConfigC(C.Structure):
    _fields_ = [("device", C.c_int32), ("n_slots", C.c_uint32), ("max_txn", C.c_uint32),
                ("max_ops_per_txn", C.c_uint32), ("max_lines", C.c_uint32), ("flags", C.c_uint32)]


class LaunchC(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("ops_per_thread", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("stage_ways", C.c_uint32), ("filter", C.c_uint32), ("dedupe", C.c_uint32),
                ("late_reads", C.c_uint32)]


class PredictorC(C.Structure):
    _fields_ = [("enable", C.c_uint32), ("train", C.c_uint32), ("stage", C.c_uint32), ("train_every", C.c_uint32),
                ("lr", C.c_float), ("pad", C.c_uint32), ("seed", C.c_uint64)]


class ServeCfgC(C.Structure):
    _fields_ = [("rate", C.c_double), ("duration_s", C.c_double), ("deadline_ms", C.c_double),
                ("budget_bytes", C.c_uint64), ("seed", C.c_uint64), ("max_batch", C.c_uint32),
                ("tpcc_pct", C.c_uint32), ("mode", C.c_uint32), ("slots", C.c_uint32)]


class ServeStatsC(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("committed", C.c_uint64), ("batches", C.c_uint64),
                ("slots", C.c_uint64), ("waited_for_slot", C.c_uint64), ("wall_s", C.c_double),
                ("throughput", C.c_double), ("mean_batch", C.c_double), ("mean_ms", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("p999_ms", C.c_double),
                ("wait_ms", C.c_double), ("launch_ms", C.c_double), ("device_ms", C.c_double)]


class ServerCfgC(C.Structure):
    _fields_ = [("deadline_ms", C.c_double), ("budget_bytes", C.c_uint64), ("max_batch", C.c_uint32),
                ("mode", C.c_uint32), ("slots", C.c_uint32), ("ycsb_ops", C.c_uint32)]


class RequestC(C.Structure):
    _fields_ = [("workload", C.c_int32), ("n", C.c_uint32), ("txn", C.c_void_p), ("lines", C.c_void_p),
                ("ops", C.c_void_p), ("vals", C.c_void_p)]


class StatsC(C.Structure):
    _fields_ = [("n_txn", C.c_uint64), ("commits", C.c_uint64), ("raw", C.c_uint64), ("war", C.c_uint64),
                ("waw", C.c_uint64), ("staged_ops", C.c_uint64), ("total_ops", C.c_uint64)]


class BatchInfoC(C.Structure):
    _fields_ = [("workload", C.c_int32), ("ops_per_txn", C.c_uint32), ("n_txn", C.c_uint64),
                ("n_op_words", C.c_uint64), ("n_updates", C.c_uint64), ("n_lines", C.c_uint64),
                ("txn_base", C.c_uint64)]


P = C.c_void_p
U32, U64, I32 = C.c_uint32, C.c_uint64, C.c_int32
SZ = C.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "ltpg_create": (C.c_int, [C.POINTER(ConfigC), C.POINTER(P)]),
    "ltpg_destroy": (C.c_int, [P]),
    "ltpg_last_error": (C.c_char_p, [P]),
    "ltpg_set_stream": (C.c_int, [P, P]),
    "ltpg_get_stream": (P, [P]),
    "ltpg_sync": (C.c_int, [P]),
    "ltpg_host_alloc": (P, [SZ]),
    "ltpg_host_free": (None, [P]),
    "ltpg_db_load_ycsb": (C.c_int, [P, U64, U64]),
    "ltpg_db_load_tpcc": (C.c_int, [P, U64, U32]),
    "ltpg_db_table_shape": (C.c_int, [P, U32, C.POINTER(U64), C.POINTER(U32)]),
    "ltpg_db_upload": (C.c_int, [P, U32, P, SZ]),
    "ltpg_db_download": (C.c_int, [P, U32, P, SZ]),
    "ltpg_gen_create_ycsb": (C.c_int, [C.POINTER(YcsbParamsC), C.POINTER(P)]),
    "ltpg_gen_create_tpcc": (C.c_int, [C.POINTER(TpccParamsC), C.POINTER(P)]),
    "ltpg_gen_destroy": (C.c_int, [P]),
    "ltpg_gen_capacity": (C.c_int, [P, C.POINTER(U64), C.POINTER(U64)]),
    "ltpg_gen_ycsb_batch": (C.c_int, [P, U64, P, P, P, C.POINTER(YcsbBatchC)]),
    "ltpg_gen_tpcc_batch": (C.c_int, [P, U64, P, P, C.POINTER(TpccBatchC)]),
    "ltpg_gen_ycsb_batch_device": (C.c_int, [P, P, U64, U32]),
    "ltpg_submit_generated": (C.c_int, [P, P, U64, U32, C.c_int, P]),
    "ltpg_batch_info_get": (C.c_int, [P, U32, C.POINTER(BatchInfoC)]),
    "ltpg_batch_download": (C.c_int, [P, U32, U32, P, C.c_size_t]),
    "ltpg_gen_tpcc_batch_device": (C.c_int, [P, P, U64, U32]),
    "ltpg_batch_upload_ycsb": (C.c_int, [P, U32, C.POINTER(YcsbBatchC)]),
    "ltpg_batch_upload_tpcc": (C.c_int, [P, U32, C.POINTER(TpccBatchC)]),
    "ltpg_execute_register": (C.c_int, [P, U32]),
    "ltpg_check_conflict": (C.c_int, [P, U32]),
    "ltpg_write_back": (C.c_int, [P, U32]),
    "ltpg_run_batch": (C.c_int, [P, U32, C.c_int]),
    "ltpg_run_batches": (C.c_int, [P, U32, U32, C.c_int]),
    "ltpg_run_ycsb_host": (C.c_int, [P, U32, C.POINTER(YcsbBatchC), C.c_int, P]),
    "ltpg_run_tpcc_host": (C.c_int, [P, U32, C.POINTER(TpccBatchC), C.c_int, P]),
    "ltpg_submit_ycsb_host": (C.c_int, [P, U32, C.POINTER(YcsbBatchC), C.c_int, P]),
    "ltpg_submit_tpcc_host": (C.c_int, [P, U32, C.POINTER(TpccBatchC), C.c_int, P]),
    "ltpg_tpcc_pack_lines": (C.c_int, [P, U64, P]),
    "ltpg_batch_upload_tpcc_packed": (C.c_int, [P, U32, C.POINTER(TpccBatchC), P]),
    "ltpg_submit_tpcc_packed_host": (C.c_int, [P, U32, C.POINTER(TpccBatchC), P, C.c_int, P]),
    "ltpg_host_wait": (C.c_int, [P, U32]),
    "ltpg_commit_bitmap": (C.c_int, [P, U32, P, SZ]),
    "ltpg_txn_flags": (C.c_int, [P, U32, P, SZ]),
    "ltpg_txn_results": (C.c_int, [P, U32, P, SZ]),
    "ltpg_batch_stats_get": (C.c_int, [P, U32, C.POINTER(StatsC)]),
    "ltpg_commit_bitmap_device": (C.c_int, [P, U32, C.POINTER(P)]),
    "ltpg_set_launch": (C.c_int, [P, C.c_int, C.POINTER(LaunchC)]),
    "ltpg_get_launch": (C.c_int, [P, C.c_int, C.POINTER(LaunchC)]),
    "ltpg_key_bucket": (U32, [U32]),
    "ltpg_stage_set": (C.c_int, [P, P, U32]),
    "ltpg_bucket_counts": (C.c_int, [P, P, C.c_int]),
    "ltpg_predictor_enable": (C.c_int, [P, C.POINTER(PredictorC)]),
    "ltpg_predictor_stats": (C.c_int, [P, C.POINTER(C.c_float), C.POINTER(U64)]),
    "ltpg_predictor_get_params": (C.c_int, [P, P, SZ]),
    "ltpg_predictor_set_params": (C.c_int, [P, P, SZ]),
    "ltpg_predictor_forward": (C.c_int, [P, P, U32, P]),
    "ltpg_predictor_gradients": (C.c_int, [P, P, P, U32, P]),
    "ltpg_serve_run": (C.c_int, [P, P, C.POINTER(ServeCfgC), C.POINTER(TpccParamsC), C.POINTER(YcsbParamsC),
                                 C.POINTER(ServeStatsC), C.POINTER(P)]),
    "ltpg_server_open": (C.c_int, [P, P, C.POINTER(ServerCfgC), C.POINTER(P)]),
    "ltpg_serve_submit": (C.c_int, [P, P, U32, C.POINTER(U64)]),
    "ltpg_serve_poll": (C.c_int, [P, U64, U32, P, P, C.POINTER(U32)]),
    "ltpg_serve_flush": (C.c_int, [P]),
    "ltpg_serve_batch_log": (C.c_int, [P, P, P, SZ, C.POINTER(SZ)]),
    "ltpg_server_close": (C.c_int, [P, C.POINTER(ServeStatsC)]),
    "ltpg_serve_record_sizes": (C.c_int, [P, C.POINTER(U64), C.POINTER(U64), C.POINTER(U64)]),
    "ltpg_serve_record_get": (C.c_int, [P, P, P, P, P, P]),
    "ltpg_serve_record_free": (C.c_int, [P]),
    "ltpg_counters": (C.c_int, [P, C.POINTER(U64), C.POINTER(U64)]),
    "ltpg_set_profiling": (C.c_int, [P, C.c_int]),
    "ltpg_kernel_times": (C.c_int, [P, U32, C.POINTER(C.c_float)]),
    "ltpg_ycsb_batch_noalloc": (C.c_int, [C.c_int, P, U64, P, P, P, U32, U32, P, P, P, P]),
    "ltpg_debug_set_epoch": (C.c_int, [P, U32]),
    "ltpg_debug_get_epoch": (C.c_int, [P, C.POINTER(U32)]),
    "ltpg_debug_noalloc_set_epoch": (C.c_int, [C.c_int, U32]),
    "ltpg_debug_noalloc_get_epoch": (C.c_int, [C.c_int, C.POINTER(U32)]),
    "ltpg_debug_barrier": (C.c_int, [P, U64, U32]),
    "ltpg_splitmix64": (U64, [U64]),
    "ltpg_hash3": (U64, [U64, U64, U64]),
}


# libltpg_bench.so (include/ltpg_bench.h): measurement only
BENCH_SIGNATURES = {
    "ltpg_microbench": (C.c_int, [C.c_int, P, C.c_int, U64, U32, C.POINTER(C.c_double)]),
}


def declared_functions(header_path):
    """Names of the functions include/ltpg.h declares (for the export test)."""
    import re
    text = open(header_path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\**(ltpg_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))
