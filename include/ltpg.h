/*
 * ltpg.h — C ABI of the GB300 deterministic batch concurrency-control engine.
 *
 * The engine runs LTPG's three-phase protocol on one GPU:
 *   1. execute + register: every operation of every transaction in a batch
 *      records its TID (= position in the batch) as the minimum reader / writer
 *      of the row it touches, and reads what it needs from the batch-start
 *      snapshot;
 *   2. check: a read conflicts (RAW) when a smaller TID registered a write of
 *      its row, a write conflicts (WAR / WAW) when a smaller TID registered a
 *      read / write of its row;
 *   3. write-back: a transaction commits iff !WAW && (!RAW || !WAR), and the
 *      writes of committed transactions are applied to the table image.
 *
 * The reference program exposes this path as three __global__ kernels plus two
 * host classes that own the buffers; it has no library interface.  Each entry
 * point below names the reference interface it replaces (paths are relative to
 * the LTPG project root; TF = LTPG/TPCC-allopt-final, Y1 = LTPG/YCSB/1).
 *
 * Conventions: every call returns an int status (LTPG_OK = 0); on failure the
 * message is available from ltpg_last_error(ctx).  No exception crosses the ABI.
 * A context is driven by one host thread at a time, like the reference's epoch
 * loop (TF/tp.cu:136-261).  Pointers named host_* are host memory; pinned memory
 * from ltpg_host_alloc() makes the copies asynchronous.
 */
#ifndef LTPG_H
#define LTPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LTPG_OK 0
#define LTPG_ERR_INVALID 1 /* bad argument or size                        */
#define LTPG_ERR_CUDA 2    /* CUDA runtime error                           */
#define LTPG_ERR_STATE 3   /* call out of order (no table, empty slot ...) */
#define LTPG_ERR_NOMEM 4   /* device or host allocation failed             */
#define LTPG_ERR_TIMEOUT 5 /* a bounded device wait gave up                */
#define LTPG_ERR_BOUNDS 6  /* a key or index in a batch is out of range    */

/* ---- workloads and run modes ------------------------------------------ */
#define LTPG_WORKLOAD_YCSB 1
#define LTPG_WORKLOAD_TPCC 2

#define LTPG_MODE_PLAIN 0      /* three kernels, one per phase                  */
#define LTPG_MODE_FUSED 1      /* tuned kernels: execute | check+write-back      */
#define LTPG_MODE_PERSISTENT 2 /* one cooperative kernel, grid barriers         */
#define LTPG_MODE_GRAPH 3      /* tuned kernels captured into a CUDA graph       */

/* ---- per-transaction conflict flags (ltpg_txn_flags) ------------------- */
#define LTPG_FLAG_RAW 0x1u
#define LTPG_FLAG_WAR 0x2u
#define LTPG_FLAG_WAW 0x4u
#define LTPG_FLAG_COMMIT 0x8u
/* A Payment by customer last name whose (name, nth) matched no customer: it
 * registers nothing, does not commit and returns 0 (the reference has no such
 * outcome; its lookup falls back to C_ID 0, TF/Genericfunction.h:37,72-74). */
#define LTPG_FLAG_NOT_FOUND 0x10u

/* ---- YCSB ----------------------------------------------------------------
 * Table: n_records rows of 10 uint64 fields, row-major (80 B per row).
 * Initial value of field f of key k = ltpg_hash3(seed, k, f).
 * A batch holds n_txn transactions of ops_per_txn operations each; the op words
 * of transaction t sit at ops[t * op_stride + j] (op_stride = ops_per_txn
 * rounded up to 4, so every transaction starts on a 16-byte boundary); unused
 * words hold LTPG_YCSB_OP_PAD.  Op word layout:
 *   bit 31      1 = update, 0 = read
 *   bits 27..30 update: field written (0..9); read: scan span s — the read
 *               covers keys key .. key + s (s = 0: a point read; keys past
 *               the table's end are left out, as the reference's scans do,
 *               Y2/Execute.h:24-32)
 *   bits 0..26  key
 * Updates carry their new values in vals[], in transaction/op order;
 * val_off[t] is the index of transaction t's first value (val_off[n_txn] =
 * number of updates).  No value is read out of bounds: a value index past
 * val_off[n_txn] or past the slot's values is reported as LTPG_ERR_BOUNDS by
 * the batch's sync, and the write-first path (late_reads = 3) also reports a
 * transaction whose update count disagrees with its offsets.  A read
 * registers and checks every key it covers.
 * Per-transaction result: sum over the reads j of (xor of the 10 fields of
 * every row the read covers) * (2j + 1), mod 2^64, read from the batch-start
 * image.
 */
#define LTPG_YCSB_FIELDS 10
#define LTPG_YCSB_OP_PAD 0xFFFFFFFFu
#define LTPG_YCSB_KEY_BITS 27
#define LTPG_YCSB_MAX_OPS 32

typedef struct {
    uint32_t n_txn;
    uint32_t ops_per_txn;
    uint32_t op_stride;
    uint32_t n_updates;
    const uint32_t *ops;     /* n_txn * op_stride */
    const uint32_t *val_off; /* n_txn + 1; NULL: made on the device from the op
                                words, and n_updates must equal the number
                                of update ops (a mismatch is reported as
                                LTPG_ERR_BOUNDS)                           */
    const uint64_t *vals;    /* n_updates         */
} ltpg_ycsb_batch;

typedef struct {
    uint64_t seed;
    uint64_t n_records;    /* keys 0 .. n_records-1                      */
    uint32_t n_txn;        /* transactions per batch                     */
    uint32_t ops_per_txn;  /* distinct keys per transaction (<= 32)      */
    uint32_t update_pct;   /* share of update operations, 0..100         */
    uint32_t rotate_every; /* new hot-set permutation every R batches; 0 = key rank order */
    double theta;          /* Zipf exponent, 0 = uniform                 */
    uint32_t scan_len;     /* 0 or 1: point reads; 2..16: every read scans
                              scan_len keys (the reference's YCSB/2: 10)  */
    uint32_t pad;
} ltpg_ycsb_params;

/* ---- TPC-C ---------------------------------------------------------------
 * Nine tables of uint64 columns, row-major.  Table ids and column counts:
 */
#define LTPG_T_WAREHOUSE 0 /*  9 cols, W rows            */
#define LTPG_T_DISTRICT 1  /* 11 cols, 10 W rows         */
#define LTPG_T_CUSTOMER 2  /* 21 cols, 30,000 W rows     */
#define LTPG_T_HISTORY 3   /*  8 cols, 30,000 W rows     */
#define LTPG_T_NEWORDER 4  /*  3 cols, 30,000 W rows     */
#define LTPG_T_ORDER 5     /*  8 cols, 30,000 W rows     */
#define LTPG_T_ORDERLINE 6 /* 10 cols, 450,000 W rows    */
#define LTPG_T_STOCK 7     /* 17 cols, 100,000 W rows    */
#define LTPG_T_ITEM 8      /*  5 cols, 100,000 rows      */
#define LTPG_TPCC_TABLES 9

#define LTPG_TPCC_NEWORDER 0
#define LTPG_TPCC_PAYMENT 1
#define LTPG_TPCC_ORDERSTATUS 2
#define LTPG_TPCC_DELIVERY 3
#define LTPG_TPCC_STOCKLEVEL 4
#define LTPG_TPCC_MAX_LINES 15

/* 32-byte transaction record.  kind_info: bits 0..7 kind, 8..15 order-line
 * count (NewOrder) or LTPG_PAY_* bits (Payment), 16..23 district, 24..31
 * customer district (Payment).
 * NewOrder: a = O_ID, b = NO_ID, c = first OL_ID.   Payment: a = H_ID,
 * b/c = low/high 32 bits of the amount in cents (int64).
 * Payment by last name (LTPG_PAY_BY_NAME): c_id holds the reference's C_LAST
 * query word, (name << 8) | nth (TF/Query.h:176-181), and the customer is the
 * nth (0-based) one of district (c_w, customer district) whose C_LAST column
 * equals name, in C_ID order; it replaces the reference's KERNEL_CID /
 * __FIND_CID_INDEX pre-phase (TF/tp.cu:11-23, TF/Genericfunction.h:29-77).
 * line_off = number of order lines of all earlier transactions of the batch.
 *
 * The other three TPC-C transactions follow the reference's all-transaction
 * variant (TA/Execute.h:1592-2231: one customer / order / order line, one
 * stock row), with the row keys computed from the record:
 *   OrderStatus: reads customer (c_w, customer district, c_id — by name with
 *     LTPG_PAY_BY_NAME as for Payment), ORDER row a and ORDER-LINE row b of
 *     warehouse w; result = C_BALANCE.
 *   Delivery: deletes NEW-ORDER row b of warehouse w (every column set to all
 *     ones), sets O_CARRIER_ID of ORDER row a (carrier in bits 8..15, 1..10)
 *     and OL_DELIVERY_D of ORDER-LINE row c, and credits customer (w,
 *     district, c_id) with that line's OL_AMOUNT (C_BALANCE +=, C_DELIVERY_CNT
 *     += 1); result = the amount.
 *   StockLevel: reads STOCK row a of warehouse w; result = S_QUANTITY. */
#define LTPG_PAY_BY_NAME 0x100u
typedef struct {
    uint32_t kind_info;
    uint32_t w;
    uint32_t c_w;
    uint32_t c_id;
    uint32_t a;
    uint32_t b;
    uint32_t c;
    uint32_t line_off;
} ltpg_tpcc_txn;

typedef struct {
    uint32_t i_id;
    uint16_t supply_w;
    uint16_t qty;
} ltpg_tpcc_line;

typedef struct {
    uint32_t n_txn;
    uint32_t n_lines;
    uint64_t txn_base; /* global number of transaction 0 (O_ENTRY_D / H_DATE) */
    const ltpg_tpcc_txn *txns;
    const ltpg_tpcc_line *lines;
} ltpg_tpcc_batch;

typedef struct {
    uint64_t seed;
    uint32_t warehouses;
    uint32_t n_txn;
    uint32_t neworder_pct; /* share of NewOrder, rest Payment         */
    uint32_t remote_line_pct; /* NewOrder remote supply, per line (1)  */
    uint32_t remote_pay_pct;  /* Payment remote customer (15)          */
    uint32_t by_name_pct;     /* Payment / OrderStatus by last name (0; TPC-C: 60) */
    uint64_t table_seed;      /* seed of the loaded tables: by-name queries
                                 name the customer a by-id Payment would pick */
    /* shares of OrderStatus, Delivery, StockLevel, taken from the non-NewOrder
     * share (0 each: NewOrder + Payment only; TPC-C mix: 45/43/4/4/4) */
    uint32_t orderstatus_pct, delivery_pct, stocklevel_pct, pad;
} ltpg_tpcc_params;

/* ---- engine context ---------------------------------------------------- */
typedef struct ltpg_ctx ltpg_ctx;

typedef struct {
    int32_t device;
    uint32_t n_slots;        /* device batch slots (>= 1)                    */
    uint32_t max_txn;        /* capacity per slot, transactions              */
    uint32_t max_ops_per_txn;/* YCSB capacity per transaction                */
    uint32_t max_lines;      /* TPC-C capacity per slot, order lines         */
    uint32_t flags;          /* LTPG_CFG_*                                   */
} ltpg_config;

/* The reference registers the NEW-ORDER insert as a read and never runs its
 * WAR check (TF/Execute_neworder.h:115,639-646); that is the default here.
 * With this flag the insert registers and checks as a write. */
#define LTPG_CFG_STRICT_INSERT 0x1u
/* By-name Payments resolve the customer with the reference's own arithmetic
 * (TF/Genericfunction.h:29-77 as its lane 0 computes it: that lane tests
 * every 32nd customer, counts each match 32 times, then walks back from the
 * end of its last block of 32, skipping position 0; no match gives C_ID 0)
 * instead of the nth-customer rule.  For parity with the reference only. */
#define LTPG_CFG_REF_NAME_LOOKUP 0x2u

typedef struct {
    uint64_t n_txn;
    uint64_t commits;
    uint64_t raw;      /* transactions with a RAW conflict */
    uint64_t war;
    uint64_t waw;
    uint64_t staged_ops;   /* registrations served from shared memory */
    uint64_t total_ops;    /* registrations issued                    */
} ltpg_batch_stats;

/* Replaces: Database / YCSBDatabase constructors + Query constructors, which
 * cudaMalloc every buffer (TF/Database.h:37-57, TF/Query.h:330-355,
 * Y1/Database.h:27-39, Y1/Query.h:142-149). */
int ltpg_create(const ltpg_config *cfg, ltpg_ctx **out);
/* Replaces: the never-run destructors (TF/Database.h:59-77, TF/Query.h:356-376). */
int ltpg_destroy(ltpg_ctx *ctx);
const char *ltpg_last_error(const ltpg_ctx *ctx);
/* Runs all device work of ctx on this stream (cudaStream_t; NULL = ctx's own). */
int ltpg_set_stream(ltpg_ctx *ctx, void *stream);
void *ltpg_get_stream(ltpg_ctx *ctx);
int ltpg_sync(ltpg_ctx *ctx);

/* Pinned host memory for fast copies (the reference's cudaMallocHost buffers,
 * TF/Query.h:338-343). */
void *ltpg_host_alloc(size_t bytes);
void ltpg_host_free(void *p);

/* ---- tables (Database.h surface) ---------------------------------------- */
/* Replaces: YCSBDatabase + initial_ycsb_data (Y1/Database.h:27-131): build the
 * table and load it into HBM. The image is generated on the device. */
int ltpg_db_load_ycsb(ltpg_ctx *ctx, uint64_t seed, uint64_t n_records);
/* Replaces: Database + initial_data (TF/Database.h:13-451). */
int ltpg_db_load_tpcc(ltpg_ctx *ctx, uint64_t seed, uint32_t warehouses);
/* Table ids for the calls below: LTPG_T_* for TPC-C, LTPG_TABLE_YCSB for YCSB. */
#define LTPG_TABLE_YCSB 100
/* Rows and columns (uint64 each) of a loaded table. */
int ltpg_db_table_shape(ltpg_ctx *ctx, uint32_t table, uint64_t *rows, uint32_t *cols);
/* H2D load of a host image / D2H download (the reference's cudaMemcpy of the
 * SNAPSHOT, TF/Database.h:445-446).  bytes must equal rows * cols * 8. */
int ltpg_db_upload(ltpg_ctx *ctx, uint32_t table, const void *host, size_t bytes);
int ltpg_db_download(ltpg_ctx *ctx, uint32_t table, void *host, size_t bytes);

/* ---- batches (Query.h surface) ------------------------------------------- */
/* Deterministic generators.  Replace MakeYCSB / MakeNeworder / MakePayment and
 * Query::initial_* (Y1/Query.h:18-117,161-188; TF/Query.h:16-212,478-525),
 * whose output depends on rand() and thread timing. */
typedef struct ltpg_gen ltpg_gen;
int ltpg_gen_create_ycsb(const ltpg_ycsb_params *p, ltpg_gen **out);
int ltpg_gen_create_tpcc(const ltpg_tpcc_params *p, ltpg_gen **out);
int ltpg_gen_destroy(ltpg_gen *g);
/* Capacity needed for one batch: ops words / values (YCSB) or txns / lines (TPC-C). */
int ltpg_gen_capacity(const ltpg_gen *g, uint64_t *cap_a, uint64_t *cap_b);
/* Fill caller buffers with batch number batch_id.  YCSB: ops (n_txn*op_stride),
 * val_off (n_txn+1), vals (capacity).  The TPC-C generator is stateful (per-
 * warehouse order / history counters advance like TF/Query.h:54-88,157-166), so
 * batches must be drawn in order. */
int ltpg_gen_ycsb_batch(ltpg_gen *g, uint64_t batch_id, uint32_t *ops, uint32_t *val_off,
                        uint64_t *vals, ltpg_ycsb_batch *out);
int ltpg_gen_tpcc_batch(ltpg_gen *g, uint64_t batch_id, ltpg_tpcc_txn *txns,
                        ltpg_tpcc_line *lines, ltpg_tpcc_batch *out);

/* Device generation: the same batch as ltpg_gen_*_batch (byte for byte),
 * made on the GPU in slot `slot` on the context stream, with no host
 * generation and no host-to-device copy (the reference generates on host
 * threads and copies, TF/Query.h:417-605).  YCSB generators are stateless
 * and may mix host and device batches.  A TPC-C generator's counters and
 * order memory move to the device at its first device batch; its host
 * batches are refused (LTPG_ERR_STATE) from then on, and batches stay in
 * order.  Device TPC-C generation needs cfg.max_lines >= 15 n_txn. */
int ltpg_gen_ycsb_batch_device(ltpg_ctx *ctx, ltpg_gen *g, uint64_t batch_id, uint32_t slot);
int ltpg_gen_tpcc_batch_device(ltpg_ctx *ctx, ltpg_gen *g, uint64_t batch_id, uint32_t slot);

/* The batch held by a slot (uploaded or generated on the device), for
 * inspection: its shape, then part `part` copied to host (YCSB 0 ops,
 * 1 val_off, 2 vals; TPC-C 0 txns, 1 lines; `bytes` must be the part's size).
 * Both synchronise the context stream. */
typedef struct {
    int32_t workload;     /* LTPG_WORKLOAD_YCSB / _TPCC */
    uint32_t ops_per_txn; /* YCSB */
    uint64_t n_txn;
    uint64_t n_op_words;  /* YCSB: n_txn * op_stride */
    uint64_t n_updates;   /* YCSB */
    uint64_t n_lines;     /* TPC-C */
    uint64_t txn_base;    /* TPC-C */
} ltpg_batch_info;
int ltpg_batch_info_get(ltpg_ctx *ctx, uint32_t slot, ltpg_batch_info *out);
int ltpg_batch_download(ltpg_ctx *ctx, uint32_t slot, uint32_t part, void *host, size_t bytes);

/* Replaces: Query::copy_to_device (TF/Query.h:532-605, Y1/Query.h:194-213).
 * Copies a host batch into device slot `slot` on the context stream.  A YCSB
 * batch without val_off has its offsets made on the device behind the copy of
 * its op words (the bytes on the wire are the op words and values only). */
int ltpg_batch_upload_ycsb(ltpg_ctx *ctx, uint32_t slot, const ltpg_ycsb_batch *b);
int ltpg_batch_upload_tpcc(ltpg_ctx *ctx, uint32_t slot, const ltpg_tpcc_batch *b);

/* ---- phases (Genericfunction.h / Execute*.h surface) --------------------- */
/* Replaces: KERNEL_EXECUTE (TF/tp.cu:24-54, Y1/ycsb.cu:9-24) → __REGISTER /
 * __READ / __WRITE (TF/Genericfunction.h:78-251). */
int ltpg_execute_register(ltpg_ctx *ctx, uint32_t slot);
/* Replaces: KERNEL_CHECK (TF/tp.cu:55-85, Y1/ycsb.cu:25-40) → __CHECK
 * (TF/Genericfunction.h:252-414). */
int ltpg_check_conflict(ltpg_ctx *ctx, uint32_t slot);
/* Replaces: KERNEL_WRITEBACK (TF/tp.cu:86-117, Y1/ycsb.cu:41-58) → write_back /
 * __WRITEBACK / __REDUCE_UPGRADE (TF/Genericfunction.h:416-518). */
int ltpg_write_back(ltpg_ctx *ctx, uint32_t slot);
/* One whole batch in the given mode (LTPG_MODE_*). */
int ltpg_run_batch(ltpg_ctx *ctx, uint32_t slot, int mode);
/* count batches in slots first..first+count-1, in order. */
int ltpg_run_batches(ltpg_ctx *ctx, uint32_t first, uint32_t count, int mode);
/* Upload + run + copy the commit bitmap back, all on the context stream and
 * synchronised before return: the host-buffer call a caller of the reference's
 * epoch loop makes per batch. */
int ltpg_run_ycsb_host(ltpg_ctx *ctx, uint32_t slot, const ltpg_ycsb_batch *b, int mode,
                       uint32_t *host_bitmap);
int ltpg_run_tpcc_host(ltpg_ctx *ctx, uint32_t slot, const ltpg_tpcc_batch *b, int mode,
                       uint32_t *host_bitmap);
/* Pipelined form of the two calls above (no reference counterpart: the
 * reference's epoch loop copies, runs and synchronises each batch in turn,
 * TF/tp.cu:136-261).  Returns once the slot's copy (on a copy stream, after
 * the slot's previous batch is finished), run and bitmap download are
 * enqueued; ltpg_host_wait(slot) returns when that bitmap is on the host, with
 * any device-side error of the batch.  The copy of one batch overlaps the
 * kernels of the previous ones.  The host buffers, pinned
 * (ltpg_host_alloc) for the copies to overlap, must stay unchanged until the
 * wait. */
int ltpg_submit_ycsb_host(ltpg_ctx *ctx, uint32_t slot, const ltpg_ycsb_batch *b, int mode,
                          uint32_t *host_bitmap);
int ltpg_submit_tpcc_host(ltpg_ctx *ctx, uint32_t slot, const ltpg_tpcc_batch *b, int mode,
                          uint32_t *host_bitmap);
int ltpg_host_wait(ltpg_ctx *ctx, uint32_t slot);
/* TPC-C order lines packed in 4 bytes for the host link: i_id in bits 0..16,
 * supply_w in bits 17..27, qty in bits 28..31 (so i_id < 2^17, supply_w <
 * 2^11 and qty < 16, which TPC-C's 100,000 items, up to 2,047 warehouses and
 * quantities 1..10 meet).  ltpg_tpcc_pack_lines packs n lines (host only; a
 * line out of those ranges is LTPG_ERR_INVALID).  The packed upload and
 * submit calls take the batch's records from b (b->lines is not read) and its
 * lines from `packed`, and unpack them on the device on the context stream
 * before the batch's kernels: half the lines' bytes on the link. */
int ltpg_tpcc_pack_lines(const ltpg_tpcc_line *lines, uint64_t n, uint32_t *packed);
int ltpg_batch_upload_tpcc_packed(ltpg_ctx *ctx, uint32_t slot, const ltpg_tpcc_batch *b, const uint32_t *packed);
int ltpg_submit_tpcc_packed_host(ltpg_ctx *ctx, uint32_t slot, const ltpg_tpcc_batch *b, const uint32_t *packed,
                                 int mode, uint32_t *host_bitmap);
/* The same pipeline with the batch made on the GPU: generator g's batch
 * batch_id (in order for TPC-C) is generated into `slot` on the copy stream,
 * so it overlaps the kernels of the batches before it, then run and its
 * bitmap queued for download; ltpg_host_wait(slot) as above. */
int ltpg_submit_generated(ltpg_ctx *ctx, ltpg_gen *g, uint64_t batch_id, uint32_t slot, int mode,
                          uint32_t *host_bitmap);

/* ---- results (statistic_query / copy_to_host surface) ------------------- */
/* Replaces: Query::copy_to_host (TF/Query.h:606-631), which reads back only
 * the commit counters. */
int ltpg_commit_bitmap(ltpg_ctx *ctx, uint32_t slot, uint32_t *host_bits, size_t words);
int ltpg_txn_flags(ltpg_ctx *ctx, uint32_t slot, uint8_t *host_flags, size_t n);
int ltpg_txn_results(ltpg_ctx *ctx, uint32_t slot, int64_t *host_results, size_t n);
int ltpg_batch_stats_get(ltpg_ctx *ctx, uint32_t slot, ltpg_batch_stats *out);
/* Device pointer of the commit bitmap of a slot (for callers that keep results
 * on the GPU). */
int ltpg_commit_bitmap_device(ltpg_ctx *ctx, uint32_t slot, const uint32_t **dev_bits);

/* ---- tuning ----------------------------------------------------------------
 * Launch shape of the tuned kernels of one workload; the autotuner writes it.
 * None of these settings can change a commit decision or the table image.
 * Defaults: 256 threads (TPC-C 128), 1 op per thread, occupancy, 4 ways,
 * filter 1, dedupe 0, late_reads 0.  The reference fixes its block sizes at
 * compile time (TF/Predefine.h:36-46) and sweeps them with scripts; here the
 * autotuner (ltpg_gb300/tune.py) searches them per workload.
 * late_reads (YCSB, strides <= 32): the execute kernel only registers; the
 * check kernel reads the rows of committed transactions once their commit
 * decision is made, and a third kernel stores the updates.  Commit decisions,
 * the table image and the results of committed transactions are unchanged;
 * an aborted transaction's result is 0 (its reads are void: it runs again in
 * a later batch).  It saves the row reads of aborted transactions. */
typedef struct {
    uint32_t block_threads;   /* threads per block of the tuned kernels: 128, 256
                                 or 512 (TPC-C: tiles of 64, 128 or 256
                                 transactions)                                  */
    uint32_t ops_per_thread;  /* YCSB op words per thread: 1, 2, 4 or 8         */
    uint32_t blocks_per_sm;   /* cap on resident blocks per SM, 0 = occupancy   */
    uint32_t stage_ways;      /* shared-memory staging entries per hot bucket   */
    uint32_t filter;          /* 1 = read the slot before its atomicMin         */
    uint32_t dedupe;          /* 1 = one atomic per key per warp (match_any; TPC-C: header ops) */
    uint32_t late_reads;      /* YCSB: rows read after the check (see above):
                                 1 = in the check kernel's tiles, 2 = in a kernel
                                 of their own, 3 = write-first registration
                                 (updates register first; a read loads its
                                 key's slot only when an update writes the key) */
} ltpg_launch;
int ltpg_set_launch(ltpg_ctx *ctx, int workload, const ltpg_launch *cfg);
int ltpg_get_launch(ltpg_ctx *ctx, int workload, ltpg_launch *cfg);

/* ---- hot-key staging ----------------------------------------------------------
 * Keys hash into LTPG_STAGE_BUCKETS buckets (ltpg_key_bucket).  Registrations of
 * keys in a staged bucket are combined in shared memory per block and reach the
 * global slot table as one atomic per key and block; a staged key's row
 * checksum is kept with its entry, so later reads of it in the block skip the
 * row read.  The staged set is chosen
 * by the contention predictor or given here; it changes speed only, never a
 * commit decision.  n = 0 turns staging off.  At most
 * LTPG_STAGE_ENTRIES / stage_ways buckets are staged (extra ones are ignored). */
#define LTPG_STAGE_BUCKETS 65536u
#define LTPG_STAGE_ENTRIES 1024u
uint32_t ltpg_key_bucket(uint32_t key);
int ltpg_stage_set(ltpg_ctx *ctx, const uint32_t *buckets, uint32_t n);
/* Per-bucket registration counts accumulated by the tuned execute kernels
 * since the last reset (exact for staged buckets, sampled 1 in 16 and scaled
 * for the others): LTPG_STAGE_BUCKETS uint32 values. */
int ltpg_bucket_counts(ltpg_ctx *ctx, uint32_t *host_counts, int reset);

/* ---- contention predictor -----------------------------------------------------
 * A small MLP (4 -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation) predicts
 * each key-hash bucket's registration count in the next batch from its counts
 * in the last 4 batches, and its top buckets become the staged set.  It is
 * trained online on the GPU (one Adam step per batch on 4,096 buckets, label =
 * the latest batch's counts).  When enabled it runs after every tuned YCSB
 * batch (inside CUDA graphs too).  It changes which keys are staged, never a
 * commit decision.  No counterpart in the reference. */
typedef struct {
    uint32_t enable;       /* 0 turns the predictor and staging off            */
    uint32_t train;        /* 1 = train online, 0 = frozen weights            */
    uint32_t stage;        /* 1 = stage the predicted top buckets             */
    uint32_t train_every;  /* reserved, 1                                     */
    float lr;              /* Adam learning rate (default 3e-3)                */
    uint32_t pad;
    uint64_t seed;         /* initial weights                                  */
} ltpg_predictor_cfg;
#define LTPG_PRED_PARAMS 4545 /* packed FP32: W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3 */
int ltpg_predictor_enable(ltpg_ctx *ctx, const ltpg_predictor_cfg *cfg);
int ltpg_predictor_stats(ltpg_ctx *ctx, float *last_loss, uint64_t *train_steps);
int ltpg_predictor_get_params(ltpg_ctx *ctx, float *host, size_t n);
int ltpg_predictor_set_params(ltpg_ctx *ctx, const float *host, size_t n);
/* Test hooks: forward pass on given features (n <= 4096, [n][4] log1p counts),
 * and the gradient of mean((y - t)^2) with respect to the packed parameters. */
int ltpg_predictor_forward(ltpg_ctx *ctx, const float *host_x, uint32_t n, float *host_y);
int ltpg_predictor_gradients(ltpg_ctx *ctx, const float *host_x, const float *host_t, uint32_t n, float *host_grad);

/* ---- serving loop ---------------------------------------------------------------
 * Continuous batching over two engines, one holding the TPC-C tables and one
 * the YCSB table.  Requests arrive open-loop (Poisson at `rate` per second for
 * `duration_s`), tpcc_pct % TPC-C (drawn in order from a pool made by the
 * generator with *tp) and the rest YCSB (pool from *yp).  A batch closes at
 * max_batch requests or when its first request has waited deadline_ms, and
 * only when a device slot is free; the slots in flight are limited by the
 * engines' slots and by budget_bytes (registration tables + batch buffers).
 * The TPC-C and YCSB parts of a batch run concurrently on two streams and the
 * next batch's upload overlaps the current kernels.  Latency = arrival to the
 * commit bitmap in host memory, over committed requests.  No counterpart in
 * the reference.  With `record` non-null, the batch boundaries and
 * every request's flags and result are kept for replay (free with
 * ltpg_serve_record_free). */
typedef struct {
    double rate;            /* arrivals per second                       */
    double duration_s;      /* arrival window                            */
    double deadline_ms;     /* batch closing deadline (2.0)              */
    uint64_t budget_bytes;  /* device budget, 0 = no limit (40 GB)       */
    uint64_t seed;
    uint32_t max_batch;     /* batch closing size (262,144)              */
    uint32_t tpcc_pct;      /* share of TPC-C requests (70)              */
    uint32_t mode;          /* LTPG_MODE_PLAIN / FUSED / PERSISTENT (GRAPH
                               captures a graph per batch size)          */
    uint32_t slots;         /* batches in flight (<= engine slots)       */
} ltpg_serve_cfg;
typedef struct {
    uint64_t submitted, committed, batches, slots, waited_for_slot;
    double wall_s, throughput, mean_batch, mean_ms, p50_ms, p99_ms, p999_ms;
    /* where latency goes: mean wait of a request until its batch closes,
     * host time to pack and enqueue a batch, device time of a batch (copies,
     * kernels, bitmap download; the longer of its TPC-C and YCSB parts) */
    double wait_ms, launch_ms, device_ms;
} ltpg_serve_stats;
typedef struct ltpg_serve_record ltpg_serve_record;
/* The request loop over generated pools, driven by ltpg_serve_submit /
 * ltpg_serve_poll below: each request is submitted at its arrival time. */
int ltpg_serve_run(ltpg_ctx *tpcc_ctx, ltpg_ctx *ycsb_ctx, const ltpg_serve_cfg *cfg, const ltpg_tpcc_params *tp,
                   const ltpg_ycsb_params *yp, ltpg_serve_stats *out, ltpg_serve_record **record);

/* Serving caller-owned transactions.  Replaces the reference's host loop that
 * stages each batch through a 2-slot prefetch (TF/Query.h:526-605): requests
 * join the forming batch as they are submitted (packed into pinned staging at
 * once); a batch closes at max_batch requests, when its TPC-C order lines
 * would pass the engine's max_lines, or when its first request has waited
 * deadline_ms (checked by every submit and poll call); it is handed to the
 * two engines when a device slot is free (slots in flight are bounded by
 * `slots`, the engines' slots and budget_bytes), the TPC-C and YCSB parts on
 * streams of their own, so batches overlap on the device.  TIDs are positions
 * within a batch's part, in submission order.  A full batch with every slot
 * in flight makes submit wait for the oldest batch.  One driving thread per
 * server, as for a context; the server sets the contexts' streams while open.
 * Request ids count from 0 in submission order; batches complete in order, so
 * the finished requests are always a prefix of the ids. */
typedef struct ltpg_server ltpg_server;
typedef struct {
    double deadline_ms;     /* batch closing deadline (2.0)                          */
    uint64_t budget_bytes;  /* registration tables + batch buffers in flight, 0 = none */
    uint32_t max_batch;     /* batch closing size (<= both engines' max_txn)         */
    uint32_t mode;          /* LTPG_MODE_PLAIN / FUSED / PERSISTENT; GRAPH is
                               accepted but captures a graph per batch size, and
                               served batches vary in size                       */
    uint32_t slots;         /* batches in flight (<= the engines' slots)             */
    uint32_t ycsb_ops;      /* op words per YCSB transaction of a batch (<= the YCSB
                               engine's max_ops_per_txn); shorter requests are
                               padded                                                */
} ltpg_server_cfg;
typedef struct {
    int32_t workload;             /* LTPG_WORKLOAD_TPCC or LTPG_WORKLOAD_YCSB           */
    uint32_t n;                   /* TPC-C: order lines; YCSB: op words (1..ycsb_ops)  */
    const ltpg_tpcc_txn *txn;     /* TPC-C: the record (its line_off is ignored)        */
    const ltpg_tpcc_line *lines;  /* TPC-C: its n order lines                           */
    const uint32_t *ops;          /* YCSB: its n op words                               */
    const uint64_t *vals;         /* YCSB: one value per update, in op order            */
} ltpg_request;
int ltpg_server_open(ltpg_ctx *tpcc_ctx, ltpg_ctx *ycsb_ctx, const ltpg_server_cfg *cfg, ltpg_server **out);
/* Admits n requests (copied before return); their ids are *first_id .. + n-1. */
int ltpg_serve_submit(ltpg_server *s, const ltpg_request *reqs, uint32_t n, uint64_t *first_id);
/* Results of requests first_id .. first_id + n - 1: *n_done = how many of them,
 * from first_id on, have finished; their flags (LTPG_FLAG_*) and results are
 * written to flags[0 .. *n_done - 1] and results[...] (either may be NULL).  A
 * request's result is kept until a poll returns it, and ids below the lowest one
 * not yet returned are forgotten (LTPG_ERR_INVALID if asked for again). */
int ltpg_serve_poll(ltpg_server *s, uint64_t first_id, uint32_t n, uint8_t *flags, int64_t *results,
                    uint32_t *n_done);
/* Closes the forming batch now and waits until every batch has finished. */
int ltpg_serve_flush(ltpg_server *s);
/* Boundaries of the batches closed so far, in order: the first request id and
 * the number of requests of batch i (for replaying a batch alone). */
int ltpg_serve_batch_log(const ltpg_server *s, uint64_t *first_ids, uint32_t *counts, size_t cap, size_t *n_batches);
/* Flushes, restores the contexts' streams, frees the server; stats (optional)
 * over its life: latency = submit to results on the host, per committed request. */
int ltpg_server_close(ltpg_server *s, ltpg_serve_stats *stats);
/* Record: batches[4 * i .. 4 * i + 3] = TPC-C pool start, count, YCSB pool
 * start, count of batch i (pool index = order of arrival within the type). */
int ltpg_serve_record_sizes(const ltpg_serve_record *r, uint64_t *n_batches, uint64_t *n_tpcc, uint64_t *n_ycsb);
int ltpg_serve_record_get(const ltpg_serve_record *r, uint64_t *batches, uint8_t *tpcc_flags, int64_t *tpcc_results,
                          uint8_t *ycsb_flags, int64_t *ycsb_results);
int ltpg_serve_record_free(ltpg_serve_record *r);

/* ---- measurement ------------------------------------------------------------- */
/* Totals since ltpg_create: transactions committed (counted on the device by
 * the write-back kernels) and kernels launched by the engine (a graph launch
 * counts its kernels). */
int ltpg_counters(ltpg_ctx *ctx, uint64_t *commits_total, uint64_t *kernel_launches);
/* When on, every batch run records CUDA events around each of its kernels
 * (also inside captured graphs); ltpg_kernel_times writes the durations in
 * milliseconds of the last run of a slot into ms4 = [execute, check, reads,
 * write-back].  A phase that runs inside another kernel reads 0: the tuned
 * modes' check kernel also writes back ([execute, check+write-back, 0, 0]),
 * YCSB late reads in the check kernel give [execute, check+reads, 0,
 * write-back], and a persistent launch puts the whole batch under execute. */
int ltpg_set_profiling(ltpg_ctx *ctx, int on);
int ltpg_kernel_times(ltpg_ctx *ctx, uint32_t slot, float *ms4);

/* ---- no-allocation batch -------------------------------------------------------
 * This entry point has no counterpart in the reference.  It runs one whole YCSB
 * batch (execute+register, check, write-back) on buffers the caller owns, and
 * allocates no device memory.  It is for callers that cannot call cudaMalloc:
 * a host runtime that owns all of the GPU's memory through its own fixed pool
 * (a database or serving process), or a latency-critical thread, where
 * cudaMalloc / cudaFree may block and cudaFree synchronises the whole device.
 * All pointers are device pointers: rows (n_records x 10 uint64, updated in
 * place), the batch arrays in the layout of ltpg_ycsb_batch, and the outputs
 * flags[n_txn], bitmap[(n_txn+31)/32], results[n_txn].  stream may be NULL.
 * Scratch (the registration table) is a static device array sized for at most
 * LTPG_NOALLOC_MAX_RECORDS records (16 MiB), held on every GPU that loads the
 * library until exit; larger tables are rejected with LTPG_ERR_INVALID.  The
 * first call on a device sets that device up (it resolves the array's device
 * address and initialises it), so make that first call before any stream
 * capture.  All calls share the one scratch array, which keeps the previous
 * call's contents (calls are told apart by an epoch tag; when the epoch would
 * pass its last value, a call first sets the array back to its cleared state):
 * calls that overlap on the GPU race and give wrong results, so issue them one
 * at a time.  The call blocks: it synchronises `stream` and reads the device
 * error word before it returns, so the batch has finished on the GPU when it
 * returns.  LTPG_ERR_BOUNDS if a key was out of range (the batch's other
 * operations still run, as in ltpg_run_batch). */
#define LTPG_NOALLOC_MAX_RECORDS (1u << 20)
int ltpg_ycsb_batch_noalloc(int device, uint64_t *rows, uint64_t n_records, const uint32_t *ops,
                            const uint32_t *val_off, const uint64_t *vals, uint32_t n_txn,
                            uint32_t ops_per_txn, uint8_t *flags, uint32_t *bitmap, int64_t *results,
                            void *stream);

/* ---- test hooks ---------------------------------------------------------------
 * For tests of rare states; no counterpart in the reference.
 * Batch epochs: each batch runs at the next epoch (1 .. 0xFFFFFFFF), which tags
 * its registration slots so that the tables never need clearing.  Before a
 * launch would run a batch past the last epoch, the engine sets every slot back
 * to the cleared state and the epoch to 1 (the reference clears its 18 tables
 * every batch instead, TF/Database.h:78-102).  ltpg_debug_set_epoch makes the
 * next batch run at `epoch` (1 .. 0xFFFFFFFF), so a test can cross that point
 * in a few batches; ltpg_debug_get_epoch reads the device's current epoch.  The
 * _noalloc_ pair does the same for the no-allocation path of `device`.
 * ltpg_debug_barrier bounds every grid-barrier wait of the persistent kernels
 * by limit_ns (0 = the default, 2 s) and makes block `skip_block` of the next
 * persistent launches never arrive at a barrier (UINT32_MAX = none), so that
 * the other blocks' waits run out: the launch then ends with LTPG_ERR_TIMEOUT
 * at the next synchronising call, no table row written, and the context stays
 * usable (the reference's epoch loop only prints and stops, TF/tp.cu:159-164). */
int ltpg_debug_set_epoch(ltpg_ctx *ctx, uint32_t epoch);
int ltpg_debug_get_epoch(ltpg_ctx *ctx, uint32_t *epoch);
int ltpg_debug_noalloc_set_epoch(int device, uint32_t epoch);
int ltpg_debug_noalloc_get_epoch(int device, uint32_t *epoch);
int ltpg_debug_barrier(ltpg_ctx *ctx, uint64_t limit_ns, uint32_t skip_block);

/* ---- hashing used by generators and the table image --------------------- */
uint64_t ltpg_splitmix64(uint64_t x);
uint64_t ltpg_hash3(uint64_t seed, uint64_t a, uint64_t b);

#ifdef __cplusplus
}
#endif
#endif /* LTPG_H */
