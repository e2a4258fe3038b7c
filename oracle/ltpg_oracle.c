/*
 * ltpg_oracle.c — CPU replay of LTPG's batch concurrency-control protocol.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine: the
 * tests, the smoke check and the CPU-baseline leg of the benchmark call it; the
 * engine never does.  It restates the protocol independently of the engine's
 * sources and shares only the data formats of include/ltpg.h.
 *
 * Parity anchor: the reference has no CPU implementation, no tests and no
 * golden vectors; its kernels are the specification restated here:
 *   registration  atomicMin of the TID into the read / write table of the row
 *                 (TF/Genericfunction.h:108-251, Y1/Genericfunction.h:150-189)
 *   check         TID > registered minimum => conflict counter += 1
 *                 (TF/Genericfunction.h:252-414, Y1/Genericfunction.h:190-233)
 *                 reads check the write table (RAW), writes check the read
 *                 table (WAR) and the write table (WAW)
 *                 (Y1/Execute.h:109-150, TF/Execute_neworder.h:426-617,
 *                 TF/Execute_payment.h:390-536)
 *   commit        waw == 0 && (raw == 0 || war == 0)
 *                 (TF/Execute_neworder.h:692, TF/Execute_payment.h:607,
 *                 Y1/Execute.h:187)
 *   hot adds      warehouse / district YTD updates skip registration and check
 *                 ("isFrequent", TF/Execute_payment.h:86-99,144-163) and are
 *                 summed for committed Payments (intent of
 *                 TF/Genericfunction.h:431-518)
 * The values written and the per-transaction results are this project's
 * definitions (the reference writes back the values it loaded, so its image
 * never changes; TF/Genericfunction.h:93-107,416-430).
 * Pins: hand-derived known-answer batches in tests/golden/, and, on a GPU, the
 * commit sets of the reference's own kernels run on the same batches.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ltpg.h"

#define NONE 0xFFFFFFFFu

/* ---- hashing (splitmix64, Steele/Lea/Flood 2014) ------------------------ */
uint64_t oracle_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
uint64_t oracle_hash3(uint64_t seed, uint64_t a, uint64_t b) {
    return oracle_splitmix64(oracle_splitmix64(oracle_splitmix64(seed) ^ a) ^ b);
}

/* ====================================================================== */
/* YCSB (Y1/Execute.h)                                                    */
/* ====================================================================== */

void oracle_ycsb_init(uint64_t *rows, uint64_t n, uint64_t seed) {
    for (uint64_t k = 0; k < n; ++k)
        for (uint32_t f = 0; f < LTPG_YCSB_FIELDS; ++f) rows[k * LTPG_YCSB_FIELDS + f] = oracle_hash3(seed, k, f);
}

static inline int op_pad(uint32_t w) { return w == LTPG_YCSB_OP_PAD; }
static inline int op_upd(uint32_t w) { return (int)(w >> 31); }
static inline uint32_t op_key(uint32_t w) { return w & ((1u << LTPG_YCSB_KEY_BITS) - 1u); }
static inline uint32_t op_field(uint32_t w) { return (w >> 27) & 0xFu; }
/* Keys a read covers: key .. key + span within the table (a range scan when
   span > 0, Y2/Execute.h:24-32, where every read scans YCSB_SCAN_SIZE keys;
   its check tests Loc + 1 for every i, Y2/Execute.h:126-132, and checks
   nothing else — here every covered key is checked, as it is registered). */
static inline uint32_t op_last(uint32_t w, uint64_t n) {
    const uint64_t last = (uint64_t)op_key(w) + (op_upd(w) ? 0u : op_field(w));
    return (uint32_t)(last < n ? last : n - 1);
}

static inline uint32_t commit_rule(uint32_t f) {
    const int raw = (f & LTPG_FLAG_RAW) != 0, war = (f & LTPG_FLAG_WAR) != 0, waw = (f & LTPG_FLAG_WAW) != 0;
    return (!waw && (!raw || !war)) ? LTPG_FLAG_COMMIT : 0u;
}

/*
 * One YCSB batch, single-threaded.  reg_r / reg_w: scratch of n entries each
 * (contents ignored on entry).  Outputs: flags[B], bitmap[(B+31)/32],
 * results[B]; rows is updated in place.  Returns the commit count, or -1 if a
 * key is out of range.
 */
int64_t oracle_ycsb_batch(uint64_t *rows, uint64_t n, const ltpg_ycsb_batch *b, uint32_t *reg_r, uint32_t *reg_w,
                          uint8_t *flags, uint32_t *bitmap, int64_t *results) {
    const uint32_t B = b->n_txn, k = b->ops_per_txn, stride = b->op_stride;
    for (uint64_t i = 0; i < (uint64_t)B * stride; ++i) {
        const uint32_t w = b->ops[i];
        if (op_pad(w)) continue;
        if (op_key(w) >= n || (op_upd(w) && op_field(w) >= LTPG_YCSB_FIELDS)) return -1;
        for (uint32_t key = op_key(w); key <= op_last(w, n); ++key) reg_r[key] = reg_w[key] = NONE;
    }
    /* phase 1: register (smallest TID wins) and read the batch-start rows */
    for (uint32_t t = 0; t < B; ++t) {
        uint64_t dig = 0;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w)) continue;
            const uint32_t key = op_key(w);
            if (op_upd(w)) {
                if (t < reg_w[key]) reg_w[key] = t;
            } else {
                uint64_t x = 0;
                for (uint32_t q = key; q <= op_last(w, n); ++q) {
                    if (t < reg_r[q]) reg_r[q] = t;
                    for (uint32_t f = 0; f < LTPG_YCSB_FIELDS; ++f) x ^= rows[(uint64_t)q * LTPG_YCSB_FIELDS + f];
                }
                dig += x * (2ull * j + 1ull);
            }
        }
        results[t] = (int64_t)dig;
    }
    /* phase 2: check */
    int64_t commits = 0;
    memset(bitmap, 0, ((size_t)B + 31) / 32 * 4);
    for (uint32_t t = 0; t < B; ++t) {
        uint32_t f = 0;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w)) continue;
            const uint32_t key = op_key(w);
            if (op_upd(w)) {
                if (reg_r[key] < t) f |= LTPG_FLAG_WAR;
                if (reg_w[key] < t) f |= LTPG_FLAG_WAW;
            } else {
                for (uint32_t q = key; q <= op_last(w, n); ++q)
                    if (reg_w[q] < t) f |= LTPG_FLAG_RAW;
            }
        }
        f |= commit_rule(f);
        flags[t] = (uint8_t)f;
        if (f & LTPG_FLAG_COMMIT) {
            bitmap[t >> 5] |= 1u << (t & 31);
            ++commits;
        }
    }
    /* phase 3: write-back of committed updates, in TID order */
    for (uint32_t t = 0; t < B; ++t) {
        if (!(flags[t] & LTPG_FLAG_COMMIT)) continue;
        uint32_t v = b->val_off[t];
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w) || !op_upd(w)) continue;
            rows[(uint64_t)op_key(w) * LTPG_YCSB_FIELDS + op_field(w)] = b->vals[v++];
        }
    }
    return commits;
}

/* ---- multi-threaded replay (CPU baseline with all host threads) ------------ */
typedef struct {
    uint64_t *rows;
    uint64_t n;
    const ltpg_ycsb_batch *b;
    uint32_t *reg_r, *reg_w;
    uint8_t *flags;
    int64_t *results;
    uint32_t t0, t1;
    pthread_barrier_t *bar;
    int64_t commits;
} ymt_arg;

static inline void atomic_min_u32(uint32_t *p, uint32_t v) {
    uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

static void *ycsb_mt_worker(void *p) {
    ymt_arg *a = (ymt_arg *)p;
    const ltpg_ycsb_batch *b = a->b;
    const uint32_t k = b->ops_per_txn, stride = b->op_stride;
    for (uint64_t i = (uint64_t)a->t0 * stride; i < (uint64_t)a->t1 * stride; ++i) {
        const uint32_t w = b->ops[i];
        if (op_pad(w)) continue;
        for (uint32_t key = op_key(w); key <= op_last(w, a->n); ++key) {
            __atomic_store_n(&a->reg_r[key], NONE, __ATOMIC_RELAXED);
            __atomic_store_n(&a->reg_w[key], NONE, __ATOMIC_RELAXED);
        }
    }
    pthread_barrier_wait(a->bar);
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        uint64_t dig = 0;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w)) continue;
            const uint32_t key = op_key(w);
            if (op_upd(w)) {
                atomic_min_u32(&a->reg_w[key], t);
            } else {
                uint64_t x = 0;
                for (uint32_t q = key; q <= op_last(w, a->n); ++q) {
                    atomic_min_u32(&a->reg_r[q], t);
                    for (uint32_t f = 0; f < LTPG_YCSB_FIELDS; ++f)
                        x ^= a->rows[(uint64_t)q * LTPG_YCSB_FIELDS + f];
                }
                dig += x * (2ull * j + 1ull);
            }
        }
        a->results[t] = (int64_t)dig;
    }
    pthread_barrier_wait(a->bar);
    int64_t commits = 0;
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        uint32_t f = 0;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w)) continue;
            const uint32_t key = op_key(w);
            if (op_upd(w)) {
                if (__atomic_load_n(&a->reg_r[key], __ATOMIC_RELAXED) < t) f |= LTPG_FLAG_WAR;
                if (__atomic_load_n(&a->reg_w[key], __ATOMIC_RELAXED) < t) f |= LTPG_FLAG_WAW;
            } else {
                for (uint32_t q = key; q <= op_last(w, a->n); ++q)
                    if (__atomic_load_n(&a->reg_w[q], __ATOMIC_RELAXED) < t) f |= LTPG_FLAG_RAW;
            }
        }
        f |= commit_rule(f);
        a->flags[t] = (uint8_t)f;
        commits += (f & LTPG_FLAG_COMMIT) != 0;
    }
    a->commits = commits;
    pthread_barrier_wait(a->bar);
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        if (!(a->flags[t] & LTPG_FLAG_COMMIT)) continue;
        uint32_t v = b->val_off[t];
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t w = b->ops[(uint64_t)t * stride + j];
            if (op_pad(w) || !op_upd(w)) continue;
            a->rows[(uint64_t)op_key(w) * LTPG_YCSB_FIELDS + op_field(w)] = b->vals[v++];
        }
    }
    return NULL;
}

/* Same protocol on nthreads host threads (keys must already be validated). */
int64_t oracle_ycsb_batch_mt(uint64_t *rows, uint64_t n, const ltpg_ycsb_batch *b, uint32_t *reg_r,
                             uint32_t *reg_w, uint8_t *flags, int64_t *results, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    ymt_arg args[256];
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)nthreads);
    const uint32_t B = b->n_txn, chunk = (B + (uint32_t)nthreads - 1) / (uint32_t)nthreads;
    for (int i = 0; i < nthreads; ++i) {
        uint32_t t0 = (uint32_t)i * chunk, t1 = t0 + chunk;
        if (t0 > B) t0 = B;
        if (t1 > B) t1 = B;
        args[i] = (ymt_arg){rows, n, b, reg_r, reg_w, flags, results, t0, t1, &bar, 0};
        pthread_create(&th[i], NULL, ycsb_mt_worker, &args[i]);
    }
    int64_t commits = 0;
    for (int i = 0; i < nthreads; ++i) {
        pthread_join(th[i], NULL);
        commits += args[i].commits;
    }
    pthread_barrier_destroy(&bar);
    return commits;
}

/* ====================================================================== */
/* TPC-C NewOrder + Payment (TF/Execute_neworder.h, TF/Execute_payment.h) */
/* ====================================================================== */

static const uint32_t TCOLS[LTPG_TPCC_TABLES] = {9, 11, 21, 8, 3, 8, 10, 17, 5};

uint64_t oracle_tpcc_rows(uint32_t table, uint32_t W) {
    static const uint64_t per_w[LTPG_TPCC_TABLES] = {1, 10, 30000, 30000, 30000, 30000, 450000, 100000, 0};
    return table == LTPG_T_ITEM ? 100000ull : per_w[table] * W;
}
uint32_t oracle_tpcc_cols(uint32_t table) { return TCOLS[table]; }

/* Initial values: ids from the row number as TF/Database.h:104-327 builds
 * them, TPC-C starting values for the columns the executors use, hashes for
 * the rest. */
uint64_t oracle_tpcc_init_value(uint64_t seed, uint32_t table, uint64_t row, uint32_t col) {
    const uint64_t h = oracle_hash3(seed ^ (0x7C3A5E1Bull * (table + 1u)), row, col);
    switch (table) {
    case LTPG_T_WAREHOUSE:
        return col == 0 ? row : col == 1 ? h % 2001u : col == 2 ? 30000000ull : h;
    case LTPG_T_DISTRICT:
        return col == 0 ? row % 10 : col == 1 ? row / 10 : col == 2 ? h % 2001u : col == 3 ? 3000000ull
               : col == 4 ? 3000u : h;
    case LTPG_T_CUSTOMER:
        switch (col) {
        case 0: return row % 3000;
        case 1: return row / 30000;
        case 2: return (row / 3000) % 10;
        case 3: return 5000000ull;
        case 4: return h % 5001u;
        case 5: return (uint64_t)(int64_t)-1000;
        case 6: return 1000u;
        case 7: return 1u;
        case 8: return 0u;
        case 13: return h % 1000u;
        default: return h;
        }
    case LTPG_T_STOCK:
        switch (col) {
        case 0: return row % 100000;
        case 1: return row / 100000;
        case 2: return 10u + h % 91u;
        case 3: case 4: case 5: return 0u;
        default: return h;
        }
    case LTPG_T_ITEM:
        return col == 0 ? row : col == 1 ? 1u + h % 10000u : col == 2 ? 100u + h % 9901u : h;
    default:
        return h;
    }
}

void oracle_tpcc_init_table(uint64_t *tab, uint32_t table, uint32_t W, uint64_t seed) {
    const uint64_t rows = oracle_tpcc_rows(table, W);
    const uint32_t cols = TCOLS[table];
    for (uint64_t r = 0; r < rows; ++r)
        for (uint32_t c = 0; c < cols; ++c) tab[r * cols + c] = oracle_tpcc_init_value(seed, table, r, c);
}

enum { R_REG = 1, W_REG = 2, C_RAW = 4, C_WAR = 8, C_WAW = 16 };
#define OP_READ (R_REG | C_RAW)
#define OP_WRITE (W_REG | C_WAR | C_WAW)

typedef struct {
    uint32_t table;
    uint64_t row;
    uint32_t flags;
} cc_op;

static inline uint32_t k_kind(uint32_t ki) { return ki & 0xFFu; }
static inline uint32_t k_cnt(uint32_t ki) { return (ki >> 8) & 0xFFu; }
static inline uint32_t k_d(uint32_t ki) { return (ki >> 16) & 0xFFu; }
static inline uint32_t k_cd(uint32_t ki) { return (ki >> 24) & 0xFFu; }
static inline int64_t amount_of(const ltpg_tpcc_txn *x) { return (int64_t)(((uint64_t)x->c << 32) | x->b); }

/* Concurrency-control ops of one transaction, in the order of the reference's
 * op_k_0 functions; returns their number, or -1 for an invalid record. */
static int txn_ops(const ltpg_tpcc_txn *x, const ltpg_tpcc_line *lines, uint32_t n_lines, uint32_t W, int strict,
                   cc_op *ops) {
    const uint32_t d = k_d(x->kind_info);
    if (x->w >= W || d >= 10 || x->c_id >= 3000) return -1;
    if (k_kind(x->kind_info) == LTPG_TPCC_NEWORDER) {
        const uint32_t cnt = k_cnt(x->kind_info);
        if (cnt > LTPG_TPCC_MAX_LINES || x->a >= 30000 || x->b >= 30000 || x->c >= 450000 ||
            (uint64_t)x->line_off + cnt > n_lines)
            return -1;
        int m = 0;
        /* op_0_0 select warehouse: read (TF/Execute_neworder.h:14-29, check_0_0 RAW :426-438) */
        ops[m++] = (cc_op){LTPG_T_WAREHOUSE, x->w, OP_READ};
        /* op_1_0 select district (:41-57, check_1_0 RAW :439-451) */
        ops[m++] = (cc_op){LTPG_T_DISTRICT, 10ull * x->w + d, OP_READ};
        /* op_2_0 select customer (:71-87, check_2_0 RAW :452-464) */
        ops[m++] = (cc_op){LTPG_T_CUSTOMER, 30000ull * x->w + 3000ull * d + x->c_id, OP_READ};
        /* op_3_0 insert NEW-ORDER: registered READ (:103-118); only check_3_1
           (WAW, :478-490) is dispatched, check_3_0 never is (:639-646) */
        ops[m++] = (cc_op){LTPG_T_NEWORDER, 30000ull * x->w + x->b, strict ? OP_WRITE : (R_REG | C_WAW)};
        /* op_4_0 insert ORDER: write (:133-148, check_4_0 WAR / check_4_1 WAW :491-516) */
        ops[m++] = (cc_op){LTPG_T_ORDER, 30000ull * x->w + x->a, OP_WRITE};
        for (uint32_t i = 0; i < cnt; ++i) {
            const ltpg_tpcc_line *ln = &lines[x->line_off + i];
            if (ln->i_id >= 100000 || ln->supply_w >= W) return -1;
            /* op_5_0 select item (:163-184, check_5_0 RAW :517-536) */
            ops[m++] = (cc_op){LTPG_T_ITEM, ln->i_id, OP_READ};
            /* op_6_0 update stock (:205-227, check_6_0 WAR / check_6_1 WAW :537-576) */
            ops[m++] = (cc_op){LTPG_T_STOCK, 100000ull * ln->supply_w + ln->i_id, OP_WRITE};
            /* op_7_0 insert ORDER-LINE (:249-273, check_7_0 WAR / check_7_1 WAW :577-617);
               the OL_ID wraps per line inside the warehouse's range */
            ops[m++] = (cc_op){LTPG_T_ORDERLINE, 450000ull * x->w + (x->c + i) % 450000u, OP_WRITE};
        }
        return m;
    }
    if (k_kind(x->kind_info) == LTPG_TPCC_ORDERSTATUS) {
        /* TA/Execute.h:1592-1770: select customer, order, order line */
        const uint32_t c_d = k_cd(x->kind_info);
        if (x->c_w >= W || c_d >= 10 || x->a >= 30000 || x->b >= 450000) return -1;
        ops[0] = (cc_op){LTPG_T_CUSTOMER, 30000ull * x->c_w + 3000ull * c_d + x->c_id, OP_READ};
        ops[1] = (cc_op){LTPG_T_ORDER, 30000ull * x->w + x->a, OP_READ};
        ops[2] = (cc_op){LTPG_T_ORDERLINE, 450000ull * x->w + x->b, OP_READ};
        return 3;
    }
    if (k_kind(x->kind_info) == LTPG_TPCC_DELIVERY) {
        /* TA/Execute.h:1772-2153: delete NEW-ORDER, select + update ORDER,
           update + select ORDER-LINE, update customer (a row read and updated
           registers and checks as both) */
        const uint32_t carrier = k_cnt(x->kind_info);
        if (x->a >= 30000 || x->b >= 30000 || x->c >= 450000 || carrier < 1 || carrier > 10) return -1;
        ops[0] = (cc_op){LTPG_T_NEWORDER, 30000ull * x->w + x->b, OP_WRITE};
        ops[1] = (cc_op){LTPG_T_ORDER, 30000ull * x->w + x->a, OP_READ | OP_WRITE};
        ops[2] = (cc_op){LTPG_T_ORDERLINE, 450000ull * x->w + x->c, OP_READ | OP_WRITE};
        ops[3] = (cc_op){LTPG_T_CUSTOMER, 30000ull * x->w + 3000ull * d + x->c_id, OP_WRITE};
        return 4;
    }
    if (k_kind(x->kind_info) == LTPG_TPCC_STOCKLEVEL) {
        /* TA/Execute.h:2155-2231: select stock */
        if (x->a >= 100000) return -1;
        ops[0] = (cc_op){LTPG_T_STOCK, 100000ull * x->w + x->a, OP_READ};
        return 1;
    }
    if (k_kind(x->kind_info) != LTPG_TPCC_PAYMENT) return -1;
    const uint32_t c_d = k_cd(x->kind_info);
    if (x->c_w >= W || c_d >= 10 || x->a >= 30000) return -1;
    const uint64_t crow = 30000ull * x->c_w + 3000ull * c_d + x->c_id;
    /* op_0_0 select warehouse (TF/Execute_payment.h:39-53, check_0_0 RAW :390-402) */
    ops[0] = (cc_op){LTPG_T_WAREHOUSE, x->w, OP_READ};
    /* op_1_0 update warehouse: hot, no registration, check with isFrequent=1
       finds no TID (:80-99, :403-430) — not a cc op */
    /* op_2_0 select district (:100-115, check_2_0 RAW :431-443) */
    ops[1] = (cc_op){LTPG_T_DISTRICT, 10ull * x->w + k_d(x->kind_info), OP_READ};
    /* op_3_0 update district: hot (:144-163) — not a cc op */
    /* op_4_0 select customer (:164-180, check_4_0 RAW :472-484) */
    ops[2] = (cc_op){LTPG_T_CUSTOMER, crow, OP_READ};
    /* op_5_0 update customer (:241-257, check_5_0 WAR / check_5_1 WAW :485-510) */
    ops[3] = (cc_op){LTPG_T_CUSTOMER, crow, OP_WRITE};
    /* op_6_0 insert HISTORY (:272-289, check_6_0 WAR / check_6_1 WAW :511-536) */
    ops[4] = (cc_op){LTPG_T_HISTORY, 30000ull * x->w + x->a, OP_WRITE};
    return 5;
}

static inline uint64_t *colp(uint64_t **tab, uint32_t table, uint64_t row, uint32_t col) {
    return tab[table] + row * TCOLS[table] + col;
}

/*
 * Payment by customer last name (LTPG_PAY_BY_NAME): c_id holds the query word
 * (name << 8) | nth of the reference's PAYMENT_QUERY.C_LAST (TF/Query.h:176-181).
 * Default rule: the nth (0-based) customer of the district whose C_LAST column
 * equals name, in C_ID order — a linear scan here (the engine uses a sorted
 * per-district index).  Returns 0 when there is no such customer.
 */
static int name_lookup(uint64_t **tab, uint32_t w, uint32_t d, uint32_t name, uint32_t nth, uint32_t *cid) {
    const uint64_t dist = 30000ull * w + 3000ull * d;
    uint32_t seen = 0;
    for (uint32_t c = 0; c < 3000; ++c) {
        if (*colp(tab, LTPG_T_CUSTOMER, dist + c, 13) != (uint64_t)name) continue;
        if (seen++ == nth) {
            *cid = c;
            return 1;
        }
    }
    return 0;
}

/*
 * LTPG_CFG_REF_NAME_LOOKUP: __FIND_CID_INDEX (TF/Genericfunction.h:29-77) as
 * lane 0 of its warp computes it.  Its shuffle `__shfl_sync(.., tmp, i)` takes
 * the loop index as source lane, i.e. the lane itself (i = lane + 32k), so
 * count = 32 * tmp: lane 0 tests positions 0, 32, 64, ... (:42-52), adding 32
 * per match, and stops once the sum reaches nth (:53-56, flag = 32 per
 * iteration).  Only lane 0 finishes (:59): walking back from flag - 1 down to 1
 * over positions holding name, it stops where the sum equals nth and
 * decrements it otherwise (:61-71); C_ID is column 0 of that row (:72), or 0
 * if the walk found nothing or the sum never reached nth (:37).  Positions past
 * the district read the next district, as the reference's flat index does;
 * past the table nothing matches (the reference reads past its array there).
 */
static uint32_t ref_name_lookup(uint64_t **tab, uint32_t W, uint32_t w, uint32_t d, uint32_t name, uint32_t nth) {
    const uint64_t dist = 30000ull * w + 3000ull * d, rows = 30000ull * W;
#define NAME_AT(row) ((row) < rows && *colp(tab, LTPG_T_CUSTOMER, (row), 13) == (uint64_t)name)
    uint32_t cum = 0, flag = 0;
    for (uint32_t i = 0; i < 3000; i += 32) {
        cum += NAME_AT(dist + i) ? 32u : 0u;
        flag += 32;
        if (cum >= nth) break;
    }
    if (cum < nth) return 0;
    uint64_t result = 0;
    for (uint32_t i = flag - 1; i > 0; --i) {
        if (!NAME_AT(dist + i)) continue;
        if (cum == nth) {
            result = dist + i;
            break;
        }
        --cum;
    }
#undef NAME_AT
    return (uint32_t)*colp(tab, LTPG_T_CUSTOMER, result, 0);
}

/*
 * One TPC-C batch, single-threaded.  tab[9]: the nine tables (updated in
 * place).  reg_r / reg_w: scratch indexed by (table, row), sized by
 * oracle_tpcc_slots(W).  Returns the commit count or -1 for an invalid batch.
 */
uint64_t oracle_tpcc_slots(uint32_t W) {
    uint64_t s = 0;
    for (uint32_t t = 0; t < LTPG_TPCC_TABLES; ++t) s += oracle_tpcc_rows(t, W);
    return s;
}

static int64_t tpcc_batch_resolved(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, const uint8_t *nf,
                                   int strict, uint32_t *reg_r, uint32_t *reg_w, uint8_t *flags, uint32_t *bitmap,
                                   int64_t *results);

/* The customer of every transaction after by-name resolution: cid[t] (the
 * record's c_id when it is not a by-name Payment) and found[t]. */
void oracle_tpcc_resolve(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, int cfg_flags, uint32_t *cid,
                         uint8_t *found) {
    for (uint32_t t = 0; t < b->n_txn; ++t) {
        const ltpg_tpcc_txn *x = &b->txns[t];
        const uint32_t c_d = k_cd(x->kind_info);
        cid[t] = x->c_id;
        found[t] = 1;
        if ((k_kind(x->kind_info) == LTPG_TPCC_PAYMENT || k_kind(x->kind_info) == LTPG_TPCC_ORDERSTATUS) &&
            (x->kind_info & LTPG_PAY_BY_NAME) && x->c_w < W && c_d < 10) {
            const uint32_t name = x->c_id >> 8, nth = x->c_id & 0xFFu;
            if (cfg_flags & LTPG_CFG_REF_NAME_LOOKUP) cid[t] = ref_name_lookup(tab, W, x->c_w, c_d, name, nth);
            else found[t] = (uint8_t)name_lookup(tab, x->c_w, c_d, name, nth, &cid[t]);
        }
    }
}

/* The records with by-name customers resolved (rx) and the not-found marks. */
static void tpcc_resolve_into(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, int cfg_flags, ltpg_tpcc_txn *rx,
                              uint8_t *nf) {
    for (uint32_t t = 0; t < b->n_txn; ++t) {
        ltpg_tpcc_txn x = b->txns[t];
        const uint32_t c_d = k_cd(x.kind_info);
        if ((k_kind(x.kind_info) == LTPG_TPCC_PAYMENT || k_kind(x.kind_info) == LTPG_TPCC_ORDERSTATUS) &&
            (x.kind_info & LTPG_PAY_BY_NAME) && x.c_w < W && c_d < 10) {
            const uint32_t name = x.c_id >> 8, nth = x.c_id & 0xFFu;
            if (cfg_flags & LTPG_CFG_REF_NAME_LOOKUP) x.c_id = ref_name_lookup(tab, W, x.c_w, c_d, name, nth);
            else if (!name_lookup(tab, x.c_w, c_d, name, nth, &x.c_id)) nf[t] = 1;
        }
        rx[t] = x;
    }
}

int64_t oracle_tpcc_batch(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, int cfg_flags, uint32_t *reg_r,
                          uint32_t *reg_w, uint8_t *flags, uint32_t *bitmap, int64_t *results) {
    /* resolve by-name Payments first (the reference's KERNEL_CID pre-phase,
       TF/tp.cu:11-23), into a copy of the records */
    const uint32_t B = b->n_txn;
    ltpg_tpcc_txn *rx = (ltpg_tpcc_txn *)malloc((size_t)(B ? B : 1) * sizeof *rx);
    uint8_t *nf = (uint8_t *)calloc(B ? B : 1, 1);
    if (!rx || !nf) {
        free(rx);
        free(nf);
        return -1;
    }
    tpcc_resolve_into(tab, W, b, cfg_flags, rx, nf);
    ltpg_tpcc_batch rb = *b;
    rb.txns = rx;
    const int64_t r = tpcc_batch_resolved(tab, W, &rb, nf, cfg_flags & LTPG_CFG_STRICT_INSERT, reg_r, reg_w, flags,
                                          bitmap, results);
    free(rx);
    free(nf);
    return r;
}

/* One transaction's registrations and execute-phase reads (its result).
   atomic: concurrent registration by several threads. */
static void tpcc_exec_one(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, int strict, const uint64_t *base,
                          uint32_t *reg_r, uint32_t *reg_w, int64_t *results, uint32_t t, int atomic) {
    cc_op ops[5 + 3 * LTPG_TPCC_MAX_LINES];
    const ltpg_tpcc_txn *x = &b->txns[t];
    const int m = txn_ops(x, b->lines, b->n_lines, W, strict, ops);
    for (int j = 0; j < m; ++j) {
        const uint64_t s = base[ops[j].table] + ops[j].row;
        if (atomic) {
            if (ops[j].flags & R_REG) atomic_min_u32(&reg_r[s], t);
            if (ops[j].flags & W_REG) atomic_min_u32(&reg_w[s], t);
        } else {
            if ((ops[j].flags & R_REG) && t < reg_r[s]) reg_r[s] = t;
            if ((ops[j].flags & W_REG) && t < reg_w[s]) reg_w[s] = t;
        }
    }
    const uint32_t d = k_d(x->kind_info);
    if (k_kind(x->kind_info) == LTPG_TPCC_NEWORDER) {
        int64_t sum = 0;
        for (uint32_t i = 0; i < k_cnt(x->kind_info); ++i) {
            const ltpg_tpcc_line *ln = &b->lines[x->line_off + i];
            sum += (int64_t)ln->qty * (int64_t)*colp(tab, LTPG_T_ITEM, ln->i_id, 2);
        }
        const int64_t disc = (int64_t)*colp(tab, LTPG_T_CUSTOMER, 30000ull * x->w + 3000ull * d + x->c_id, 4);
        const int64_t wtax = (int64_t)*colp(tab, LTPG_T_WAREHOUSE, x->w, 1);
        const int64_t dtax = (int64_t)*colp(tab, LTPG_T_DISTRICT, 10ull * x->w + d, 2);
        results[t] = sum * (10000 - disc) * (10000 + wtax + dtax) / 100000000;
    } else if (k_kind(x->kind_info) == LTPG_TPCC_PAYMENT) {
        const uint64_t crow = 30000ull * x->c_w + 3000ull * k_cd(x->kind_info) + x->c_id;
        results[t] = (int64_t)*colp(tab, LTPG_T_CUSTOMER, crow, 5) - amount_of(x);
    } else if (k_kind(x->kind_info) == LTPG_TPCC_ORDERSTATUS) {  /* C_BALANCE */
        const uint64_t crow = 30000ull * x->c_w + 3000ull * k_cd(x->kind_info) + x->c_id;
        results[t] = (int64_t)*colp(tab, LTPG_T_CUSTOMER, crow, 5);
    } else if (k_kind(x->kind_info) == LTPG_TPCC_DELIVERY) {  /* the line's OL_AMOUNT */
        results[t] = (int64_t)*colp(tab, LTPG_T_ORDERLINE, 450000ull * x->w + x->c, 8);
    } else {  /* StockLevel: S_QUANTITY */
        results[t] = (int64_t)*colp(tab, LTPG_T_STOCK, 100000ull * x->w + x->a, 2);
    }
}

/* One transaction's conflict flags and commit bit. */
static uint32_t tpcc_check_one(uint32_t W, const ltpg_tpcc_batch *b, int strict, const uint64_t *base,
                               const uint32_t *reg_r, const uint32_t *reg_w, uint32_t t) {
    cc_op ops[5 + 3 * LTPG_TPCC_MAX_LINES];
    const int m = txn_ops(&b->txns[t], b->lines, b->n_lines, W, strict, ops);
    uint32_t f = 0;
    for (int j = 0; j < m; ++j) {
        const uint64_t s = base[ops[j].table] + ops[j].row;
        if ((ops[j].flags & C_RAW) && reg_w[s] < t) f |= LTPG_FLAG_RAW;
        if ((ops[j].flags & C_WAR) && reg_r[s] < t) f |= LTPG_FLAG_WAR;
        if ((ops[j].flags & C_WAW) && reg_w[s] < t) f |= LTPG_FLAG_WAW;
    }
    return f | commit_rule(f);
}

/* Write-back of one committed transaction.  atomic: the warehouse / district
   YTD adds (the only rows several committed transactions write) are atomic. */
static void tpcc_write_one(uint64_t **tab, const ltpg_tpcc_batch *b, const int64_t *results, uint32_t t,
                           int atomic) {
    const ltpg_tpcc_txn *x = &b->txns[t];
    const uint32_t d = k_d(x->kind_info);
    const uint64_t date = b->txn_base + t;
    if (k_kind(x->kind_info) == LTPG_TPCC_NEWORDER) {
        const uint32_t cnt = k_cnt(x->kind_info);
        int all_local = 1;
        for (uint32_t i = 0; i < cnt; ++i) {
            const ltpg_tpcc_line *ln = &b->lines[x->line_off + i];
            const uint64_t srow = 100000ull * ln->supply_w + ln->i_id;
            all_local &= ln->supply_w == x->w;
            uint64_t *s = colp(tab, LTPG_T_STOCK, srow, 0);
            /* S_QUANTITY rule of TPC-C clause 2.4.2.2 */
            s[2] = s[2] >= (uint64_t)ln->qty + 10u ? s[2] - ln->qty : s[2] - ln->qty + 91u;
            s[3] += ln->qty;
            s[4] += 1;
            s[5] += ln->supply_w != x->w;
            uint64_t *o = colp(tab, LTPG_T_ORDERLINE, 450000ull * x->w + (x->c + i) % 450000u, 0);
            o[0] = x->a; o[1] = d; o[2] = x->w; o[3] = i + 1; o[4] = ln->i_id; o[5] = ln->supply_w;
            o[6] = 0; o[7] = ln->qty; o[8] = (uint64_t)ln->qty * *colp(tab, LTPG_T_ITEM, ln->i_id, 2);
            o[9] = *colp(tab, LTPG_T_STOCK, srow, 6 + d);
        }
        uint64_t *o = colp(tab, LTPG_T_ORDER, 30000ull * x->w + x->a, 0);
        o[0] = x->a; o[1] = d; o[2] = x->w; o[3] = x->c_id; o[4] = date; o[5] = 0; o[6] = cnt;
        o[7] = (uint64_t)all_local;
        uint64_t *no = colp(tab, LTPG_T_NEWORDER, 30000ull * x->w + x->b, 0);
        no[0] = x->a; no[1] = d; no[2] = x->w;
    } else if (k_kind(x->kind_info) == LTPG_TPCC_DELIVERY) {
        uint64_t *no = colp(tab, LTPG_T_NEWORDER, 30000ull * x->w + x->b, 0);
        no[0] = no[1] = no[2] = ~0ull; /* deleted */
        *colp(tab, LTPG_T_ORDER, 30000ull * x->w + x->a, 5) = k_cnt(x->kind_info);   /* O_CARRIER_ID */
        *colp(tab, LTPG_T_ORDERLINE, 450000ull * x->w + x->c, 6) = date;              /* OL_DELIVERY_D */
        uint64_t *c = colp(tab, LTPG_T_CUSTOMER, 30000ull * x->w + 3000ull * d + x->c_id, 0);
        c[5] = (uint64_t)((int64_t)c[5] + results[t]);                                 /* C_BALANCE */
        c[8] += 1;                                                                     /* C_DELIVERY_CNT */
    } else if (k_kind(x->kind_info) != LTPG_TPCC_PAYMENT) {
        /* OrderStatus, StockLevel: read-only */
    } else {
        const int64_t amt = amount_of(x);
        const uint32_t c_d = k_cd(x->kind_info);
        uint64_t *wy = colp(tab, LTPG_T_WAREHOUSE, x->w, 2), *dy = colp(tab, LTPG_T_DISTRICT, 10ull * x->w + d, 3);
        if (atomic) {
            __atomic_fetch_add(wy, (uint64_t)amt, __ATOMIC_RELAXED);
            __atomic_fetch_add(dy, (uint64_t)amt, __ATOMIC_RELAXED);
        } else {
            *wy += (uint64_t)amt;
            *dy += (uint64_t)amt;
        }
        uint64_t *c = colp(tab, LTPG_T_CUSTOMER, 30000ull * x->c_w + 3000ull * c_d + x->c_id, 0);
        c[5] = (uint64_t)((int64_t)c[5] - amt);
        c[6] = (uint64_t)((int64_t)c[6] + amt);
        c[7] += 1;
        uint64_t *h = colp(tab, LTPG_T_HISTORY, 30000ull * x->w + x->a, 0);
        h[0] = x->c_id; h[1] = c_d; h[2] = x->c_w; h[3] = d; h[4] = x->w; h[5] = (uint64_t)amt; h[6] = date;
        h[7] = 0;
    }
}

static void tpcc_bases(uint32_t W, uint64_t *base) {
    uint64_t acc = 0;
    for (uint32_t t = 0; t < LTPG_TPCC_TABLES; ++t) {
        base[t] = acc;
        acc += oracle_tpcc_rows(t, W);
    }
}

static int64_t tpcc_batch_resolved(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, const uint8_t *nf,
                                   int strict, uint32_t *reg_r, uint32_t *reg_w, uint8_t *flags, uint32_t *bitmap,
                                   int64_t *results) {
    uint64_t base[LTPG_TPCC_TABLES];
    tpcc_bases(W, base);
    cc_op ops[5 + 3 * LTPG_TPCC_MAX_LINES];
    const uint32_t B = b->n_txn;
    /* validate and clear the touched slots */
    for (uint32_t t = 0; t < B; ++t) {
        if (nf[t]) continue;
        const int m = txn_ops(&b->txns[t], b->lines, b->n_lines, W, strict, ops);
        if (m < 0) return -1;
        for (int j = 0; j < m; ++j) reg_r[base[ops[j].table] + ops[j].row] = reg_w[base[ops[j].table] + ops[j].row] = NONE;
    }
    /* phase 1: register + reads of the execute phase */
    for (uint32_t t = 0; t < B; ++t) {
        if (nf[t]) results[t] = 0;
        else tpcc_exec_one(tab, W, b, strict, base, reg_r, reg_w, results, t, 0);
    }
    /* phase 2: check */
    int64_t commits = 0;
    memset(bitmap, 0, ((size_t)B + 31) / 32 * 4);
    for (uint32_t t = 0; t < B; ++t) {
        if (nf[t]) {
            flags[t] = LTPG_FLAG_NOT_FOUND;
            continue;
        }
        const uint32_t f = tpcc_check_one(W, b, strict, base, reg_r, reg_w, t);
        flags[t] = (uint8_t)f;
        if (f & LTPG_FLAG_COMMIT) {
            bitmap[t >> 5] |= 1u << (t & 31);
            ++commits;
        }
    }
    /* phase 3: write-back of committed transactions in TID order */
    for (uint32_t t = 0; t < B; ++t)
        if (flags[t] & LTPG_FLAG_COMMIT) tpcc_write_one(tab, b, results, t, 0);
    return commits;
}

/* ---- multi-threaded TPC-C replay (CPU baseline with all host threads) ----
   The same phases on nthreads threads, a barrier between them.  Registration
   is an atomic minimum; write-back order does not matter: every row but the
   warehouse / district YTD (atomic adds) has at most one committed writer,
   and the columns write-back reads (item price, S_DIST_xx) are never
   written. */
typedef struct {
    uint64_t **tab;
    uint32_t W;
    const ltpg_tpcc_batch *b;
    const uint8_t *nf;
    int strict;
    const uint64_t *base;
    uint32_t *reg_r, *reg_w;
    uint8_t *flags;
    uint32_t *bitmap;
    int64_t *results;
    uint32_t t0, t1;
    pthread_barrier_t *bar;
    int *err;
    int64_t commits;
} tmt_arg;

static void *tpcc_mt_worker(void *p) {
    tmt_arg *a = (tmt_arg *)p;
    cc_op ops[5 + 3 * LTPG_TPCC_MAX_LINES];
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        if (a->nf[t]) continue;
        const int m = txn_ops(&a->b->txns[t], a->b->lines, a->b->n_lines, a->W, a->strict, ops);
        if (m < 0) {
            __atomic_store_n(a->err, 1, __ATOMIC_RELAXED);
            break;
        }
        for (int j = 0; j < m; ++j) {
            const uint64_t s = a->base[ops[j].table] + ops[j].row;
            __atomic_store_n(&a->reg_r[s], NONE, __ATOMIC_RELAXED);
            __atomic_store_n(&a->reg_w[s], NONE, __ATOMIC_RELAXED);
        }
    }
    pthread_barrier_wait(a->bar);
    if (__atomic_load_n(a->err, __ATOMIC_RELAXED)) return NULL;
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        if (a->nf[t]) a->results[t] = 0;
        else tpcc_exec_one(a->tab, a->W, a->b, a->strict, a->base, a->reg_r, a->reg_w, a->results, t, 1);
    }
    pthread_barrier_wait(a->bar);
    int64_t commits = 0;
    for (uint32_t t = a->t0; t < a->t1; ++t) {
        if (a->nf[t]) {
            a->flags[t] = LTPG_FLAG_NOT_FOUND;
            continue;
        }
        const uint32_t f = tpcc_check_one(a->W, a->b, a->strict, a->base, a->reg_r, a->reg_w, t);
        a->flags[t] = (uint8_t)f;
        if (f & LTPG_FLAG_COMMIT) {
            __atomic_fetch_or(&a->bitmap[t >> 5], 1u << (t & 31), __ATOMIC_RELAXED);
            ++commits;
        }
    }
    a->commits = commits;
    pthread_barrier_wait(a->bar);
    for (uint32_t t = a->t0; t < a->t1; ++t)
        if (a->flags[t] & LTPG_FLAG_COMMIT) tpcc_write_one(a->tab, a->b, a->results, t, 1);
    return NULL;
}

/* oracle_tpcc_batch on nthreads host threads: the same outputs and image. */
int64_t oracle_tpcc_batch_mt(uint64_t **tab, uint32_t W, const ltpg_tpcc_batch *b, int cfg_flags, uint32_t *reg_r,
                             uint32_t *reg_w, uint8_t *flags, uint32_t *bitmap, int64_t *results, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    const uint32_t B = b->n_txn;
    ltpg_tpcc_txn *rx = (ltpg_tpcc_txn *)malloc((size_t)(B ? B : 1) * sizeof *rx);
    uint8_t *nf = (uint8_t *)calloc(B ? B : 1, 1);
    if (!rx || !nf) {
        free(rx);
        free(nf);
        return -1;
    }
    tpcc_resolve_into(tab, W, b, cfg_flags, rx, nf);
    ltpg_tpcc_batch rb = *b;
    rb.txns = rx;
    uint64_t base[LTPG_TPCC_TABLES];
    tpcc_bases(W, base);
    memset(bitmap, 0, ((size_t)B + 31) / 32 * 4);
    pthread_t th[256];
    tmt_arg args[256];
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)nthreads);
    int err = 0;
    const uint32_t chunk = (B + (uint32_t)nthreads - 1) / (uint32_t)nthreads;
    for (int i = 0; i < nthreads; ++i) {
        uint32_t t0 = (uint32_t)i * chunk, t1 = t0 + chunk;
        if (t0 > B) t0 = B;
        if (t1 > B) t1 = B;
        args[i] = (tmt_arg){tab, W, &rb, nf, cfg_flags & LTPG_CFG_STRICT_INSERT, base, reg_r, reg_w, flags,
                            bitmap, results, t0, t1, &bar, &err, 0};
        pthread_create(&th[i], NULL, tpcc_mt_worker, &args[i]);
    }
    int64_t commits = 0;
    for (int i = 0; i < nthreads; ++i) {
        pthread_join(th[i], NULL);
        commits += args[i].commits;
    }
    pthread_barrier_destroy(&bar);
    free(rx);
    free(nf);
    return err ? -1 : commits;
}
