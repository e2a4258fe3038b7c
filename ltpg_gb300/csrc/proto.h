// proto.h — protocol constants and pure functions shared by host and device code.
//
// Everything here is integer arithmetic with one definition for the generator,
// the kernels and the host checks, so the three cannot drift apart.
#pragma once
#include <stdint.h>
#include "../../include/ltpg.h"

#if defined(__CUDACC__)
#define LTPG_HD __host__ __device__ __forceinline__
#else
#define LTPG_HD static inline
#endif

namespace ltpg {

// ---- hashing ----------------------------------------------------------------
// splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): one step from state x.
LTPG_HD uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
LTPG_HD uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
    return splitmix64(splitmix64(splitmix64(seed) ^ a) ^ b);
}

// ---- registration slot tags ---------------------------------------------------
// A registration slot holds the minimum TID of the current batch in its low 32
// bits and a batch tag in its high 32 bits.  The tag of batch epoch e is
// 0xFFFFFFFF - e, so a newer batch has a smaller tag and its atomicMin
// overwrites entries left by older batches: the tables never need clearing
// (the reference memsets 18 tables per batch, TF/Database.h:78-102).
LTPG_HD uint64_t slot_tag(uint32_t epoch) { return (uint64_t)(0xFFFFFFFFu - epoch) << 32; }
LTPG_HD uint32_t slot_min(uint64_t v, uint32_t epoch) {
    return (uint32_t)(v >> 32) == 0xFFFFFFFFu - epoch ? (uint32_t)v : 0xFFFFFFFFu;
}

// ---- YCSB op words -------------------------------------------------------------
constexpr uint32_t YCSB_KEY_MASK = (1u << LTPG_YCSB_KEY_BITS) - 1u;
LTPG_HD bool ycsb_is_pad(uint32_t w) { return w == LTPG_YCSB_OP_PAD; }
LTPG_HD bool ycsb_is_update(uint32_t w) { return (w >> 31) != 0; }
LTPG_HD uint32_t ycsb_field(uint32_t w) { return (w >> 27) & 0xFu; }
LTPG_HD uint32_t ycsb_key(uint32_t w) { return w & YCSB_KEY_MASK; }
// A read's field bits name a range scan of span + 1 consecutive keys (0: a
// point read); keys past the table's end are left out (Y2/Execute.h:24-32).
LTPG_HD uint32_t ycsb_span(uint32_t w) { return ycsb_is_update(w) ? 0u : ((w >> 27) & 0xFu); }
LTPG_HD uint32_t ycsb_word(uint32_t key, bool update, uint32_t field) {
    return (update ? 0x80000000u : 0u) | ((field & 0xFu) << 27) | (key & YCSB_KEY_MASK);
}
LTPG_HD uint32_t ycsb_stride(uint32_t k) { return (k + 3u) & ~3u; }

// ---- TPC-C layout ---------------------------------------------------------------
constexpr uint32_t TPCC_COLS[LTPG_TPCC_TABLES] = {9, 11, 21, 8, 3, 8, 10, 17, 5};
LTPG_HD uint32_t tpcc_cols(uint32_t table) {
    switch (table) {
    case LTPG_T_WAREHOUSE: return 9;
    case LTPG_T_DISTRICT: return 11;
    case LTPG_T_CUSTOMER: return 21;
    case LTPG_T_HISTORY: return 8;
    case LTPG_T_NEWORDER: return 3;
    case LTPG_T_ORDER: return 8;
    case LTPG_T_ORDERLINE: return 10;
    case LTPG_T_STOCK: return 17;
    default: return 5;
    }
}
LTPG_HD uint64_t tpcc_rows(uint32_t table, uint32_t W) {
    switch (table) {
    case LTPG_T_WAREHOUSE: return W;
    case LTPG_T_DISTRICT: return 10ull * W;
    case LTPG_T_CUSTOMER: return 30000ull * W;
    case LTPG_T_HISTORY: return 30000ull * W;
    case LTPG_T_NEWORDER: return 30000ull * W;
    case LTPG_T_ORDER: return 30000ull * W;
    case LTPG_T_ORDERLINE: return 450000ull * W;
    case LTPG_T_STOCK: return 100000ull * W;
    default: return 100000ull;
    }
}
// Registration slots of all nine tables in one flat array: slot = base + row.
LTPG_HD uint64_t tpcc_slot_base(uint32_t table, uint32_t W) {
    uint64_t b = 0;
    for (uint32_t t = 0; t < table; ++t) b += tpcc_rows(t, W);
    return b;
}

// Column numbers used by the executors (schema of TF/Datastructure.h:3-118;
// money columns are int64 cents, taxes and discounts basis points).
enum : uint32_t {
    W_ID = 0, W_TAX = 1, W_YTD = 2,
    D_ID = 0, D_W_ID = 1, D_TAX = 2, D_YTD = 3, D_NEXT_O_ID = 4,
    C_ID = 0, C_W_ID = 1, C_D_ID = 2, C_CREDIT_LIM = 3, C_DISCOUNT = 4, C_BALANCE = 5,
    C_YTD_PAYMENT = 6, C_PAYMENT_CNT = 7, C_DELIVERY_CNT = 8, C_DATA = 9, C_CREDIT = 10,
    C_LAST = 13,
    H_C_ID = 0, H_C_D_ID = 1, H_C_W_ID = 2, H_D_ID = 3, H_W_ID = 4, H_AMOUNT = 5, H_DATE = 6,
    H_DATA = 7,
    NO_O_ID = 0, NO_D_ID = 1, NO_W_ID = 2,
    O_ID = 0, O_D_ID = 1, O_W_ID = 2, O_C_ID = 3, O_ENTRY_D = 4, O_CARRIER_ID = 5,
    O_OL_CNT = 6, O_ALL_LOCAL = 7,
    OL_O_ID = 0, OL_D_ID = 1, OL_W_ID = 2, OL_NUMBER = 3, OL_I_ID = 4, OL_SUPPLY_W_ID = 5,
    OL_DELIVERY_D = 6, OL_QUANTITY = 7, OL_AMOUNT = 8, OL_DIST_INFO = 9,
    S_I_ID = 0, S_W_ID = 1, S_QUANTITY = 2, S_YTD = 3, S_ORDER_CNT = 4, S_REMOTE_CNT = 5,
    S_DIST_01 = 6, S_DATA = 16,
    I_ID = 0, I_IM_ID = 1, I_PRICE = 2, I_NAME = 3, I_DATA = 4,
};

// Registration / check kinds of one concurrency-control operation.
enum : uint32_t {
    OPF_REG_R = 1u,   // atomicMin into the read slot
    OPF_REG_W = 2u,   // atomicMin into the write slot
    OPF_CHK_RAW = 4u, // smaller writer registered -> RAW
    OPF_CHK_WAR = 8u, // smaller reader registered -> WAR
    OPF_CHK_WAW = 16u // smaller writer registered -> WAW
};
constexpr uint32_t OPF_READ = OPF_REG_R | OPF_CHK_RAW;
constexpr uint32_t OPF_WRITE = OPF_REG_W | OPF_CHK_WAR | OPF_CHK_WAW;
// NEW-ORDER insert as the reference does it: registered as a read
// (TF/Execute_neworder.h:115) and, because check_3_0 is never dispatched
// (TF/Execute_neworder.h:639-646), checked only for WAW (check_3_1, :478-490).
constexpr uint32_t OPF_NO_INSERT_COMPAT = OPF_REG_R | OPF_CHK_WAW;
// A row read and then updated by one transaction (the reference registers and
// checks it as a read op and a write op of the same row, TA/Execute.h:1772-2153).
constexpr uint32_t OPF_RW = OPF_READ | OPF_WRITE;

LTPG_HD uint32_t tpcc_kind(uint32_t kind_info) { return kind_info & 0xFFu; }
LTPG_HD uint32_t tpcc_ol_cnt(uint32_t kind_info) { return (kind_info >> 8) & 0xFFu; }
LTPG_HD uint32_t tpcc_d(uint32_t kind_info) { return (kind_info >> 16) & 0xFFu; }
LTPG_HD uint32_t tpcc_c_d(uint32_t kind_info) { return (kind_info >> 24) & 0xFFu; }
LTPG_HD uint32_t tpcc_n_ops(uint32_t kind_info) {
    switch (tpcc_kind(kind_info)) {
    case LTPG_TPCC_NEWORDER: return 5u + 3u * tpcc_ol_cnt(kind_info);
    case LTPG_TPCC_PAYMENT: return 5u;
    case LTPG_TPCC_ORDERSTATUS: return 3u;
    case LTPG_TPCC_DELIVERY: return 4u;
    default: return 1u;
    }
}
// Ops that can conflict, apart from order lines (the tuned kernels' header
// ops): reads of WAREHOUSE, DISTRICT and ITEM rows never can (no transaction
// registers a write there), so NewOrder and Payment keep ops j = 2, 3, 4 and
// the other kinds all of theirs.
LTPG_HD uint32_t tpcc_n_head(uint32_t kind_info) {
    switch (tpcc_kind(kind_info)) {
    case LTPG_TPCC_DELIVERY: return 4u;
    case LTPG_TPCC_STOCKLEVEL: return 1u;
    default: return 3u;
    }
}
LTPG_HD uint32_t tpcc_head_j(uint32_t kind_info, uint32_t k) {
    const uint32_t kind = tpcc_kind(kind_info);
    return (kind == LTPG_TPCC_NEWORDER || kind == LTPG_TPCC_PAYMENT) ? k + 2u : k;
}
LTPG_HD bool tpcc_customer_by_name(uint32_t kind_info) {
    const uint32_t kind = tpcc_kind(kind_info);
    return (kind == LTPG_TPCC_PAYMENT || kind == LTPG_TPCC_ORDERSTATUS) && (kind_info & LTPG_PAY_BY_NAME);
}
// First concurrency-control op of transaction t: NewOrder has 5 + 3 per line,
// Payment 5, so the offset follows from t and the line prefix alone.
LTPG_HD uint64_t tpcc_op_off(uint32_t t, uint32_t line_off) { return 5ull * t + 3ull * line_off; }
LTPG_HD int64_t tpcc_amount(const ltpg_tpcc_txn &x) {
    return (int64_t)(((uint64_t)x.c << 32) | (uint64_t)x.b);
}
LTPG_HD uint64_t tpcc_cust_row(uint32_t w, uint32_t d, uint32_t c) {
    return 30000ull * w + 3000ull * d + c;
}
LTPG_HD uint64_t tpcc_ol_row(uint32_t w, uint32_t ol_id, uint32_t i) {
    return 450000ull * w + (ol_id + i) % 450000u;
}

// Row and op flags of op j of a transaction (j < tpcc_n_ops).  `line` must be
// the transaction's line (j - 5) / 3 for NewOrder ops j >= 5.
struct TpccOp {
    uint32_t table;
    uint64_t row;
    uint32_t flags;
};
LTPG_HD TpccOp tpcc_op(const ltpg_tpcc_txn &x, uint32_t j, const ltpg_tpcc_line &ln,
                       uint32_t strict_insert) {
    TpccOp op;
    const uint32_t d = tpcc_d(x.kind_info);
    if (tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER) {
        switch (j) {
        case 0: op.table = LTPG_T_WAREHOUSE; op.row = x.w; op.flags = OPF_READ; return op;
        case 1: op.table = LTPG_T_DISTRICT; op.row = 10ull * x.w + d; op.flags = OPF_READ; return op;
        case 2: op.table = LTPG_T_CUSTOMER; op.row = tpcc_cust_row(x.w, d, x.c_id); op.flags = OPF_READ; return op;
        case 3: op.table = LTPG_T_NEWORDER; op.row = 30000ull * x.w + x.b;
            op.flags = strict_insert ? OPF_WRITE : OPF_NO_INSERT_COMPAT; return op;
        case 4: op.table = LTPG_T_ORDER; op.row = 30000ull * x.w + x.a; op.flags = OPF_WRITE; return op;
        default: break;
        }
        const uint32_t i = (j - 5u) / 3u, sub = (j - 5u) % 3u;
        if (sub == 0) { op.table = LTPG_T_ITEM; op.row = ln.i_id; op.flags = OPF_READ; }
        else if (sub == 1) { op.table = LTPG_T_STOCK; op.row = 100000ull * ln.supply_w + ln.i_id; op.flags = OPF_WRITE; }
        else { op.table = LTPG_T_ORDERLINE; op.row = tpcc_ol_row(x.w, x.c, i); op.flags = OPF_WRITE; }
        return op;
    }
    const uint32_t c_d = tpcc_c_d(x.kind_info);
    switch (tpcc_kind(x.kind_info)) {
    case LTPG_TPCC_ORDERSTATUS:  // TA/Execute.h:1592-1770
        if (j == 0) { op.table = LTPG_T_CUSTOMER; op.row = tpcc_cust_row(x.c_w, c_d, x.c_id); }
        else if (j == 1) { op.table = LTPG_T_ORDER; op.row = 30000ull * x.w + x.a; }
        else { op.table = LTPG_T_ORDERLINE; op.row = 450000ull * x.w + x.b; }
        op.flags = OPF_READ;
        return op;
    case LTPG_TPCC_DELIVERY:  // TA/Execute.h:1772-2153
        if (j == 0) { op.table = LTPG_T_NEWORDER; op.row = 30000ull * x.w + x.b; op.flags = OPF_WRITE; }
        else if (j == 1) { op.table = LTPG_T_ORDER; op.row = 30000ull * x.w + x.a; op.flags = OPF_RW; }
        else if (j == 2) { op.table = LTPG_T_ORDERLINE; op.row = 450000ull * x.w + x.c; op.flags = OPF_RW; }
        else { op.table = LTPG_T_CUSTOMER; op.row = tpcc_cust_row(x.w, d, x.c_id); op.flags = OPF_WRITE; }
        return op;
    case LTPG_TPCC_STOCKLEVEL:  // TA/Execute.h:2155-2231
        op.table = LTPG_T_STOCK; op.row = 100000ull * x.w + x.a; op.flags = OPF_READ;
        return op;
    default: break;
    }
    switch (j) {
    case 0: op.table = LTPG_T_WAREHOUSE; op.row = x.w; op.flags = OPF_READ; return op;
    case 1: op.table = LTPG_T_DISTRICT; op.row = 10ull * x.w + d; op.flags = OPF_READ; return op;
    case 2: op.table = LTPG_T_CUSTOMER; op.row = tpcc_cust_row(x.c_w, c_d, x.c_id); op.flags = OPF_READ; return op;
    case 3: op.table = LTPG_T_CUSTOMER; op.row = tpcc_cust_row(x.c_w, c_d, x.c_id); op.flags = OPF_WRITE; return op;
    default: op.table = LTPG_T_HISTORY; op.row = 30000ull * x.w + x.a; op.flags = OPF_WRITE; return op;
    }
}

// Initial value of column col of row `row` of a TPC-C table.  Ids follow the
// row numbering of TF/Database.h:104-327; the other columns are hashes, and
// the arithmetic columns get TPC-C-shaped starting values (clause 4.3.3.1).
LTPG_HD uint64_t tpcc_init_value(uint64_t seed, uint32_t table, uint64_t row, uint32_t col) {
    const uint64_t h = hash3(seed ^ (0x7C3A5E1Bull * (table + 1u)), row, col);
    switch (table) {
    case LTPG_T_WAREHOUSE:
        if (col == W_ID) return row;
        if (col == W_TAX) return h % 2001u;
        if (col == W_YTD) return 30000000ull;
        return h;
    case LTPG_T_DISTRICT:
        if (col == D_ID) return row % 10u;
        if (col == D_W_ID) return row / 10u;
        if (col == D_TAX) return h % 2001u;
        if (col == D_YTD) return 3000000ull;
        if (col == D_NEXT_O_ID) return 3000u;
        return h;
    case LTPG_T_CUSTOMER:
        if (col == C_ID) return row % 3000u;
        if (col == C_W_ID) return row / 30000u;
        if (col == C_D_ID) return (row / 3000u) % 10u;
        if (col == C_CREDIT_LIM) return 5000000ull;
        if (col == C_DISCOUNT) return h % 5001u;
        if (col == C_BALANCE) return (uint64_t)(int64_t)-1000;
        if (col == C_YTD_PAYMENT) return 1000u;
        if (col == C_PAYMENT_CNT) return 1u;
        if (col == C_DELIVERY_CNT) return 0u;
        if (col == C_LAST) return h % 1000u;
        return h;
    case LTPG_T_STOCK:
        if (col == S_I_ID) return row % 100000u;
        if (col == S_W_ID) return row / 100000u;
        if (col == S_QUANTITY) return 10u + h % 91u;
        if (col == S_YTD || col == S_ORDER_CNT || col == S_REMOTE_CNT) return 0u;
        return h;
    case LTPG_T_ITEM:
        if (col == I_ID) return row;
        if (col == I_IM_ID) return 1u + h % 10000u;
        if (col == I_PRICE) return 100u + h % 9901u;
        return h;
    default:
        return h;
    }
}

// NewOrder total in cents: sum(amount) * (1 - discount) * (1 + w_tax + d_tax),
// rates in basis points, rounded down (TPC-C clause 2.4.2.2).  With at most 15
// lines of 10 items at 100.00 the product stays below 2^48.
LTPG_HD int64_t neworder_total(int64_t sum_amount, uint64_t disc, uint64_t wtax, uint64_t dtax) {
    return sum_amount * (int64_t)(10000u - disc) * (int64_t)(10000u + wtax + dtax) / 100000000;
}

// Commit rule of the reference (TF/Execute_neworder.h:692, Y1/Execute.h:187).
LTPG_HD bool commits(uint32_t f) {
    return !(f & LTPG_FLAG_WAW) && (!(f & LTPG_FLAG_RAW) || !(f & LTPG_FLAG_WAR));
}

// New stock quantity after ordering qty (TPC-C clause 2.4.2.2).
LTPG_HD uint64_t stock_after(uint64_t q, uint64_t qty) {
    return q >= qty + 10u ? q - qty : q - qty + 91u;
}

}  // namespace ltpg
