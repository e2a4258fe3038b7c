// tpcc.cu — TPC-C NewOrder + Payment executors: table image and plain path.
//
// Concurrency-control ops per transaction follow NEWORDER_NAMESPACE and
// PAYMENT_NAMESPACE of the reference (TF/Execute_neworder.h:14-336,426-617,
// TF/Execute_payment.h:39-303,390-536); see tpcc_op() in proto.h.  The
// warehouse and district YTD updates of Payment are hot commutative adds that
// neither register nor check (the "isFrequent" path, TF/Execute_payment.h:86-99,
// 144-163); they are applied as exact int64 adds for committed Payments only.
//
// Transactions are ragged (5 + 3 * lines ops for NewOrder, 5 for Payment).  A
// block takes a tile of transactions, lays their ops out back to back by an
// in-tile prefix sum, and its threads walk that flat list, so short and long
// transactions cost the same per op (the reference leaves lanes idle per
// missing order line, TF/Execute_neworder.h:174-183).
#include "devutil.cuh"

namespace ltpg {

struct TpccDev {
    uint64_t *tab[LTPG_TPCC_TABLES];
    uint64_t rows[LTPG_TPCC_TABLES];
    uint64_t base[LTPG_TPCC_TABLES];
    const uint64_t *name_idx;
    uint32_t W;
    uint32_t strict;
    uint32_t ref_names;
};

static TpccDev make_dev(ltpg_ctx *c) {
    TpccDev d{};
    for (int t = 0; t < LTPG_TPCC_TABLES; ++t) {
        d.tab[t] = c->tpcc.tab[t];
        d.rows[t] = c->tpcc.rows[t];
        d.base[t] = c->tpcc.base[t];
    }
    d.name_idx = c->tpcc.name_idx;
    d.W = c->tpcc.W;
    d.strict = (c->cfg.flags & LTPG_CFG_STRICT_INSERT) ? 1u : 0u;
    d.ref_names = (c->cfg.flags & LTPG_CFG_REF_NAME_LOOKUP) ? 1u : 0u;
    return d;
}

__device__ __forceinline__ uint64_t *col_ptr(const TpccDev &db, uint32_t table, uint64_t row, uint32_t col) {
    return db.tab[table] + row * tpcc_cols(table) + col;
}
__device__ __forceinline__ uint64_t ld_col(const TpccDev &db, uint32_t table, uint64_t row, uint32_t col) {
    return __ldg(col_ptr(db, table, row, col));
}

// Field ranges of a transaction record (the keys the reference computes in
// op_k_0 would silently alias other rows if a field were out of range).
__device__ __forceinline__ bool txn_valid(const ltpg_tpcc_txn &x, uint32_t W, uint32_t n_lines) {
    const uint32_t kind = tpcc_kind(x.kind_info);
    if (x.w >= W || tpcc_d(x.kind_info) >= 10u || x.c_id >= 3000u) return false;
    switch (kind) {
    case LTPG_TPCC_NEWORDER: {
        const uint32_t cnt = tpcc_ol_cnt(x.kind_info);
        return cnt <= LTPG_TPCC_MAX_LINES && x.a < 30000u && x.b < 30000u && x.c < 450000u &&
               (uint64_t)x.line_off + cnt <= n_lines;
    }
    case LTPG_TPCC_PAYMENT: return x.c_w < W && tpcc_c_d(x.kind_info) < 10u && x.a < 30000u;
    case LTPG_TPCC_ORDERSTATUS:
        return x.c_w < W && tpcc_c_d(x.kind_info) < 10u && x.a < 30000u && x.b < 450000u;
    case LTPG_TPCC_DELIVERY: {
        const uint32_t carrier = tpcc_ol_cnt(x.kind_info);
        return x.a < 30000u && x.b < 30000u && x.c < 450000u && carrier >= 1u && carrier <= 10u;
    }
    case LTPG_TPCC_STOCKLEVEL: return x.a < 100000u;
    default: return false;
    }
}
__device__ __forceinline__ bool line_valid(const ltpg_tpcc_line &ln, uint32_t W) {
    return ln.i_id < 100000u && ln.supply_w < W;
}

// ---- table image (Database::initial_data, TF/Database.h:349-451) ------------
__global__ void tpcc_init_kernel(uint64_t *__restrict__ tab, uint64_t rows, uint32_t cols, uint32_t table,
                                 uint64_t seed) {
    const uint64_t total = rows * cols;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x)
        tab[i] = tpcc_init_value(seed, table, i / cols, (uint32_t)(i % cols));
}

cudaError_t tpcc_init_tables(ltpg_ctx *c) {
    for (uint32_t t = 0; t < LTPG_TPCC_TABLES; ++t) {
        tpcc_init_kernel<<<c->sm_count * 8, 256, 0, c->stream>>>(c->tpcc.tab[t], c->tpcc.rows[t], tpcc_cols(t), t,
                                                                  c->tpcc_seed);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaMemsetAsync(c->tpcc.reg, 0xFF, c->tpcc.n_slots * sizeof(RegSlot), c->stream);
}

// ---- customer last-name index (replaces INDEX.customer_name_index and its
// 3,000-entry warp scan, TF/Datastructure.h:131-134, TF/Genericfunction.h:29-77)
// One block per district sorts the district's keys (C_LAST << 32 | C_ID) in
// shared memory (bitonic, 4,096 slots); a lookup is then a binary search in a
// 24 KB run that stays in L2.
constexpr uint32_t NAME_SORT = 4096;

__global__ void __launch_bounds__(1024) tpcc_name_index_kernel(const uint64_t *__restrict__ cust,
                                                               uint64_t *__restrict__ idx) {
    __shared__ unsigned long long k[NAME_SORT];
    const uint64_t r0 = (uint64_t)blockIdx.x * 3000u;
    for (uint32_t i = threadIdx.x; i < NAME_SORT; i += blockDim.x) {
        unsigned long long v = ~0ull;
        if (i < 3000u) {
            const uint64_t name = cust[(r0 + i) * tpcc_cols(LTPG_T_CUSTOMER) + C_LAST];
            v = ((name < 0xFFFFFFFFull ? name : 0xFFFFFFFFull) << 32) | i;
        }
        k[i] = v;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= NAME_SORT; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < NAME_SORT; i += blockDim.x) {
                const uint32_t j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0u;
                    const unsigned long long a = k[i], b = k[j];
                    if ((a > b) == up) {
                        k[i] = b;
                        k[j] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < 3000u; i += blockDim.x) idx[r0 + i] = k[i];
}

cudaError_t tpcc_build_name_index(ltpg_ctx *c) {
    if (!c->tpcc.W || !c->tpcc.name_idx) return cudaSuccess;
    tpcc_name_index_kernel<<<c->tpcc.W * 10u, 1024, 0, c->stream>>>(c->tpcc.tab[LTPG_T_CUSTOMER], c->tpcc.name_idx);
    return cudaGetLastError();
}

// The nth (0-based) customer of district (w, d) whose C_LAST is name, in C_ID
// order: the first index key >= name << 32, then nth further.
__device__ __forceinline__ bool name_lookup(const TpccDev &db, uint32_t w, uint32_t d, uint32_t name, uint32_t nth,
                                            uint32_t &cid) {
    const uint64_t *k = db.name_idx + (10ull * w + d) * 3000u;
    const uint64_t target = (uint64_t)name << 32;
    uint32_t lo = 0, hi = 3000u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(k + mid) < target) lo = mid + 1u;
        else hi = mid;
    }
    const uint32_t p = lo + nth;
    if (p >= 3000u) return false;
    const uint64_t v = __ldg(k + p);
    if ((v >> 32) != name) return false;
    cid = (uint32_t)v;
    return true;
}

// The reference's __FIND_CID_INDEX (TF/Genericfunction.h:29-77) as its lane 0
// computes it: the lane's shuffle reads its own match flag 32 times, so it
// tests customers 0, 32, 64, ... and counts each match 32 times until the
// count reaches nth; it then walks back from the end of its last block of 32
// (down to position 1) over customers with that name, counting down to nth,
// and returns the C_ID column of the row it stops at; otherwise C_ID 0.
// Positions past the district read the next district's rows, as the
// reference's index does; past the table they match nothing.
__device__ __forceinline__ uint32_t ref_name_lookup(const TpccDev &db, uint32_t w, uint32_t d, uint32_t name,
                                                    uint32_t nth) {
    const uint64_t dist = 30000ull * w + 3000ull * d, rows = db.rows[LTPG_T_CUSTOMER];
    auto name_at = [&](uint64_t row) {
        return row < rows && ld_col(db, LTPG_T_CUSTOMER, row, C_LAST) == (uint64_t)name;
    };
    uint32_t cum = 0, flag = 0;
    for (uint32_t i = 0; i < 3000u; i += 32u) {
        cum += name_at(dist + i) ? 32u : 0u;
        flag += 32u;
        if (cum >= nth) break;
    }
    if (cum < nth) return 0u;
    uint64_t result = 0;
    for (uint32_t i = flag - 1u; i > 0u; --i) {
        if (!name_at(dist + i)) continue;
        if (cum == nth) {
            result = dist + i;
            break;
        }
        --cum;
    }
    return (uint32_t)ld_col(db, LTPG_T_CUSTOMER, result, C_ID);
}

// Marks a by-name Payment whose customer was not found (kept in the
// shared-memory copy of the record only; a Payment's bits 8..15 are flags,
// a NewOrder's its line count).
constexpr uint32_t KI_NOT_FOUND = 0x200u;
__device__ __forceinline__ bool txn_not_found(const ltpg_tpcc_txn &x) {
    const uint32_t kind = tpcc_kind(x.kind_info);
    return (kind == LTPG_TPCC_PAYMENT || kind == LTPG_TPCC_ORDERSTATUS) && (x.kind_info & KI_NOT_FOUND);
}

// Resolves a by-name Payment or OrderStatus in place: c_id becomes the
// customer's C_ID.  Returns false when the customer is not found;
// out-of-range fields are left for txn_valid to reject.
__device__ __forceinline__ bool resolve_by_name(const TpccDev &db, ltpg_tpcc_txn &x) {
    if (!tpcc_customer_by_name(x.kind_info)) return true;
    const uint32_t c_d = tpcc_c_d(x.kind_info);
    if (x.c_w >= db.W || c_d >= 10u) return true;
    const uint32_t name = x.c_id >> 8, nth = x.c_id & 0xFFu;
    if (db.ref_names) {
        x.c_id = ref_name_lookup(db, x.c_w, c_d, name, nth);
        return true;
    }
    uint32_t cid;
    if (!name_lookup(db, x.c_w, c_d, name, nth, cid)) return false;
    x.c_id = cid;
    return true;
}

constexpr uint32_t PT = 64;    // transactions per tile (plain path)
constexpr uint32_t PBS = 256;  // threads per block (plain path)
// Tuned path: a block of 2P threads walks tiles of P transactions; P = 64
// (128-thread blocks, so a tile's barriers hold 4 warps) by default, 128 or
// 256 by the launch setting block_threads (256 / 512).

template <uint32_t N>
struct TileHdrN {
    ltpg_tpcc_txn x[N];
    uint32_t off[N + 1];
    uint32_t ok[N];
};
using TileHdr = TileHdrN<PT>;

// Loads a tile and lays out its ops (n_ops_of = ops per transaction).
template <class H, class F>
__device__ __forceinline__ uint32_t load_tile(H &h, const ltpg_tpcc_txn *__restrict__ txns, uint32_t t0,
                                              uint32_t nt, const TpccDev &db, uint32_t n_lines, DevCtl *ctl,
                                              F n_ops_of) {
    if (threadIdx.x < nt) {
        const uint4 *p = reinterpret_cast<const uint4 *>(txns + t0 + threadIdx.x);
        const uint4 a = ld_nc_u4(p), b = ld_nc_u4(p + 1);
        ltpg_tpcc_txn x;
        x.kind_info = a.x; x.w = a.y; x.c_w = a.z; x.c_id = a.w;
        x.a = b.x; x.b = b.y; x.c = b.z; x.line_off = b.w;
        const bool found = resolve_by_name(db, x);
        if (!found) x.kind_info |= KI_NOT_FOUND;
        h.x[threadIdx.x] = x;
        const bool ok = found && txn_valid(x, db.W, n_lines);
        if (!ok && found) report_error(ctl, DERR_BOUNDS, t0 + threadIdx.x);
        h.ok[threadIdx.x] = ok;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // warp 0: prefix sum of the tile's op counts
        uint32_t carry = 0;
        for (uint32_t base = 0; base < nt; base += 32) {
            const uint32_t i = base + threadIdx.x;
            const int n = i < nt ? (int)n_ops_of(i) : 0;
            const int incl = warp_incl_scan(n);
            if (i < nt) h.off[i] = carry + (uint32_t)(incl - n);
            carry += (uint32_t)__shfl_sync(FULL, incl, 31);
        }
        if (threadIdx.x == 0) h.off[nt] = carry;
    }
    __syncthreads();
    return h.off[nt];
}

// Transaction of flat op e: the last i with off[i] <= e.
template <class H>
__device__ __forceinline__ uint32_t tile_owner(const H &h, uint32_t nt, uint32_t e) {
    uint32_t lo = 0, hi = nt;  // off[lo] <= e < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (h.off[mid] <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ ltpg_tpcc_line load_line(const ltpg_tpcc_line *__restrict__ lines, uint64_t idx) {
    const uint2 v = __ldg(reinterpret_cast<const uint2 *>(lines) + idx);
    ltpg_tpcc_line ln;
    ln.i_id = v.x;
    ln.supply_w = (uint16_t)(v.y & 0xFFFFu);
    ln.qty = (uint16_t)(v.y >> 16);
    return ln;
}

// The execute-phase read that gives a non-NewOrder transaction its result, if
// op j is the op holding it: Payment j = 2 (C_BALANCE - amount), OrderStatus
// j = 0 (C_BALANCE), Delivery j = 2 (the line's OL_AMOUNT), StockLevel j = 0
// (S_QUANTITY).  Batch-start image.
__device__ __forceinline__ bool result_read(const TpccDev &db, const ltpg_tpcc_txn &x, uint32_t j, const TpccOp &op,
                                            long long &out) {
    switch (tpcc_kind(x.kind_info)) {
    case LTPG_TPCC_PAYMENT:
        if (j != 2u) return false;
        out = (long long)ld_col(db, LTPG_T_CUSTOMER, op.row, C_BALANCE) - tpcc_amount(x);
        return true;
    case LTPG_TPCC_ORDERSTATUS:
        if (j != 0u) return false;
        out = (long long)ld_col(db, LTPG_T_CUSTOMER, op.row, C_BALANCE);
        return true;
    case LTPG_TPCC_DELIVERY:
        if (j != 2u) return false;
        out = (long long)ld_col(db, LTPG_T_ORDERLINE, op.row, OL_AMOUNT);
        return true;
    case LTPG_TPCC_STOCKLEVEL:
        out = (long long)ld_col(db, LTPG_T_STOCK, op.row, S_QUANTITY);
        return true;
    default: return false;
    }
}

// ---- plain phase 1: execute + register (KERNEL_EXECUTE, TF/tp.cu:24-54) ----
__global__ void __launch_bounds__(PBS) tpcc_exec_plain(const ltpg_tpcc_txn *__restrict__ txns, uint32_t B,
                                                       const ltpg_tpcc_line *__restrict__ lines,
                                                       const uint64_t *__restrict__ hdr, TpccDev db,
                                                       RegSlot *__restrict__ reg, int64_t *__restrict__ results,
                                                       DevCtl *ctl) {
    const uint32_t n_lines = (uint32_t)hdr[0];
    __shared__ TileHdr h;
    __shared__ unsigned long long sum[PT];
    __shared__ uint32_t wtax[PT], dtax[PT], disc[PT];
    __shared__ long long res[PT];
    const uint64_t tag = slot_tag(ctl->epoch);
    const uint32_t t0 = blockIdx.x * PT, nt = min(PT, B - t0);
    if (threadIdx.x < PT) sum[threadIdx.x] = 0ull;
    const uint32_t total = load_tile(h, txns, t0, nt, db, n_lines, ctl,
                                     [&](uint32_t i) { return h.ok[i] ? tpcc_n_ops(h.x[i].kind_info) : 0u; });
    for (uint32_t e = threadIdx.x; e < total; e += PBS) {
        const uint32_t i = tile_owner(h, nt, e), j = e - h.off[i];
        const ltpg_tpcc_txn &x = h.x[i];
        const bool no = tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER;
        ltpg_tpcc_line ln{0, 0, 0};
        if (no && j >= 5) {
            ln = load_line(lines, (uint64_t)x.line_off + (j - 5) / 3);
            if (!line_valid(ln, db.W)) {
                report_error(ctl, DERR_BOUNDS, t0 + i);
                continue;
            }
        }
        const TpccOp op = tpcc_op(x, j, ln, db.strict);
        RegSlot *s = reg + db.base[op.table] + op.row;
        const unsigned long long v = tag | (t0 + i);
        if (op.flags & OPF_REG_R) red_min(&s->r, v);
        if (op.flags & OPF_REG_W) red_min(&s->w, v);
        // Reads of the execute phase (batch-start snapshot).
        if (no) {
            if (j == 0) wtax[i] = (uint32_t)ld_col(db, LTPG_T_WAREHOUSE, op.row, W_TAX);
            else if (j == 1) dtax[i] = (uint32_t)ld_col(db, LTPG_T_DISTRICT, op.row, D_TAX);
            else if (j == 2) disc[i] = (uint32_t)ld_col(db, LTPG_T_CUSTOMER, op.row, C_DISCOUNT);
            else if (op.table == LTPG_T_ITEM)
                atomicAdd(&sum[i], (unsigned long long)ln.qty * ld_col(db, LTPG_T_ITEM, op.row, I_PRICE));
        } else {
            long long r;
            if (result_read(db, x, j, op, r)) res[i] = r;
        }
    }
    __syncthreads();
    if (threadIdx.x < nt) {
        const uint32_t i = threadIdx.x;
        int64_t r = 0;
        if (h.ok[i])
            r = tpcc_kind(h.x[i].kind_info) == LTPG_TPCC_NEWORDER
                    ? neworder_total((int64_t)sum[i], disc[i], wtax[i], dtax[i])
                    : (int64_t)res[i];
        results[t0 + i] = r;
    }
}

// ---- plain phase 2: check (KERNEL_CHECK, TF/tp.cu:55-85) ---------------------
__global__ void __launch_bounds__(PBS) tpcc_check_plain(const ltpg_tpcc_txn *__restrict__ txns, uint32_t B,
                                                        const ltpg_tpcc_line *__restrict__ lines,
                                                        const uint64_t *__restrict__ hdr, TpccDev db,
                                                        const RegSlot *__restrict__ reg,
                                                        uint8_t *__restrict__ flags, DevCtl *ctl) {
    const uint32_t n_lines = (uint32_t)hdr[0];
    __shared__ TileHdr h;
    __shared__ uint32_t fl[PT];
    const uint32_t epoch = ctl->epoch;
    const uint32_t t0 = blockIdx.x * PT, nt = min(PT, B - t0);
    if (threadIdx.x < PT) fl[threadIdx.x] = 0u;
    const uint32_t total = load_tile(h, txns, t0, nt, db, n_lines, ctl,
                                     [&](uint32_t i) { return h.ok[i] ? tpcc_n_ops(h.x[i].kind_info) : 0u; });
    for (uint32_t e = threadIdx.x; e < total; e += PBS) {
        const uint32_t i = tile_owner(h, nt, e), j = e - h.off[i];
        const ltpg_tpcc_txn &x = h.x[i];
        ltpg_tpcc_line ln{0, 0, 0};
        if (tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER && j >= 5) {
            ln = load_line(lines, (uint64_t)x.line_off + (j - 5) / 3);
            if (!line_valid(ln, db.W)) continue;
        }
        const TpccOp op = tpcc_op(x, j, ln, db.strict);
        const ulonglong2 s = ld_slot(reg + db.base[op.table] + op.row);
        const uint32_t rmin = slot_min(s.x, epoch), wmin = slot_min(s.y, epoch), t = t0 + i;
        uint32_t f = 0;
        if ((op.flags & OPF_CHK_RAW) && wmin < t) f |= LTPG_FLAG_RAW;
        if ((op.flags & OPF_CHK_WAR) && rmin < t) f |= LTPG_FLAG_WAR;
        if ((op.flags & OPF_CHK_WAW) && wmin < t) f |= LTPG_FLAG_WAW;
        if (f) atomicOr(&fl[i], f);
    }
    __syncthreads();
    if (threadIdx.x < nt) {
        uint32_t f = fl[threadIdx.x];
        if (h.ok[threadIdx.x] && commits(f)) f |= LTPG_FLAG_COMMIT;
        if (txn_not_found(h.x[threadIdx.x])) f |= LTPG_FLAG_NOT_FOUND;
        flags[t0 + threadIdx.x] = (uint8_t)f;
    }
}

// Write op q of a committed transaction.  NewOrder: 0 ORDER insert, 1
// NEW-ORDER insert, 2+2i stock update of line i, 3+2i ORDER-LINE insert of
// line i.  Payment: 0 W_YTD add, 1 D_YTD add, 2 customer update, 3 HISTORY
// insert.  Delivery: 0 NEW-ORDER delete, 1 ORDER carrier, 2 ORDER-LINE delivery
// date, 3 customer credit (`result` = the line's OL_AMOUNT read by the execute
// phase).  Rows written here have exactly one committed writer in the batch
// (a second one would have seen WAW), so plain read-modify-writes are safe;
// the YTD adds are commutative and use atomics.
__device__ __forceinline__ uint32_t tpcc_n_writes(uint32_t kind_info) {
    switch (tpcc_kind(kind_info)) {
    case LTPG_TPCC_NEWORDER: return 2u + 2u * tpcc_ol_cnt(kind_info);
    case LTPG_TPCC_PAYMENT: return 4u;
    case LTPG_TPCC_DELIVERY: return 4u;
    default: return 0u;  // OrderStatus, StockLevel: read-only
    }
}

template <bool kHotDirect>
__device__ __forceinline__ void tpcc_apply_write(const TpccDev &db, const ltpg_tpcc_txn &x, uint32_t q,
                                                 const ltpg_tpcc_line *__restrict__ lines, uint64_t date,
                                                 long long *hot_w, long long *hot_d, int64_t result) {
    const uint32_t d = tpcc_d(x.kind_info);
    if (tpcc_kind(x.kind_info) == LTPG_TPCC_DELIVERY) {
        if (q == 0) {
            uint64_t *o = col_ptr(db, LTPG_T_NEWORDER, 30000ull * x.w + x.b, 0);
            o[NO_O_ID] = o[NO_D_ID] = o[NO_W_ID] = ~0ull;  // deleted
        } else if (q == 1) {
            *col_ptr(db, LTPG_T_ORDER, 30000ull * x.w + x.a, O_CARRIER_ID) = tpcc_ol_cnt(x.kind_info);
        } else if (q == 2) {
            *col_ptr(db, LTPG_T_ORDERLINE, 450000ull * x.w + x.c, OL_DELIVERY_D) = date;
        } else {
            uint64_t *cst = col_ptr(db, LTPG_T_CUSTOMER, tpcc_cust_row(x.w, d, x.c_id), 0);
            cst[C_BALANCE] = (uint64_t)((int64_t)cst[C_BALANCE] + result);
            cst[C_DELIVERY_CNT] += 1u;
        }
        return;
    }
    if (tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER) {
        const uint32_t cnt = tpcc_ol_cnt(x.kind_info);
        if (q == 0) {
            uint64_t *o = col_ptr(db, LTPG_T_ORDER, 30000ull * x.w + x.a, 0);
            bool all_local = true;
            for (uint32_t i = 0; i < cnt; ++i) all_local &= load_line(lines, (uint64_t)x.line_off + i).supply_w == x.w;
            o[O_ID] = x.a; o[O_D_ID] = d; o[O_W_ID] = x.w; o[O_C_ID] = x.c_id;
            o[O_ENTRY_D] = date; o[O_CARRIER_ID] = 0; o[O_OL_CNT] = cnt; o[O_ALL_LOCAL] = all_local;
            return;
        }
        if (q == 1) {
            uint64_t *o = col_ptr(db, LTPG_T_NEWORDER, 30000ull * x.w + x.b, 0);
            o[NO_O_ID] = x.a; o[NO_D_ID] = d; o[NO_W_ID] = x.w;
            return;
        }
        const uint32_t i = (q - 2) / 2;
        const ltpg_tpcc_line ln = load_line(lines, (uint64_t)x.line_off + i);
        const uint64_t srow = 100000ull * ln.supply_w + ln.i_id;
        if ((q & 1u) == 0u) {
            // Atomic, so that an order listing one stock row twice (the
            // reference's generator draws distinct items, a caller's batch
            // need not) updates it once per line.  Order does not matter: for
            // S_QUANTITY in [10, 100] and quantities <= 91 the rule keeps the
            // value in [10, 100], so after any set of lines it is
            // 10 + ((q - sum - 10) mod 91) whatever their order; the counters
            // add.  No other committed transaction writes the row (WAW).
            uint64_t *s = col_ptr(db, LTPG_T_STOCK, srow, 0);
            unsigned long long *qp = reinterpret_cast<unsigned long long *>(s + S_QUANTITY);
            unsigned long long cur = *qp;
            for (uint32_t tries = 0; tries < 64u; ++tries) {  // contenders: the order's own lines
                const unsigned long long prev = atomicCAS(qp, cur, (unsigned long long)stock_after(cur, ln.qty));
                if (prev == cur) break;
                cur = prev;
            }
            red_add_u64(reinterpret_cast<unsigned long long *>(s + S_YTD), ln.qty);
            red_add_u64(reinterpret_cast<unsigned long long *>(s + S_ORDER_CNT), 1ull);
            if (ln.supply_w != x.w) red_add_u64(reinterpret_cast<unsigned long long *>(s + S_REMOTE_CNT), 1ull);
        } else {
            uint64_t *o = col_ptr(db, LTPG_T_ORDERLINE, tpcc_ol_row(x.w, x.c, i), 0);
            o[OL_O_ID] = x.a; o[OL_D_ID] = d; o[OL_W_ID] = x.w; o[OL_NUMBER] = i + 1u;
            o[OL_I_ID] = ln.i_id; o[OL_SUPPLY_W_ID] = ln.supply_w; o[OL_DELIVERY_D] = 0u;
            o[OL_QUANTITY] = ln.qty;
            o[OL_AMOUNT] = (uint64_t)ln.qty * ld_col(db, LTPG_T_ITEM, ln.i_id, I_PRICE);
            o[OL_DIST_INFO] = ld_col(db, LTPG_T_STOCK, srow, S_DIST_01 + d);
        }
        return;
    }
    const int64_t amt = tpcc_amount(x);
    const uint32_t c_d = tpcc_c_d(x.kind_info);
    if (q == 0) {
        if (kHotDirect) red_add_u64(reinterpret_cast<unsigned long long *>(col_ptr(db, LTPG_T_WAREHOUSE, x.w, W_YTD)),
                                    (unsigned long long)amt);
        else atomicAdd(reinterpret_cast<unsigned long long *>(hot_w + x.w), (unsigned long long)amt);
    } else if (q == 1) {
        if (kHotDirect)
            red_add_u64(reinterpret_cast<unsigned long long *>(col_ptr(db, LTPG_T_DISTRICT, 10ull * x.w + d, D_YTD)),
                        (unsigned long long)amt);
        else atomicAdd(reinterpret_cast<unsigned long long *>(hot_d + 10u * x.w + d), (unsigned long long)amt);
    } else if (q == 2) {
        uint64_t *cst = col_ptr(db, LTPG_T_CUSTOMER, tpcc_cust_row(x.c_w, c_d, x.c_id), 0);
        cst[C_BALANCE] = (uint64_t)((int64_t)cst[C_BALANCE] - amt);
        cst[C_YTD_PAYMENT] = (uint64_t)((int64_t)cst[C_YTD_PAYMENT] + amt);
        cst[C_PAYMENT_CNT] += 1u;
    } else {
        uint64_t *hh = col_ptr(db, LTPG_T_HISTORY, 30000ull * x.w + x.a, 0);
        hh[H_C_ID] = x.c_id; hh[H_C_D_ID] = c_d; hh[H_C_W_ID] = x.c_w; hh[H_D_ID] = d;
        hh[H_W_ID] = x.w; hh[H_AMOUNT] = (uint64_t)amt; hh[H_DATE] = date; hh[H_DATA] = 0u;
    }
}

// ---- plain phase 3: write-back (KERNEL_WRITEBACK, TF/tp.cu:86-117) ----------
__global__ void __launch_bounds__(PBS) tpcc_writeback_plain(const ltpg_tpcc_txn *__restrict__ txns, uint32_t B,
                                                            const ltpg_tpcc_line *__restrict__ lines,
                                                            const uint64_t *__restrict__ hdr, TpccDev db,
                                                            const int64_t *__restrict__ results,
                                                            const uint8_t *__restrict__ flags,
                                                            uint32_t *__restrict__ bitmap, DevStats *st,
                                                            DevCtl *ctl) {
    const uint32_t n_lines = (uint32_t)hdr[0];
    const uint64_t txn_base = hdr[1];
    __shared__ TileHdr h;
    __shared__ uint8_t fl[PT];
    const uint32_t t0 = blockIdx.x * PT, nt = min(PT, B - t0);
    if (threadIdx.x < PT) {
        const uint32_t f = threadIdx.x < nt ? flags[t0 + threadIdx.x] : 0u;
        fl[threadIdx.x] = (uint8_t)f;
        const unsigned bal = __ballot_sync(FULL, (f & LTPG_FLAG_COMMIT) != 0u);
        const unsigned braw = __ballot_sync(FULL, (f & LTPG_FLAG_RAW) != 0u);
        const unsigned bwar = __ballot_sync(FULL, (f & LTPG_FLAG_WAR) != 0u);
        const unsigned bwaw = __ballot_sync(FULL, (f & LTPG_FLAG_WAW) != 0u);
        if ((threadIdx.x & 31) == 0 && threadIdx.x < nt) {
            bitmap[(t0 + threadIdx.x) >> 5] = bal;
            if (bal) {
                red_add_u64(&st->commits, __popc(bal));
                red_add_u64(&ctl->total_commits, __popc(bal));
            }
            if (braw) red_add_u64(&st->raw, __popc(braw));
            if (bwar) red_add_u64(&st->war, __popc(bwar));
            if (bwaw) red_add_u64(&st->waw, __popc(bwaw));
        }
    }
    __syncthreads();
    const uint32_t total = load_tile(h, txns, t0, nt, db, n_lines, ctl, [&](uint32_t i) {
        return (h.ok[i] && (fl[i] & LTPG_FLAG_COMMIT)) ? tpcc_n_writes(h.x[i].kind_info) : 0u;
    });
    for (uint32_t e = threadIdx.x; e < total; e += PBS) {
        const uint32_t i = tile_owner(h, nt, e), q = e - h.off[i];
        tpcc_apply_write<true>(db, h.x[i], q, lines, txn_base + t0 + i, nullptr, nullptr, results[t0 + i]);
    }
    finish_batch(ctl);
}

cudaError_t tpcc_phase(ltpg_ctx *c, Slot &s, int phase) {
    const uint32_t B = s.n_txn;
    if (B == 0) return cudaSuccess;
    const TpccDev db = make_dev(c);
    const uint32_t grid = (B + PT - 1) / PT;
    if (phase == 0) {
        cudaError_t e = cudaMemsetAsync(s.stats, 0, sizeof(DevStats), c->stream);
        if (e != cudaSuccess) return e;
        tpcc_exec_plain<<<grid, PBS, 0, c->stream>>>(s.txns, B, s.lines, s.dev_hdr, db, c->tpcc.reg, s.results,
                                                     c->ctl);
    } else if (phase == 1) {
        tpcc_check_plain<<<grid, PBS, 0, c->stream>>>(s.txns, B, s.lines, s.dev_hdr, db, c->tpcc.reg, s.flags,
                                                      c->ctl);
    } else {
        tpcc_writeback_plain<<<grid, PBS, 0, c->stream>>>(s.txns, B, s.lines, s.dev_hdr, db, s.results, s.flags,
                                                          s.bitmap, s.stats, c->ctl);
    }
    return cudaGetLastError();
}

}  // namespace ltpg


// ============================================================================
// Tuned path: the same tiles, with deduplicated + filtered registration, check
// and write-back fused, and the hot W_YTD / D_YTD adds of a block summed in
// shared memory and flushed once per block (one atomic per warehouse and per
// district instead of one per Payment).
// ============================================================================
#include "stage.cuh"

namespace ltpg {

constexpr uint32_t HOT_SMEM_MAX_W = 256;  // shared-memory YTD sums up to 256 warehouses

struct TpccTunedArgs {
    const ltpg_tpcc_txn *txns;
    const ltpg_tpcc_line *lines;
    const uint64_t *hdr;  // {n_lines, txn_base} of the slot
    uint32_t B;
    TpccDev db;
    RegSlot *reg;
    int64_t *results;
    uint8_t *flags;
    uint32_t *bitmap;
    DevStats *st;
    DevCtl *ctl;
    uint32_t filter;
    uint32_t dedupe;  // one registration per distinct slot of a warp (header ops)
};

__device__ __forceinline__ uint64_t ld_ca_u64t(const unsigned long long *p) {
    uint64_t v;
    asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

// Tables that no NewOrder or Payment registers a write on: WAREHOUSE and
// DISTRICT (their YTD updates are unregistered hot adds, D_NEXT_O_ID is
// host-assigned, TF/Query.h:54-88) and ITEM (read-only).  A read of such a row
// never sees RAW, and its registration can never give a writer WAR, so the
// tuned kernels neither register nor check those reads; the outcome is the
// plain path's, which keeps the reference's full op list.
//
// What remains is uniform: every transaction has three header ops (tpcc_op
// j = 2, 3, 4 — NewOrder: customer read, NEW-ORDER insert, ORDER insert;
// Payment: customer read, customer write, HISTORY insert) and every order line
// two (stock write, ORDER-LINE insert: j = 5 + 3i + 1, + 2).  A block walks its
// tile's header ops, three lanes per transaction, then its lines, one lane per
// line, so the lanes of a warp run the same code.  Lanes are in TID order in
// both passes, so the lowest lane of a warp's same-slot group holds the
// smallest TID.

// One registration; `dedupe`: one atomic per distinct slot of the warp,
// `filter`: skipped when the slot already holds a smaller tag.  Warp-uniform.
__device__ __forceinline__ void tuned_register(const TpccTunedArgs &a, bool valid, uint64_t slot_idx, bool is_w,
                                               unsigned long long mine, bool dedupe, bool filter) {
    bool leader = valid;
    if (dedupe) {
        const unsigned long long mkey = valid ? (slot_idx << 1) | (is_w ? 1ull : 0ull) : ~0ull;
        const unsigned peers = __match_any_sync(FULL, mkey);
        leader = valid && (__ffs(peers) - 1) == (int)(threadIdx.x & 31);
    }
    if (!leader) return;
    RegSlot *s = a.reg + slot_idx;
    unsigned long long *p = is_w ? &s->w : &s->r;
    if (!filter || ld_ca_u64t(p) > mine) red_min_exec(p, mine);
}

// Order line e of a tile whose line prefix is h.off: owner transaction and
// the line's index within it.
template <class H>
__device__ __forceinline__ void tile_line(const H &h, uint32_t nt, uint32_t e, uint32_t &i, uint32_t &li) {
    i = tile_owner(h, nt, e);
    li = e - h.off[i];
}

// Loads a tile, lays out its order lines and returns their number; hk = header
// lanes per transaction (4 if the tile holds a Delivery, else 3).
template <class H>
__device__ __forceinline__ uint32_t load_tile_lines(H &h, const TpccTunedArgs &a, uint32_t t0, uint32_t nt,
                                                    uint32_t n_lines, uint32_t &hk) {
    const uint32_t total = load_tile(h, a.txns, t0, nt, a.db, n_lines, a.ctl, [&](uint32_t i) {
        return (h.ok[i] && tpcc_kind(h.x[i].kind_info) == LTPG_TPCC_NEWORDER) ? tpcc_ol_cnt(h.x[i].kind_info) : 0u;
    });
    const bool dl = threadIdx.x < nt && tpcc_kind(h.x[threadIdx.x].kind_info) == LTPG_TPCC_DELIVERY;
    hk = __syncthreads_or(dl) ? 4u : 3u;
    return total;
}

// Work item e of a tile: e < hk nt is header op k = e % hk of transaction
// e / hk (valid when k < tpcc_n_head), the rest are order lines.  Each item
// has up to two registrations: the header op, or the line's stock write and
// ORDER-LINE insert.
struct TileItem {
    uint32_t i, k, li;
    bool head, valid, two;
    ltpg_tpcc_line ln;
    TpccOp op;
};
template <class H>
__device__ __forceinline__ TileItem tile_item(const TpccTunedArgs &a, const H &h, uint32_t nt, uint32_t hk,
                                              uint32_t e, uint32_t n_items, uint32_t t0, bool report) {
    TileItem it{0, 0, 0, false, false, false, {0, 0, 0}, {0, 0, 0}};
    if (e >= n_items) return it;
    const uint32_t n_head = hk * nt;
    if (e < n_head) {
        it.head = true;
        it.i = e / hk;
        it.k = e - hk * it.i;
        const uint32_t ki = h.x[it.i].kind_info;
        it.valid = h.ok[it.i] != 0u && it.k < tpcc_n_head(ki);
        if (it.valid) it.op = tpcc_op(h.x[it.i], tpcc_head_j(ki, it.k), it.ln, a.db.strict);
        return it;
    }
    tile_line(h, nt, e - n_head, it.i, it.li);
    it.ln = load_line(a.lines, (uint64_t)h.x[it.i].line_off + it.li);
    it.valid = line_valid(it.ln, a.db.W);
    if (!it.valid && report) report_error(a.ctl, DERR_BOUNDS, t0 + it.i);
    it.two = it.valid;
    return it;
}

template <uint32_t P>
__device__ __forceinline__ void tpcc_exec_tiles(const TpccTunedArgs &a, TileHdrN<P> &h, uint64_t tag) {
    const uint32_t n_lines = (uint32_t)a.hdr[0];
    __shared__ unsigned long long sum[P];
    __shared__ uint32_t wtax[P], dtax[P], disc[P];
    __shared__ long long res[P];
    const bool filt = a.filter != 0u;
    const uint32_t n_tiles = (a.B + P - 1) / P;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t t0 = tile * P, nt = min(P, a.B - t0);
        if (threadIdx.x < P) sum[threadIdx.x] = 0ull;
        uint32_t hk;
        const uint32_t lines_n = load_tile_lines(h, a, t0, nt, n_lines, hk);
        const uint32_t n_items = hk * nt + lines_n;
        for (uint32_t base = 0; base < n_items; base += blockDim.x) {
            const TileItem it = tile_item(a, h, nt, hk, base + threadIdx.x, n_items, t0, true);
            const ltpg_tpcc_txn &x = h.x[it.i];
            const unsigned long long mine = tag | (t0 + it.i);
            // header: the op (customer rows repeat under NURand, the inserts are
            // unique per batch); line: the stock write, then the ORDER-LINE insert
            const uint64_t srow = 100000ull * it.ln.supply_w + it.ln.i_id;
            const uint64_t s1 = it.head ? a.db.base[it.op.table] + it.op.row : a.db.base[LTPG_T_STOCK] + srow;
            const bool w1 = it.head ? (it.op.flags & OPF_REG_W) != 0u : true;
            const bool f1 = filt && (it.head ? it.op.table == LTPG_T_CUSTOMER : true);
            tuned_register(a, it.valid, s1, w1, mine, a.dedupe != 0u, f1);
            // second registration: a line's ORDER-LINE insert, or the read half
            // of a header op that reads and writes its row (Delivery)
            const bool rw = it.head && (it.op.flags & OPF_REG_R) && (it.op.flags & OPF_REG_W);
            const uint64_t s2 = it.head ? s1 : a.db.base[LTPG_T_ORDERLINE] + tpcc_ol_row(x.w, x.c, it.li);
            tuned_register(a, it.two || (it.valid && rw), s2, !it.head, mine, false, false);
            if (!it.valid) continue;
            if (!it.head) {
                atomicAdd(&sum[it.i], (unsigned long long)it.ln.qty * ld_col(a.db, LTPG_T_ITEM, it.ln.i_id, I_PRICE));
            } else if (tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER) {
                if (it.k == 0u) {
                    wtax[it.i] = (uint32_t)ld_col(a.db, LTPG_T_WAREHOUSE, x.w, W_TAX);
                    dtax[it.i] = (uint32_t)ld_col(a.db, LTPG_T_DISTRICT, 10ull * x.w + tpcc_d(x.kind_info), D_TAX);
                    disc[it.i] = (uint32_t)ld_col(a.db, LTPG_T_CUSTOMER, it.op.row, C_DISCOUNT);
                }
            } else {
                long long r;
                if (result_read(a.db, x, tpcc_head_j(x.kind_info, it.k), it.op, r)) res[it.i] = r;
            }
        }
        __syncthreads();
        if (threadIdx.x < nt) {
            const uint32_t i = threadIdx.x;
            int64_t r = 0;
            if (h.ok[i])
                r = tpcc_kind(h.x[i].kind_info) == LTPG_TPCC_NEWORDER
                        ? neworder_total((int64_t)sum[i], disc[i], wtax[i], dtax[i])
                        : (int64_t)res[i];
            a.results[t0 + i] = r;
        }
        __syncthreads();
    }
}

// hot: 11 W int64 sums in shared memory (W <= HOT_SMEM_MAX_W), or null.
template <uint32_t P>
__device__ __forceinline__ void tpcc_checkwb_tiles(const TpccTunedArgs &a, TileHdrN<P> &h, uint32_t epoch,
                                                   long long *hot) {
    const uint32_t n_lines = (uint32_t)a.hdr[0];
    const uint64_t txn_base = a.hdr[1];
    __shared__ uint32_t fl[P];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n_tiles = (a.B + P - 1) / P;
    unsigned long long c_com = 0, c_raw = 0, c_war = 0, c_waw = 0;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t t0 = tile * P, nt = min(P, a.B - t0);
        if (threadIdx.x < P) fl[threadIdx.x] = 0u;
        uint32_t hk;
        const uint32_t lines_n = load_tile_lines(h, a, t0, nt, n_lines, hk);
        const uint32_t n_items = hk * nt + lines_n;
        // header ops and order lines in one pass (reads of WAREHOUSE, DISTRICT
        // and ITEM rows cannot conflict; see tpcc_exec_tiles)
        for (uint32_t e = threadIdx.x; e < n_items; e += blockDim.x) {
            const TileItem it = tile_item(a, h, nt, hk, e, n_items, t0, false);
            if (!it.valid) continue;
            const uint32_t t = t0 + it.i;
            uint32_t f = 0;
            if (it.head) {
                const ulonglong2 s = ld_slot(a.reg + a.db.base[it.op.table] + it.op.row);
                const uint32_t rmin = slot_min(s.x, epoch), wmin = slot_min(s.y, epoch);
                if ((it.op.flags & OPF_CHK_RAW) && wmin < t) f |= LTPG_FLAG_RAW;
                if ((it.op.flags & OPF_CHK_WAR) && rmin < t) f |= LTPG_FLAG_WAR;
                if ((it.op.flags & OPF_CHK_WAW) && wmin < t) f |= LTPG_FLAG_WAW;
            } else {
                // stock write and ORDER-LINE insert: WAR and WAW each
                const ltpg_tpcc_txn &x = h.x[it.i];
                const ulonglong2 s1 = ld_slot(a.reg + a.db.base[LTPG_T_STOCK] + 100000ull * it.ln.supply_w + it.ln.i_id);
                const ulonglong2 s2 = ld_slot(a.reg + a.db.base[LTPG_T_ORDERLINE] + tpcc_ol_row(x.w, x.c, it.li));
                if (slot_min(s1.x, epoch) < t || slot_min(s2.x, epoch) < t) f |= LTPG_FLAG_WAR;
                if (slot_min(s1.y, epoch) < t || slot_min(s2.y, epoch) < t) f |= LTPG_FLAG_WAW;
            }
            if (f) atomicOr(&fl[it.i], f);
        }
        __syncthreads();
        if (threadIdx.x < P) {
            uint32_t f = threadIdx.x < nt ? fl[threadIdx.x] : 0u;
            const bool com = threadIdx.x < nt && h.ok[threadIdx.x] && commits(f);
            if (com) f |= LTPG_FLAG_COMMIT;
            if (threadIdx.x < nt && txn_not_found(h.x[threadIdx.x])) f |= LTPG_FLAG_NOT_FOUND;
            if (threadIdx.x < nt) {
                a.flags[t0 + threadIdx.x] = (uint8_t)f;
                fl[threadIdx.x] = f;
            }
            const unsigned bal = __ballot_sync(FULL, com);
            const unsigned braw = __ballot_sync(FULL, (f & LTPG_FLAG_RAW) != 0u);
            const unsigned bwar = __ballot_sync(FULL, (f & LTPG_FLAG_WAR) != 0u);
            const unsigned bwaw = __ballot_sync(FULL, (f & LTPG_FLAG_WAW) != 0u);
            if (lane == 0 && threadIdx.x < nt) {
                a.bitmap[(t0 + threadIdx.x) >> 5] = bal;
                c_com += __popc(bal);
                c_raw += __popc(braw);
                c_war += __popc(bwar);
                c_waw += __popc(bwaw);
            }
        }
        __syncthreads();
        // committed write ops, laid out back to back (ballot/prefix compaction)
        if (threadIdx.x < 32) {
            uint32_t carry = 0;
            for (uint32_t b0 = 0; b0 < nt; b0 += 32) {
                const uint32_t i = b0 + threadIdx.x;
                const int n = (i < nt && (fl[i] & LTPG_FLAG_COMMIT)) ? (int)tpcc_n_writes(h.x[i].kind_info) : 0;
                const int incl = warp_incl_scan(n);
                if (i < nt) h.off[i] = carry + (uint32_t)(incl - n);
                carry += (uint32_t)__shfl_sync(FULL, incl, 31);
            }
            if (threadIdx.x == 0) h.off[nt] = carry;
        }
        __syncthreads();
        const uint32_t wtotal = h.off[nt];
        for (uint32_t e = threadIdx.x; e < wtotal; e += blockDim.x) {
            const uint32_t i = tile_owner(h, nt, e);
            if (hot) tpcc_apply_write<false>(a.db, h.x[i], e - h.off[i], a.lines, txn_base + t0 + i, hot,
                                             hot + a.db.W, a.results[t0 + i]);
            else tpcc_apply_write<true>(a.db, h.x[i], e - h.off[i], a.lines, txn_base + t0 + i, nullptr,
                                        nullptr, a.results[t0 + i]);
        }
        __syncthreads();
    }
    if (lane == 0) {
        if (c_com) {
            red_add_u64(&a.st->commits, c_com);
            red_add_u64(&a.ctl->total_commits, c_com);
        }
        if (c_raw) red_add_u64(&a.st->raw, c_raw);
        if (c_war) red_add_u64(&a.st->war, c_war);
        if (c_waw) red_add_u64(&a.st->waw, c_waw);
    }
}

__device__ __forceinline__ void hot_init(long long *hot, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) hot[i] = 0;
    __syncthreads();
}
__device__ __forceinline__ void hot_flush(const TpccDev &db, const long long *hot) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 11u * db.W; i += blockDim.x) {
        const long long v = hot[i];
        if (!v) continue;
        uint64_t *p = i < db.W ? col_ptr(db, LTPG_T_WAREHOUSE, i, W_YTD) : col_ptr(db, LTPG_T_DISTRICT, i - db.W, D_YTD);
        red_add_u64(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
    }
}

template <uint32_t P>
__global__ void __launch_bounds__(2 * P) tpcc_exec_tuned(TpccTunedArgs a) {
    __shared__ TileHdrN<P> h;
    tpcc_exec_tiles<P>(a, h, slot_tag(a.ctl->epoch));
}

template <uint32_t P>
__global__ void __launch_bounds__(2 * P) tpcc_checkwb_tuned(TpccTunedArgs a) {
    __shared__ TileHdrN<P> h;
    extern __shared__ __align__(16) long long hot_dyn[];
    long long *hot = a.db.W <= HOT_SMEM_MAX_W ? hot_dyn : nullptr;
    if (hot) hot_init(hot, 11u * a.db.W);
    tpcc_checkwb_tiles<P>(a, h, a.ctl->epoch, hot);
    if (hot) hot_flush(a.db, hot);
    finish_batch(a.ctl);
}

// One cooperative kernel per batch: execute+register, a bounded grid barrier,
// check + write-back.  What the second phase loads that the first wrote:
// registration slots (ld_slot: ld.global.cg, served by L2) and the tile's
// results (written by the same block, ordered by __syncthreads).  Table rows
// are read through the read-only path only in the first phase, before any
// row is written; the second phase's read-modify-writes (C_BALANCE,
// S_QUANTITY by atomicCAS) touch rows that one committed transaction writes
// (WAW), whose batch-start value is what they must see.
template <uint32_t P>
__global__ void __launch_bounds__(2 * P) tpcc_persistent(TpccTunedArgs a) {
    __shared__ TileHdrN<P> h;
    extern __shared__ __align__(16) long long hot_dyn[];
    long long *hot = a.db.W <= HOT_SMEM_MAX_W ? hot_dyn : nullptr;
    const uint32_t epoch = a.ctl->epoch;
    if (hot) hot_init(hot, 11u * a.db.W);
    tpcc_exec_tiles<P>(a, h, slot_tag(epoch));
    if (grid_barrier(a.ctl)) tpcc_checkwb_tiles<P>(a, h, epoch, hot);
    if (hot) hot_flush(a.db, hot);
    finish_batch(a.ctl);
}

template <uint32_t P>
static cudaError_t tpcc_launch_tuned(ltpg_ctx *c, const TpccTunedArgs &a_in, int mode) {
    TpccTunedArgs a = a_in;
    constexpr uint32_t threads = 2 * P;
    const size_t smem = a.db.W <= HOT_SMEM_MAX_W ? 11u * a.db.W * sizeof(long long) : 0u;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, mode == LTPG_MODE_PERSISTENT ? (const void *)tpcc_persistent<P> : (const void *)tpcc_checkwb_tuned<P>,
        threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (c->launch_c.blocks_per_sm && (int)c->launch_c.blocks_per_sm < per_sm) per_sm = (int)c->launch_c.blocks_per_sm;
    const uint32_t n_tiles = (a.B + P - 1) / P;
    const uint32_t grid = std::min<uint32_t>(n_tiles, (uint32_t)(per_sm * c->sm_count));
    if (mode == LTPG_MODE_PERSISTENT) {
        prof_mark(c, 0);
        void *args[] = {&a};
        count_launch(c);
        e = cudaLaunchCooperativeKernel((const void *)tpcc_persistent<P>, dim3(grid), dim3(threads), args, smem,
                                        c->stream);
        if (e != cudaSuccess) return e;
        for (int m = 1; m < PROF_MARKS; ++m) prof_mark(c, m);
        return cudaSuccess;
    }
    prof_mark(c, 0);
    count_launch(c);
    tpcc_exec_tuned<P><<<grid, threads, 0, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 1);
    count_launch(c);
    tpcc_checkwb_tuned<P><<<grid, threads, smem, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int m = 2; m < PROF_MARKS; ++m) prof_mark(c, m);
    return cudaSuccess;
}

cudaError_t tpcc_run_tuned(ltpg_ctx *c, Slot &s, int mode) {
    if (s.n_txn == 0) return cudaSuccess;
    TpccTunedArgs a;
    a.txns = s.txns;
    a.lines = s.lines;
    a.hdr = s.dev_hdr;
    a.B = s.n_txn;
    a.db = make_dev(c);
    a.reg = c->tpcc.reg;
    a.results = s.results;
    a.flags = s.flags;
    a.bitmap = s.bitmap;
    a.st = s.stats;
    a.ctl = c->ctl;
    a.filter = c->launch_c.filter;
    a.dedupe = c->launch_c.dedupe;
    cudaError_t e = cudaMemsetAsync(s.stats, 0, sizeof(DevStats), c->stream);
    if (e != cudaSuccess) return e;
    // block_threads 128 / 256 / 512: tiles of 64 / 128 / 256 transactions
    switch (c->launch_c.block) {
    case 256: return tpcc_launch_tuned<128>(c, a, mode);
    case 512: return tpcc_launch_tuned<256>(c, a, mode);
    default: return tpcc_launch_tuned<64>(c, a, mode);
    }
}

// Packed order lines (ltpg_tpcc_pack_lines) back to ltpg_tpcc_line: one
// 4-byte load and one 8-byte store per line.
__global__ void __launch_bounds__(256) tpcc_unpack_lines_kernel(const uint32_t *__restrict__ packed, uint64_t n,
                                                                 ltpg_tpcc_line *__restrict__ lines) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        const uint32_t p = __ldg(packed + i);
        reinterpret_cast<uint2 *>(lines)[i] = make_uint2(p & 0x1FFFFu, ((p >> 17) & 0x7FFu) | ((p >> 28) << 16));
    }
}

cudaError_t tpcc_unpack_lines(Slot &s, cudaStream_t st) {
    const uint64_t n = s.n_lines;
    if (!n) return cudaSuccess;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((n + 255) / 256, 4096);
    tpcc_unpack_lines_kernel<<<grid, 256, 0, st>>>(s.packed_lines, n, s.lines);
    return cudaGetLastError();
}

}  // namespace ltpg
