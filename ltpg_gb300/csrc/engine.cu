// engine.cu — the C ABI: context, tables, batch slots, phase dispatch, results.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>

#include "engine.h"

using namespace ltpg;

namespace {

int fail(ltpg_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(ltpg_ctx *c, cudaError_t e, const char *what) {
    return fail(c, LTPG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)

template <class T>
cudaError_t dev_alloc(T **p, uint64_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void **)p, count * sizeof(T));
}
template <class T>
void dev_free(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

void free_slot(Slot &s) {
    dev_free(s.ops);
    dev_free(s.val_off);
    dev_free(s.vals);
    dev_free(s.off_blocks);
    dev_free(s.txns);
    dev_free(s.lines);
    dev_free(s.packed_lines);
    dev_free(s.dev_hdr);
    dev_free(s.flags);
    dev_free(s.bitmap);
    dev_free(s.results);
    dev_free(s.stats);
    if (s.copied) cudaEventDestroy(s.copied);
    if (s.done) cudaEventDestroy(s.done);
    s = Slot{};
}

void drop_graphs(ltpg_ctx *c) {
    for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

// Output buffers of a slot, sized for n transactions.
int ensure_outputs(ltpg_ctx *c, Slot &s, uint64_t n) {
    if (s.cap_out >= n && s.stats) return LTPG_OK;
    dev_free(s.flags);
    dev_free(s.bitmap);
    dev_free(s.results);
    dev_free(s.stats);
    const uint64_t cap = std::max<uint64_t>(n, c->cfg.max_txn);
    // a multiple of 4 bytes: write-first registration ORs conflict bits into
    // the flag bytes with 32-bit atomics
    CK(dev_alloc(&s.flags, (cap + 3) / 4 * 4), "alloc flags");
    CK(dev_alloc(&s.bitmap, (cap + 31) / 32 + 1), "alloc bitmap");
    CK(dev_alloc(&s.results, cap), "alloc results");
    CK(dev_alloc(&s.stats, 1), "alloc stats");
    CK(cudaMemset(s.stats, 0, sizeof(DevStats)), "clear stats");
    s.cap_out = cap;
    drop_graphs(c);
    return LTPG_OK;
}

// Reads and clears the device error word; call after a synchronisation.
int check_device_error(ltpg_ctx *c) {
    DevCtl h;
    CK(cudaMemcpy(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost), "read control block");
    if (h.error == 0) return LTPG_OK;
    const uint32_t error = h.error, index = h.err_index;
    // clear the error and any barrier / completion state a failed kernel left
    h.error = 0;
    h.err_index = 0;
    h.done = 0;
    h.barrier_count = 0;
    CK(cudaMemcpy(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice), "clear error");
    char buf[160];
    if (error & DERR_TIMEOUT) {
        snprintf(buf, sizeof buf, "device wait timed out (block %u)", index);
        return fail(c, LTPG_ERR_TIMEOUT, buf);
    }
    snprintf(buf, sizeof buf, "key or index out of range in batch (transaction %u)", index);
    return fail(c, LTPG_ERR_BOUNDS, buf);
}

int ensure_prof_events(ltpg_ctx *c) {
    const size_t need = c->slots.size() * PROF_MARKS;
    while (c->prof_events.size() < need) {
        cudaEvent_t ev;
        CK(cudaEventCreate(&ev), "event create");
        c->prof_events.push_back(ev);
    }
    return LTPG_OK;
}

Slot *get_slot(ltpg_ctx *c, uint32_t slot) {
    if (!c || slot >= c->slots.size()) return nullptr;
    return &c->slots[slot];
}

}  // namespace

namespace ltpg {

__global__ void ctl_set_epoch_kernel(DevCtl *ctl, uint32_t epoch) {
    ctl->epoch = epoch;
    ctl->done = 0u;
}

cudaError_t ctl_set_epoch(DevCtl *ctl, uint32_t epoch, cudaStream_t st) {
    ctl_set_epoch_kernel<<<1, 1, 0, st>>>(ctl, epoch);
    return cudaGetLastError();
}

int epoch_reserve(ltpg_ctx *c, uint64_t batches) {
    if (c->epoch_next + batches - 1 <= kEpochLast) {
        c->epoch_next += batches;
        return LTPG_OK;
    }
    // The batches would pass the last epoch: every slot back to the cleared
    // state (all ones: tag 0xFFFFFFFF, which no epoch from 1 on carries) and
    // the epoch to 1, on the context stream ahead of the batches.  The kernels
    // read the epoch from device memory, so captured graphs stay valid.
    if (batches > kEpochLast) return fail(c, LTPG_ERR_INVALID, "too many batches in one launch");
    if (c->ycsb.reg)
        CK(cudaMemsetAsync(c->ycsb.reg, 0xFF, c->ycsb.n * sizeof(RegSlot), c->stream), "clear YCSB slots");
    if (c->tpcc.reg)
        CK(cudaMemsetAsync(c->tpcc.reg, 0xFF, c->tpcc.n_slots * sizeof(RegSlot), c->stream), "clear TPC-C slots");
    CK(ctl_set_epoch(c->ctl, 1u, c->stream), "reset epoch");
    c->epoch_next = 1 + batches;
    return LTPG_OK;
}

void drop_graphs_ctx(ltpg_ctx *c) { drop_graphs(c); }
void prof_mark(ltpg_ctx *c, int i) {
    if (!c->profiling) return;
    const size_t k = (size_t)c->cur_slot * PROF_MARKS + (size_t)i;
    if (k >= c->prof_events.size()) return;
    if (c->capturing) cudaEventRecordWithFlags(c->prof_events[k], c->stream, cudaEventRecordExternal);
    else cudaEventRecord(c->prof_events[k], c->stream);
}
}  // namespace ltpg

extern "C" {

int ltpg_create(const ltpg_config *cfg, ltpg_ctx **out) {
    if (!cfg || !out) return LTPG_ERR_INVALID;
    *out = nullptr;
    if (cfg->n_slots == 0 || cfg->n_slots > 4096 || cfg->max_txn == 0 || cfg->max_txn > (1u << 26))
        return LTPG_ERR_INVALID;
    if (cfg->max_ops_per_txn > LTPG_YCSB_MAX_OPS) return LTPG_ERR_INVALID;
    ltpg_ctx *c = new (std::nothrow) ltpg_ctx();
    if (!c) return LTPG_ERR_NOMEM;
    c->cfg = *cfg;
    if (c->cfg.max_ops_per_txn == 0) c->cfg.max_ops_per_txn = 16;
    if (c->cfg.max_lines == 0) c->cfg.max_lines = c->cfg.max_txn * 10u;
    c->device = cfg->device;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->ctl, sizeof(DevCtl));
    if (e == cudaSuccess) {
        DevCtl h{};
        h.epoch = 1;
        e = cudaMemcpy(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        if (c->ctl) cudaFree(c->ctl);
        if (c->own_stream) cudaStreamDestroy(c->own_stream);
        delete c;
        return LTPG_ERR_CUDA;
    }
    c->stream = c->own_stream;
    c->slots.resize(cfg->n_slots);
    c->launch_c.block = 128;  // the tuned TPC-C kernels' default block (64-transaction tiles)
    *out = c;
    return LTPG_OK;
}

int ltpg_destroy(ltpg_ctx *c) {
    if (!c) return LTPG_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    for (auto ev : c->prof_events) cudaEventDestroy(ev);
    predictor_free(c);
    for (auto &s : c->slots) free_slot(s);
    dev_free(c->ycsb.rows);
    dev_free(c->ycsb.reg);
    dev_free(c->ycsb.wbits);
    dev_free(c->ycsb.upd);
    for (auto &t : c->tpcc.tab) dev_free(t);
    dev_free(c->tpcc.reg);
    dev_free(c->tpcc.name_idx);
    dev_free(c->stage_map);
    dev_free(c->stage_bits);
    dev_free(c->stage_rank);
    dev_free(c->bucket_counts);
    dev_free(c->ctl);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return LTPG_OK;
}

const char *ltpg_last_error(const ltpg_ctx *c) { return c ? c->err.c_str() : "null context"; }

int ltpg_set_stream(ltpg_ctx *c, void *stream) {
    if (!c) return LTPG_ERR_INVALID;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return LTPG_OK;
}
void *ltpg_get_stream(ltpg_ctx *c) { return c ? (void *)c->stream : nullptr; }

int ltpg_sync(ltpg_ctx *c) {
    if (!c) return LTPG_ERR_INVALID;
    CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    return check_device_error(c);
}

void *ltpg_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}
void ltpg_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

// ---- tables -----------------------------------------------------------------
int ltpg_db_load_ycsb(ltpg_ctx *c, uint64_t seed, uint64_t n) {
    if (!c) return LTPG_ERR_INVALID;
    if (n == 0 || n > (1ull << LTPG_YCSB_KEY_BITS)) return fail(c, LTPG_ERR_INVALID, "YCSB table size out of range");
    CK(cudaSetDevice(c->device), "set device");
    CK(cudaStreamSynchronize(c->stream), "sync");
    drop_graphs(c);
    dev_free(c->ycsb.rows);
    dev_free(c->ycsb.reg);
    dev_free(c->ycsb.wbits);
    c->ycsb.n = 0;
    CK(dev_alloc(&c->ycsb.rows, n * LTPG_YCSB_FIELDS), "alloc YCSB table");
    CK(dev_alloc(&c->ycsb.reg, n), "alloc YCSB registration table");
    CK(dev_alloc(&c->ycsb.wbits, (n + 31) / 32), "alloc YCSB writer bitmap");
    c->ycsb.n = n;
    c->ycsb_seed = seed;
    CK(ycsb_init_table(c), "init YCSB table");
    return ltpg_sync(c);
}

int ltpg_db_load_tpcc(ltpg_ctx *c, uint64_t seed, uint32_t W) {
    if (!c) return LTPG_ERR_INVALID;
    if (W == 0 || W > 4096) return fail(c, LTPG_ERR_INVALID, "warehouse count out of range");
    CK(cudaSetDevice(c->device), "set device");
    CK(cudaStreamSynchronize(c->stream), "sync");
    drop_graphs(c);
    for (auto &t : c->tpcc.tab) dev_free(t);
    dev_free(c->tpcc.reg);
    dev_free(c->tpcc.name_idx);
    c->tpcc = TpccDb{};
    uint64_t total = 0;
    for (uint32_t t = 0; t < LTPG_TPCC_TABLES; ++t) {
        c->tpcc.rows[t] = tpcc_rows(t, W);
        c->tpcc.base[t] = total;
        total += c->tpcc.rows[t];
        CK(dev_alloc(&c->tpcc.tab[t], c->tpcc.rows[t] * TPCC_COLS[t]), "alloc TPC-C table");
    }
    if (total >= (1ull << 32)) return fail(c, LTPG_ERR_INVALID, "too many rows for 32-bit slots");
    CK(dev_alloc(&c->tpcc.reg, total), "alloc TPC-C registration table");
    CK(dev_alloc(&c->tpcc.name_idx, c->tpcc.rows[LTPG_T_CUSTOMER]), "alloc customer name index");
    c->tpcc.n_slots = total;
    c->tpcc.W = W;
    c->tpcc_seed = seed;
    CK(tpcc_init_tables(c), "init TPC-C tables");
    CK(tpcc_build_name_index(c), "build customer name index");
    return ltpg_sync(c);
}

}  // extern "C"

namespace {
// table id: 0..8 TPC-C tables, 100 = YCSB table.
int table_ptr(ltpg_ctx *c, uint32_t table, uint64_t **p, uint64_t *count) {
    if (table == LTPG_TABLE_YCSB) {
        if (!c->ycsb.rows) return fail(c, LTPG_ERR_STATE, "no YCSB table loaded");
        *p = c->ycsb.rows;
        *count = c->ycsb.n * LTPG_YCSB_FIELDS;
        return LTPG_OK;
    }
    if (table < LTPG_TPCC_TABLES) {
        if (!c->tpcc.W) return fail(c, LTPG_ERR_STATE, "no TPC-C tables loaded");
        *p = c->tpcc.tab[table];
        *count = c->tpcc.rows[table] * TPCC_COLS[table];
        return LTPG_OK;
    }
    return fail(c, LTPG_ERR_INVALID, "unknown table id");
}
}  // namespace

extern "C" {

int ltpg_db_table_shape(ltpg_ctx *c, uint32_t table, uint64_t *rows, uint32_t *cols) {
    if (!c || !rows || !cols) return LTPG_ERR_INVALID;
    uint64_t *p;
    uint64_t n;
    int r = table_ptr(c, table, &p, &n);
    if (r) return r;
    *cols = table == LTPG_TABLE_YCSB ? LTPG_YCSB_FIELDS : TPCC_COLS[table];
    *rows = n / *cols;
    return LTPG_OK;
}

int ltpg_db_upload(ltpg_ctx *c, uint32_t table, const void *host, size_t bytes) {
    if (!c || !host) return LTPG_ERR_INVALID;
    uint64_t *p;
    uint64_t n;
    int r = table_ptr(c, table, &p, &n);
    if (r) return r;
    if (bytes != n * 8) return fail(c, LTPG_ERR_INVALID, "image size mismatch");
    CK(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, c->stream), "upload table");
    if (table == LTPG_T_CUSTOMER) CK(tpcc_build_name_index(c), "build customer name index");
    return ltpg_sync(c);
}

int ltpg_db_download(ltpg_ctx *c, uint32_t table, void *host, size_t bytes) {
    if (!c || !host) return LTPG_ERR_INVALID;
    uint64_t *p;
    uint64_t n;
    int r = table_ptr(c, table, &p, &n);
    if (r) return r;
    if (bytes != n * 8) return fail(c, LTPG_ERR_INVALID, "image size mismatch");
    CK(cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, c->stream), "download table");
    return ltpg_sync(c);
}

// ---- batches ---------------------------------------------------------------------
}  // extern "C"

namespace ltpg {

int slot_prepare_ycsb(ltpg_ctx *c, uint32_t slot, uint32_t n_txn, uint32_t k, uint32_t n_updates, Slot **out) {
    Slot *s = get_slot(c, slot);
    if (!s) return fail(c, LTPG_ERR_INVALID, "bad slot or batch");
    if (!c->ycsb.rows) return fail(c, LTPG_ERR_STATE, "no YCSB table loaded");
    if (n_txn == 0 || n_txn > c->cfg.max_txn) return fail(c, LTPG_ERR_INVALID, "batch larger than max_txn");
    if (k == 0 || k > c->cfg.max_ops_per_txn) return fail(c, LTPG_ERR_INVALID, "bad ops_per_txn / op_stride");
    if (n_updates > (uint64_t)n_txn * k) return fail(c, LTPG_ERR_INVALID, "too many updates");
    if (!s->ops) {
        const uint64_t cap_ops = (uint64_t)c->cfg.max_txn * ycsb_stride(c->cfg.max_ops_per_txn);
        const uint64_t cap_vals = (uint64_t)c->cfg.max_txn * c->cfg.max_ops_per_txn;
        CK(dev_alloc(&s->ops, cap_ops), "alloc ops");
        CK(dev_alloc(&s->val_off, (uint64_t)c->cfg.max_txn + 1), "alloc val_off");
        CK(dev_alloc(&s->off_blocks, ((uint64_t)c->cfg.max_txn + 1023) / 1024 + 1), "alloc offset sums");
        CK(dev_alloc(&s->vals, cap_vals), "alloc vals");
        s->cap_ops = cap_ops;
        s->cap_vals = cap_vals;
        if (c->ycsb.upd_cap < cap_vals) {
            dev_free(c->ycsb.upd);
            c->ycsb.upd_cap = 0;
            CK(dev_alloc(&c->ycsb.upd, cap_vals), "alloc update list");
            c->ycsb.upd_cap = cap_vals;
        }
        s->cap_txn_y = c->cfg.max_txn;
    }
    int r = ensure_outputs(c, *s, n_txn);
    if (r) return r;
    if (s->workload != LTPG_WORKLOAD_YCSB || s->n_txn != n_txn || s->k != k) drop_graphs(c);
    s->workload = LTPG_WORKLOAD_YCSB;
    s->n_txn = n_txn;
    s->k = k;
    s->stride = ycsb_stride(k);
    s->n_updates = n_updates;
    *out = s;
    return LTPG_OK;
}

int slot_prepare_tpcc(ltpg_ctx *c, uint32_t slot, uint32_t n_txn, uint64_t n_lines, uint64_t txn_base, Slot **out) {
    Slot *s = get_slot(c, slot);
    if (!s) return fail(c, LTPG_ERR_INVALID, "bad slot or batch");
    if (!c->tpcc.W) return fail(c, LTPG_ERR_STATE, "no TPC-C tables loaded");
    if (n_txn == 0 || n_txn > c->cfg.max_txn) return fail(c, LTPG_ERR_INVALID, "batch larger than max_txn");
    if (n_lines > c->cfg.max_lines) return fail(c, LTPG_ERR_INVALID, "batch has more lines than max_lines");
    if (!s->txns) {
        CK(dev_alloc(&s->txns, c->cfg.max_txn), "alloc txns");
        CK(dev_alloc(&s->lines, (uint64_t)c->cfg.max_lines + 1), "alloc lines");
        CK(dev_alloc(&s->dev_hdr, 2), "alloc slot header");
        s->cap_txn_c = c->cfg.max_txn;
        s->cap_lines = c->cfg.max_lines;
    }
    int r = ensure_outputs(c, *s, n_txn);
    if (r) return r;
    if (s->workload != LTPG_WORKLOAD_TPCC || s->n_txn != n_txn) drop_graphs(c);
    s->workload = LTPG_WORKLOAD_TPCC;
    s->n_txn = n_txn;
    s->n_lines = (uint32_t)n_lines;
    s->txn_base = txn_base;
    *out = s;
    return LTPG_OK;
}

int ctx_fail(ltpg_ctx *c, int code, const char *msg) { return fail(c, code, msg); }
int ctx_cuda_fail(ltpg_ctx *c, cudaError_t e, const char *what) { return cuda_fail(c, e, what); }

}  // namespace ltpg

namespace {
// derive_st: the stream that makes the value offsets of a batch without them
// (after the op words' copy on st; null: the offsets are left to the caller).
int upload_ycsb(ltpg_ctx *c, uint32_t slot, const ltpg_ycsb_batch *b, cudaStream_t st, cudaStream_t derive_st) {
    if (!c || !b) return c ? fail(c, LTPG_ERR_INVALID, "bad slot or batch") : LTPG_ERR_INVALID;
    if (b->ops_per_txn == 0 || b->op_stride != ycsb_stride(b->ops_per_txn))
        return fail(c, LTPG_ERR_INVALID, "bad ops_per_txn / op_stride");
    if (!b->ops || (b->n_updates && !b->vals)) return fail(c, LTPG_ERR_INVALID, "null batch array");
    Slot *s = nullptr;
    int r = slot_prepare_ycsb(c, slot, b->n_txn, b->ops_per_txn, b->n_updates, &s);
    if (r) return r;
    const uint64_t n_ops = (uint64_t)b->n_txn * b->op_stride;
    CK(cudaMemcpyAsync(s->ops, b->ops, n_ops * 4, cudaMemcpyHostToDevice, st), "upload ops");
    if (b->val_off)
        CK(cudaMemcpyAsync(s->val_off, b->val_off, ((uint64_t)b->n_txn + 1) * 4, cudaMemcpyHostToDevice, st),
           "upload val_off");
    else if (derive_st)  // made on the device from the op words, behind their copy
        CK(ycsb_derive_offsets(c, *s, derive_st), "value offsets");
    if (b->n_updates)
        CK(cudaMemcpyAsync(s->vals, b->vals, (uint64_t)b->n_updates * 8, cudaMemcpyHostToDevice, st), "upload vals");
    return LTPG_OK;
}

// packed: the order lines in the 4-byte form (b->lines unused), copied to the
// slot's packed buffer; unpack_st: the stream that unpacks them (null: left to
// the caller).
int upload_tpcc(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b, cudaStream_t st,
                const uint32_t *packed = nullptr, cudaStream_t unpack_st = nullptr) {
    if (!c || !b) return c ? fail(c, LTPG_ERR_INVALID, "bad slot or batch") : LTPG_ERR_INVALID;
    if (!b->txns || (b->n_lines && !b->lines && !packed)) return fail(c, LTPG_ERR_INVALID, "null batch array");
    Slot *s = nullptr;
    int r = slot_prepare_tpcc(c, slot, b->n_txn, b->n_lines, b->txn_base, &s);
    if (r) return r;
    CK(cudaMemcpyAsync(s->txns, b->txns, (uint64_t)b->n_txn * sizeof(ltpg_tpcc_txn), cudaMemcpyHostToDevice, st),
       "upload txns");
    if (b->n_lines && packed) {
        if (!s->packed_lines) CK(dev_alloc(&s->packed_lines, s->cap_lines + 1), "alloc packed lines");
        CK(cudaMemcpyAsync(s->packed_lines, packed, (uint64_t)b->n_lines * 4, cudaMemcpyHostToDevice, st),
           "upload packed lines");
        if (unpack_st) CK(tpcc_unpack_lines(*s, unpack_st), "unpack lines");
    } else if (b->n_lines) {
        CK(cudaMemcpyAsync(s->lines, b->lines, (uint64_t)b->n_lines * sizeof(ltpg_tpcc_line),
                           cudaMemcpyHostToDevice, st),
           "upload lines");
    }
    s->host_hdr[0] = b->n_lines;
    s->host_hdr[1] = b->txn_base;
    // pageable source: the runtime stages it before returning, so the next
    // upload may overwrite host_hdr at once
    CK(cudaMemcpyAsync(s->dev_hdr, s->host_hdr, sizeof s->host_hdr, cudaMemcpyHostToDevice, st),
       "upload slot header");
    return LTPG_OK;
}
}  // namespace

extern "C" {

int ltpg_batch_upload_ycsb(ltpg_ctx *c, uint32_t slot, const ltpg_ycsb_batch *b) {
    return c ? upload_ycsb(c, slot, b, c->stream, c->stream) : LTPG_ERR_INVALID;
}
int ltpg_batch_upload_tpcc(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b) {
    return c ? upload_tpcc(c, slot, b, c->stream) : LTPG_ERR_INVALID;
}
int ltpg_batch_upload_tpcc_packed(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b, const uint32_t *packed) {
    if (!c) return LTPG_ERR_INVALID;
    if (b && b->n_lines && !packed) return fail(c, LTPG_ERR_INVALID, "null packed lines");
    return upload_tpcc(c, slot, b, c->stream, packed, c->stream);
}
int ltpg_tpcc_pack_lines(const ltpg_tpcc_line *lines, uint64_t n, uint32_t *packed) {
    if (n && (!lines || !packed)) return LTPG_ERR_INVALID;
    for (uint64_t i = 0; i < n; ++i) {
        const ltpg_tpcc_line &l = lines[i];
        if (l.i_id >= (1u << 17) || l.supply_w >= (1u << 11) || l.qty >= 16u) return LTPG_ERR_INVALID;
        packed[i] = l.i_id | ((uint32_t)l.supply_w << 17) | ((uint32_t)l.qty << 28);
    }
    return LTPG_OK;
}

}  // extern "C"

namespace {

int run_phase(ltpg_ctx *c, uint32_t slot, int phase) {
    Slot *s = get_slot(c, slot);
    if (!s) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    c->cur_slot = slot;
    if (s->workload != LTPG_WORKLOAD_YCSB && s->workload != LTPG_WORKLOAD_TPCC)
        return fail(c, LTPG_ERR_STATE, "slot holds no batch");
    // a batch's epoch is taken at its first phase and advanced by its last
    if (phase == 0 && !c->capturing) {
        int r = epoch_reserve(c, 1);
        if (r) return r;
    }
    count_launch(c);
    cudaError_t e;
    if (s->workload == LTPG_WORKLOAD_YCSB) e = ycsb_phase(c, *s, phase);
    else if (s->workload == LTPG_WORKLOAD_TPCC) e = tpcc_phase(c, *s, phase);
    else return fail(c, LTPG_ERR_STATE, "slot holds no batch");
    if (e != cudaSuccess) return cuda_fail(c, e, "phase launch");
    return LTPG_OK;
}

int run_one(ltpg_ctx *c, uint32_t slot, int mode) {
    Slot *s = get_slot(c, slot);
    if (!s) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    c->cur_slot = slot;
    if (s->workload != LTPG_WORKLOAD_YCSB && s->workload != LTPG_WORKLOAD_TPCC)
        return fail(c, LTPG_ERR_STATE, "slot holds no batch");
    if (mode == LTPG_MODE_PLAIN) {  // intervals: execute, check, (no reads), write-back
        static const int after[3][2] = {{1, 1}, {2, 3}, {4, 4}};
        prof_mark(c, 0);
        for (int p = 0; p < 3; ++p) {
            int r = run_phase(c, slot, p);
            if (r) return r;
            prof_mark(c, after[p][0]);
            if (after[p][1] != after[p][0]) prof_mark(c, after[p][1]);
        }
        return LTPG_OK;
    }
    cudaError_t e;
    if (s->workload == LTPG_WORKLOAD_YCSB) e = ycsb_run_tuned(c, *s, mode);
    else if (s->workload == LTPG_WORKLOAD_TPCC) e = tpcc_run_tuned(c, *s, mode);
    else return fail(c, LTPG_ERR_STATE, "slot holds no batch");
    if (e != cudaSuccess) return cuda_fail(c, e, "tuned launch");
    return LTPG_OK;
}

}  // namespace

extern "C" {

int ltpg_execute_register(ltpg_ctx *c, uint32_t slot) { return run_phase(c, slot, 0); }
int ltpg_check_conflict(ltpg_ctx *c, uint32_t slot) { return run_phase(c, slot, 1); }
int ltpg_write_back(ltpg_ctx *c, uint32_t slot) { return run_phase(c, slot, 2); }

int ltpg_run_batch(ltpg_ctx *c, uint32_t slot, int mode) {
    if (!c) return LTPG_ERR_INVALID;
    if (mode == LTPG_MODE_GRAPH) return ltpg_run_batches(c, slot, 1, mode);
    if (mode < LTPG_MODE_PLAIN || mode > LTPG_MODE_GRAPH) return fail(c, LTPG_ERR_INVALID, "bad mode");
    if (mode != LTPG_MODE_PLAIN) {  // the plain mode reserves in its execute phase
        int r = epoch_reserve(c, 1);
        if (r) return r;
    }
    return run_one(c, slot, mode);
}

int ltpg_run_batches(ltpg_ctx *c, uint32_t first, uint32_t count, int mode) {
    if (!c) return LTPG_ERR_INVALID;
    if (count == 0) return LTPG_OK;
    if ((uint64_t)first + count > c->slots.size()) return fail(c, LTPG_ERR_INVALID, "slot range out of bounds");
    if (mode != LTPG_MODE_GRAPH) {
        for (uint32_t i = 0; i < count; ++i) {
            int r = ltpg_run_batch(c, first + i, mode);
            if (r) return r;
        }
        return LTPG_OK;
    }
    const int wl = c->slots[first].workload;
    for (uint32_t i = 0; i < count; ++i) {
        const int w = c->slots[first + i].workload;
        if (w != LTPG_WORKLOAD_YCSB && w != LTPG_WORKLOAD_TPCC) return fail(c, LTPG_ERR_STATE, "slot holds no batch");
    }
    int r = epoch_reserve(c, count);
    if (r) return r;
    for (auto &g : c->graphs)
        if (g.first == first && g.count == count && g.workload == wl) {
            CK(cudaGraphLaunch(g.exec, c->stream), "graph launch");
            count_launch(c, g.kernels);
            return LTPG_OK;
        }
    // Capture the fused kernels of `count` batches into one graph.  The batch
    // epoch lives in device memory and is advanced by the kernels themselves,
    // so the graph can be replayed as is.
    cudaStream_t cap = c->stream;
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    const uint64_t launches0 = c->launches;
    c->capturing = true;
    for (uint32_t i = 0; i < count && r == LTPG_OK; ++i) r = run_one(c, first + i, LTPG_MODE_FUSED);
    c->capturing = false;
    const uint64_t kernels = c->launches - launches0;
    c->launches = launches0;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    if (r) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    c->graphs.push_back({first, count, wl, exec, kernels});
    CK(cudaGraphLaunch(exec, c->stream), "graph launch");
    count_launch(c, kernels);
    return LTPG_OK;
}

int ltpg_run_ycsb_host(ltpg_ctx *c, uint32_t slot, const ltpg_ycsb_batch *b, int mode, uint32_t *host_bitmap) {
    int r = ltpg_batch_upload_ycsb(c, slot, b);
    if (r) return r;
    r = ltpg_run_batch(c, slot, mode);
    if (r) return r;
    if (host_bitmap) {
        Slot &s = c->slots[slot];
        CK(cudaMemcpyAsync(host_bitmap, s.bitmap, ((uint64_t)s.n_txn + 31) / 32 * 4, cudaMemcpyDeviceToHost,
                           c->stream),
           "bitmap download");
    }
    return ltpg_sync(c);
}

int ltpg_run_tpcc_host(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b, int mode, uint32_t *host_bitmap) {
    int r = ltpg_batch_upload_tpcc(c, slot, b);
    if (r) return r;
    r = ltpg_run_batch(c, slot, mode);
    if (r) return r;
    if (host_bitmap) {
        Slot &s = c->slots[slot];
        CK(cudaMemcpyAsync(host_bitmap, s.bitmap, ((uint64_t)s.n_txn + 31) / 32 * 4, cudaMemcpyDeviceToHost,
                           c->stream),
           "bitmap download");
    }
    return ltpg_sync(c);
}

// Pipelined host calls: the batch is copied on the copy stream once the slot's
// previous use is over, the run waits for the copy on the compute stream, and
// the bitmap download follows the run; nothing blocks the caller, so the copy
// of the next batch overlaps this one's kernels.
extern "C++" {
namespace {
// derive: make the YCSB value offsets on the compute stream once the copy is
// done (a batch uploaded without them): kernels on the copy stream would wait
// there for SMs held by the previous batch and hold up the next copy.
template <class Up>
int submit_host(ltpg_ctx *c, uint32_t slot, int mode, uint32_t *host_bitmap, Up upload, bool derive = false,
                bool unpack = false) {
    Slot *s = get_slot(c, slot);
    if (!s) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    if (!c->copy_stream) CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "create copy stream");
    if (!s->copied) CK(cudaEventCreateWithFlags(&s->copied, cudaEventDisableTiming), "create event");
    if (!s->done) {
        CK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming), "create event");
        CK(cudaEventRecord(s->done, c->stream), "record event");
    }
    CK(cudaStreamWaitEvent(c->copy_stream, s->done, 0), "wait for the slot");
    int r = upload(c->copy_stream);
    if (r) return r;
    CK(cudaEventRecord(s->copied, c->copy_stream), "record copy");
    CK(cudaStreamWaitEvent(c->stream, s->copied, 0), "wait for the copy");
    if (derive) CK(ycsb_derive_offsets(c, *s, c->stream), "value offsets");
    if (unpack) CK(tpcc_unpack_lines(*s, c->stream), "unpack lines");
    r = ltpg_run_batch(c, slot, mode);
    if (r) return r;
    if (host_bitmap)
        CK(cudaMemcpyAsync(host_bitmap, s->bitmap, ((uint64_t)s->n_txn + 31) / 32 * 4, cudaMemcpyDeviceToHost,
                           c->stream),
           "bitmap download");
    CK(cudaEventRecord(s->done, c->stream), "record done");
    return LTPG_OK;
}
}  // namespace
}  // extern "C++"

int ltpg_submit_ycsb_host(ltpg_ctx *c, uint32_t slot, const ltpg_ycsb_batch *b, int mode, uint32_t *host_bitmap) {
    if (!c) return LTPG_ERR_INVALID;
    return submit_host(
        c, slot, mode, host_bitmap, [&](cudaStream_t st) { return upload_ycsb(c, slot, b, st, nullptr); },
        b && !b->val_off);
}

int ltpg_submit_tpcc_host(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b, int mode, uint32_t *host_bitmap) {
    if (!c) return LTPG_ERR_INVALID;
    return submit_host(c, slot, mode, host_bitmap, [&](cudaStream_t st) { return upload_tpcc(c, slot, b, st); });
}

int ltpg_submit_tpcc_packed_host(ltpg_ctx *c, uint32_t slot, const ltpg_tpcc_batch *b, const uint32_t *packed,
                                 int mode, uint32_t *host_bitmap) {
    if (!c) return LTPG_ERR_INVALID;
    if (b && b->n_lines && !packed) return fail(c, LTPG_ERR_INVALID, "null packed lines");
    return submit_host(
        c, slot, mode, host_bitmap, [&](cudaStream_t st) { return upload_tpcc(c, slot, b, st, packed, nullptr); },
        false, b && b->n_lines != 0);
}

int ltpg_submit_generated(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot, int mode,
                          uint32_t *host_bitmap) {
    if (!c || !g) return c ? fail(c, LTPG_ERR_INVALID, "null generator") : LTPG_ERR_INVALID;
    return submit_host(c, slot, mode, host_bitmap,
                       [&](cudaStream_t st) { return gen_device_batch(c, g, batch_id, slot, st); });
}

int ltpg_host_wait(ltpg_ctx *c, uint32_t slot) {
    Slot *s = get_slot(c, slot);
    if (!s) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    if (s->done) CK(cudaEventSynchronize(s->done), "wait for the slot");
    return check_device_error(c);
}

// ---- results -----------------------------------------------------------------
int ltpg_batch_info_get(ltpg_ctx *c, uint32_t slot, ltpg_batch_info *out) {
    Slot *s = get_slot(c, slot);
    if (!s || !out) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    *out = ltpg_batch_info{};
    // counts made on the device (device generation) are read from it
    if (s->workload == LTPG_WORKLOAD_YCSB) {
        uint32_t nu = 0;
        CK(cudaMemcpyAsync(&nu, s->val_off + s->n_txn, 4, cudaMemcpyDeviceToHost, c->stream), "read update count");
        int r = ltpg_sync(c);
        if (r) return r;
        out->workload = LTPG_WORKLOAD_YCSB;
        out->ops_per_txn = s->k;
        out->n_txn = s->n_txn;
        out->n_op_words = (uint64_t)s->n_txn * s->stride;
        out->n_updates = nu;
        return LTPG_OK;
    }
    if (s->workload == LTPG_WORKLOAD_TPCC) {
        uint64_t h[2] = {0, 0};
        CK(cudaMemcpyAsync(h, s->dev_hdr, sizeof h, cudaMemcpyDeviceToHost, c->stream), "read slot header");
        int r = ltpg_sync(c);
        if (r) return r;
        out->workload = LTPG_WORKLOAD_TPCC;
        out->n_txn = s->n_txn;
        out->n_lines = h[0];
        out->txn_base = h[1];
        return LTPG_OK;
    }
    return fail(c, LTPG_ERR_STATE, "slot holds no batch");
}

int ltpg_batch_download(ltpg_ctx *c, uint32_t slot, uint32_t part, void *host, size_t bytes) {
    ltpg_batch_info bi;
    int r = ltpg_batch_info_get(c, slot, &bi);
    if (r) return r;
    const uint64_t n = bi.n_txn;
    Slot *s = get_slot(c, slot);
    const void *src = nullptr;
    size_t need = 0;
    if (s->workload == LTPG_WORKLOAD_YCSB) {
        if (part == 0) src = s->ops, need = bi.n_op_words * 4;
        else if (part == 1) src = s->val_off, need = (n + 1) * 4;
        else if (part == 2) src = s->vals, need = bi.n_updates * 8;
    } else {
        if (part == 0) src = s->txns, need = n * sizeof(ltpg_tpcc_txn);
        else if (part == 1) src = s->lines, need = bi.n_lines * sizeof(ltpg_tpcc_line);
    }
    if (!src) return fail(c, LTPG_ERR_INVALID, "no such batch part");
    if (bytes != need) return fail(c, LTPG_ERR_INVALID, "buffer size differs from the batch part");
    if (need && !host) return fail(c, LTPG_ERR_INVALID, "null buffer");  // an empty part needs none
    if (need) CK(cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, c->stream), "batch download");
    return ltpg_sync(c);
}

int ltpg_commit_bitmap(ltpg_ctx *c, uint32_t slot, uint32_t *host_bits, size_t words) {
    Slot *s = get_slot(c, slot);
    if (!s || !host_bits) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    const size_t need = ((size_t)s->n_txn + 31) / 32;
    if (words < need) return fail(c, LTPG_ERR_INVALID, "bitmap buffer too small");
    CK(cudaMemcpyAsync(host_bits, s->bitmap, need * 4, cudaMemcpyDeviceToHost, c->stream), "bitmap download");
    return ltpg_sync(c);
}

int ltpg_txn_flags(ltpg_ctx *c, uint32_t slot, uint8_t *host, size_t n) {
    Slot *s = get_slot(c, slot);
    if (!s || !host) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    if (n < s->n_txn) return fail(c, LTPG_ERR_INVALID, "flags buffer too small");
    CK(cudaMemcpyAsync(host, s->flags, s->n_txn, cudaMemcpyDeviceToHost, c->stream), "flags download");
    return ltpg_sync(c);
}

int ltpg_txn_results(ltpg_ctx *c, uint32_t slot, int64_t *host, size_t n) {
    Slot *s = get_slot(c, slot);
    if (!s || !host) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    if (n < s->n_txn) return fail(c, LTPG_ERR_INVALID, "results buffer too small");
    CK(cudaMemcpyAsync(host, s->results, (size_t)s->n_txn * 8, cudaMemcpyDeviceToHost, c->stream),
       "results download");
    return ltpg_sync(c);
}

int ltpg_batch_stats_get(ltpg_ctx *c, uint32_t slot, ltpg_batch_stats *out) {
    Slot *s = get_slot(c, slot);
    if (!s || !out) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    DevStats h{};
    CK(cudaMemcpyAsync(&h, s->stats, sizeof h, cudaMemcpyDeviceToHost, c->stream), "stats download");
    int r = ltpg_sync(c);
    if (r) return r;
    out->n_txn = s->n_txn;
    out->commits = h.commits;
    out->raw = h.raw;
    out->war = h.war;
    out->waw = h.waw;
    out->staged_ops = h.staged_ops;
    out->total_ops = h.total_ops;
    return LTPG_OK;
}

int ltpg_commit_bitmap_device(ltpg_ctx *c, uint32_t slot, const uint32_t **dev_bits) {
    Slot *s = get_slot(c, slot);
    if (!s || !dev_bits) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    *dev_bits = s->bitmap;
    return LTPG_OK;
}

int ltpg_set_launch(ltpg_ctx *c, int workload, const ltpg_launch *cfg) {
    if (!c || !cfg) return LTPG_ERR_INVALID;
    if (workload != LTPG_WORKLOAD_YCSB && workload != LTPG_WORKLOAD_TPCC)
        return fail(c, LTPG_ERR_INVALID, "unknown workload");
    if (cfg->block_threads != 128 && cfg->block_threads != 256 && cfg->block_threads != 512)
        return fail(c, LTPG_ERR_INVALID, "block_threads in {128, 256, 512}");
    const uint32_t opt = cfg->ops_per_thread;
    if (opt != 1 && opt != 2 && opt != 4 && opt != 8) return fail(c, LTPG_ERR_INVALID, "ops_per_thread in {1, 2, 4, 8}");
    if (cfg->stage_ways < 1 || cfg->stage_ways > 8) return fail(c, LTPG_ERR_INVALID, "stage_ways in [1, 8]");
    if (cfg->late_reads > 3) return fail(c, LTPG_ERR_INVALID, "late_reads in {0, 1, 2, 3}");
    LaunchCfg &l = workload == LTPG_WORKLOAD_YCSB ? c->launch_y : c->launch_c;
    l.block = cfg->block_threads;
    l.per_thread = cfg->ops_per_thread;
    l.blocks_per_sm = cfg->blocks_per_sm;
    l.ways = cfg->stage_ways;
    l.filter = cfg->filter ? 1u : 0u;
    l.dedupe = cfg->dedupe ? 1u : 0u;
    l.late_reads = cfg->late_reads;
    drop_graphs(c);
    return LTPG_OK;
}

int ltpg_get_launch(ltpg_ctx *c, int workload, ltpg_launch *cfg) {
    if (!c || !cfg) return LTPG_ERR_INVALID;
    if (workload != LTPG_WORKLOAD_YCSB && workload != LTPG_WORKLOAD_TPCC)
        return fail(c, LTPG_ERR_INVALID, "unknown workload");
    const LaunchCfg &l = workload == LTPG_WORKLOAD_YCSB ? c->launch_y : c->launch_c;
    cfg->block_threads = l.block;
    cfg->ops_per_thread = l.per_thread;
    cfg->blocks_per_sm = l.blocks_per_sm;
    cfg->stage_ways = l.ways;
    cfg->filter = l.filter;
    cfg->dedupe = l.dedupe;
    cfg->late_reads = l.late_reads;
    return LTPG_OK;
}

int ltpg_counters(ltpg_ctx *c, uint64_t *commits_total, uint64_t *kernel_launches) {
    if (!c || !commits_total || !kernel_launches) return LTPG_ERR_INVALID;
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, &c->ctl->total_commits, sizeof v, cudaMemcpyDeviceToHost, c->stream), "counter download");
    int r = ltpg_sync(c);
    if (r) return r;
    *commits_total = v;
    *kernel_launches = c->launches;
    return LTPG_OK;
}

int ltpg_set_profiling(ltpg_ctx *c, int on) {
    if (!c) return LTPG_ERR_INVALID;
    if (on) {
        int r = ensure_prof_events(c);
        if (r) return r;
    }
    if (c->profiling != (on != 0)) drop_graphs(c);
    c->profiling = on != 0;
    return LTPG_OK;
}

int ltpg_kernel_times(ltpg_ctx *c, uint32_t slot, float *ms4) {
    Slot *s = get_slot(c, slot);
    if (!s || !ms4) return c ? fail(c, LTPG_ERR_INVALID, "bad slot") : LTPG_ERR_INVALID;
    if (!c->profiling) return fail(c, LTPG_ERR_STATE, "profiling is off");
    CK(cudaStreamSynchronize(c->stream), "sync");
    cudaEvent_t *ev = &c->prof_events[(size_t)slot * PROF_MARKS];
    for (int i = 0; i < PROF_MARKS - 1; ++i) {
        float ms = 0.f;
        cudaError_t e = cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        ms4[i] = e == cudaSuccess ? ms : 0.f;
        if (e != cudaSuccess) cudaGetLastError();
    }
    return LTPG_OK;
}

// ---- test hooks ------------------------------------------------------------------
int ltpg_debug_set_epoch(ltpg_ctx *c, uint32_t epoch) {
    if (!c) return LTPG_ERR_INVALID;
    if (epoch == 0u) return fail(c, LTPG_ERR_INVALID, "epoch 0 carries the cleared slots' tag");
    CK(cudaSetDevice(c->device), "set device");
    CK(ctl_set_epoch(c->ctl, epoch, c->stream), "set epoch");
    c->epoch_next = epoch;
    return ltpg_sync(c);
}

int ltpg_debug_get_epoch(ltpg_ctx *c, uint32_t *epoch) {
    if (!c || !epoch) return LTPG_ERR_INVALID;
    CK(cudaMemcpyAsync(epoch, &c->ctl->epoch, sizeof *epoch, cudaMemcpyDeviceToHost, c->stream), "read epoch");
    return ltpg_sync(c);
}

int ltpg_debug_barrier(ltpg_ctx *c, uint64_t limit_ns, uint32_t skip_block) {
    if (!c) return LTPG_ERR_INVALID;
    CK(cudaSetDevice(c->device), "set device");
    CK(cudaStreamSynchronize(c->stream), "sync");
    DevCtl h;
    CK(cudaMemcpy(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost), "read control block");
    h.barrier_limit_ns = limit_ns;
    h.barrier_skip = skip_block == UINT32_MAX ? 0u : skip_block + 1u;
    CK(cudaMemcpy(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice), "write control block");
    return LTPG_OK;
}

uint32_t ltpg_key_bucket(uint32_t key) { return (key * 0x9E3779B1u) >> 16; }

int ltpg_stage_set(ltpg_ctx *c, const uint32_t *buckets, uint32_t n) {
    if (!c || (n && !buckets)) return LTPG_ERR_INVALID;
    if (!c->stage_map) {
        CK(dev_alloc(&c->stage_map, LTPG_STAGE_BUCKETS), "alloc stage map");
        CK(dev_alloc(&c->stage_bits, LTPG_STAGE_BUCKETS / 32), "alloc stage bits");
        CK(dev_alloc(&c->stage_rank, LTPG_STAGE_BUCKETS / 32), "alloc stage rank");
        CK(dev_alloc(&c->bucket_counts, LTPG_STAGE_BUCKETS), "alloc bucket counts");
        CK(cudaMemset(c->bucket_counts, 0, LTPG_STAGE_BUCKETS * 4), "clear bucket counts");
    }
    // the first LTPG_STAGE_ENTRIES / ways distinct buckets of the list are staged;
    // a staged bucket's group is its rank among the staged buckets
    const uint32_t ways = c->launch_y.ways ? c->launch_y.ways : 4u;
    const uint32_t groups = LTPG_STAGE_ENTRIES / ways;
    std::vector<uint32_t> bits(LTPG_STAGE_BUCKETS / 32, 0u), rank(LTPG_STAGE_BUCKETS / 32, 0u);
    uint32_t taken = 0;
    for (uint32_t i = 0; i < n && taken < groups; ++i) {
        if (buckets[i] >= LTPG_STAGE_BUCKETS) return fail(c, LTPG_ERR_INVALID, "bucket out of range");
        uint32_t &w = bits[buckets[i] >> 5];
        const uint32_t bit = 1u << (buckets[i] & 31u);
        if (!(w & bit)) {
            w |= bit;
            ++taken;
        }
    }
    std::vector<uint16_t> map(LTPG_STAGE_BUCKETS, 0xFFFFu);
    uint32_t acc = 0;
    for (uint32_t wi = 0; wi < LTPG_STAGE_BUCKETS / 32; ++wi) {
        rank[wi] = acc;
        for (uint32_t bi = 0; bi < 32; ++bi)
            if (bits[wi] >> bi & 1u) map[wi * 32 + bi] = (uint16_t)acc++;
    }
    CK(cudaMemcpyAsync(c->stage_map, map.data(), LTPG_STAGE_BUCKETS * 2, cudaMemcpyHostToDevice, c->stream),
       "upload stage map");
    CK(cudaMemcpyAsync(c->stage_bits, bits.data(), LTPG_STAGE_BUCKETS / 8, cudaMemcpyHostToDevice, c->stream),
       "upload stage bits");
    CK(cudaMemcpyAsync(c->stage_rank, rank.data(), LTPG_STAGE_BUCKETS / 8, cudaMemcpyHostToDevice, c->stream),
       "upload stage rank");
    CK(cudaStreamSynchronize(c->stream), "sync");
    const uint32_t on = n ? 1u : 0u;
    if (on != c->stage_on) drop_graphs(c);
    c->stage_on = on;
    return LTPG_OK;
}

int ltpg_bucket_counts(ltpg_ctx *c, uint32_t *host, int reset) {
    if (!c || !host) return LTPG_ERR_INVALID;
    if (!c->bucket_counts) {
        memset(host, 0, LTPG_STAGE_BUCKETS * 4);
        return LTPG_OK;
    }
    CK(cudaMemcpyAsync(host, c->bucket_counts, LTPG_STAGE_BUCKETS * 4, cudaMemcpyDeviceToHost, c->stream),
       "download bucket counts");
    if (reset) CK(cudaMemsetAsync(c->bucket_counts, 0, LTPG_STAGE_BUCKETS * 4, c->stream), "reset counts");
    return ltpg_sync(c);
}

}  // extern "C"
