// serve.cpp — continuous-batching request loop over two engines (TPC-C, YCSB).
//
// Requests arrive open-loop (Poisson, seeded) as a mix of TPC-C NewOrder /
// Payment transactions and YCSB transactions, drawn in order from pools made
// by the deterministic generators.  The loop admits every request whose
// arrival time has passed into the forming batch, closes the batch when it
// holds max_batch requests or its first request has waited deadline_ms, and
// hands the two sub-batches to their engines on their own streams, so TPC-C
// and YCSB kernels run concurrently and the next batch's host-to-device copy
// overlaps the current batch's kernels.  A batch can only close when both
// engines have a free slot; the number of slots in flight is bounded by the
// device-memory budget (batch buffers + registration tables, the tables kept
// resident).  A request's latency is the time from its arrival to the moment
// its batch's commit bitmap is in host memory.  With record = 1, the batch
// boundaries and every request's flags and result are kept, so a test can
// replay the batches one by one and compare.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <random>
#include <vector>

#include "engine.h"

using namespace ltpg;

namespace {

using Clock = std::chrono::steady_clock;

struct Pinned {
    void *p = nullptr;
    size_t n = 0;
    ~Pinned() { ltpg_host_free(p); }
    bool reserve(size_t bytes) {
        if (bytes <= n) return true;
        ltpg_host_free(p);
        p = ltpg_host_alloc(bytes);
        n = p ? bytes : 0;
        return p != nullptr;
    }
};

struct SlotState {
    bool busy = false;
    cudaEvent_t done_c = nullptr, done_y = nullptr;
    cudaEvent_t start = nullptr;  // recorded when the batch is handed to the engines
    double t_close = 0;           // host time the batch closed
    uint64_t c_start = 0, c_count = 0, y_start = 0, y_count = 0;
    uint64_t c_packed = 0, y_packed = 0;  // requests of the forming batch already in the staging buffers
    double arrival_first = 0;
    Pinned c_txns, c_lines, y_ops, y_voff, y_vals;   // host staging of the batch
    Pinned c_bits, y_bits, c_flags, y_flags, c_res, y_res;
    std::vector<ltpg_tpcc_txn> tmp_txn;
};

double percentile(std::vector<double> &v, double q) {
    if (v.empty()) return 0.0;
    size_t k = (size_t)std::min<double>(v.size() - 1, std::floor(q * (v.size() - 1)));
    std::nth_element(v.begin(), v.begin() + k, v.end());
    return v[k];
}

}  // namespace

struct ltpg_serve_record {
    std::vector<uint64_t> batches;  // per batch: c_start, c_count, y_start, y_count
    std::vector<uint8_t> c_flags, y_flags;
    std::vector<int64_t> c_res, y_res;
};

extern "C" {

int ltpg_serve_run(ltpg_ctx *tc, ltpg_ctx *yc, const ltpg_serve_cfg *cfg, const ltpg_tpcc_params *tp,
                   const ltpg_ycsb_params *yp, ltpg_serve_stats *out, ltpg_serve_record **record) {
    if (!tc || !yc || !cfg || !tp || !yp || !out) return LTPG_ERR_INVALID;
    if (cfg->rate <= 0 || cfg->duration_s <= 0 || cfg->max_batch == 0 || cfg->tpcc_pct > 100)
        return LTPG_ERR_INVALID;
    if (cfg->max_batch > tc->cfg.max_txn || cfg->max_batch > yc->cfg.max_txn) return LTPG_ERR_INVALID;
    if (!tc->tpcc.W || !yc->ycsb.rows) return LTPG_ERR_STATE;
    const uint32_t n_slots = std::min<uint32_t>(cfg->slots ? cfg->slots : 4, std::min<uint32_t>(
                                                   (uint32_t)tc->slots.size(), (uint32_t)yc->slots.size()));
    // ---- memory budget: registration tables + n_slots batch slots of each engine
    const uint64_t per_txn_c = 32 + 8 * LTPG_TPCC_MAX_LINES + 1 + 8 + 1;
    const uint64_t per_txn_y = 4ull * ((yp->ops_per_txn + 3) & ~3u) + 4 + 8ull * yp->ops_per_txn + 1 + 8 + 1;
    const uint64_t tables = tc->tpcc.n_slots * sizeof(RegSlot) + yc->ycsb.n * sizeof(RegSlot);
    const uint64_t slot_bytes = (uint64_t)cfg->max_batch * (per_txn_c + per_txn_y);
    uint32_t allowed = n_slots;
    if (cfg->budget_bytes) {
        if (tables >= cfg->budget_bytes) return LTPG_ERR_NOMEM;
        allowed = (uint32_t)std::min<uint64_t>(n_slots, (cfg->budget_bytes - tables) / std::max<uint64_t>(1, slot_bytes));
        if (allowed == 0) return LTPG_ERR_NOMEM;
    }
    // ---- request pools and arrival times (before the clock starts)
    const uint64_t expected = (uint64_t)(cfg->rate * cfg->duration_s);
    std::mt19937_64 rng(cfg->seed ^ 0x5E57ull);
    std::exponential_distribution<double> gap(cfg->rate);
    std::uniform_int_distribution<int> pct(0, 99);
    std::vector<double> arrival;
    std::vector<uint8_t> is_tpcc;
    arrival.reserve(expected + expected / 8 + 16);
    double tt = 0;
    uint64_t n_c = 0, n_y = 0;
    while (true) {
        tt += gap(rng);
        if (tt > cfg->duration_s) break;
        arrival.push_back(tt);
        const bool c = pct(rng) < (int)cfg->tpcc_pct;
        is_tpcc.push_back(c);
        n_c += c;
        n_y += !c;
    }
    const uint64_t N = arrival.size();
    // TPC-C pool: consecutive generator batches
    std::vector<ltpg_tpcc_txn> c_pool;
    std::vector<ltpg_tpcc_line> c_lines;
    std::vector<uint64_t> c_line_off;  // global line offset of each pool transaction
    {
        ltpg_tpcc_params p = *tp;
        p.n_txn = std::max<uint32_t>(1, std::min<uint64_t>(p.n_txn, n_c ? n_c : 1));
        ltpg_gen *g = nullptr;
        if (ltpg_gen_create_tpcc(&p, &g)) return LTPG_ERR_INVALID;
        std::vector<ltpg_tpcc_txn> tx(p.n_txn);
        std::vector<ltpg_tpcc_line> ln((size_t)p.n_txn * LTPG_TPCC_MAX_LINES);
        uint64_t bid = 0;
        while (c_pool.size() < n_c) {
            ltpg_tpcc_batch b;
            ltpg_gen_tpcc_batch(g, bid++, tx.data(), ln.data(), &b);
            for (uint32_t t = 0; t < b.n_txn && c_pool.size() < n_c; ++t) {
                c_line_off.push_back(c_lines.size());
                c_pool.push_back(tx[t]);
                const uint32_t cnt = tpcc_kind(tx[t].kind_info) == LTPG_TPCC_NEWORDER ? tpcc_ol_cnt(tx[t].kind_info) : 0;
                for (uint32_t i = 0; i < cnt; ++i) c_lines.push_back(ln[tx[t].line_off + i]);
            }
        }
        c_line_off.push_back(c_lines.size());
        ltpg_gen_destroy(g);
    }
    // YCSB pool
    const uint32_t ky = yp->ops_per_txn, sy = (ky + 3) & ~3u;
    std::vector<uint32_t> y_ops;
    std::vector<uint64_t> y_vals;
    std::vector<uint64_t> y_voff;  // global value offset of each pool transaction
    {
        ltpg_ycsb_params p = *yp;
        p.n_txn = std::max<uint32_t>(1, std::min<uint64_t>(p.n_txn, n_y ? n_y : 1));
        ltpg_gen *g = nullptr;
        if (ltpg_gen_create_ycsb(&p, &g)) return LTPG_ERR_INVALID;
        std::vector<uint32_t> ops((size_t)p.n_txn * sy), voff(p.n_txn + 1);
        std::vector<uint64_t> vals((size_t)p.n_txn * ky);
        uint64_t bid = 0, have = 0;
        while (have < n_y) {
            ltpg_ycsb_batch b;
            ltpg_gen_ycsb_batch(g, bid++, ops.data(), voff.data(), vals.data(), &b);
            const uint64_t take = std::min<uint64_t>(b.n_txn, n_y - have);
            for (uint64_t t = 0; t < take; ++t) y_voff.push_back(y_vals.size() + voff[t]);
            y_ops.insert(y_ops.end(), ops.begin(), ops.begin() + take * sy);
            y_vals.insert(y_vals.end(), vals.begin(), vals.begin() + voff[take]);
            have += take;
        }
        y_voff.push_back(y_vals.size());
        ltpg_gen_destroy(g);
    }
    // ---- slots, streams
    std::vector<SlotState> slots(allowed);
    cudaStream_t cs_c, cs_y, cp_c, cp_y;
    cudaSetDevice(tc->device);
    cudaStreamCreateWithFlags(&cs_c, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&cp_c, cudaStreamNonBlocking);
    cudaSetDevice(yc->device);
    cudaStreamCreateWithFlags(&cs_y, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&cp_y, cudaStreamNonBlocking);
    for (auto &s : slots) {
        cudaEventCreate(&s.done_c);
        cudaEventCreate(&s.done_y);
        cudaEventCreate(&s.start);
    }
    // pinned staging for the largest batch, reserved before the clock starts
    for (auto &s : slots) {
        const uint64_t m = cfg->max_batch;
        if (!s.c_txns.reserve(m * sizeof(ltpg_tpcc_txn)) || !s.c_lines.reserve((m * LTPG_TPCC_MAX_LINES + 1) * 8) ||
            !s.c_bits.reserve((m + 31) / 32 * 4) || !s.c_flags.reserve(m) || !s.c_res.reserve(m * 8) ||
            !s.y_ops.reserve(m * sy * 4) || !s.y_voff.reserve((m + 1) * 4) || !s.y_vals.reserve((m * ky + 1) * 8) ||
            !s.y_bits.reserve((m + 31) / 32 * 4) || !s.y_flags.reserve(m) || !s.y_res.reserve(m * 8))
            return LTPG_ERR_NOMEM;
    }
    cudaEvent_t up_c, up_y;
    cudaEventCreateWithFlags(&up_c, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&up_y, cudaEventDisableTiming);
    ltpg_serve_record *rec = nullptr;
    if (record) {
        rec = new (std::nothrow) ltpg_serve_record();
        if (!rec) return LTPG_ERR_NOMEM;
        rec->c_flags.assign(n_c, 0);
        rec->y_flags.assign(n_y, 0);
        rec->c_res.assign(n_c, 0);
        rec->y_res.assign(n_y, 0);
    }
    std::vector<double> lat;  // committed requests' latencies (ms)
    lat.reserve(N);
    double wait_sum = 0, pack_sum = 0, dev_sum = 0;  // latency parts (s): close wait per request, per batch
    std::vector<double> arr_c(n_c), arr_y(n_y);
    {
        uint64_t ic = 0, iy = 0;
        for (uint64_t i = 0; i < N; ++i) (is_tpcc[i] ? arr_c[ic++] : arr_y[iy++]) = arrival[i];
    }
    uint64_t next = 0, pos_c = 0, pos_y = 0;  // next arrival; next pool index per type
    uint64_t form_start = 0;                  // first arrival of the forming batch
    uint64_t batches = 0, committed = 0, waited_for_slot = 0;
    double batch_sizes = 0;
    int rc = LTPG_OK;
    const int mode = (int)cfg->mode;
    const double deadline = cfg->deadline_ms * 1e-3;
    const Clock::time_point t0 = Clock::now();
    auto now_s = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };

    auto complete = [&](SlotState &s, double t_done) {
        float ms_c = 0.f, ms_y = 0.f;
        cudaEventElapsedTime(&ms_c, s.start, s.done_c);
        cudaEventElapsedTime(&ms_y, s.start, s.done_y);
        dev_sum += std::max(ms_c, ms_y) * 1e-3;
        (void)t_done;
        // latency of every committed request of the batch
        const uint32_t *bc = static_cast<const uint32_t *>(s.c_bits.p);
        const uint32_t *by = static_cast<const uint32_t *>(s.y_bits.p);
        for (uint64_t i = 0; i < s.c_count; ++i)
            if (bc[i >> 5] >> (i & 31) & 1u) {
                lat.push_back((t_done - arr_c[s.c_start + i]) * 1e3);
                ++committed;
            }
        for (uint64_t i = 0; i < s.y_count; ++i)
            if (by[i >> 5] >> (i & 31) & 1u) {
                lat.push_back((t_done - arr_y[s.y_start + i]) * 1e3);
                ++committed;
            }
        if (rec) {
            memcpy(&rec->c_flags[s.c_start], s.c_flags.p, s.c_count);
            memcpy(&rec->y_flags[s.y_start], s.y_flags.p, s.y_count);
            memcpy(&rec->c_res[s.c_start], s.c_res.p, s.c_count * 8);
            memcpy(&rec->y_res[s.y_start], s.y_res.p, s.y_count * 8);
        }
        s.busy = false;
    };

    // Packs pool requests [c_start + c_packed, c_end) and [y_start + y_packed,
    // y_end) into the slot's pinned staging: called as requests are admitted,
    // so a batch is mostly packed when it closes.
    auto pack_upto = [&](SlotState &s, uint64_t c_end, uint64_t y_end) {
        const uint64_t c_from = s.c_start + s.c_packed;
        if (c_end > c_from) {
            const uint64_t l0 = c_line_off[s.c_start];
            ltpg_tpcc_txn *tx = static_cast<ltpg_tpcc_txn *>(s.c_txns.p);
            for (uint64_t i = c_from; i < c_end; ++i) {
                tx[i - s.c_start] = c_pool[i];
                tx[i - s.c_start].line_off = (uint32_t)(c_line_off[i] - l0);
            }
            memcpy(static_cast<ltpg_tpcc_line *>(s.c_lines.p) + (c_line_off[c_from] - l0), c_lines.data() + c_line_off[c_from],
                   (c_line_off[c_end] - c_line_off[c_from]) * 8);
            s.c_packed = c_end - s.c_start;
        }
        const uint64_t y_from = s.y_start + s.y_packed;
        if (y_end > y_from) {
            const uint64_t v0 = y_voff[s.y_start];
            memcpy(static_cast<uint32_t *>(s.y_ops.p) + (y_from - s.y_start) * sy, y_ops.data() + y_from * sy,
                   (y_end - y_from) * sy * 4);
            uint32_t *vo = static_cast<uint32_t *>(s.y_voff.p);
            for (uint64_t i = y_from; i < y_end; ++i) vo[i - s.y_start] = (uint32_t)(y_voff[i] - v0);
            memcpy(static_cast<uint64_t *>(s.y_vals.p) + (y_voff[y_from] - v0), y_vals.data() + y_voff[y_from],
                   (y_voff[y_end] - y_voff[y_from]) * 8);
            s.y_packed = y_end - s.y_start;
        }
    };

    // Hands a closed, packed batch to the two engines.
    auto launch = [&](SlotState &s, uint32_t slot_idx) -> int {
        const uint64_t nc = s.c_count, ny = s.y_count;
        pack_upto(s, s.c_start + nc, s.y_start + ny);
        cudaEventRecord(s.start, cp_c);
        // ---- TPC-C sub-batch
        if (nc) {
            const uint64_t l0 = c_line_off[s.c_start], l1 = c_line_off[s.c_start + nc];
            ltpg_tpcc_batch b{(uint32_t)nc, (uint32_t)(l1 - l0), s.c_start, static_cast<ltpg_tpcc_txn *>(s.c_txns.p),
                              static_cast<ltpg_tpcc_line *>(s.c_lines.p)};
            ltpg_set_stream(tc, cp_c);
            int r = ltpg_batch_upload_tpcc(tc, slot_idx, &b);
            if (r) return r;
            cudaEventRecord(up_c, cp_c);
            cudaStreamWaitEvent(cs_c, up_c, 0);
            ltpg_set_stream(tc, cs_c);
            if ((r = ltpg_run_batch(tc, slot_idx, mode))) return r;
            const uint32_t *dbits;
            ltpg_commit_bitmap_device(tc, slot_idx, &dbits);
            cudaMemcpyAsync(s.c_bits.p, dbits, (nc + 31) / 32 * 4, cudaMemcpyDeviceToHost, cs_c);
            if (rec) {
                cudaMemcpyAsync(s.c_flags.p, tc->slots[slot_idx].flags, nc, cudaMemcpyDeviceToHost, cs_c);
                cudaMemcpyAsync(s.c_res.p, tc->slots[slot_idx].results, nc * 8, cudaMemcpyDeviceToHost, cs_c);
            }
        }
        cudaEventRecord(s.done_c, cs_c);
        // ---- YCSB sub-batch
        if (ny) {
            const uint64_t v0 = y_voff[s.y_start], v1 = y_voff[s.y_start + ny];
            uint32_t *vo = static_cast<uint32_t *>(s.y_voff.p);
            vo[ny] = (uint32_t)(v1 - v0);
            ltpg_ycsb_batch b{(uint32_t)ny, ky, sy, (uint32_t)(v1 - v0), static_cast<uint32_t *>(s.y_ops.p), vo,
                              static_cast<uint64_t *>(s.y_vals.p)};
            ltpg_set_stream(yc, cp_y);
            int r = ltpg_batch_upload_ycsb(yc, slot_idx, &b);
            if (r) return r;
            cudaEventRecord(up_y, cp_y);
            cudaStreamWaitEvent(cs_y, up_y, 0);
            ltpg_set_stream(yc, cs_y);
            if ((r = ltpg_run_batch(yc, slot_idx, mode))) return r;
            const uint32_t *dbits;
            ltpg_commit_bitmap_device(yc, slot_idx, &dbits);
            cudaMemcpyAsync(s.y_bits.p, dbits, (ny + 31) / 32 * 4, cudaMemcpyDeviceToHost, cs_y);
            if (rec) {
                cudaMemcpyAsync(s.y_flags.p, yc->slots[slot_idx].flags, ny, cudaMemcpyDeviceToHost, cs_y);
                cudaMemcpyAsync(s.y_res.p, yc->slots[slot_idx].results, ny * 8, cudaMemcpyDeviceToHost, cs_y);
            }
        }
        cudaEventRecord(s.done_y, cs_y);
        s.busy = true;
        s.c_packed = s.y_packed = 0;
        if (rec) {
            rec->batches.push_back(s.c_start);
            rec->batches.push_back(nc);
            rec->batches.push_back(s.y_start);
            rec->batches.push_back(ny);
        }
        return LTPG_OK;
    };

    uint32_t rr = 0;           // next slot in round-robin order (batches complete in order)
    uint64_t form_c = 0;       // TPC-C requests in the forming batch (the rest are YCSB)
    bool form_packing = false; // the forming batch is being packed into slots[rr]
    while (rc == LTPG_OK) {
        const double t = now_s();
        // completions
        for (uint32_t k = 0; k < allowed; ++k) {
            SlotState &s = slots[(rr + k) % allowed];
            if (!s.busy) continue;
            if (cudaEventQuery(s.done_c) == cudaSuccess && cudaEventQuery(s.done_y) == cudaSuccess)
                complete(s, now_s());
        }
        // admission: requests that have arrived join the forming batch
        uint64_t form_end = next;
        while (form_end < N && arrival[form_end] <= t && form_end - form_start < cfg->max_batch) {
            form_c += is_tpcc[form_end];
            ++form_end;
        }
        next = form_end;
        const uint64_t size = next - form_start;
        // pack the admitted requests now if the forming batch's slot is free
        SlotState &fs = slots[rr];
        if (!fs.busy && size > 0) {
            if (!form_packing) {
                fs.c_start = pos_c;
                fs.y_start = pos_y;
                fs.c_packed = fs.y_packed = 0;
                form_packing = true;
            }
            pack_upto(fs, pos_c + form_c, pos_y + (size - form_c));
        }
        const bool full = size >= cfg->max_batch;
        const bool due = size > 0 && t - arrival[form_start] >= deadline;
        const bool drain = next >= N && size > 0;
        if (full || due || drain) {
            SlotState &s = slots[rr];
            if (s.busy) {
                ++waited_for_slot;  // all slots in flight: the batch keeps forming
            } else {
                const uint64_t nc = form_c;
                if (!form_packing) {
                    s.c_packed = s.y_packed = 0;
                }
                s.c_start = pos_c;
                s.c_count = nc;
                s.y_start = pos_y;
                s.y_count = size - nc;
                s.arrival_first = arrival[form_start];
                s.t_close = t;
                for (uint64_t i = form_start; i < next; ++i) wait_sum += t - arrival[i];
                pos_c += nc;
                pos_y += size - nc;
                rc = launch(s, rr);
                pack_sum += now_s() - t;
                batches++;
                batch_sizes += (double)size;
                form_start = next;
                form_c = 0;
                form_packing = false;
                rr = (rr + 1) % allowed;
            }
        }
        if (next >= N && form_start >= N) {
            bool any = false;
            for (auto &s : slots) any |= s.busy;
            if (!any) break;
        }
    }
    const double wall = now_s();
    ltpg_set_stream(tc, nullptr);
    ltpg_set_stream(yc, nullptr);
    cudaStreamSynchronize(cs_c);
    cudaStreamSynchronize(cs_y);
    for (auto &s : slots) {
        cudaEventDestroy(s.done_c);
        cudaEventDestroy(s.done_y);
        cudaEventDestroy(s.start);
    }
    cudaEventDestroy(up_c);
    cudaEventDestroy(up_y);
    cudaStreamDestroy(cs_c);
    cudaStreamDestroy(cp_c);
    cudaStreamDestroy(cs_y);
    cudaStreamDestroy(cp_y);
    if (rc == LTPG_OK) {
        int r1 = ltpg_sync(tc), r2 = ltpg_sync(yc);
        rc = r1 ? r1 : r2;
    }
    memset(out, 0, sizeof *out);
    out->submitted = N;
    out->committed = committed;
    out->batches = batches;
    out->slots = allowed;
    out->waited_for_slot = waited_for_slot;
    out->wall_s = wall;
    out->throughput = wall > 0 ? committed / wall : 0;
    out->mean_batch = batches ? batch_sizes / batches : 0;
    double sum = 0;
    for (double v : lat) sum += v;
    out->mean_ms = lat.empty() ? 0 : sum / lat.size();
    out->p50_ms = percentile(lat, 0.50);
    out->p99_ms = percentile(lat, 0.99);
    out->p999_ms = percentile(lat, 0.999);
    out->wait_ms = N ? wait_sum * 1e3 / N : 0;
    out->launch_ms = batches ? pack_sum * 1e3 / batches : 0;
    out->device_ms = batches ? dev_sum * 1e3 / batches : 0;
    if (record) *record = rec;
    return rc;
}

int ltpg_serve_record_sizes(const ltpg_serve_record *r, uint64_t *n_batches, uint64_t *n_tpcc, uint64_t *n_ycsb) {
    if (!r || !n_batches || !n_tpcc || !n_ycsb) return LTPG_ERR_INVALID;
    *n_batches = r->batches.size() / 4;
    *n_tpcc = r->c_flags.size();
    *n_ycsb = r->y_flags.size();
    return LTPG_OK;
}

int ltpg_serve_record_get(const ltpg_serve_record *r, uint64_t *batches, uint8_t *tpcc_flags, int64_t *tpcc_results,
                          uint8_t *ycsb_flags, int64_t *ycsb_results) {
    if (!r) return LTPG_ERR_INVALID;
    if (batches) memcpy(batches, r->batches.data(), r->batches.size() * 8);
    if (tpcc_flags) memcpy(tpcc_flags, r->c_flags.data(), r->c_flags.size());
    if (tpcc_results) memcpy(tpcc_results, r->c_res.data(), r->c_res.size() * 8);
    if (ycsb_flags) memcpy(ycsb_flags, r->y_flags.data(), r->y_flags.size());
    if (ycsb_results) memcpy(ycsb_results, r->y_res.data(), r->y_res.size() * 8);
    return LTPG_OK;
}

int ltpg_serve_record_free(ltpg_serve_record *r) {
    delete r;
    return LTPG_OK;
}

}  // extern "C"
