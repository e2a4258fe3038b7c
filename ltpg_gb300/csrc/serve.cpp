// serve.cpp — continuous batching of caller-submitted transactions over two
// engines (TPC-C, YCSB), and the Poisson request loop built on it.
//
// A server owns the forming batch and the batches in flight.  Submitted
// requests are packed at once into the forming batch's pinned host staging
// (one set of staging buffers per batch in flight, plus the forming one), so
// closing a batch costs its copies and launches, not its packing.  A batch
// closes at max_batch requests, when its TPC-C order lines would pass the
// engine's max_lines, or when its first request has waited deadline_ms; it is
// handed to the engines when a device slot is free: the TPC-C part on one pair
// of streams (copy, compute), the YCSB part on another, so the two parts and
// successive batches overlap on the device.  Each engine runs its batches in
// order on its compute stream, so batches complete in order and the finished
// requests are always a prefix of the request ids.  A request's flags and
// result come back with its batch (pinned device-to-host copies behind the
// kernels) and are kept until a poll returns them.
//
// The reference stages caller batches through a two-slot prefetch on host
// threads and runs one batch at a time (TF/Query.h:526-605, TF/tp.cu:136-261);
// here admission, batch closing and overlap are the server's.
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
    Pinned() = default;
    Pinned(const Pinned &) = delete;
    Pinned &operator=(const Pinned &) = delete;
    ~Pinned() { ltpg_host_free(p); }
    bool reserve(size_t bytes) {
        if (bytes <= n) return true;
        ltpg_host_free(p);
        p = ltpg_host_alloc(bytes);
        n = p ? bytes : 0;
        return p != nullptr;
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

// Pinned host staging of one batch; bound to that batch until its uploads
// (recorded by up_c / up_y on the copy streams) are done.
struct Staging {
    Pinned c_txns, c_lines, y_ops, y_voff, y_vals;
    cudaEvent_t up_c = nullptr, up_y = nullptr;
    bool pending = false;
};

// A device slot of both engines with the batch it runs.
struct DevSlot {
    bool busy = false;
    cudaEvent_t start = nullptr, done_c = nullptr, done_y = nullptr;
    Pinned c_flags, c_res, y_flags, y_res;  // results, copied back behind the kernels
    uint64_t first_id = 0;
    uint32_t n = 0, n_c = 0, n_y = 0;
    std::vector<uint32_t> map;      // per request: (index in its part << 1) | (1 for YCSB)
    std::vector<double> t_submit;   // per request, server clock (s)
};

struct Res {
    int64_t result;
    uint8_t flags, done, returned;
};

double percentile(std::vector<double> &v, double q) {
    if (v.empty()) return 0.0;
    size_t k = (size_t)std::min<double>(v.size() - 1, std::floor(q * (v.size() - 1)));
    std::nth_element(v.begin(), v.begin() + k, v.end());
    return v[k];
}

}  // namespace

struct ltpg_server {
    ltpg_ctx *tc = nullptr, *yc = nullptr;
    void *tc_stream0 = nullptr, *yc_stream0 = nullptr;  // the contexts' streams before open
    double deadline_s = 0.002;
    uint32_t max_batch = 0, mode = 0, allowed = 0, ky = 0, sy = 0;
    uint64_t max_lines = 0;
    cudaStream_t cs_c = nullptr, cp_c = nullptr, cs_y = nullptr, cp_y = nullptr;
    std::vector<Staging> stage;  // allowed + 1 sets
    std::vector<DevSlot> dev;    // allowed slots, used in order
    uint32_t hf = 0;             // staging set of the forming batch
    uint32_t next_dev = 0, oldest = 0, in_flight = 0;
    // the forming batch
    uint64_t form_first = 0;
    uint32_t form_n = 0, form_c = 0, form_y = 0;
    uint64_t form_lines = 0, form_vals = 0;
    double form_t_first = 0;
    std::vector<uint32_t> form_map;
    std::vector<double> form_t;
    // request ids and results
    uint64_t next_id = 0, base_id = 0;
    std::deque<Res> res;
    uint64_t c_total = 0;  // TPC-C requests in the batches closed so far (txn_base of the next)
    std::vector<uint64_t> log_first;
    std::vector<uint32_t> log_n, log_c;
    // statistics
    Clock::time_point t0;
    double t_last_done = 0;
    std::vector<double> lat;
    uint64_t committed = 0, batches = 0, waited_for_slot = 0;
    double wait_sum = 0, launch_sum = 0, dev_sum = 0;
    int error = LTPG_OK;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void destroy(ltpg_server *s) {
    for (auto &g : s->stage) {
        if (g.up_c) cudaEventDestroy(g.up_c);
        if (g.up_y) cudaEventDestroy(g.up_y);
    }
    for (auto &d : s->dev) {
        if (d.start) cudaEventDestroy(d.start);
        if (d.done_c) cudaEventDestroy(d.done_c);
        if (d.done_y) cudaEventDestroy(d.done_y);
    }
    for (cudaStream_t st : {s->cs_c, s->cp_c, s->cs_y, s->cp_y})
        if (st) cudaStreamDestroy(st);
    delete s;
}

// Records the first error; later calls return it.
int fail(ltpg_server *s, int code) {
    if (s->error == LTPG_OK) s->error = code;
    return code;
}

// Finishes the oldest batch in flight (waiting for it when block): its
// requests' flags, results and latencies.  Returns false if none finished.
bool complete_oldest(ltpg_server *s, bool block) {
    if (s->in_flight == 0) return false;
    DevSlot &d = s->dev[s->oldest];
    if (block) {
        if (cudaEventSynchronize(d.done_c) != cudaSuccess || cudaEventSynchronize(d.done_y) != cudaSuccess) {
            fail(s, LTPG_ERR_CUDA);
            return false;
        }
    } else if (cudaEventQuery(d.done_c) != cudaSuccess || cudaEventQuery(d.done_y) != cudaSuccess) {
        return false;
    }
    const double t_done = s->now();
    float ms_c = 0.f, ms_y = 0.f;
    cudaEventElapsedTime(&ms_c, d.start, d.done_c);
    cudaEventElapsedTime(&ms_y, d.start, d.done_y);
    s->dev_sum += std::max(ms_c, ms_y) * 1e-3;
    const uint8_t *cf = d.c_flags.as<uint8_t>(), *yf = d.y_flags.as<uint8_t>();
    const int64_t *cr = d.c_res.as<int64_t>(), *yr = d.y_res.as<int64_t>();
    for (uint32_t i = 0; i < d.n; ++i) {
        const uint32_t m = d.map[i], k = m >> 1;
        Res &r = s->res[d.first_id + i - s->base_id];
        r.flags = (m & 1u) ? yf[k] : cf[k];
        r.result = (m & 1u) ? yr[k] : cr[k];
        r.done = 1;
        if (r.flags & LTPG_FLAG_COMMIT) {
            ++s->committed;
            s->lat.push_back((t_done - d.t_submit[i]) * 1e3);
        }
    }
    s->t_last_done = t_done;
    d.busy = false;
    s->oldest = (s->oldest + 1) % s->allowed;
    --s->in_flight;
    return true;
}

// The staging set of a new forming batch must be free of its last batch's uploads.
int begin_forming(ltpg_server *s, double t) {
    Staging &g = s->stage[s->hf];
    if (g.pending) {
        if (cudaEventSynchronize(g.up_c) != cudaSuccess || cudaEventSynchronize(g.up_y) != cudaSuccess)
            return fail(s, LTPG_ERR_CUDA);
        g.pending = false;
    }
    s->form_first = s->next_id;
    s->form_t_first = t;
    s->form_n = s->form_c = s->form_y = 0;
    s->form_lines = s->form_vals = 0;
    s->form_map.clear();
    s->form_t.clear();
    return LTPG_OK;
}

// Hands the forming batch to the engines.  Without a free device slot it
// waits for the oldest batch when block, else leaves the batch forming.
int close_batch(ltpg_server *s, bool block) {
    if (s->form_n == 0) return LTPG_OK;
    const double t = s->now();
    DevSlot &d = s->dev[s->next_dev];
    if (d.busy) {
        if (!block) {
            ++s->waited_for_slot;
            return LTPG_OK;
        }
        ++s->waited_for_slot;
        while (d.busy)
            if (!complete_oldest(s, true)) return fail(s, s->error ? s->error : LTPG_ERR_CUDA);
    }
    Staging &g = s->stage[s->hf];
    const uint32_t slot = s->next_dev;
    cudaEventRecord(d.start, s->cp_c);
    cudaStreamWaitEvent(s->cp_y, d.start, 0);
    int r = LTPG_OK;
    if (s->form_c) {
        ltpg_tpcc_batch b{s->form_c, (uint32_t)s->form_lines, s->c_total, g.c_txns.as<ltpg_tpcc_txn>(),
                          g.c_lines.as<ltpg_tpcc_line>()};
        ltpg_set_stream(s->tc, s->cp_c);
        if ((r = ltpg_batch_upload_tpcc(s->tc, slot, &b))) return fail(s, r);
        cudaEventRecord(g.up_c, s->cp_c);
        cudaStreamWaitEvent(s->cs_c, g.up_c, 0);
        ltpg_set_stream(s->tc, s->cs_c);
        if ((r = ltpg_run_batch(s->tc, slot, (int)s->mode))) return fail(s, r);
        const Slot &es = s->tc->slots[slot];
        cudaMemcpyAsync(d.c_flags.p, es.flags, s->form_c, cudaMemcpyDeviceToHost, s->cs_c);
        cudaMemcpyAsync(d.c_res.p, es.results, (size_t)s->form_c * 8, cudaMemcpyDeviceToHost, s->cs_c);
    } else {
        cudaEventRecord(g.up_c, s->cp_c);
        cudaStreamWaitEvent(s->cs_c, d.start, 0);
    }
    cudaEventRecord(d.done_c, s->cs_c);
    if (s->form_y) {
        g.y_voff.as<uint32_t>()[s->form_y] = (uint32_t)s->form_vals;
        ltpg_ycsb_batch b{s->form_y, s->ky, s->sy, (uint32_t)s->form_vals, g.y_ops.as<uint32_t>(),
                          g.y_voff.as<uint32_t>(), g.y_vals.as<uint64_t>()};
        ltpg_set_stream(s->yc, s->cp_y);
        if ((r = ltpg_batch_upload_ycsb(s->yc, slot, &b))) return fail(s, r);
        cudaEventRecord(g.up_y, s->cp_y);
        cudaStreamWaitEvent(s->cs_y, g.up_y, 0);
        ltpg_set_stream(s->yc, s->cs_y);
        if ((r = ltpg_run_batch(s->yc, slot, (int)s->mode))) return fail(s, r);
        const Slot &es = s->yc->slots[slot];
        cudaMemcpyAsync(d.y_flags.p, es.flags, s->form_y, cudaMemcpyDeviceToHost, s->cs_y);
        cudaMemcpyAsync(d.y_res.p, es.results, (size_t)s->form_y * 8, cudaMemcpyDeviceToHost, s->cs_y);
    } else {
        cudaEventRecord(g.up_y, s->cp_y);
        cudaStreamWaitEvent(s->cs_y, d.start, 0);
    }
    cudaEventRecord(d.done_y, s->cs_y);
    if (cudaGetLastError() != cudaSuccess) return fail(s, LTPG_ERR_CUDA);
    g.pending = true;
    d.busy = true;
    d.first_id = s->form_first;
    d.n = s->form_n;
    d.n_c = s->form_c;
    d.n_y = s->form_y;
    d.map.swap(s->form_map);
    d.t_submit.swap(s->form_t);
    for (double ts : d.t_submit) s->wait_sum += t - ts;
    s->log_first.push_back(s->form_first);
    s->log_n.push_back(s->form_n);
    s->log_c.push_back(s->form_c);
    s->c_total += s->form_c;
    ++s->batches;
    ++s->in_flight;
    s->next_dev = (s->next_dev + 1) % s->allowed;
    s->hf = (s->hf + 1) % (uint32_t)s->stage.size();
    s->form_n = 0;
    s->launch_sum += s->now() - t;
    return LTPG_OK;
}

// Finished batches, then the forming batch's deadline.
int progress(ltpg_server *s) {
    while (complete_oldest(s, false)) {
    }
    if (s->error) return s->error;
    if (s->form_n && s->now() - s->form_t_first >= s->deadline_s) return close_batch(s, false);
    return LTPG_OK;
}

int check_request(const ltpg_server *s, const ltpg_request &q) {
    if (q.workload == LTPG_WORKLOAD_TPCC) {
        if (!q.txn || (q.n && !q.lines) || q.n > LTPG_TPCC_MAX_LINES || q.n > s->max_lines) return LTPG_ERR_INVALID;
        const bool no = tpcc_kind(q.txn->kind_info) == LTPG_TPCC_NEWORDER;
        if (no ? q.n != tpcc_ol_cnt(q.txn->kind_info) : q.n != 0) return LTPG_ERR_INVALID;
        return LTPG_OK;
    }
    if (q.workload == LTPG_WORKLOAD_YCSB) {
        if (!q.ops || q.n == 0 || q.n > s->ky) return LTPG_ERR_INVALID;
        for (uint32_t j = 0; j < q.n; ++j)
            if (!ycsb_is_pad(q.ops[j]) && ycsb_is_update(q.ops[j]) && !q.vals) return LTPG_ERR_INVALID;
        return LTPG_OK;
    }
    return LTPG_ERR_INVALID;
}

// Packs one request into the forming batch's staging.
void pack(ltpg_server *s, const ltpg_request &q, double t) {
    Staging &g = s->stage[s->hf];
    if (q.workload == LTPG_WORKLOAD_TPCC) {
        ltpg_tpcc_txn x = *q.txn;
        x.line_off = (uint32_t)s->form_lines;
        g.c_txns.as<ltpg_tpcc_txn>()[s->form_c] = x;
        if (q.n) memcpy(g.c_lines.as<ltpg_tpcc_line>() + s->form_lines, q.lines, (size_t)q.n * sizeof(ltpg_tpcc_line));
        s->form_lines += q.n;
        s->form_map.push_back(s->form_c << 1);
        ++s->form_c;
    } else {
        uint32_t *w = g.y_ops.as<uint32_t>() + (size_t)s->form_y * s->sy;
        uint64_t *v = g.y_vals.as<uint64_t>() + s->form_vals;
        g.y_voff.as<uint32_t>()[s->form_y] = (uint32_t)s->form_vals;
        uint32_t nu = 0;
        for (uint32_t j = 0; j < s->sy; ++j) {
            const uint32_t op = j < q.n ? q.ops[j] : LTPG_YCSB_OP_PAD;
            w[j] = op;
            if (!ycsb_is_pad(op) && ycsb_is_update(op)) {
                v[nu] = q.vals[nu];
                ++nu;
            }
        }
        s->form_vals += nu;
        s->form_map.push_back((s->form_y << 1) | 1u);
        ++s->form_y;
    }
    s->form_t.push_back(t);
    ++s->form_n;
    s->res.push_back(Res{0, 0, 0, 0});
    ++s->next_id;
}

// Submission with given submit times (t == nullptr: now).
int submit(ltpg_server *s, const ltpg_request *reqs, uint32_t n, uint64_t *first_id, const double *t_submit) {
    if (s->error) return s->error;
    int r = progress(s);
    if (r) return r;
    if (first_id) *first_id = s->next_id;
    for (uint32_t i = 0; i < n; ++i) {
        const ltpg_request &q = reqs[i];
        if ((r = check_request(s, q))) return r;
        const double t = t_submit ? t_submit[i] : s->now();
        const bool lines_full =
            q.workload == LTPG_WORKLOAD_TPCC && s->form_lines + q.n > s->max_lines;
        if (s->form_n && (s->form_n >= s->max_batch || lines_full))
            if ((r = close_batch(s, true))) return r;
        if (s->form_n == 0 && (r = begin_forming(s, t))) return r;
        pack(s, q, t);
    }
    if (s->form_n >= s->max_batch && (r = close_batch(s, true))) return r;
    return progress(s);
}

int flush(ltpg_server *s) {
    if (s->error) return s->error;
    int r = close_batch(s, true);
    if (r) return r;
    while (s->in_flight)
        if (!complete_oldest(s, true)) return fail(s, s->error ? s->error : LTPG_ERR_CUDA);
    // device-side errors of the batches (out-of-range keys) are reported here
    int r1 = ltpg_sync(s->tc), r2 = ltpg_sync(s->yc);
    if (r1 || r2) return fail(s, r1 ? r1 : r2);
    return LTPG_OK;
}

void fill_stats(const ltpg_server *s, ltpg_serve_stats *out) {
    std::vector<double> lat = s->lat;
    memset(out, 0, sizeof *out);
    out->submitted = s->next_id;
    out->committed = s->committed;
    out->batches = s->batches;
    out->slots = s->allowed;
    out->waited_for_slot = s->waited_for_slot;
    out->wall_s = s->t_last_done;
    out->throughput = s->t_last_done > 0 ? s->committed / s->t_last_done : 0;
    out->mean_batch = s->batches ? (double)s->next_id / s->batches : 0;
    double sum = 0;
    for (double v : lat) sum += v;
    out->mean_ms = lat.empty() ? 0 : sum / lat.size();
    out->p50_ms = percentile(lat, 0.50);
    out->p99_ms = percentile(lat, 0.99);
    out->p999_ms = percentile(lat, 0.999);
    out->wait_ms = s->next_id ? s->wait_sum * 1e3 / s->next_id : 0;
    out->launch_ms = s->batches ? s->launch_sum * 1e3 / s->batches : 0;
    out->device_ms = s->batches ? s->dev_sum * 1e3 / s->batches : 0;
}

}  // namespace

struct ltpg_serve_record {
    std::vector<uint64_t> batches;  // per batch: c_start, c_count, y_start, y_count
    std::vector<uint8_t> c_flags, y_flags;
    std::vector<int64_t> c_res, y_res;
};

extern "C" {

int ltpg_server_open(ltpg_ctx *tc, ltpg_ctx *yc, const ltpg_server_cfg *cfg, ltpg_server **out) {
    if (!tc || !yc || !cfg || !out || tc == yc) return LTPG_ERR_INVALID;
    *out = nullptr;
    if (cfg->max_batch == 0 || cfg->max_batch > tc->cfg.max_txn || cfg->max_batch > yc->cfg.max_txn)
        return LTPG_ERR_INVALID;
    if (cfg->ycsb_ops == 0 || cfg->ycsb_ops > yc->cfg.max_ops_per_txn || cfg->deadline_ms < 0 ||
        cfg->mode > LTPG_MODE_GRAPH)
        return LTPG_ERR_INVALID;
    if (!tc->tpcc.W || !yc->ycsb.rows) return LTPG_ERR_STATE;
    const uint32_t n_slots = std::min<uint32_t>(cfg->slots ? cfg->slots : 4,
                                                std::min<uint32_t>((uint32_t)tc->slots.size(),
                                                                   (uint32_t)yc->slots.size()));
    const uint32_t ky = cfg->ycsb_ops, sy = ycsb_stride(ky);
    const uint64_t max_lines = std::min<uint64_t>(tc->cfg.max_lines, (uint64_t)cfg->max_batch * LTPG_TPCC_MAX_LINES);
    // memory budget: the registration tables stay resident; each batch in
    // flight holds a slot of each engine
    const uint64_t per_txn_c = 32 + 8ull * LTPG_TPCC_MAX_LINES + 1 + 8 + 1;
    const uint64_t per_txn_y = 4ull * sy + 4 + 8ull * ky + 1 + 8 + 1;
    const uint64_t tables = tc->tpcc.n_slots * sizeof(RegSlot) + yc->ycsb.n * sizeof(RegSlot);
    const uint64_t slot_bytes = (uint64_t)cfg->max_batch * (per_txn_c + per_txn_y);
    uint32_t allowed = n_slots;
    if (cfg->budget_bytes) {
        if (tables >= cfg->budget_bytes) return LTPG_ERR_NOMEM;
        allowed = (uint32_t)std::min<uint64_t>(n_slots, (cfg->budget_bytes - tables) / std::max<uint64_t>(1, slot_bytes));
        if (allowed == 0) return LTPG_ERR_NOMEM;
    }
    ltpg_server *s = new (std::nothrow) ltpg_server();
    if (!s) return LTPG_ERR_NOMEM;
    s->tc = tc;
    s->yc = yc;
    s->tc_stream0 = ltpg_get_stream(tc) == tc->own_stream ? nullptr : ltpg_get_stream(tc);
    s->yc_stream0 = ltpg_get_stream(yc) == yc->own_stream ? nullptr : ltpg_get_stream(yc);
    s->deadline_s = cfg->deadline_ms * 1e-3;
    s->max_batch = cfg->max_batch;
    s->mode = cfg->mode;
    s->allowed = allowed;
    s->ky = ky;
    s->sy = sy;
    s->max_lines = max_lines;
    bool ok = cudaSetDevice(tc->device) == cudaSuccess;
    for (cudaStream_t *st : {&s->cs_c, &s->cp_c})
        ok = ok && cudaStreamCreateWithFlags(st, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaSetDevice(yc->device) == cudaSuccess;
    for (cudaStream_t *st : {&s->cs_y, &s->cp_y})
        ok = ok && cudaStreamCreateWithFlags(st, cudaStreamNonBlocking) == cudaSuccess;
    s->stage = std::vector<Staging>(allowed + 1);
    s->dev = std::vector<DevSlot>(allowed);
    const uint64_t m = cfg->max_batch;
    for (auto &g : s->stage) {
        ok = ok && g.c_txns.reserve(m * sizeof(ltpg_tpcc_txn)) && g.c_lines.reserve((max_lines + 1) * 8) &&
             g.y_ops.reserve(m * sy * 4) && g.y_voff.reserve((m + 1) * 4) && g.y_vals.reserve((m * ky + 1) * 8);
        ok = ok && cudaEventCreateWithFlags(&g.up_c, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&g.up_y, cudaEventDisableTiming) == cudaSuccess;
    }
    for (auto &d : s->dev) {
        ok = ok && d.c_flags.reserve(m) && d.c_res.reserve(m * 8) && d.y_flags.reserve(m) && d.y_res.reserve(m * 8);
        ok = ok && cudaEventCreate(&d.start) == cudaSuccess && cudaEventCreate(&d.done_c) == cudaSuccess &&
             cudaEventCreate(&d.done_y) == cudaSuccess;
    }
    if (!ok) {
        destroy(s);
        return LTPG_ERR_NOMEM;
    }
    s->t0 = Clock::now();
    *out = s;
    return LTPG_OK;
}

int ltpg_serve_submit(ltpg_server *s, const ltpg_request *reqs, uint32_t n, uint64_t *first_id) {
    if (!s || (n && !reqs)) return LTPG_ERR_INVALID;
    return submit(s, reqs, n, first_id, nullptr);
}

int ltpg_serve_poll(ltpg_server *s, uint64_t first_id, uint32_t n, uint8_t *flags, int64_t *results,
                    uint32_t *n_done) {
    if (!s || !n_done) return LTPG_ERR_INVALID;
    *n_done = 0;
    int r = progress(s);
    if (r) return r;
    if (first_id < s->base_id) return LTPG_ERR_INVALID;
    uint32_t k = 0;
    while (k < n && first_id + k < s->next_id) {
        Res &q = s->res[first_id + k - s->base_id];
        if (!q.done) break;
        if (flags) flags[k] = q.flags;
        if (results) results[k] = q.result;
        q.returned = 1;
        ++k;
    }
    *n_done = k;
    while (!s->res.empty() && s->res.front().returned) {
        s->res.pop_front();
        ++s->base_id;
    }
    return LTPG_OK;
}

int ltpg_serve_flush(ltpg_server *s) { return s ? flush(s) : LTPG_ERR_INVALID; }

int ltpg_serve_batch_log(const ltpg_server *s, uint64_t *first_ids, uint32_t *counts, size_t cap, size_t *n_batches) {
    if (!s || !n_batches) return LTPG_ERR_INVALID;
    *n_batches = s->log_first.size();
    const size_t k = std::min(cap, s->log_first.size());
    if (first_ids) memcpy(first_ids, s->log_first.data(), k * 8);
    if (counts) memcpy(counts, s->log_n.data(), k * 4);
    return LTPG_OK;
}

int ltpg_server_close(ltpg_server *s, ltpg_serve_stats *stats) {
    if (!s) return LTPG_ERR_INVALID;
    const int r = flush(s);
    if (stats) fill_stats(s, stats);
    ltpg_set_stream(s->tc, s->tc_stream0);
    ltpg_set_stream(s->yc, s->yc_stream0);
    cudaStreamSynchronize(s->cs_c);
    cudaStreamSynchronize(s->cs_y);
    destroy(s);
    return r;
}

// ---- the request loop over generated pools ----------------------------------
int ltpg_serve_run(ltpg_ctx *tc, ltpg_ctx *yc, const ltpg_serve_cfg *cfg, const ltpg_tpcc_params *tp,
                   const ltpg_ycsb_params *yp, ltpg_serve_stats *out, ltpg_serve_record **record) {
    if (!tc || !yc || !cfg || !tp || !yp || !out) return LTPG_ERR_INVALID;
    if (cfg->rate <= 0 || cfg->duration_s <= 0 || cfg->max_batch == 0 || cfg->tpcc_pct > 100)
        return LTPG_ERR_INVALID;
    if (yp->ops_per_txn == 0 || yp->ops_per_txn > LTPG_YCSB_MAX_OPS) return LTPG_ERR_INVALID;
    // ---- arrival times and request pools (before the clock starts)
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
    std::vector<uint64_t> c_line_off;  // line offset of each pool transaction
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
    const uint32_t ky = yp->ops_per_txn, sy = ycsb_stride(ky);
    std::vector<uint32_t> y_ops;
    std::vector<uint64_t> y_vals;
    std::vector<uint64_t> y_voff;  // value offset of each pool transaction
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
    // ---- the server; each request is submitted at its arrival time
    ltpg_server_cfg sc{cfg->deadline_ms, cfg->budget_bytes, cfg->max_batch, cfg->mode, cfg->slots, ky};
    ltpg_server *s = nullptr;
    int rc = ltpg_server_open(tc, yc, &sc, &s);
    if (rc) return rc;
    std::vector<ltpg_request> reqs;
    reqs.reserve(4096);
    uint64_t next = 0, pos_c = 0, pos_y = 0;
    while (rc == LTPG_OK && next < N) {
        const double t = s->now();
        reqs.clear();
        const uint64_t from = next;
        while (next < N && arrival[next] <= t && reqs.size() < 4096) {
            ltpg_request q{};
            if (is_tpcc[next]) {
                q.workload = LTPG_WORKLOAD_TPCC;
                q.txn = &c_pool[pos_c];
                q.lines = c_lines.data() + c_line_off[pos_c];
                q.n = (uint32_t)(c_line_off[pos_c + 1] - c_line_off[pos_c]);
                ++pos_c;
            } else {
                q.workload = LTPG_WORKLOAD_YCSB;
                q.ops = y_ops.data() + pos_y * sy;
                q.vals = y_vals.data() + y_voff[pos_y];
                q.n = ky;
                ++pos_y;
            }
            reqs.push_back(q);
            ++next;
        }
        rc = reqs.empty() ? progress(s) : submit(s, reqs.data(), (uint32_t)reqs.size(), nullptr, &arrival[from]);
    }
    if (rc == LTPG_OK) rc = flush(s);
    ltpg_serve_record *rec = nullptr;
    if (rc == LTPG_OK && record) {
        rec = new (std::nothrow) ltpg_serve_record();
        if (!rec) rc = LTPG_ERR_NOMEM;
    }
    if (rec) {
        // per request, in submission order: flags and results by type; batch
        // boundaries as pool ranges per type
        std::vector<uint8_t> f(N);
        std::vector<int64_t> r(N);
        uint32_t got = 0;
        for (uint64_t i = 0; i < N && rc == LTPG_OK; i += got) {
            const uint32_t want = (uint32_t)std::min<uint64_t>(N - i, 1u << 20);
            rc = ltpg_serve_poll(s, i, want, f.data() + i, r.data() + i, &got);
            if (rc == LTPG_OK && got == 0) rc = LTPG_ERR_STATE;
        }
        for (uint64_t i = 0; i < N; ++i) {
            if (is_tpcc[i]) {
                rec->c_flags.push_back(f[i]);
                rec->c_res.push_back(r[i]);
            } else {
                rec->y_flags.push_back(f[i]);
                rec->y_res.push_back(r[i]);
            }
        }
        uint64_t cs = 0, ys = 0;
        for (size_t b = 0; b < s->log_first.size(); ++b) {
            const uint64_t nc = s->log_c[b], ny = s->log_n[b] - nc;
            rec->batches.insert(rec->batches.end(), {cs, nc, ys, ny});
            cs += nc;
            ys += ny;
        }
    }
    const int rc_close = ltpg_server_close(s, out);
    if (rc == LTPG_OK) rc = rc_close;
    if (record) *record = rc == LTPG_OK ? rec : nullptr;
    if (rc != LTPG_OK) delete rec;
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
