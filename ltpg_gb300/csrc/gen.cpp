// gen.cpp — deterministic batch generators (the Query.h surface).
//
// The reference draws every batch from libc rand() seeded with time(0) and
// called from up to 100 racing threads (Random.h:12,47-53; Y1/Query.h:229-250;
// TF/Query.h:640-671), so its batches cannot be reproduced.  Here every
// transaction owns a splitmix64 stream seeded by (seed, batch, position): the
// same parameters give the same bytes on any host, with any thread count.
//
// Compiled with -ffp-contract=off so the double arithmetic of the Zipf sampler
// rounds identically on x86-64 and aarch64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "proto.h"

using namespace ltpg;

namespace {

constexpr uint64_t DOM_YCSB_OPS = 0x59435342ull;   // "YCSB"
constexpr uint64_t DOM_YCSB_VAL = 0x56414C55ull;   // "VALU"
constexpr uint64_t DOM_YCSB_PERM = 0x5045524Dull;  // "PERM"
constexpr uint64_t DOM_TPCC = 0x54504343ull;       // "TPCC"

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // Uniform in [0, n) by Lemire's multiply-shift (no modulo bias worth noting
    // at these sizes, integer only).
    uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
    // Uniform in [a, b].
    uint64_t range(uint64_t a, uint64_t b) { return a + below(b - a + 1); }
    double unit() { return (double)(next() >> 11) * 0x1.0p-53; }
};

// Bijection of [0, n) keyed by k: a 4-round Feistel network over the smallest
// even bit width covering n, with cycle walking back into range.
struct Perm {
    uint64_t n = 0, key = 0;
    uint32_t half = 1;
    void init(uint64_t n_, uint64_t key_) {
        n = n_;
        key = key_;
        uint32_t bits = 2;
        while (bits < 64 && (1ull << bits) < n) bits += 2;
        half = bits / 2;
    }
    uint64_t round_fn(uint64_t x, uint32_t r) const {
        return splitmix64(x ^ (key + 0x1234567ull * (r + 1))) & ((1ull << half) - 1);
    }
    uint64_t once(uint64_t x) const {
        const uint64_t m = (1ull << half) - 1;
        uint64_t l = x >> half, rr = x & m;
        for (uint32_t r = 0; r < 4; ++r) {
            uint64_t t = l ^ round_fn(rr, r);
            l = rr;
            rr = t;
        }
        return (l << half) | rr;
    }
    uint64_t operator()(uint64_t x) const {
        uint64_t y = once(x);
        while (y >= n) y = once(y);
        return y;
    }
};

// Zipfian ranks by the method of Gray, Sundaresan, Englert, Baclawski and
// Weinberger, "Quickly generating billion-record synthetic databases" (SIGMOD
// 1994), the sampler YCSB uses.  Rank 0 is the most popular.
struct Zipf {
    uint64_t n = 0;
    double theta = 0, zetan = 0, alpha = 0, eta = 0, half_pow = 0;
    void init(uint64_t n_, double th) {
        n = n_;
        theta = th;
        if (theta == 0.0) return;
        double z = 0.0;
        for (uint64_t i = 1; i <= n; ++i) z += 1.0 / std::pow((double)i, theta);
        zetan = z;
        const double zeta2 = 1.0 + std::pow(0.5, theta);
        alpha = 1.0 / (1.0 - theta);
        eta = (1.0 - std::pow(2.0 / (double)n, 1.0 - theta)) / (1.0 - zeta2 / zetan);
        half_pow = std::pow(0.5, theta);
    }
    uint64_t sample(Rng &r) const {
        if (theta == 0.0) return r.below(n);
        const double u = r.unit();
        const double uz = u * zetan;
        if (uz < 1.0) return 0;
        if (uz < 1.0 + half_pow) return n > 1 ? 1 : 0;
        uint64_t v = (uint64_t)((double)n * std::pow(eta * u - eta + 1.0, alpha));
        return v < n ? v : n - 1;
    }
};

}  // namespace

struct ltpg_gen {
    int kind = 0;
    ltpg_ycsb_params y{};
    ltpg_tpcc_params c{};
    Zipf zipf;
    // TPC-C per-warehouse counters (TF/Query.h:54-88,157-166).
    std::vector<uint32_t> o_id, no_id, ol_id, h_id;
    // By-name Payments: C_LAST of every customer of the loaded image and its
    // rank among the customers of its district with that name, in C_ID order.
    std::vector<uint16_t> cust_name;
    std::vector<uint8_t> cust_rank;
    // OrderStatus / Delivery: the orders this generator made, per warehouse
    // (indexed by O_ID): customer, district, first OL_ID, line count; how many
    // were made and delivered.
    std::vector<uint16_t> o_cust;
    std::vector<uint8_t> o_dist, o_cnt;
    std::vector<uint32_t> o_ol;
    std::vector<uint64_t> made, delivered;
    uint64_t next_batch = 0, txn_base = 0;
};

extern "C" {

uint64_t ltpg_splitmix64(uint64_t x) { return splitmix64(x); }
uint64_t ltpg_hash3(uint64_t seed, uint64_t a, uint64_t b) { return hash3(seed, a, b); }

int ltpg_gen_create_ycsb(const ltpg_ycsb_params *p, ltpg_gen **out) {
    if (!p || !out) return LTPG_ERR_INVALID;
    if (p->n_records == 0 || p->n_records > (1ull << LTPG_YCSB_KEY_BITS)) return LTPG_ERR_INVALID;
    if (p->ops_per_txn == 0 || p->ops_per_txn > LTPG_YCSB_MAX_OPS) return LTPG_ERR_INVALID;
    if (p->ops_per_txn > p->n_records || p->update_pct > 100 || p->n_txn == 0) return LTPG_ERR_INVALID;
    if (!(p->theta >= 0.0 && p->theta < 1.0)) return LTPG_ERR_INVALID;
    if (p->scan_len > 16) return LTPG_ERR_INVALID;
    ltpg_gen *g = new (std::nothrow) ltpg_gen();
    if (!g) return LTPG_ERR_NOMEM;
    g->kind = LTPG_WORKLOAD_YCSB;
    g->y = *p;
    g->zipf.init(p->n_records, p->theta);
    *out = g;
    return LTPG_OK;
}

int ltpg_gen_create_tpcc(const ltpg_tpcc_params *p, ltpg_gen **out) {
    if (!p || !out) return LTPG_ERR_INVALID;
    if (p->warehouses == 0 || p->warehouses > 65535 || p->n_txn == 0) return LTPG_ERR_INVALID;
    if (p->neworder_pct > 100 || p->remote_line_pct > 100 || p->remote_pay_pct > 100 || p->by_name_pct > 100)
        return LTPG_ERR_INVALID;
    if ((uint64_t)p->neworder_pct + p->orderstatus_pct + p->delivery_pct + p->stocklevel_pct > 100)
        return LTPG_ERR_INVALID;
    ltpg_gen *g = new (std::nothrow) ltpg_gen();
    if (!g) return LTPG_ERR_NOMEM;
    g->kind = LTPG_WORKLOAD_TPCC;
    g->c = *p;
    g->o_id.assign(p->warehouses, 0);
    g->no_id.assign(p->warehouses, 0);
    g->ol_id.assign(p->warehouses, 0);
    g->h_id.assign(p->warehouses, 0);
    if (p->orderstatus_pct || p->delivery_pct) {
        const size_t n = 30000ull * p->warehouses;
        g->o_cust.assign(n, 0);
        g->o_dist.assign(n, 0);
        g->o_cnt.assign(n, 0);
        g->o_ol.assign(n, 0);
        g->made.assign(p->warehouses, 0);
        g->delivered.assign(p->warehouses, 0);
    }
    if (p->by_name_pct) {
        // names of the initial image (tpcc_init_value: C_LAST < 1000)
        const uint64_t n = 30000ull * p->warehouses;
        g->cust_name.resize(n);
        g->cust_rank.resize(n);
        std::vector<uint16_t> seen(1000);
        for (uint64_t d0 = 0; d0 < n; d0 += 3000) {
            std::fill(seen.begin(), seen.end(), 0);
            for (uint64_t row = d0; row < d0 + 3000; ++row) {
                const uint32_t name = (uint32_t)tpcc_init_value(p->table_seed, LTPG_T_CUSTOMER, row, C_LAST);
                g->cust_name[row] = (uint16_t)name;
                g->cust_rank[row] = (uint8_t)std::min<uint32_t>(seen[name]++, 255u);
            }
        }
    }
    *out = g;
    return LTPG_OK;
}

int ltpg_gen_destroy(ltpg_gen *g) {
    delete g;
    return LTPG_OK;
}

int ltpg_gen_capacity(const ltpg_gen *g, uint64_t *cap_a, uint64_t *cap_b) {
    if (!g || !cap_a || !cap_b) return LTPG_ERR_INVALID;
    if (g->kind == LTPG_WORKLOAD_YCSB) {
        *cap_a = (uint64_t)g->y.n_txn * ycsb_stride(g->y.ops_per_txn);
        *cap_b = (uint64_t)g->y.n_txn * g->y.ops_per_txn;
    } else {
        *cap_a = g->c.n_txn;
        *cap_b = (uint64_t)g->c.n_txn * LTPG_TPCC_MAX_LINES;
    }
    return LTPG_OK;
}

int ltpg_gen_ycsb_batch(ltpg_gen *g, uint64_t batch_id, uint32_t *ops, uint32_t *val_off,
                        uint64_t *vals, ltpg_ycsb_batch *out) {
    if (!g || g->kind != LTPG_WORKLOAD_YCSB || !ops || !val_off || !vals || !out) return LTPG_ERR_INVALID;
    const ltpg_ycsb_params &p = g->y;
    const uint32_t B = p.n_txn, k = p.ops_per_txn, stride = ycsb_stride(k);
    Perm perm;
    const bool rotate = p.rotate_every != 0;
    if (rotate) perm.init(p.n_records, hash3(p.seed ^ DOM_YCSB_PERM, batch_id / p.rotate_every, 0));

    // Pass 1: op words and per-transaction update counts, in parallel over
    // transactions (each has its own stream, so the split does not matter).
    auto fill = [&](uint32_t t0, uint32_t t1) {
        uint32_t keys[LTPG_YCSB_MAX_OPS];
        for (uint32_t t = t0; t < t1; ++t) {
            Rng r(hash3(p.seed ^ DOM_YCSB_OPS, batch_id, t));
            uint32_t nupd = 0;
            uint32_t *w = ops + (uint64_t)t * stride;
            for (uint32_t j = 0; j < k; ++j) {
                uint64_t key = 0;
                for (uint32_t attempt = 0;; ++attempt) {
                    uint64_t rank = g->zipf.sample(r);
                    key = rotate ? perm(rank) : rank;
                    if (attempt >= 64) {  // pathological tiny tables: walk to a free key
                        for (;;) {
                            bool dup = false;
                            for (uint32_t q = 0; q < j; ++q) dup |= keys[q] == key;
                            if (!dup) break;
                            key = (key + 1) % p.n_records;
                        }
                        break;
                    }
                    bool dup = false;
                    for (uint32_t q = 0; q < j; ++q) dup |= keys[q] == key;
                    if (!dup) break;
                }
                keys[j] = (uint32_t)key;
                const bool upd = r.below(100) < p.update_pct;
                const uint32_t field = (uint32_t)r.below(LTPG_YCSB_FIELDS);
                // a read scans scan_len keys when scan_len >= 2 (span in the field bits)
                const uint32_t span = p.scan_len >= 2u ? p.scan_len - 1u : 0u;
                w[j] = ycsb_word((uint32_t)key, upd, upd ? field : span);
                nupd += upd;
            }
            for (uint32_t j = k; j < stride; ++j) w[j] = LTPG_YCSB_OP_PAD;
            val_off[t + 1] = nupd;
        }
    };
    unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if ((uint64_t)B * k < 200000) nth = 1;
    std::vector<std::thread> th;
    const uint32_t chunk = (B + nth - 1) / nth;
    for (unsigned i = 0; i < nth; ++i) {
        uint32_t t0 = i * chunk, t1 = std::min(B, t0 + chunk);
        if (t0 >= t1) break;
        th.emplace_back(fill, t0, t1);
    }
    for (auto &x : th) x.join();
    val_off[0] = 0;
    for (uint32_t t = 0; t < B; ++t) val_off[t + 1] += val_off[t];
    // Pass 2: update values splitmix64(seed, txn, op) in transaction/op order.
    const uint64_t txn0 = batch_id * (uint64_t)B;
    for (uint32_t t = 0; t < B; ++t) {
        uint32_t v = val_off[t];
        const uint32_t *w = ops + (uint64_t)t * stride;
        for (uint32_t j = 0; j < k; ++j)
            if (ycsb_is_update(w[j])) vals[v++] = hash3(p.seed ^ DOM_YCSB_VAL, txn0 + t, j);
    }
    out->n_txn = B;
    out->ops_per_txn = k;
    out->op_stride = stride;
    out->n_updates = val_off[B];
    out->ops = ops;
    out->val_off = val_off;
    out->vals = vals;
    return LTPG_OK;
}

int ltpg_gen_tpcc_batch(ltpg_gen *g, uint64_t batch_id, ltpg_tpcc_txn *txns,
                        ltpg_tpcc_line *lines, ltpg_tpcc_batch *out) {
    if (!g || g->kind != LTPG_WORKLOAD_TPCC || !txns || !lines || !out) return LTPG_ERR_INVALID;
    if (batch_id != g->next_batch) return LTPG_ERR_STATE;  // counters advance in batch order
    const ltpg_tpcc_params &p = g->c;
    const uint32_t W = p.warehouses;
    // NURand of the reference, without the run-time constant C (Random.h:72-75).
    auto nurand = [](Rng &r, uint64_t A, uint64_t x, uint64_t y) {
        return ((r.range(0, A) | r.range(x, y)) % (y - x + 1)) + x;
    };
    auto other_w = [&](Rng &r, uint32_t w) {
        uint32_t o = (uint32_t)r.below(W - 1);
        return o >= w ? o + 1 : o;
    };
    uint32_t nl = 0;
    for (uint32_t t = 0; t < p.n_txn; ++t) {
        Rng r(hash3(p.seed ^ DOM_TPCC, batch_id, t));
        ltpg_tpcc_txn &x = txns[t];
        memset(&x, 0, sizeof x);
        x.line_off = nl;
        // kind: NewOrder, then OrderStatus, Delivery, StockLevel, else Payment
        const uint32_t u = (uint32_t)r.below(100);
        const bool is_no = u < p.neworder_pct;
        const uint32_t c_os = p.neworder_pct + p.orderstatus_pct, c_dl = c_os + p.delivery_pct,
                       c_sl = c_dl + p.stocklevel_pct;
        const uint32_t w = (uint32_t)r.below(W), d = (uint32_t)r.below(10);
        x.w = w;
        const bool tracking = !g->made.empty();
        // by last name (TF/Query.h:174-181): the query names customer (cw, cd,
        // c) by its C_LAST and its rank among that name's holders
        auto by_name = [&](uint32_t cw, uint32_t cd) {
            if (p.by_name_pct && r.below(100) < p.by_name_pct) {
                const uint64_t row = 30000ull * cw + 3000ull * cd + x.c_id;
                if (g->cust_rank[row] < 255u) {
                    x.kind_info |= LTPG_PAY_BY_NAME;
                    x.c_id = ((uint32_t)g->cust_name[row] << 8) | g->cust_rank[row];
                }
            }
        };
        if (!is_no && u < c_os) {
            // OrderStatus (TA/Query.h:214-246): a recent order of warehouse w
            // and one of its lines, read with its customer
            uint32_t cd = d, o, ol;
            if (tracking && g->made[w]) {
                const uint64_t back = r.below(std::min<uint64_t>(g->made[w], 1000));
                o = (uint32_t)((g->o_id[w] + 30000u - 1u - (uint32_t)back) % 30000u);
                const size_t k = 30000ull * w + o;
                cd = g->o_dist[k];
                x.c_id = g->o_cust[k];
                ol = (uint32_t)((g->o_ol[k] + r.below(std::max<uint32_t>(1u, g->o_cnt[k]))) % 450000u);
            } else {
                x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
                o = (uint32_t)r.below(30000);
                ol = (uint32_t)r.below(450000);
            }
            x.kind_info = LTPG_TPCC_ORDERSTATUS | (cd << 16) | (cd << 24);
            x.c_w = w;
            x.a = o;
            x.b = ol;
            by_name(w, cd);
            continue;
        }
        if (!is_no && u < c_dl) {
            // Delivery (TA/Query.h:247-269): the oldest undelivered order of w
            uint32_t cd = d, o, ol;
            if (tracking && g->delivered[w] < g->made[w]) {
                if (g->made[w] - g->delivered[w] > 30000u) g->delivered[w] = g->made[w] - 30000u;
                o = (uint32_t)(g->delivered[w]++ % 30000u);
                const size_t k = 30000ull * w + o;
                cd = g->o_dist[k];
                x.c_id = g->o_cust[k];
                ol = g->o_ol[k];
            } else {
                x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
                o = (uint32_t)r.below(30000);
                ol = (uint32_t)r.below(450000);
            }
            const uint32_t carrier = (uint32_t)r.range(1, 10);
            x.kind_info = LTPG_TPCC_DELIVERY | (carrier << 8) | (cd << 16);
            x.c_w = w;
            x.a = o;
            x.b = o;  // NO_ID and O_ID advance together (TF/Query.h:54-88)
            x.c = ol;
            continue;
        }
        if (!is_no && u < c_sl) {
            // StockLevel (TA/Query.h:270-296): one stock row of w
            const uint32_t threshold = (uint32_t)r.range(10, 20);
            x.kind_info = LTPG_TPCC_STOCKLEVEL | (threshold << 8) | (d << 16);
            x.c_w = w;
            x.a = (uint32_t)nurand(r, 8191, 1, 100000) - 1;
            continue;
        }
        if (is_no) {
            const uint32_t cnt = (uint32_t)r.range(5, LTPG_TPCC_MAX_LINES);
            x.kind_info = LTPG_TPCC_NEWORDER | (cnt << 8) | (d << 16);
            x.c_w = w;
            x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
            x.a = g->o_id[w];
            g->o_id[w] = (g->o_id[w] + 1) % 30000u;
            x.b = g->no_id[w];
            g->no_id[w] = (g->no_id[w] + 1) % 30000u;
            x.c = g->ol_id[w];
            g->ol_id[w] = (g->ol_id[w] + cnt) % 450000u;
            if (tracking) {
                const size_t k = 30000ull * w + x.a;
                g->o_cust[k] = (uint16_t)x.c_id;
                g->o_dist[k] = (uint8_t)d;
                g->o_ol[k] = x.c;
                g->o_cnt[k] = (uint8_t)cnt;
                g->made[w]++;
            }
            for (uint32_t i = 0; i < cnt; ++i) {
                ltpg_tpcc_line &ln = lines[nl + i];
                uint32_t item;
                for (;;) {  // distinct items within an order (TF/Query.h:103-114)
                    item = (uint32_t)nurand(r, 8191, 1, 100000) - 1;
                    bool dup = false;
                    for (uint32_t q = 0; q < i; ++q) dup |= lines[nl + q].i_id == item;
                    if (!dup) break;
                }
                ln.i_id = item;
                const bool remote = W > 1 && r.below(100) < p.remote_line_pct;
                ln.supply_w = (uint16_t)(remote ? other_w(r, w) : w);
                ln.qty = (uint16_t)r.range(1, 10);
            }
            nl += cnt;
        } else {
            const bool remote = W > 1 && r.below(100) < p.remote_pay_pct;
            uint32_t c_w = w, c_d = d;
            if (remote) {
                c_w = other_w(r, w);
                c_d = (uint32_t)r.below(10);
            }
            x.kind_info = LTPG_TPCC_PAYMENT | (d << 16) | (c_d << 24);
            x.c_w = c_w;
            x.c_id = (uint32_t)nurand(r, 1023, 1, 3000) - 1;
            const uint64_t amount = r.range(100, 500000);
            x.a = g->h_id[w];
            g->h_id[w] = (g->h_id[w] + 1) % 30000u;
            x.b = (uint32_t)amount;
            x.c = (uint32_t)(amount >> 32);
            by_name(c_w, c_d);
        }
    }
    out->n_txn = p.n_txn;
    out->n_lines = nl;
    out->txn_base = g->txn_base;
    out->txns = txns;
    out->lines = lines;
    g->txn_base += p.n_txn;
    g->next_batch++;
    return LTPG_OK;
}

}  // extern "C"
