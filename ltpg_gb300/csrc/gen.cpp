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

#include "gen_state.h"

using namespace ltpg;

using namespace ltpg::gen;

namespace {

void zipf_init(Zipf &z, uint64_t n, double theta) {
    z = Zipf{};
    z.n = n;
    z.theta = theta;
    if (theta == 0.0) return;
    double sum = 0.0;
    for (uint64_t i = 1; i <= n; ++i) sum += 1.0 / std::pow((double)i, theta);
    z.zetan = sum;
    const double zeta2 = 1.0 + std::pow(0.5, theta);
    z.alpha = 1.0 / (1.0 - theta);
    z.eta = (1.0 - std::pow(2.0 / (double)n, 1.0 - theta)) / (1.0 - zeta2 / z.zetan);
    z.half_pow = std::pow(0.5, theta);
}

}  // namespace

const FixTables &host_fix_tables() {
    static const FixTables t = [] {
        FixTables x;
        fix_tables_fill(x);
        return x;
    }();
    return t;
}

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
    zipf_init(g->zipf, p->n_records, p->theta);
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
    if (g) gen_dev_free(g);
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
    const FixTables &tab = host_fix_tables();
    auto fill = [&](uint32_t t0, uint32_t t1) {
        for (uint32_t t = t0; t < t1; ++t)
            val_off[t + 1] = ycsb_txn(p, g->zipf, tab, rotate ? &perm : nullptr, batch_id, t, ops + (uint64_t)t * stride);
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
            if (ycsb_is_update(w[j])) vals[v++] = ycsb_value(p, txn0 + t, j);
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
    if (g->dev_bound) return LTPG_ERR_STATE;  // the counters live on the device
    const ltpg_tpcc_params &p = g->c;
    const bool tracking = !g->made.empty();
    const uint16_t *cname = g->cust_name.data();
    const uint8_t *crank = g->cust_rank.data();
    uint32_t nl = 0;
    for (uint32_t t = 0; t < p.n_txn; ++t) {
        Rng r(hash3(p.seed ^ DOM_TPCC, batch_id, t));
        ltpg_tpcc_txn &x = txns[t];
        memset(&x, 0, sizeof x);
        x.line_off = nl;
        const TpccHead h = tpcc_head(p, r);
        const uint32_t w = h.w;
        x.w = w;
        auto order = [&](uint32_t o) {
            const size_t k = 30000ull * w + o;
            return TpccOrder{g->o_cust[k], g->o_dist[k], g->o_ol[k], g->o_cnt[k]};
        };
        switch (h.kind) {
        case LTPG_TPCC_ORDERSTATUS:
            tpcc_orderstatus(p, r, h, x, tracking ? g->made[w] : 0u, g->o_id[w], order, cname, crank);
            break;
        case LTPG_TPCC_DELIVERY: {
            const bool tracked = tracking && g->delivered[w] < g->made[w];
            uint32_t o = 0;
            if (tracked) {
                if (g->made[w] - g->delivered[w] > 30000u) g->delivered[w] = g->made[w] - 30000u;
                o = (uint32_t)(g->delivered[w]++ % 30000u);
            }
            tpcc_delivery(r, h, x, tracked, o, order);
            break;
        }
        case LTPG_TPCC_STOCKLEVEL:
            tpcc_stocklevel(r, h, x);
            break;
        case LTPG_TPCC_NEWORDER:
            x.a = g->o_id[w];
            g->o_id[w] = (g->o_id[w] + 1) % 30000u;
            x.b = g->no_id[w];
            g->no_id[w] = (g->no_id[w] + 1) % 30000u;
            x.c = g->ol_id[w];
            g->ol_id[w] = (g->ol_id[w] + h.cnt) % 450000u;
            tpcc_neworder(p, r, h, x, lines + nl);
            if (tracking) {
                const size_t k = 30000ull * w + x.a;
                g->o_cust[k] = (uint16_t)x.c_id;
                g->o_dist[k] = (uint8_t)h.d;
                g->o_ol[k] = x.c;
                g->o_cnt[k] = (uint8_t)h.cnt;
                g->made[w]++;
            }
            nl += h.cnt;
            break;
        default:  // Payment
            x.a = g->h_id[w];
            g->h_id[w] = (g->h_id[w] + 1) % 30000u;
            tpcc_payment(p, r, h, x, cname, crank);
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
