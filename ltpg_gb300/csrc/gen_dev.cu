// gen_dev.cu — the deterministic batch generators on the GPU: the batches of
// gen.cpp, byte for byte, made directly in a slot's device buffers (no host
// generation, no host-to-device copy).
//
// Compiled with -fmad=false: the Zipf sampler's double arithmetic (gen.h) must
// round exactly like the host's.
//
// YCSB: one thread per transaction draws its op words (gen::ycsb_txn), an
// inclusive scan of the update counts gives val_off, and one thread per
// transaction writes its update values.
//
// TPC-C: the host generator is a loop whose per-warehouse counters (O_ID,
// NO_ID, OL_ID, H_ID) and order memory (for OrderStatus and Delivery) carry
// from one transaction to the next.  Each value a transaction reads is its
// warehouse's value at batch start plus a count over the batch's earlier
// transactions of the same warehouse, so the loop becomes:
//   1. head: kind, warehouse, district and line count of every transaction
//      (its first draws), counted per chunk of transactions and warehouse;
//   2. line offsets: an inclusive scan of the line counts;
//   3. the chunk counts scanned over chunks, and per-warehouse list starts;
//   4. ranks: per transaction the batch's earlier NewOrders (and their lines,
//      Payments, Deliveries) of its warehouse; each warehouse's NewOrders and
//      Deliveries listed in batch order;
//   5. NewOrder, Payment and StockLevel records;
//   6. Delivery's oldest-undelivered counter, the only true recurrence: one
//      sequential walk per warehouse over its Deliveries;
//   7. OrderStatus and Delivery records, each remembered order read from the
//      batch's NewOrder that made it or from the order memory at batch start;
//   8. state: counters, order memory (last writer of each O_ID), slot header.
#include <algorithm>
#include <new>

#include "engine.h"
#include "gen_state.h"

using namespace ltpg;
using namespace ltpg::gen;

namespace {

constexpr uint32_t TB = 256;          // threads per block of the per-transaction kernels
constexpr uint32_t SCAN_T = 1024;     // threads per block of the scan
constexpr uint32_t SCAN_V = 4;        // values per scan thread
constexpr uint32_t SCAN_BLOCK = SCAN_T * SCAN_V;
constexpr uint32_t DL_TRACKED = 0x80000000u;
constexpr uint64_t MAX_CHUNK_COUNTERS = 8ull << 20;  // per class, chunks x warehouses

__device__ __forceinline__ uint32_t warp_scan_incl(uint32_t v) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// Inclusive scan over the threads of a block of SCAN_T threads.
__device__ __forceinline__ uint32_t block_scan_incl(uint32_t v, uint32_t *sh) {
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint32_t x = warp_scan_incl(v);
    if (lane == 31u) sh[wid] = x;
    __syncthreads();
    if (wid == 0) sh[lane] = warp_scan_incl(sh[lane]);
    __syncthreads();
    if (wid > 0) x += sh[wid - 1];
    __syncthreads();
    return x;
}

// In-place inclusive scan, pass 1: each block scans SCAN_BLOCK values and
// records its total.
__global__ void __launch_bounds__(SCAN_T) scan_blocks(uint32_t *a, uint32_t n, uint32_t *blk) {
    __shared__ uint32_t sh[32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_BLOCK + (uint64_t)threadIdx.x * SCAN_V;
    uint32_t v[SCAN_V], s = 0;
#pragma unroll
    for (uint32_t j = 0; j < SCAN_V; ++j) {
        v[j] = base + j < n ? a[base + j] : 0u;
        s += v[j];
        v[j] = s;
    }
    const uint32_t excl = block_scan_incl(s, sh) - s;
#pragma unroll
    for (uint32_t j = 0; j < SCAN_V; ++j)
        if (base + j < n) a[base + j] = v[j] + excl;
    if (threadIdx.x == SCAN_T - 1) blk[blockIdx.x] = excl + s;
}
// Pass 2: one block scans the block totals, SCAN_BLOCK at a time.
__global__ void __launch_bounds__(SCAN_T) scan_totals(uint32_t *blk, uint32_t nb) {
    __shared__ uint32_t sh[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < nb; b0 += SCAN_BLOCK) {
        const uint32_t base = b0 + threadIdx.x * SCAN_V;
        uint32_t v[SCAN_V], s = 0;
#pragma unroll
        for (uint32_t j = 0; j < SCAN_V; ++j) {
            v[j] = base + j < nb ? blk[base + j] : 0u;
            s += v[j];
            v[j] = s;
        }
        const uint32_t c0 = carry;
        const uint32_t incl = block_scan_incl(s, sh);
        const uint32_t excl = incl - s + c0;
#pragma unroll
        for (uint32_t j = 0; j < SCAN_V; ++j)
            if (base + j < nb) blk[base + j] = v[j] + excl;
        __syncthreads();
        if (threadIdx.x == SCAN_T - 1) carry = c0 + incl;
        __syncthreads();
    }
}
// Pass 3: block b adds the totals of blocks 0 .. b-1.
__global__ void __launch_bounds__(SCAN_T) scan_add(uint32_t *a, uint32_t n, const uint32_t *blk) {
    if (blockIdx.x == 0) return;
    const uint32_t add = blk[blockIdx.x - 1];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_BLOCK + (uint64_t)threadIdx.x * SCAN_V;
#pragma unroll
    for (uint32_t j = 0; j < SCAN_V; ++j)
        if (base + j < n) a[base + j] += add;
}

cudaError_t inclusive_scan(uint32_t *a, uint32_t n, uint32_t *blk, cudaStream_t st, uint64_t &launches) {
    if (n == 0) return cudaSuccess;
    const uint32_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    scan_blocks<<<nb, SCAN_T, 0, st>>>(a, n, blk);
    ++launches;
    if (nb > 1) {
        scan_totals<<<1, SCAN_T, 0, st>>>(blk, nb);
        scan_add<<<nb, SCAN_T, 0, st>>>(a, n, blk);
        launches += 2;
    }
    return cudaGetLastError();
}
uint32_t scan_scratch(uint32_t n) { return (n + SCAN_BLOCK - 1) / SCAN_BLOCK + 1; }

// ---- YCSB ----------------------------------------------------------------------
struct YcsbGenArgs {
    ltpg_ycsb_params p;
    Zipf zipf;
    const FixTables *tab;
    Perm perm;
    bool rotate;
    uint64_t batch_id;
    uint32_t *ops, *val_off;
    uint64_t *vals;
};

__global__ void __launch_bounds__(TB) ycsb_gen_ops(YcsbGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) a.val_off[0] = 0;
    if (t >= a.p.n_txn) return;
    const uint32_t stride = ycsb_stride(a.p.ops_per_txn);
    a.val_off[t + 1] =
        ycsb_txn(a.p, a.zipf, *a.tab, a.rotate ? &a.perm : nullptr, a.batch_id, t, a.ops + (uint64_t)t * stride);
}

__global__ void __launch_bounds__(TB) ycsb_gen_vals(YcsbGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.p.n_txn) return;
    const uint32_t k = a.p.ops_per_txn, stride = ycsb_stride(k);
    const uint64_t txn = a.batch_id * (uint64_t)a.p.n_txn + t;
    uint32_t v = a.val_off[t];
    const uint32_t *w = a.ops + (uint64_t)t * stride;
    for (uint32_t j = 0; j < k; ++j)
        if (ycsb_is_update(w[j])) a.vals[v++] = ycsb_value(a.p, txn, j);
}

// ---- TPC-C ---------------------------------------------------------------------
enum { CL_NO = 0, CL_OL = 1, CL_PAY = 2, CL_DL = 3 };

struct TpccGenArgs {
    ltpg_tpcc_params p;
    uint64_t batch_id, txn_base;
    uint32_t B, W, G, C;  // transactions, warehouses, chunks, transactions per chunk
    uint32_t tracking;
    // generator state
    uint32_t *o_id, *no_id, *ol_id, *h_id;
    uint64_t *made, *delivered;
    uint16_t *o_cust;
    uint8_t *o_dist, *o_cnt;
    uint32_t *o_ol;
    const uint16_t *cust_name;
    const uint8_t *cust_rank;
    // per-batch scratch
    uint32_t *incl;     // B: inclusive scan of line counts
    uint32_t *nob;      // B: the batch's earlier NewOrders of the same warehouse
    uint32_t *aux;      // B: per kind (see tpcc_gen_rank, tpcc_gen_dl_walk)
    uint32_t *cc;       // 4 W G chunk counters [class][w][chunk]
    uint32_t *tot;      // 4 W batch totals [class][w]
    uint32_t *no_start, *dl_start;  // W + 1 list starts
    uint32_t *no_list;  // NewOrders by (warehouse, rank)
    uint64_t *dl_list;  // Deliveries by (warehouse, rank): nob << 32 | TID
    // slot
    ltpg_tpcc_txn *txns;
    ltpg_tpcc_line *lines;
    uint64_t *hdr;
};

__device__ __forceinline__ Rng tpcc_rng(const TpccGenArgs &a, uint32_t t) {
    return Rng(hash3(a.p.seed ^ DOM_TPCC, a.batch_id, t));
}
__device__ __forceinline__ uint32_t *ccp(const TpccGenArgs &a, uint32_t cl, uint32_t w, uint32_t g) {
    return a.cc + ((uint64_t)cl * a.W + w) * a.G + g;
}
__device__ __forceinline__ void store_txn(ltpg_tpcc_txn *dst, const ltpg_tpcc_txn &x) {
    uint4 *p = reinterpret_cast<uint4 *>(dst);
    p[0] = make_uint4(x.kind_info, x.w, x.c_w, x.c_id);
    p[1] = make_uint4(x.a, x.b, x.c, x.line_off);
}

// 1. Heads, line counts, chunk counters.
__global__ void __launch_bounds__(TB) tpcc_gen_head(TpccGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.B) return;
    Rng r = tpcc_rng(a, t);
    const TpccHead h = tpcc_head(a.p, r);
    a.incl[t] = h.cnt;
    const uint32_t g = t / a.C;
    if (h.kind == LTPG_TPCC_NEWORDER) {
        atomicAdd(ccp(a, CL_NO, h.w, g), 1u);
        atomicAdd(ccp(a, CL_OL, h.w, g), h.cnt);
    } else if (h.kind == LTPG_TPCC_PAYMENT) {
        atomicAdd(ccp(a, CL_PAY, h.w, g), 1u);
    } else if (h.kind == LTPG_TPCC_DELIVERY) {
        atomicAdd(ccp(a, CL_DL, h.w, g), 1u);
    }
}

// 3a. One warp per (class, warehouse): exclusive scan of its chunk counters.
__global__ void __launch_bounds__(TB) tpcc_gen_chunk_scan(TpccGenArgs a) {
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (gw >= 4u * a.W) return;
    uint32_t *c = a.cc + (uint64_t)gw * a.G;
    uint32_t carry = 0;
    for (uint32_t g0 = 0; g0 < a.G; g0 += 32) {
        const uint32_t g = g0 + lane;
        const uint32_t v = g < a.G ? c[g] : 0u;
        const uint32_t incl = warp_scan_incl(v);
        if (g < a.G) c[g] = carry + incl - v;
        carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) a.tot[gw] = carry;
}

// 3b. One block: list starts of each warehouse's NewOrders and Deliveries.
__global__ void __launch_bounds__(SCAN_T) tpcc_gen_starts(TpccGenArgs a) {
    __shared__ uint32_t sh[32];
    __shared__ uint32_t carry[2];
    if (threadIdx.x < 2) carry[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t w0 = 0; w0 < a.W; w0 += SCAN_T) {
        const uint32_t w = w0 + threadIdx.x;
        const uint32_t vn = w < a.W ? a.tot[CL_NO * a.W + w] : 0u;
        const uint32_t vd = w < a.W ? a.tot[CL_DL * a.W + w] : 0u;
        const uint32_t cn = carry[0], cd = carry[1];
        const uint32_t in = block_scan_incl(vn, sh);
        const uint32_t id = block_scan_incl(vd, sh);
        if (w < a.W) {
            a.no_start[w] = cn + in - vn;
            a.dl_start[w] = cd + id - vd;
        }
        __syncthreads();
        if (threadIdx.x == SCAN_T - 1) {
            carry[0] = cn + in;
            carry[1] = cd + id;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.no_start[a.W] = carry[0];
        a.dl_start[a.W] = carry[1];
    }
}

// 4. One warp per chunk, 32 transactions per step in batch order.  A lane
// counts the step's earlier lanes of its warehouse by shuffles; the
// warehouse's running counters of the chunk (the chunk counters, now
// prefixes) are advanced by the step's last lane of that warehouse.
//   nob[t]  NewOrders of w before t in the batch (every kind)
//   aux[t]  NewOrder: lines of w's earlier NewOrders; Payment: earlier
//           Payments of w; Delivery: earlier Deliveries of w
__global__ void __launch_bounds__(TB) tpcc_gen_rank(TpccGenArgs a) {
    const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (g >= a.G) return;
    const uint32_t t_end = min(a.B, (g + 1) * a.C);
    for (uint32_t base = g * a.C; base < t_end; base += 32) {
        const uint32_t t = base + lane;
        const bool valid = t < t_end;
        TpccHead h{0u, 0xFFFFFFFFu, 0u, 0u};
        if (valid) {
            Rng r = tpcc_rng(a, t);
            h = tpcc_head(a.p, r);
        }
        const uint32_t key = valid ? h.w : 0xFFFFFFFFu;
        uint32_t pno = 0, pol = 0, ppay = 0, pdl = 0;
        bool last = valid;
        for (uint32_t src = 0; src < 32; ++src) {
            const uint32_t kw = __shfl_sync(0xFFFFFFFFu, key, src);
            const uint32_t kk = __shfl_sync(0xFFFFFFFFu, h.kind, src);
            const uint32_t kc = __shfl_sync(0xFFFFFFFFu, h.cnt, src);
            if (kw != key || !valid) continue;
            if (src < lane) {
                pno += kk == LTPG_TPCC_NEWORDER;
                pol += kk == LTPG_TPCC_NEWORDER ? kc : 0u;
                ppay += kk == LTPG_TPCC_PAYMENT;
                pdl += kk == LTPG_TPCC_DELIVERY;
            } else if (src > lane) {
                last = false;
            }
        }
        uint32_t bno = 0, bol = 0, bpay = 0, bdl = 0;
        if (valid) {
            bno = *ccp(a, CL_NO, h.w, g);
            bol = *ccp(a, CL_OL, h.w, g);
            bpay = *ccp(a, CL_PAY, h.w, g);
            bdl = *ccp(a, CL_DL, h.w, g);
            const uint32_t nb = bno + pno;
            a.nob[t] = nb;
            uint32_t aux = 0;
            if (h.kind == LTPG_TPCC_NEWORDER) {
                aux = bol + pol;
                a.no_list[a.no_start[h.w] + nb] = t;
            } else if (h.kind == LTPG_TPCC_PAYMENT) {
                aux = bpay + ppay;
            } else if (h.kind == LTPG_TPCC_DELIVERY) {
                aux = bdl + pdl;
                a.dl_list[a.dl_start[h.w] + aux] = ((uint64_t)nb << 32) | t;
            }
            a.aux[t] = aux;
        }
        __syncwarp();
        if (last) {
            const bool no = h.kind == LTPG_TPCC_NEWORDER;
            *ccp(a, CL_NO, h.w, g) = bno + pno + (no ? 1u : 0u);
            *ccp(a, CL_OL, h.w, g) = bol + pol + (no ? h.cnt : 0u);
            *ccp(a, CL_PAY, h.w, g) = bpay + ppay + (h.kind == LTPG_TPCC_PAYMENT ? 1u : 0u);
            *ccp(a, CL_DL, h.w, g) = bdl + pdl + (h.kind == LTPG_TPCC_DELIVERY ? 1u : 0u);
        }
        __syncwarp();
    }
}

// 5. NewOrder, Payment, StockLevel records.
__global__ void __launch_bounds__(TB) tpcc_gen_main(TpccGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.B) return;
    Rng r = tpcc_rng(a, t);
    const TpccHead h = tpcc_head(a.p, r);
    if (h.kind == LTPG_TPCC_ORDERSTATUS || h.kind == LTPG_TPCC_DELIVERY) return;
    ltpg_tpcc_txn x{};
    x.line_off = a.incl[t] - h.cnt;
    x.w = h.w;
    if (h.kind == LTPG_TPCC_NEWORDER) {
        const uint32_t s = a.nob[t];
        x.a = (uint32_t)(((uint64_t)a.o_id[h.w] + s) % 30000u);
        x.b = (uint32_t)(((uint64_t)a.no_id[h.w] + s) % 30000u);
        x.c = (uint32_t)(((uint64_t)a.ol_id[h.w] + a.aux[t]) % 450000u);
        tpcc_neworder(a.p, r, h, x, a.lines + x.line_off);
    } else if (h.kind == LTPG_TPCC_PAYMENT) {
        x.a = (uint32_t)(((uint64_t)a.h_id[h.w] + a.aux[t]) % 30000u);
        tpcc_payment(a.p, r, h, x, a.cust_name, a.cust_rank);
    } else {
        tpcc_stocklevel(r, h, x);
    }
    store_txn(a.txns + t, x);
}

// 6. Oldest undelivered order, per warehouse in batch order.  aux[t] of a
// Delivery becomes DL_TRACKED | O_ID, or 0 when w had no undelivered order.
__global__ void __launch_bounds__(TB) tpcc_gen_dl_walk(TpccGenArgs a) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= a.W) return;
    uint64_t D = a.delivered[w];
    const uint64_t M0 = a.made[w];
    const uint32_t i1 = a.dl_start[w + 1];
    for (uint32_t i = a.dl_start[w]; i < i1; i += 4) {
        uint64_t e[4];
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) e[j] = i + j < i1 ? a.dl_list[i + j] : 0ull;
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) {
            if (i + j >= i1) break;
            const uint32_t t = (uint32_t)e[j];
            const uint64_t M = M0 + (e[j] >> 32);
            uint32_t v = 0;
            if (D < M) {
                if (M - D > 30000u) D = M - 30000u;
                v = DL_TRACKED | (uint32_t)(D % 30000u);
                ++D;
            }
            a.aux[t] = v;
        }
    }
    a.delivered[w] = D;
}

// 7. OrderStatus and Delivery records.
__global__ void __launch_bounds__(TB) tpcc_gen_osdl(TpccGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.B) return;
    Rng r = tpcc_rng(a, t);
    const TpccHead h = tpcc_head(a.p, r);
    if (h.kind != LTPG_TPCC_ORDERSTATUS && h.kind != LTPG_TPCC_DELIVERY) return;
    const uint32_t w = h.w, nb = a.nob[t];
    const uint32_t o_id_t = (uint32_t)(((uint64_t)a.o_id[w] + nb) % 30000u);
    // The order with O_ID o as the host loop sees it at t: made by the batch's
    // NewOrder of rank nb - 1 - delta when that is >= 0, else remembered.
    auto order = [&](uint32_t o) {
        const uint32_t delta = (o_id_t + 30000u - 1u - o) % 30000u;
        if (delta < nb) {
            const ltpg_tpcc_txn y = a.txns[a.no_list[a.no_start[w] + nb - 1u - delta]];
            return TpccOrder{y.c_id, tpcc_d(y.kind_info), y.c, tpcc_ol_cnt(y.kind_info)};
        }
        const size_t k = 30000ull * w + o;
        return TpccOrder{a.o_cust[k], a.o_dist[k], a.o_ol[k], a.o_cnt[k]};
    };
    ltpg_tpcc_txn x{};
    x.line_off = a.incl[t];
    x.w = w;
    if (h.kind == LTPG_TPCC_ORDERSTATUS) {
        const uint64_t made = a.tracking ? a.made[w] + nb : 0u;
        tpcc_orderstatus(a.p, r, h, x, made, o_id_t, order, a.cust_name, a.cust_rank);
    } else {
        const uint32_t v = a.tracking ? a.aux[t] : 0u;
        tpcc_delivery(r, h, x, (v & DL_TRACKED) != 0u, v & ~DL_TRACKED, order);
    }
    store_txn(a.txns + t, x);
}

// 8. Order memory (the batch's last NewOrder of each O_ID), counters, header.
__global__ void __launch_bounds__(TB) tpcc_gen_state(TpccGenArgs a) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < a.B && a.tracking) {
        const ltpg_tpcc_txn x = a.txns[t];
        if (tpcc_kind(x.kind_info) == LTPG_TPCC_NEWORDER && a.nob[t] + 30000u >= a.tot[CL_NO * a.W + x.w]) {
            const size_t k = 30000ull * x.w + x.a;
            a.o_cust[k] = (uint16_t)x.c_id;
            a.o_dist[k] = (uint8_t)tpcc_d(x.kind_info);
            a.o_ol[k] = x.c;
            a.o_cnt[k] = (uint8_t)tpcc_ol_cnt(x.kind_info);
        }
    }
    if (t < a.W) {
        const uint32_t n_no = a.tot[CL_NO * a.W + t];
        a.o_id[t] = (uint32_t)(((uint64_t)a.o_id[t] + n_no) % 30000u);
        a.no_id[t] = (uint32_t)(((uint64_t)a.no_id[t] + n_no) % 30000u);
        a.ol_id[t] = (uint32_t)(((uint64_t)a.ol_id[t] + a.tot[CL_OL * a.W + t]) % 450000u);
        a.h_id[t] = (uint32_t)(((uint64_t)a.h_id[t] + a.tot[CL_PAY * a.W + t]) % 30000u);
        if (a.tracking) a.made[t] += n_no;
    }
    if (t == 0) {
        a.hdr[0] = a.incl[a.B - 1];
        a.hdr[1] = a.txn_base;
    }
}

uint32_t blocks(uint64_t n, uint32_t per) { return (uint32_t)((n + per - 1) / per); }

}  // namespace

// Device side of a generator: YCSB, the sampler's power tables; TPC-C, the
// generator's state and the scratch of one batch.
struct ltpg_gen_dev {
    int device = -1;
    FixTables *tab = nullptr;
    uint32_t G = 0, C = 0;
    uint32_t *o_id = nullptr, *no_id = nullptr, *ol_id = nullptr, *h_id = nullptr;
    uint64_t *made = nullptr, *delivered = nullptr;
    uint16_t *o_cust = nullptr;
    uint8_t *o_dist = nullptr, *o_cnt = nullptr;
    uint32_t *o_ol = nullptr;
    uint16_t *cust_name = nullptr;
    uint8_t *cust_rank = nullptr;
    uint32_t *incl = nullptr, *nob = nullptr, *aux = nullptr, *cc = nullptr, *tot = nullptr;
    uint32_t *no_start = nullptr, *dl_start = nullptr, *no_list = nullptr, *blk = nullptr;
    uint64_t *dl_list = nullptr;
    std::vector<void *> owned;
};

namespace {

template <class T>
cudaError_t dalloc(ltpg_gen_dev *d, T **p, uint64_t n) {
    *p = nullptr;
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e == cudaSuccess) d->owned.push_back(*p);
    return e;
}
template <class T>
cudaError_t dput(ltpg_gen_dev *d, T **p, const std::vector<T> &h) {
    cudaError_t e = dalloc(d, p, h.size());
    if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

void free_dev(ltpg_gen_dev *d) {
    if (!d) return;
    int cur = -1;
    cudaGetDevice(&cur);
    if (d->device >= 0 && d->device != cur) cudaSetDevice(d->device);
    for (void *p : d->owned) cudaFree(p);
    if (d->device >= 0 && d->device != cur && cur >= 0) cudaSetDevice(cur);
    delete d;
}

// Copies the host state of a TPC-C generator to the device (first device batch).
cudaError_t bind_tpcc(ltpg_gen *g, int device) {
    ltpg_gen_dev *d = new (std::nothrow) ltpg_gen_dev();
    if (!d) return cudaErrorMemoryAllocation;
    d->device = device;
    const uint32_t B = g->c.n_txn, W = g->c.warehouses;
    d->C = 1024;
    if ((uint64_t)((B + d->C - 1) / d->C) * W > MAX_CHUNK_COUNTERS) {
        const uint64_t g_max = std::max<uint64_t>(1, MAX_CHUNK_COUNTERS / W);
        d->C = (uint32_t)(((B + g_max - 1) / g_max + 31) / 32 * 32);
    }
    d->G = (B + d->C - 1) / d->C;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    ok(dput(d, &d->o_id, g->o_id));
    ok(dput(d, &d->no_id, g->no_id));
    ok(dput(d, &d->ol_id, g->ol_id));
    ok(dput(d, &d->h_id, g->h_id));
    if (!g->made.empty()) {
        ok(dput(d, &d->made, g->made));
        ok(dput(d, &d->delivered, g->delivered));
        ok(dput(d, &d->o_cust, g->o_cust));
        ok(dput(d, &d->o_dist, g->o_dist));
        ok(dput(d, &d->o_cnt, g->o_cnt));
        ok(dput(d, &d->o_ol, g->o_ol));
    }
    if (!g->cust_name.empty()) {
        ok(dput(d, &d->cust_name, g->cust_name));
        ok(dput(d, &d->cust_rank, g->cust_rank));
    }
    ok(dalloc(d, &d->incl, B));
    ok(dalloc(d, &d->nob, B));
    ok(dalloc(d, &d->aux, B));
    ok(dalloc(d, &d->cc, 4ull * W * d->G));
    ok(dalloc(d, &d->tot, 4ull * W));
    ok(dalloc(d, &d->no_start, (uint64_t)W + 1));
    ok(dalloc(d, &d->dl_start, (uint64_t)W + 1));
    ok(dalloc(d, &d->no_list, B));
    ok(dalloc(d, &d->dl_list, B));
    ok(dalloc(d, &d->blk, scan_scratch(B)));
    if (e != cudaSuccess) {
        free_dev(d);
        return e;
    }
    g->dev = d;
    g->dev_bound = true;
    return cudaSuccess;
}

// The YCSB generator's power tables on the device (first device batch).
cudaError_t bind_ycsb(ltpg_gen *g, int device) {
    ltpg_gen_dev *d = new (std::nothrow) ltpg_gen_dev();
    if (!d) return cudaErrorMemoryAllocation;
    d->device = device;
    cudaError_t e = dalloc(d, &d->tab, 1);
    if (e == cudaSuccess) e = cudaMemcpy(d->tab, &host_fix_tables(), sizeof(FixTables), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_dev(d);
        return e;
    }
    g->dev = d;
    return cudaSuccess;
}

}  // namespace

void gen_dev_free(ltpg_gen *g) {
    free_dev(g->dev);
    g->dev = nullptr;
}

extern "C" {

}  // extern "C"

namespace {

int gen_ycsb(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot, cudaStream_t st) {
    const ltpg_ycsb_params &p = g->y;
    if (cudaSetDevice(c->device) != cudaSuccess) return ctx_fail(c, LTPG_ERR_CUDA, "set device");
    if (p.n_records > c->ycsb.n) return ctx_fail(c, LTPG_ERR_INVALID, "generator keys exceed the loaded table");
    if (g->dev && g->dev->device != c->device)
        return ctx_fail(c, LTPG_ERR_INVALID, "generator tables live on another device");
    Slot *s = nullptr;
    int r = slot_prepare_ycsb(c, slot, p.n_txn, p.ops_per_txn, 0, &s);
    if (r) return r;
    cudaError_t e0 = cudaSuccess;
    if (!g->dev && (e0 = bind_ycsb(g, c->device)) != cudaSuccess) return ctx_cuda_fail(c, e0, "generator tables");
    YcsbGenArgs a;
    a.p = p;
    a.zipf = g->zipf;
    a.tab = g->dev->tab;
    a.rotate = p.rotate_every != 0;
    if (a.rotate) a.perm.init(p.n_records, hash3(p.seed ^ DOM_YCSB_PERM, batch_id / p.rotate_every, 0));
    a.batch_id = batch_id;
    a.ops = s->ops;
    a.val_off = s->val_off;
    a.vals = s->vals;
    const uint32_t nb = blocks(p.n_txn, TB);
    ycsb_gen_ops<<<nb, TB, 0, st>>>(a);
    count_launch(c);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        // the scan's block totals borrow the slot's vals buffer, whose values
        // are written after the scan
        uint64_t launches = 0;
        e = inclusive_scan(s->val_off + 1, p.n_txn, reinterpret_cast<uint32_t *>(s->vals), st, launches);
        count_launch(c, launches);
    }
    if (e == cudaSuccess) {
        ycsb_gen_vals<<<nb, TB, 0, st>>>(a);
        count_launch(c);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? LTPG_OK : ctx_cuda_fail(c, e, "device YCSB generation");
}

int gen_tpcc(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot, cudaStream_t st) {
    if (batch_id != g->next_batch) return ctx_fail(c, LTPG_ERR_STATE, "TPC-C batches are drawn in order");
    const ltpg_tpcc_params &p = g->c;
    if (cudaSetDevice(c->device) != cudaSuccess) return ctx_fail(c, LTPG_ERR_CUDA, "set device");
    if (p.warehouses > c->tpcc.W) return ctx_fail(c, LTPG_ERR_INVALID, "generator warehouses exceed the loaded tables");
    if (g->dev && g->dev->device != c->device)
        return ctx_fail(c, LTPG_ERR_INVALID, "generator state lives on another device");
    const uint64_t max_lines = (uint64_t)p.n_txn * LTPG_TPCC_MAX_LINES;
    if (max_lines > c->cfg.max_lines)
        return ctx_fail(c, LTPG_ERR_INVALID, "device generation needs max_lines >= 15 n_txn");
    Slot *s = nullptr;
    int r = slot_prepare_tpcc(c, slot, p.n_txn, max_lines, g->txn_base, &s);
    if (r) return r;
    cudaError_t e = cudaSuccess;
    if (!g->dev && (e = bind_tpcc(g, c->device)) != cudaSuccess) return ctx_cuda_fail(c, e, "generator state to device");
    ltpg_gen_dev *d = g->dev;
    TpccGenArgs a;
    a.p = p;
    a.batch_id = batch_id;
    a.txn_base = g->txn_base;
    a.B = p.n_txn;
    a.W = p.warehouses;
    a.G = d->G;
    a.C = d->C;
    a.tracking = d->made != nullptr;
    a.o_id = d->o_id;
    a.no_id = d->no_id;
    a.ol_id = d->ol_id;
    a.h_id = d->h_id;
    a.made = d->made;
    a.delivered = d->delivered;
    a.o_cust = d->o_cust;
    a.o_dist = d->o_dist;
    a.o_cnt = d->o_cnt;
    a.o_ol = d->o_ol;
    a.cust_name = d->cust_name;
    a.cust_rank = d->cust_rank;
    a.incl = d->incl;
    a.nob = d->nob;
    a.aux = d->aux;
    a.cc = d->cc;
    a.tot = d->tot;
    a.no_start = d->no_start;
    a.dl_start = d->dl_start;
    a.no_list = d->no_list;
    a.dl_list = d->dl_list;
    a.txns = s->txns;
    a.lines = s->lines;
    a.hdr = s->dev_hdr;
    const uint32_t nb = blocks(a.B, TB);
    uint64_t launches = 0;
    e = cudaMemsetAsync(a.cc, 0, 4ull * a.W * a.G * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        tpcc_gen_head<<<nb, TB, 0, st>>>(a);
        ++launches;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = inclusive_scan(a.incl, a.B, d->blk, st, launches);
    if (e == cudaSuccess) {
        tpcc_gen_chunk_scan<<<blocks(4ull * a.W * 32, TB), TB, 0, st>>>(a);
        tpcc_gen_starts<<<1, SCAN_T, 0, st>>>(a);
        tpcc_gen_rank<<<blocks((uint64_t)a.G * 32, TB), TB, 0, st>>>(a);
        tpcc_gen_main<<<nb, TB, 0, st>>>(a);
        launches += 4;
        if (a.tracking) {
            tpcc_gen_dl_walk<<<blocks(a.W, TB), TB, 0, st>>>(a);
            ++launches;
        }
        tpcc_gen_osdl<<<nb, TB, 0, st>>>(a);
        tpcc_gen_state<<<blocks(std::max(a.B, a.W), TB), TB, 0, st>>>(a);
        launches += 2;
        e = cudaGetLastError();
    }
    count_launch(c, launches);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "device TPC-C generation");
    g->txn_base += p.n_txn;
    g->next_batch++;
    return LTPG_OK;
}

}  // namespace

namespace ltpg {
int gen_device_batch(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot, cudaStream_t st) {
    if (!c || !g) return c ? ctx_fail(c, LTPG_ERR_INVALID, "null generator") : LTPG_ERR_INVALID;
    if (g->kind == LTPG_WORKLOAD_YCSB) return gen_ycsb(c, g, batch_id, slot, st);
    if (g->kind == LTPG_WORKLOAD_TPCC) return gen_tpcc(c, g, batch_id, slot, st);
    return ctx_fail(c, LTPG_ERR_INVALID, "unknown generator");
}
}  // namespace ltpg

extern "C" {

int ltpg_gen_ycsb_batch_device(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot) {
    if (!c || !g || g->kind != LTPG_WORKLOAD_YCSB)
        return c ? ctx_fail(c, LTPG_ERR_INVALID, "not a YCSB generator") : LTPG_ERR_INVALID;
    return gen_ycsb(c, g, batch_id, slot, c->stream);
}

int ltpg_gen_tpcc_batch_device(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot) {
    if (!c || !g || g->kind != LTPG_WORKLOAD_TPCC)
        return c ? ctx_fail(c, LTPG_ERR_INVALID, "not a TPC-C generator") : LTPG_ERR_INVALID;
    return gen_tpcc(c, g, batch_id, slot, c->stream);
}

}  // extern "C"
