// ycsb_tuned.cu — tuned YCSB path: fused kernels, CUDA-graph and persistent modes.
//
// Same protocol and outputs as the plain path (ycsb.cu); only the schedule
// changes:
//   * execute+register walks block tiles of whole transactions, reading four op
//     words per thread with one 128-bit load;
//   * a registration goes (a) to a shared-memory staging entry when the
//     predictor marked its key's bucket hot, else (b) through a warp-level
//     dedupe (__match_any_sync: only the smallest TID of each key in the warp
//     issues), then (c) an L1 read of the slot skips the atomic when the slot
//     already holds a smaller value.  Slot values only decrease (newer batch
//     tags are smaller, and within a batch atomicMin only lowers), so any value
//     observed, stale or not, is >= the current one: the skip is exact;
//   * check and write-back run in one kernel: the commit decision of a tile is
//     made in shared memory, then each committed transaction's thread stores
//     its updates in op order;
//   * late reads (a launch setting): execute only registers, the check kernel
//     reads the rows of the committed transactions after the tile's commit
//     decision, and a third kernel stores the updates, so that no aborted
//     transaction's rows are read;
//   * write-first registration (late reads 3): the updates register first,
//     then each read touches its key's slot only when an update writes the
//     key; the read registration also lists the updates by value index, and
//     the check and the write-back walk that list instead of the op words.
#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "stage.cuh"

namespace ltpg {

struct YcsbTunedArgs {
    const uint32_t *ops;
    const uint32_t *val_off;
    const uint64_t *vals;
    uint32_t B, k, stride, tile;  // tile = transactions per block tile (multiple of 32)
    uint64_t *rows;
    uint64_t n;
    RegSlot *reg;
    int64_t *results;
    uint8_t *flags;
    uint32_t *bitmap;
    DevStats *st;
    DevCtl *ctl;
    const uint16_t *stage_map;
    const uint32_t *stage_bits;
    const uint32_t *stage_rank;
    uint32_t *bucket_counts;
    uint32_t ways, stage_entries;
    uint32_t filter;
    uint32_t lpt;  // lanes per transaction of the one-op-per-lane kernels: stride rounded up to a power of two (0: > 32)
    uint32_t late; // late reads: 0 off, 1 in the check kernel's tiles, 2 in a kernel of their own,
                   // 3 write-first registration
    uint32_t *wbits;  // write-first: one bit per key, set for keys an update of the batch writes
    uint2 *upd;        // write-first update list: entry u = {TID, op word} of the u-th update (0 entries: none)
    uint64_t upd_cap;  // entries of the update list
    uint64_t vals_cap; // values the slot holds (bound of every value index)
};

__device__ __forceinline__ uint64_t ld_ca_u64(const unsigned long long *p) {
    uint64_t v;
    asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_ca_u32(const unsigned *p) {
    uint32_t v;
    asm volatile("ld.global.ca.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// kCoh (the persistent kernel, where the phases share one launch): every
// load of a word that an earlier phase of the launch wrote, or that this
// phase writes (slots, writer bits, flag bytes), is a GPU-scope relaxed load
// served by L2 (ld_gpu_*), never an L1 or read-only-path load, which could
// return a line cached before the grid barrier.  Op words, values and rows
// (read before the write-back) are written by no phase and keep the
// read-only path.  In the separate kernels L1 starts empty at every kernel.
template <bool kCoh>
__device__ __forceinline__ uint64_t ld_filter_u64(const unsigned long long *p) {
    return kCoh ? ld_gpu_u64(p) : ld_ca_u64(p);
}
template <bool kCoh>
__device__ __forceinline__ uint32_t ld_wbits(const uint32_t *p) {
    return kCoh ? ld_gpu_u32(p) : __ldg(p);
}
template <bool kCoh>
__device__ __forceinline__ uint32_t ld_flag(const uint8_t *p) {
    return kCoh ? ld_gpu_u8(p) : (uint32_t)*p;
}

// ---- execute + register over all tiles assigned to this block ----------------
template <bool kStage>
__device__ __forceinline__ void exec_tiles(const YcsbTunedArgs &a, unsigned long long *dig, StageEnt *tab,
                                           uint64_t tag) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nvec_tile = a.tile * a.stride / 4;
    const uint32_t n_tiles = (a.B + a.tile - 1) / a.tile;
    uint32_t counted = 0;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t t0 = tile * a.tile;
        const uint32_t nt = min(a.tile, a.B - t0);
        const uint32_t nvec = nt * a.stride / 4;
        for (uint32_t i = threadIdx.x; i < a.tile; i += blockDim.x) dig[i] = 0ull;
        __syncthreads();
        const uint4 *vp = reinterpret_cast<const uint4 *>(a.ops + (uint64_t)t0 * a.stride);
        for (uint32_t base = 0; base < nvec_tile; base += blockDim.x) {
            const uint32_t v = base + threadIdx.x;
            const bool act = v < nvec;
            const uint4 w4 = act ? ld_nc_u4(vp + v) : make_uint4(LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD,
                                                                  LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD);
            const uint32_t lt = act ? (v * 4) / a.stride : 0;
            const uint32_t j0 = v * 4 - lt * a.stride;
            const uint32_t t = t0 + lt;
            const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
            unsigned long long part = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t w = words[q];
                bool valid = act && !ycsb_is_pad(w);
                const uint32_t key = ycsb_key(w);
                const bool upd = ycsb_is_update(w);
                if (valid && key >= a.n) {
                    report_error(a.ctl, DERR_BOUNDS, t);
                    valid = false;
                }
                bool staged = false;
                if (kStage && valid) {
                    const uint32_t b = key_bucket(key);
                    const uint32_t g = __ldg(a.stage_map + b);
                    if (g != STAGE_NONE && (g + 1) * a.ways <= a.stage_entries) {
                        StageEnt *e = stage_find(tab, g, a.ways, key);
                        if (e) {
                            atomicMin(upd ? &e->wmin : &e->rmin, t);
                            atomicAdd(&e->cnt, 1u);
                            staged = true;
                        }
                    }
                    if (!staged && (t % COUNT_SAMPLE) == 0u) {
                        atomicAdd(a.bucket_counts + b, COUNT_SAMPLE);
                        ++counted;
                    }
                }
                const bool need = valid && !staged;
                const uint32_t mkey = need ? (key | (upd ? 0x80000000u : 0u)) : 0xFFFFFFFFu;
                const unsigned peers = __match_any_sync(FULL, mkey);
                // lanes are in transaction order, so the lowest peer holds the smallest TID
                if (need && (__ffs(peers) - 1) == (int)lane) {
                    unsigned long long *slot = upd ? &a.reg[key].w : &a.reg[key].r;
                    const unsigned long long mine = tag | t;
                    if (!a.filter || ld_ca_u64(slot) > mine) red_min(slot, mine);
                }
                if (valid && !upd) {
                    const char *p = reinterpret_cast<const char *>(a.rows + (uint64_t)key * LTPG_YCSB_FIELDS);
                    const ulonglong2 r0 = ld_nc16(p), r1 = ld_nc16(p + 16), r2 = ld_nc16(p + 32),
                                     r3 = ld_nc16(p + 48), r4 = ld_nc16(p + 64);
                    const unsigned long long x = r0.x ^ r0.y ^ r1.x ^ r1.y ^ r2.x ^ r2.y ^ r3.x ^ r3.y ^ r4.x ^ r4.y ^
                                                 scan_rest(a.reg, a.rows, a.n, w, tag | t, a.filter != 0u);
                    part += x * (2ull * (j0 + q) + 1ull);
                }
            }
            if (part) atomicAdd(&dig[lt], part);
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x) a.results[t0 + i] = (int64_t)dig[i];
    }
    (void)counted;
}

// Stores the updates of committed transaction t in op order: a transaction
// that updates a field twice leaves its later value (as a sequential replay
// does), and no two committed transactions write one row (WAW).
__device__ __forceinline__ void write_txn_updates(const YcsbTunedArgs &a, uint32_t t) {
    uint32_t v = a.val_off[t];
    if (v == a.val_off[t + 1]) return;
    // value indices stay below the batch's value count and the slot's
    // capacity: offsets that disagree with the op words are reported
    const uint64_t nv = min((uint64_t)__ldg(a.val_off + a.B), a.vals_cap);
    const uint4 *tw = reinterpret_cast<const uint4 *>(a.ops + (uint64_t)t * a.stride);
    for (uint32_t q4 = 0; q4 < a.stride / 4u; ++q4) {
        const uint4 w4 = ld_nc_u4(tw + q4);
        const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t x = words[q];
            if (ycsb_is_pad(x) || !ycsb_is_update(x)) continue;
            const uint32_t key = ycsb_key(x), fld = ycsb_field(x);
            if (v >= nv) {
                report_error(a.ctl, DERR_BOUNDS, t);
                return;
            }
            if (key < a.n && fld < LTPG_YCSB_FIELDS) a.rows[(uint64_t)key * LTPG_YCSB_FIELDS + fld] = a.vals[v];
            ++v;
        }
    }
}

// Late reads of one tile whose commit flags are in fl: the lpt lanes of a
// transaction (a power of two, aligned in the warp) take one op each; the
// point reads of committed transactions are gathered five lanes to a row (one
// 16-byte chunk each, six rows per round), a range scan by the whole warp over
// its contiguous rows.  results[t] = sum over reads of xor(row) * (2j + 1), as
// at execute; 0 for an aborted transaction.  No row is written before the
// next kernel, so every read sees the batch-start image.
// Per-warp shared scratch of the late reads: the keys of the warp's point
// reads by rank, and the xor of each one's row.
struct LateScratch {
    uint32_t key[32];
    unsigned long long x[32];
};

// This warp's scratch; one array per kernel, whichever late-read loops it runs.
__device__ __forceinline__ LateScratch *late_scratch() {
    __shared__ LateScratch scratch[16];  // blocks of up to 512 threads
    return scratch + (threadIdx.x >> 5);
}

// One step of the lanes of a warp (all 32 call it): lane j of transaction t
// (own: the lane holds an op slot of a transaction; com: t committed).
__device__ __forceinline__ void late_read_step(const YcsbTunedArgs &a, LateScratch *ws, uint32_t t, uint32_t j,
                                               bool own, bool com) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lpt = a.lpt;
    const uint32_t grp = lane / 5, chunk = lane % 5;
    {
        const uint32_t w = com && j < a.stride ? __ldg(a.ops + (uint64_t)t * a.stride + j) : LTPG_YCSB_OP_PAD;
        const uint32_t key = ycsb_key(w);
        const bool rd = !ycsb_is_pad(w) && !ycsb_is_update(w) && key < a.n;
        const bool scan = rd && ycsb_span(w) != 0u;
        const unsigned need = __ballot_sync(FULL, rd && !scan);
        const uint32_t n_need = __popc(need);
        unsigned long long x = 0;
        if (n_need) {  // warp-uniform
            // round r: lane group g (five lanes, one 16-byte chunk each) reads
            // the row of the (6r + g)-th point read; its first lane folds the
            // chunks and leaves the row's xor under that rank
            const uint32_t my_rank = __popc(need & ((1u << lane) - 1u));
            const bool mine = (need >> lane) & 1u;
            if (mine) ws->key[my_rank] = key;
            __syncwarp();
            ulonglong2 ch[6];
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const uint32_t idx = (uint32_t)r * 6u + grp;
                const bool go = grp < 6 && idx < n_need;
                const uint32_t k_src = go ? ws->key[idx] : 0u;
                ch[r] = go ? ld_nc16_issue(reinterpret_cast<const char *>(a.rows + (uint64_t)k_src * LTPG_YCSB_FIELDS) +
                                           16u * chunk)
                           : make_ulonglong2(0ull, 0ull);
            }
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                if ((uint32_t)r * 6u >= n_need) break;  // warp-uniform
                const unsigned long long c0 = ch[r].x ^ ch[r].y;
                unsigned long long c = c0 ^ __shfl_down_sync(FULL, c0, 1);
                c ^= __shfl_down_sync(FULL, c, 2);
                const unsigned long long rowx = c ^ __shfl_down_sync(FULL, c0, 4);
                const uint32_t idx = (uint32_t)r * 6u + grp;
                if (chunk == 0u && grp < 6 && idx < n_need) ws->x[idx] = rowx;
            }
            __syncwarp();
            if (mine) x = ws->x[my_rank];
            __syncwarp();  // the next step reuses the scratch
        }
        const uint32_t last = scan ? (uint32_t)scan_last(w, a.n) : 0u;
        for (unsigned m = __ballot_sync(FULL, scan); m; m &= m - 1u) {
            const uint32_t src = (uint32_t)__ffs(m) - 1u;
            const uint32_t k0 = __shfl_sync(FULL, key, src), k1 = __shfl_sync(FULL, last, src);
            const uint32_t chunks = (k1 - k0 + 1u) * 5u;
            const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(a.rows + (uint64_t)k0 * LTPG_YCSB_FIELDS);
            unsigned long long c_all = 0;
            for (uint32_t c = lane; c < chunks; c += 32u) {
                const ulonglong2 q = ld_nc16(p + c);
                c_all ^= q.x ^ q.y;
            }
            for (uint32_t o = 16; o >= 1u; o >>= 1) c_all ^= __shfl_xor_sync(FULL, c_all, o);
            if (lane == src) x = c_all;
        }
        unsigned long long part = rd ? x * (2ull * j + 1ull) : 0ull;
        for (uint32_t o = lpt >> 1; o >= 1; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
        if (own && j == 0u) a.results[t] = (int64_t)part;
    }
}

__device__ __forceinline__ void late_read_tile(const YcsbTunedArgs &a, const uint32_t *fl, uint32_t t0,
                                               uint32_t nt) {
    LateScratch *ws = late_scratch();
    const uint32_t lsh = (uint32_t)__ffs(a.lpt) - 1u;
    const uint32_t nl = a.tile << lsh;
    for (uint32_t base = 0; base < nl; base += blockDim.x) {
        const uint32_t v = base + threadIdx.x;
        const uint32_t lt = v >> lsh, j = v & (a.lpt - 1u);
        const bool own = v < nl && lt < nt;
        late_read_step(a, ws, t0 + lt, j, own, own && (fl[lt] & LTPG_FLAG_COMMIT) != 0u);
    }
}

// Late reads as a kernel of their own (late_reads = 2), after the check: the
// lanes of the whole batch, lpt per transaction, commit flags from global memory.
template <bool kCoh>
__device__ __forceinline__ void late_read_loop(const YcsbTunedArgs &a) {
    LateScratch *ws = late_scratch();
    const uint32_t lsh = (uint32_t)__ffs(a.lpt) - 1u;
    const uint64_t nw = (uint64_t)a.B << lsh;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nw; base += step) {
        const uint64_t v = base + threadIdx.x;
        const bool own = v < nw;
        const uint32_t t = (uint32_t)(v >> lsh), j = (uint32_t)v & (a.lpt - 1u);
        // the commit decision from the conflict bits (the check kernel of late
        // reads 2 also set COMMIT; write-first leaves it to the write-back)
        late_read_step(a, ws, t, j, own,
                       own && commits(ld_flag<kCoh>(a.flags + t) & (LTPG_FLAG_RAW | LTPG_FLAG_WAR | LTPG_FLAG_WAW)));
    }
}

// The grid-stride kernels below are instantiated per block size (BS = 128,
// 256, 512: launch setting block_threads), each with launch bounds of its own
// block: bounds above the block change the compiler's register choice (the
// read kernel takes 58 registers under 512-thread bounds against 40 under
// 256, and loses a third of its resident warps).
template <int BS>
__global__ void __launch_bounds__(BS) ycsb_read_late(YcsbTunedArgs a) { late_read_loop<false>(a); }

// ---- write-first registration (late_reads = 3) ---------------------------------
// The same RAW / WAR / WAW outcome with at most one random slot access per op
// instead of two.  (1) The updates register (write word) and set their key's
// bit in a writer bitmap.  (2) A read whose key has no writer in the batch has
// no RAW and no WAR to cause, and touches no slot; any other read loads its
// key's slot once: the write word is final, so RAW = (smallest writer < t),
// and the read registers in the read word.  A key with a writer thus gets
// every one of its reads registered, as in the protocol.  (3) The updates load
// their slot for WAR and WAW.  The flag bytes collect the conflict bits of (2)
// and (3).  (4) The committed reads gather their rows (late_read_loop; commit
// from the conflict bits); (5) the write-back decides the commits, writes the
// final flags, bitmap and counters, and stores.  Checking the updates in a
// kernel of their own keeps their slot loads out of the path of the row
// reads: 81 % of the warps of a 16-op, 5 %-update batch hold an update.

// 16-byte slot load through L1: the write words are final after (1), and L1
// is invalidated between dependent kernels; a read word seen stale is never
// below the current one, so skipping a red.min on it stays exact.
__device__ __forceinline__ ulonglong2 ld_slot_ca(const RegSlot *p) {
    ulonglong2 v;
    asm volatile("ld.global.ca.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}

// (1) the updates' registrations and writer bits: four op words per thread
// (transactions are 4-word aligned); every op's key is bounds-checked here.
// Also zeroes the flag bytes, which (2) and (3) OR the conflict bits into.
template <bool kCoh>
__device__ __forceinline__ void wf_register_writes(const YcsbTunedArgs &a, uint64_t tag) {
    const uint64_t nvec = (uint64_t)a.B * a.stride / 4u;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((uint64_t)a.B + 3) / 4; i += step)
        reinterpret_cast<unsigned *>(a.flags)[i] = 0u;
    const uint4 *vp = reinterpret_cast<const uint4 *>(a.ops);
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvec; v += step) {
        const uint4 w4 = ld_nc_u4(vp + v);
        const uint32_t t = (uint32_t)(v * 4u / a.stride);
        const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t w = words[q];
            if (ycsb_is_pad(w)) continue;
            const uint32_t key = ycsb_key(w);
            if (key >= a.n) {
                report_error(a.ctl, DERR_BOUNDS, t);
                continue;
            }
            if (!ycsb_is_update(w)) continue;
            unsigned long long *slot = &a.reg[key].w;
            const unsigned long long mine = tag | t;
            if (!a.filter || ld_filter_u64<kCoh>(slot) > mine) red_min(slot, mine);
            // bits are only set within a batch: a bit seen set needs no atomic
            // (hot keys' updates would otherwise all hit one word)
            unsigned *bw = a.wbits + (key >> 5);
            const uint32_t seen = kCoh ? ld_gpu_u32(bw) : ld_ca_u32(bw);
            if (!((seen >> (key & 31u)) & 1u)) atomicOr(bw, 1u << (key & 31u));
        }
    }
}

// One key of a read: RAW against the final write word, registration when the
// key has a writer.  Returns the RAW bit.  A key outside the writer bitmap has
// no writer in the batch: no RAW, nothing to register, and no slot load (the
// bitmap, 1/128 of the slot table, stays in L2).
template <bool kCoh>
__device__ __forceinline__ bool wf_read_key(const YcsbTunedArgs &a, uint64_t key, uint32_t t, uint32_t epoch,
                                            unsigned long long mine) {
    if (!((ld_wbits<kCoh>(a.wbits + (key >> 5)) >> (key & 31u)) & 1u)) return false;
    const ulonglong2 s = kCoh ? ld_gpu_slot(a.reg + key) : ld_slot_ca(a.reg + key);
    const uint32_t wmin = slot_min(s.y, epoch);
    if (wmin != 0xFFFFFFFFu && s.x > mine) red_min(&a.reg[key].r, mine);
    return wmin < t;
}

// The update list: the batch's u-th update (u = its value index, val_off[t]
// + its rank among transaction t's updates) is stored as {t, op word}, so that
// the check and the write-back walk the updates alone instead of every op word.
// A lane holds op vector seg of its transaction (vpt = stride / 4 vectors, at
// most 8).  With vpt a power of two the transaction's vectors are consecutive
// lanes of one warp and a segmented scan gives each lane the updates of the
// earlier vectors; otherwise the lane counts them in those vectors itself
// (loads that its neighbours made a moment before).  The transaction's last
// lane checks its update count against its value range: the list positions are
// only as good as val_off, so a batch whose offsets disagree with its op words
// is reported (LTPG_ERR_BOUNDS) and its positions are never used past the
// list.  Called by whole warps.
__device__ __forceinline__ uint32_t vec_updates(const uint32_t *w) {
    uint32_t n = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) n += (!ycsb_is_pad(w[q]) && ycsb_is_update(w[q])) ? 1u : 0u;
    return n;
}
__device__ __forceinline__ void wf_list_updates(const YcsbTunedArgs &a, bool act, uint64_t v, uint32_t t,
                                                const uint32_t *words) {
    const uint32_t vpt = a.stride / 4u, seg = (uint32_t)(v % vpt);
    const bool pow2 = (vpt & (vpt - 1u)) == 0u;
    const uint32_t off = act ? __ldg(a.val_off + t) : 0u;
    const uint32_t end = act && seg == vpt - 1u ? __ldg(a.val_off + t + 1) : 0u;
    const uint32_t n_upd = vec_updates(words);
    uint32_t incl = n_upd;
    if (pow2) {
        for (uint32_t o = 1; o < vpt; o <<= 1) {
            const uint32_t x = __shfl_up_sync(FULL, incl, o);
            if (seg >= o) incl += x;
        }
    } else if (act) {
        const uint4 *vp = reinterpret_cast<const uint4 *>(a.ops) + (v - seg);
        for (uint32_t q = 0; q < seg; ++q) {
            const uint4 w4 = ld_nc_u4(vp + q);
            const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
            incl += vec_updates(w);
        }
    }
    if (act && seg == vpt - 1u && end - off != incl) report_error(a.ctl, DERR_BOUNDS, t);
    uint64_t u = (uint64_t)off + (incl - n_upd);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (!act || ycsb_is_pad(words[q]) || !ycsb_is_update(words[q])) continue;
        if (u < a.upd_cap) a.upd[u] = make_uint2(t, words[q]);
        else report_error(a.ctl, DERR_BOUNDS, t);
        ++u;
    }
}

// (2) reads: four op words per thread (one 16-byte load); the writer-bitmap
// words of the thread's reads are loaded together, then the slots of those
// with a writer; the RAW bit is OR-ed into the transaction's flag byte
// (zeroed by (1)) with a 32-bit atomic.
// kList: the pass also writes the update list (wf_list_updates); its stores
// wait behind the slot loads this pass is bound by.
template <bool kCoh, bool kList = false>
__device__ __forceinline__ void wf_register_reads(const YcsbTunedArgs &a, uint32_t epoch) {
    const uint64_t tag = slot_tag(epoch);
    const uint64_t nvec = (uint64_t)a.B * a.stride / 4u;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    const uint4 *vp = reinterpret_cast<const uint4 *>(a.ops);
    // a block-uniform loop, so that whole warps reach the warp-wide calls below
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nvec; base += step) {
        const uint64_t v = base + threadIdx.x;
        const bool act = v < nvec;
        const uint4 w4 = act ? ld_nc_u4(vp + v)
                             : make_uint4(LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD);
        const uint32_t t = act ? (uint32_t)(v * 4u / a.stride) : 0xFFFFFFFFu;
        const unsigned long long mine = tag | t;
        const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
        if (kList) wf_list_updates(a, act, v, t, words);
        bool rd[4];
        uint32_t bits[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t w = words[q], key = ycsb_key(w);
            rd[q] = !ycsb_is_pad(w) && !ycsb_is_update(w) && key < a.n;
            bits[q] = rd[q] ? ld_wbits<kCoh>(a.wbits + (key >> 5)) : 0u;
        }
        ulonglong2 s[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t key = ycsb_key(words[q]);
            s[q] = (bits[q] >> (key & 31u)) & 1u ? (kCoh ? ld_gpu_slot(a.reg + key) : ld_slot_ca(a.reg + key))
                                                 : make_ulonglong2(~0ull, ~0ull);
        }
        bool raw = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t w = words[q], key = ycsb_key(w);
            const uint32_t wmin = slot_min(s[q].y, epoch);
            if (wmin != 0xFFFFFFFFu && s[q].x > mine) red_min(&a.reg[key].r, mine);
            raw |= wmin < t;
            if (rd[q] && ycsb_span(w)) {  // a range scan: the keys after the first
                const uint64_t last = scan_last(w, a.n);
                for (uint64_t k2 = (uint64_t)key + 1; k2 <= last; ++k2)
                    raw |= wf_read_key<kCoh>(a, k2, t, epoch, mine);
            }
        }
        // one atomic per transaction: the lowest of its threads in the warp
        // ORs the bit when any of them saw RAW
        const unsigned peers = __match_any_sync(FULL, t);
        const bool any = (__ballot_sync(FULL, raw) & peers) != 0u;
        if (act && any && (threadIdx.x & 31u) == (uint32_t)__ffs(peers) - 1u)
            atomicOr(reinterpret_cast<unsigned *>(a.flags) + (t >> 2), LTPG_FLAG_RAW << (8u * (t & 3u)));
    }
}


template <int BS>
__global__ void __launch_bounds__(BS) ycsb_wf_writes(YcsbTunedArgs a) {
    wf_register_writes<false>(a, slot_tag(a.ctl->epoch));
}

// ---- write-first with the update list (stride / 4 a power of two <= 8) --------
template <int BS>
__global__ void __launch_bounds__(BS) ycsb_wf_reads_list(YcsbTunedArgs a) {
    wf_register_reads<false, true>(a, a.ctl->epoch);
}

// Entries of the batch's update list: val_off[B], bounded by the list.
__device__ __forceinline__ uint64_t upd_count(const YcsbTunedArgs &a) {
    const uint64_t n = __ldg(a.val_off + a.B);
    return n < a.upd_cap ? n : a.upd_cap;
}

// (3) over the update list: each update's WAR / WAW, OR-ed into its
// transaction's flag byte.  Four entries per thread and step, their entry and
// slot loads issued together.
// An entry of the update list; kCoh: written earlier in the same launch (the
// persistent kernel), so loaded coherently at L2.
template <bool kCoh>
__device__ __forceinline__ uint2 ld_upd(const uint2 *p) {
    return kCoh ? ld_gpu_u2(p) : __ldg(p);
}

template <bool kCoh>
__device__ __forceinline__ void wf_check_list(const YcsbTunedArgs &a, uint32_t epoch) {
    const uint64_t nu = upd_count(a);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u0 < nu; u0 += 4 * step) {
        uint2 e[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint64_t u = u0 + (uint64_t)q * step;
            e[q] = u < nu ? ld_upd<kCoh>(a.upd + u) : make_uint2(0xFFFFFFFFu, 0u);
        }
        bool ok[4];
        ulonglong2 sl[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            ok[q] = e[q].x < a.B && ycsb_key(e[q].y) < a.n;
            sl[q] = ok[q] ? (kCoh ? ld_gpu_slot(a.reg + ycsb_key(e[q].y)) : ld_slot(a.reg + ycsb_key(e[q].y)))
                          : make_ulonglong2(~0ull, ~0ull);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t f = 0;
            if (slot_min(sl[q].x, epoch) < e[q].x) f |= LTPG_FLAG_WAR;
            if (slot_min(sl[q].y, epoch) < e[q].x) f |= LTPG_FLAG_WAW;
            if (ok[q] && f)
                atomicOr(reinterpret_cast<unsigned *>(a.flags) + (e[q].x >> 2), f << (8u * (e[q].x & 3u)));
        }
    }
}
template <int BS>
__global__ void __launch_bounds__(BS) ycsb_wf_check_list(YcsbTunedArgs a) { wf_check_list<false>(a, a.ctl->epoch); }

// ---- check + write-back over all tiles assigned to this block ------------------
// fl: tile flags.  kLate = 0: the third pass stores the committed updates;
// 1: it reads the committed transactions' rows (late_read_tile); 2: there is
// no third pass (the reads have a kernel of their own).  With late reads the
// updates are stored by a later kernel.
template <int kLate>
__device__ __forceinline__ void checkwb_tiles(const YcsbTunedArgs &a, uint32_t *fl,
                                              uint32_t epoch) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nvec_tile = a.tile * a.stride / 4;
    const uint32_t n_tiles = (a.B + a.tile - 1) / a.tile;
    unsigned long long c_com = 0, c_raw = 0, c_war = 0, c_waw = 0;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t t0 = tile * a.tile;
        const uint32_t nt = min(a.tile, a.B - t0);
        const uint32_t nvec = nt * a.stride / 4;
        for (uint32_t i = threadIdx.x; i < a.tile; i += blockDim.x) fl[i] = 0u;
        __syncthreads();
        const uint4 *vp = reinterpret_cast<const uint4 *>(a.ops + (uint64_t)t0 * a.stride);
        // pass 1: conflict flags per transaction
        for (uint32_t base = 0; base < nvec_tile; base += blockDim.x) {
            const uint32_t v = base + threadIdx.x;
            if (v >= nvec) continue;
            const uint4 w4 = ld_nc_u4(vp + v);
            const uint32_t lt = (v * 4) / a.stride;
            const uint32_t t = t0 + lt;
            const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
            uint32_t f = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t w = words[q];
                if (ycsb_is_pad(w) || ycsb_key(w) >= a.n) continue;
                const ulonglong2 s = ld_slot(a.reg + ycsb_key(w));
                const uint32_t rmin = slot_min(s.x, epoch), wmin = slot_min(s.y, epoch);
                if (ycsb_is_update(w)) {
                    if (rmin < t) f |= LTPG_FLAG_WAR;
                    if (wmin < t) f |= LTPG_FLAG_WAW;
                } else if (wmin < t || scan_rest_raw(a.reg, a.n, w, t, epoch)) {
                    f |= LTPG_FLAG_RAW;
                }
            }
            if (f) atomicOr(&fl[lt], f);
        }
        __syncthreads();
        // pass 2: commit decision, flags, bitmap words (tile is a multiple of 32)
        for (uint32_t i = threadIdx.x; i < a.tile; i += blockDim.x) {
            uint32_t f = i < nt ? fl[i] : 0u;
            const bool com = i < nt && commits(f);
            if (com) f |= LTPG_FLAG_COMMIT;
            if (i < nt) {
                a.flags[t0 + i] = (uint8_t)f;
                fl[i] = f;
            }
            const unsigned bal = __ballot_sync(FULL, com);
            const unsigned braw = __ballot_sync(FULL, (f & LTPG_FLAG_RAW) != 0u);
            const unsigned bwar = __ballot_sync(FULL, (f & LTPG_FLAG_WAR) != 0u);
            const unsigned bwaw = __ballot_sync(FULL, (f & LTPG_FLAG_WAW) != 0u);
            if (lane == 0 && i < nt) {
                a.bitmap[(t0 + i) >> 5] = bal;
                c_com += __popc(bal);
                c_raw += __popc(braw);
                c_war += __popc(bwar);
                c_waw += __popc(bwaw);
            }
        }
        __syncthreads();
        // pass 3: committed updates, one thread per transaction in op order
        // (or, with late reads, the committed transactions' row reads)
        if (kLate == 1) {
            late_read_tile(a, fl, t0, nt);
        } else if (kLate == 0) {
            for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x)
                if (fl[i] & LTPG_FLAG_COMMIT) write_txn_updates(a, t0 + i);
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

// ---- fast execute+register: transactions of 2^m words, no block barriers -----
// Each thread takes OPS consecutive op words of one transaction (one 4-, 8- or
// 16-byte load); the lpt = stride / OPS lanes of a transaction are adjacent and
// aligned inside a warp, so the per-transaction read checksum is a segmented
// shuffle reduction and the kernel needs no shared memory outside staging.
// All row loads and slot reads of a thread's ops are issued before any of them
// is consumed, to keep many requests in flight per SM.
template <int OPS>
struct OpVec;
template <>
struct OpVec<1> {
    static __device__ __forceinline__ void load(const uint32_t *p, uint32_t *w) { w[0] = __ldg(p); }
};
template <>
struct OpVec<2> {
    static __device__ __forceinline__ void load(const uint32_t *p, uint32_t *w) {
        uint2 v;
        asm("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
        w[0] = v.x;
        w[1] = v.y;
    }
};
template <>
struct OpVec<4> {
    static __device__ __forceinline__ void load(const uint32_t *p, uint32_t *w) {
        const uint4 v = ld_nc_u4(p);
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    }
};

template <int OPS, bool kStage, bool kFilter, bool kDedupe, int BS>
__global__ void __launch_bounds__(BS) ycsb_exec_fast(YcsbTunedArgs a, uint32_t lpt) {
    extern __shared__ __align__(16) char smem[];
    StageEnt *tab = reinterpret_cast<StageEnt *>(smem);
    const uint64_t tag = slot_tag(a.ctl->epoch);
    const uint32_t lane = threadIdx.x & 31;
    if (kStage) {
        stage_init(tab, a.stage_entries);
        __syncthreads();
    }
    const uint32_t nv = a.B * lpt;  // op vectors in the batch
    const uint32_t step = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < nv; base += step) {
        const uint32_t v = base + threadIdx.x;
        const bool act = v < nv;
        uint32_t w[OPS];
        if (act) OpVec<OPS>::load(a.ops + (uint64_t)v * OPS, w);
        else
#pragma unroll
            for (int q = 0; q < OPS; ++q) w[q] = LTPG_YCSB_OP_PAD;
        const uint32_t t = v / lpt;
        const uint32_t j0 = (v % lpt) * OPS;
        bool rd[OPS], need[OPS];
        uint32_t key[OPS];
#pragma unroll
        for (int q = 0; q < OPS; ++q) {
            bool valid = act && !ycsb_is_pad(w[q]);
            key[q] = ycsb_key(w[q]);
            if (valid && key[q] >= a.n) {
                report_error(a.ctl, DERR_BOUNDS, t);
                valid = false;
            }
            rd[q] = valid && !ycsb_is_update(w[q]);
            need[q] = valid;
            if (kStage && valid) {
                const uint32_t b = key_bucket(key[q]);
                const uint32_t g = __ldg(a.stage_map + b);
                if (g != STAGE_NONE && (g + 1) * a.ways <= a.stage_entries) {
                    StageEnt *e = stage_find(tab, g, a.ways, key[q]);
                    if (e) {
                        atomicMin(ycsb_is_update(w[q]) ? &e->wmin : &e->rmin, t);
                        atomicAdd(&e->cnt, 1u);
                        need[q] = false;
                    }
                }
                if (need[q] && (t % COUNT_SAMPLE) == 0u) atomicAdd(a.bucket_counts + b, COUNT_SAMPLE);
            }
        }
        // issue every load of this thread's ops
        ulonglong2 r[OPS][5];
        uint64_t cur[OPS];
#pragma unroll
        for (int q = 0; q < OPS; ++q) {
            const char *p = reinterpret_cast<const char *>(a.rows + (uint64_t)key[q] * LTPG_YCSB_FIELDS);
#pragma unroll
            for (int i = 0; i < 5; ++i) r[q][i] = rd[q] ? ld_nc16_issue(p + 16 * i) : make_ulonglong2(0ull, 0ull);
            unsigned long long *slot = ycsb_is_update(w[q]) ? &a.reg[key[q]].w : &a.reg[key[q]].r;
            cur[q] = (kFilter && need[q]) ? ld_ca_u64(slot) : ~0ull;
        }
        // registration: optionally one atomic per distinct (key, kind) of the
        // warp, optionally skipped when the slot already holds a smaller value
#pragma unroll
        for (int q = 0; q < OPS; ++q) {
            bool leader = need[q];
            if (kDedupe) {
                const uint32_t mkey = need[q] ? (key[q] | (ycsb_is_update(w[q]) ? 0x80000000u : 0u)) : 0xFFFFFFFFu;
                const unsigned peers = __match_any_sync(FULL, mkey);
                // lanes are in transaction order, so the lowest peer holds the smallest TID
                leader = need[q] && (__ffs(peers) - 1) == (int)lane;
            }
            const unsigned long long mine = tag | t;
            if (leader && cur[q] > mine)
                red_min(ycsb_is_update(w[q]) ? &a.reg[key[q]].w : &a.reg[key[q]].r, mine);
        }
        unsigned long long part = 0;
#pragma unroll
        for (int q = 0; q < OPS; ++q) {
            unsigned long long x = r[q][0].x ^ r[q][0].y ^ r[q][1].x ^ r[q][1].y ^ r[q][2].x ^ r[q][2].y ^
                                   r[q][3].x ^ r[q][3].y ^ r[q][4].x ^ r[q][4].y;
            if (rd[q]) x ^= scan_rest(a.reg, a.rows, a.n, w[q], tag | t, kFilter);
            part += rd[q] ? x * (2ull * (j0 + q) + 1ull) : 0ull;
        }
        for (uint32_t o = lpt >> 1; o >= 1; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
        if (act && (v % lpt) == 0u) a.results[t] = (int64_t)part;
    }
    if (kStage) {
        __syncthreads();
        const uint32_t ops = stage_flush(tab, a.stage_entries, a.reg, tag, a.bucket_counts);
        if (ops) red_add_u64(&a.st->staged_ops, ops);
    }
}

// ---- cooperative execute+register: one op per lane, rows read by 5 lanes ----
// A warp takes whole transactions, lpt lanes each (the stride rounded up to a
// power of two <= 32; lanes past the stride hold padding ops).  Each lane
// registers its own op; then the rows of the
// warp's reads are fetched six at a time, five lanes per row, each lane one
// contiguous 16-byte chunk, so a row costs one or two cache-line requests
// instead of five.  The five chunks are xor-folded within their lane group and
// handed back to the lane that owns the op.
// kReads = false (late reads): registration only; the rows are read after the
// check, by the committed transactions alone (late_read_tile).
template <bool kStage, bool kFilter, bool kDedupe, bool kReads>
__device__ __forceinline__ void coop_exec_loop(const YcsbTunedArgs &a, StageEnt *tab, const uint32_t *sbits,
                                               const uint32_t *srank, uint64_t tag) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lanes_below = (1u << lane) - 1u;
    const uint32_t lpt = a.lpt;  // lanes per transaction, a power of two
    const uint32_t lsh = (uint32_t)__ffs(lpt) - 1u;
    const uint32_t groups = a.ways ? a.stage_entries / a.ways : 0u;
    const uint64_t nw = (uint64_t)a.B << lsh;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t grp = lane / 5, chunk = lane % 5;  // row-read lane groups (6 x 5 lanes)
    bool scans = false;  // some read of this thread's was a range scan
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nw; base += step) {
        const uint64_t v = base + threadIdx.x;
        const bool act = v < nw;
        const uint32_t t = (uint32_t)(v >> lsh);
        const uint32_t j = (uint32_t)v & (lpt - 1u);
        const uint32_t w = act && j < a.stride ? __ldg(a.ops + (uint64_t)t * a.stride + j) : LTPG_YCSB_OP_PAD;
        bool valid = act && !ycsb_is_pad(w);
        const uint32_t key = ycsb_key(w);
        if (valid && key >= a.n) {
            report_error(a.ctl, DERR_BOUNDS, t);
            valid = false;
        }
        const bool upd = ycsb_is_update(w);
        const bool rd = valid && !upd;
        StageEnt *e = nullptr;
        bool have_dig = false;
        unsigned long long x = 0;
        if (kStage && valid) {
            const uint32_t b = key_bucket(key);
            const uint32_t g = stage_group(sbits, srank, b);
            if (g < groups) e = stage_find(tab, g, a.ways, key);
            if (!e && (t % COUNT_SAMPLE) == 0u) atomicAdd(a.bucket_counts + b, COUNT_SAMPLE);
            if (kReads && e && rd && *reinterpret_cast<volatile uint32_t *>(&e->dig_ok)) {
                __threadfence_block();
                x = *reinterpret_cast<volatile unsigned long long *>(&e->dig);
                have_dig = true;
            }
        }
        // one row read per distinct key of the warp: peers share the leader's
        unsigned peers = 1u << lane;
        if (kDedupe || kStage) peers = __match_any_sync(FULL, valid ? (key | (upd ? 0x80000000u : 0u)) : 0xFFFFFFFFu);
        const uint32_t leader_lane = (uint32_t)__ffs(peers) - 1u;
        const bool leader = valid && leader_lane == lane;
        // rows still to read, compacted: round r reads the (6r + g)-th of them
        const unsigned need = kReads ? __ballot_sync(FULL, rd && !have_dig && leader) : 0u;
        const uint32_t n_need = __popc(need);
        ulonglong2 ch[6];
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const uint32_t idx = (uint32_t)r * 6u + grp;
            const bool go = kReads && grp < 6 && idx < n_need;
            const uint32_t src = go ? __fns(need, 0, (int)idx + 1) : 0u;
            const uint32_t k_src = __shfl_sync(FULL, key, src & 31u);
            ch[r] = go ? ld_nc16_issue(reinterpret_cast<const char *>(a.rows + (uint64_t)k_src * LTPG_YCSB_FIELDS) +
                                       16u * chunk)
                       : make_ulonglong2(0ull, 0ull);
        }
        // registration: staged rows in shared memory, the rest through the
        // warp dedupe and the slot filter
        const bool need_global = valid && !e;
        uint64_t cur = ~0ull;
        unsigned long long *slot = upd ? &a.reg[key].w : &a.reg[key].r;
        if (kFilter && need_global) cur = ld_ca_u64(slot);
        if (kStage && e && leader) {
            atomicMin(upd ? &e->wmin : &e->rmin, t);
            atomicAdd(&e->cnt, (uint32_t)__popc(peers));
        }
        const unsigned long long mine = tag | t;
        if (need_global && (kDedupe ? leader : true) && cur > mine) red_min_exec(slot, mine);
        scans |= rd && ycsb_span(w) != 0u;
        if (!kReads) continue;
        // fold the five chunks of each row onto its group's first lane (5g),
        // then hand the row's xor to the lane that owns the op
        const uint32_t my_rank = __popc(need & lanes_below);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            if ((uint32_t)r * 6u >= n_need) break;  // warp-uniform
            const unsigned long long c0 = ch[r].x ^ ch[r].y;
            unsigned long long c = c0 ^ __shfl_down_sync(FULL, c0, 1);  // lane 5g: chunks 0,1
            c ^= __shfl_down_sync(FULL, c, 2);                          // lane 5g: chunks 0..3
            const unsigned long long rowx = c ^ __shfl_down_sync(FULL, c0, 4);  // + chunk 4
            const uint32_t op0 = (uint32_t)r * 6u;
            const unsigned long long got = __shfl_sync(FULL, rowx, ((my_rank - op0) * 5u) & 31u);
            if (((need >> lane) & 1u) && my_rank >= op0 && my_rank < op0 + 6u) x = got;
        }
        {
            const unsigned long long from_leader = __shfl_sync(FULL, x, leader_lane);
            if (!have_dig) x = from_leader;
        }
        if (kStage && e && rd && !have_dig && leader) {  // publish the checksum for later reads in this block
            e->dig = x;
            __threadfence_block();
            *reinterpret_cast<volatile uint32_t *>(&e->dig_ok) = 1u;
        }
        unsigned long long part = rd ? x * (2ull * j + 1ull) : 0ull;
        for (uint32_t o = lpt >> 1; o >= 1; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
        if (act && j == 0u) a.results[t] = (int64_t)part;
    }
    // Range scans: the keys after each scan's first, in a second pass over the
    // block's ops (kept out of the loop above, whose code is the point-read
    // path: with the scan code inside, that loop ran 6 % slower on point-read
    // batches).  The same thread leads a transaction in both passes, so its
    // result is completed in program order.
    if (__syncthreads_or(scans)) {
        for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nw; base += step) {
            const uint64_t v = base + threadIdx.x;
            const bool act = v < nw;
            const uint32_t t = (uint32_t)(v >> lsh);
            const uint32_t j = (uint32_t)v & (lpt - 1u);
            const uint32_t w = act && j < a.stride ? __ldg(a.ops + (uint64_t)t * a.stride + j) : LTPG_YCSB_OP_PAD;
            const bool rd = act && !ycsb_is_pad(w) && ycsb_key(w) < a.n && ycsb_span(w) != 0u;
            const uint32_t key = ycsb_key(w);
            const uint32_t last = rd ? (uint32_t)scan_last(w, a.n) : 0u;
            // the warp takes its scans one at a time: all lanes read the
            // scan's rows as one contiguous range (16 B chunks, coalesced) and
            // register its keys after the first, one key per lane
            unsigned long long xf = 0, xa = 0;  // this lane's scan: first row, all rows
            for (unsigned m = __ballot_sync(FULL, rd); m; m &= m - 1u) {
                const uint32_t src = (uint32_t)__ffs(m) - 1u;
                const uint32_t k0 = __shfl_sync(FULL, key, src), k1 = __shfl_sync(FULL, last, src);
                const uint32_t ts = __shfl_sync(FULL, t, src);
                const uint32_t chunks = kReads ? (k1 - k0 + 1u) * 5u : 0u;
                const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(a.rows + (uint64_t)k0 * LTPG_YCSB_FIELDS);
                unsigned long long c_all = 0, c_first = 0;
                for (uint32_t c = lane; c < chunks; c += 32u) {
                    const ulonglong2 q = ld_nc16(p + c);
                    c_all ^= q.x ^ q.y;
                    if (c < 5u) c_first ^= q.x ^ q.y;
                }
                if (lane < k1 - k0) {
                    unsigned long long *slot = &a.reg[(uint64_t)k0 + 1u + lane].r;
                    const unsigned long long mine = tag | ts;
                    if (!kFilter || ld_ca_u64(slot) > mine) red_min(slot, mine);
                }
                if (!kReads) continue;
                for (uint32_t o = 16; o >= 1u; o >>= 1) {
                    c_all ^= __shfl_xor_sync(FULL, c_all, o);
                    c_first ^= __shfl_xor_sync(FULL, c_first, o);
                }
                if (lane == src) {
                    xa = c_all;
                    xf = c_first;
                }
            }
            if (!kReads) continue;
            // the first pass added x_first * (2j + 1); the read's term is
            // x_all * (2j + 1): add the difference (mod 2^64)
            unsigned long long part = rd ? (xa - xf) * (2ull * j + 1ull) : 0ull;
            for (uint32_t o = lpt >> 1; o >= 1; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
            if (act && j == 0u && part) a.results[t] = (int64_t)((unsigned long long)a.results[t] + part);
        }
    }
}

template <bool kStage, bool kFilter, bool kDedupe, bool kReads, int BS>
__global__ void __launch_bounds__(BS) ycsb_exec_coop(YcsbTunedArgs a) {
    extern __shared__ __align__(16) char smem[];
    uint32_t *sbits = reinterpret_cast<uint32_t *>(smem);
    uint32_t *srank = sbits + STAGE_WORDS;
    StageEnt *tab = reinterpret_cast<StageEnt *>(srank + STAGE_WORDS);
    const uint64_t tag = slot_tag(a.ctl->epoch);
    if (kStage) {
        for (uint32_t i = threadIdx.x; i < STAGE_WORDS; i += blockDim.x) {
            sbits[i] = __ldg(a.stage_bits + i);
            srank[i] = __ldg(a.stage_rank + i);
        }
        stage_init(tab, a.stage_entries);
        __syncthreads();
    }
    coop_exec_loop<kStage, kFilter, kDedupe, kReads>(a, tab, sbits, srank, tag);
    if (kStage) {
        __syncthreads();
        const uint32_t ops = stage_flush(tab, a.stage_entries, a.reg, tag, a.bucket_counts);
        if (ops) red_add_u64(&a.st->staged_ops, ops);
    }
}

// Shared memory layout: [dig: tile u64][fl: tile u32][stage table]
__host__ __device__ __forceinline__ size_t ycsb_smem_bytes(uint32_t tile, uint32_t threads, uint32_t stage_entries) {
    (void)threads;
    const size_t a = ((size_t)tile * 8 + 15) / 16 * 16;
    const size_t b = ((size_t)tile * 4 + 15) / 16 * 16;
    return a + b + (size_t)stage_entries * sizeof(StageEnt);
}

struct SmemPtrs {
    unsigned long long *dig;
    uint32_t *fl;
    StageEnt *tab;
};
__device__ __forceinline__ SmemPtrs carve(char *base, uint32_t tile) {
    SmemPtrs p;
    const size_t a = ((size_t)tile * 8 + 15) / 16 * 16;
    const size_t b = ((size_t)tile * 4 + 15) / 16 * 16;
    p.dig = reinterpret_cast<unsigned long long *>(base);
    p.fl = reinterpret_cast<uint32_t *>(base + a);
    p.tab = reinterpret_cast<StageEnt *>(base + a + b);
    return p;
}

template <bool kStage>
__global__ void __launch_bounds__(512) ycsb_exec_tuned(YcsbTunedArgs a) {
    extern __shared__ __align__(16) char smem[];
    const SmemPtrs p = carve(smem, a.tile);
    const uint64_t tag = slot_tag(a.ctl->epoch);
    if (kStage) {
        stage_init(p.tab, a.stage_entries);
        __syncthreads();
    }
    exec_tiles<kStage>(a, p.dig, p.tab, tag);
    if (kStage) {
        __syncthreads();
        const uint32_t ops = stage_flush(p.tab, a.stage_entries, a.reg, tag, a.bucket_counts);
        if (ops) red_add_u64(&a.st->staged_ops, ops);
    }
}

template <int kLate>
__global__ void __launch_bounds__(512) ycsb_checkwb_tuned(YcsbTunedArgs a) {
    extern __shared__ __align__(16) char smem[];
    const SmemPtrs p = carve(smem, a.tile);
    checkwb_tiles<kLate>(a, p.fl, a.ctl->epoch);
    if (!kLate) finish_batch(a.ctl);
}

// Write-back after late reads: one thread per transaction; a committed one
// stores its updates.  kDecide (write-first registration): the flags hold the
// conflict bits only, and this pass makes the commit decision and writes the
// final flags, the bitmap (a warp's ballot over 32 consecutive transactions is
// one bitmap word) and the counters.  kStore = false: the decision only (the
// update-list write-back stores from the list).
template <bool kDecide, bool kCoh, bool kStore = true>
__device__ __forceinline__ void writeback_late_loop(const YcsbTunedArgs &a) {
    const uint32_t step = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long c_com = 0, c_raw = 0, c_war = 0, c_waw = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < a.B; base += step) {
        const uint32_t t = base + threadIdx.x;
        const bool act = t < a.B;
        const uint32_t f = act ? ld_flag<kCoh>(a.flags + t) : 0u;
        bool com;
        if (kDecide) {
            com = act && commits(f);
            if (act) a.flags[t] = (uint8_t)(f | (com ? LTPG_FLAG_COMMIT : 0u));
            const unsigned bc = __ballot_sync(FULL, com);
            const unsigned br = __ballot_sync(FULL, (f & LTPG_FLAG_RAW) != 0u);
            const unsigned bwr = __ballot_sync(FULL, (f & LTPG_FLAG_WAR) != 0u);
            const unsigned bww = __ballot_sync(FULL, (f & LTPG_FLAG_WAW) != 0u);
            if (lane == 0u && act) {
                a.bitmap[t >> 5] = bc;
                c_com += __popc(bc);
                c_raw += __popc(br);
                c_war += __popc(bwr);
                c_waw += __popc(bww);
            }
        } else {
            com = (f & LTPG_FLAG_COMMIT) != 0u;
        }
        if (kStore && com) write_txn_updates(a, t);
    }
    if (kDecide && lane == 0u) {
        if (c_com) {
            red_add_u64(&a.st->commits, c_com);
            red_add_u64(&a.ctl->total_commits, c_com);
        }
        if (c_raw) red_add_u64(&a.st->raw, c_raw);
        if (c_war) red_add_u64(&a.st->war, c_war);
        if (c_waw) red_add_u64(&a.st->waw, c_waw);
    }
}

// Late reads 2: the check kernel made the decisions; this one stores.
template <int BS>
__global__ void __launch_bounds__(BS) ycsb_writeback_late(YcsbTunedArgs a) {
    writeback_late_loop<false, false>(a);
    finish_batch(a.ctl);
}

// Write-back over the update list: the decision per transaction (flags,
// bitmap, counters: writeback_late_loop with no stores), then one update per
// thread.  An update of a committing transaction stores its value unless a
// later op of the same transaction writes the same field: op order decides, as
// in a sequential replay (the transaction's entries are consecutive).  The
// decision is a function of the conflict bits, which nothing changes here, so
// an update that reads its transaction's flag byte before or after the first
// loop adds COMMIT to it decides the same.
template <bool kCoh>
__device__ __forceinline__ void writeback_list(const YcsbTunedArgs &a) {
    writeback_late_loop<true, kCoh, false>(a);
    // a batch whose registration reported an error (a key past the table, or
    // offsets that disagree with the op words, which leave list positions
    // unwritten) stores nothing
    const uint64_t nu = ld_gpu_u32(&a.ctl->error) ? 0ull : upd_count(a);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += step) {
        const uint2 e = ld_upd<kCoh>(a.upd + u);
        const uint32_t key = ycsb_key(e.y), fld = ycsb_field(e.y);
        if (e.x >= a.B || key >= a.n || fld >= LTPG_YCSB_FIELDS) continue;
        if (!commits(ld_gpu_u8(a.flags + e.x) & (LTPG_FLAG_RAW | LTPG_FLAG_WAR | LTPG_FLAG_WAW))) continue;
        bool last = true;
        for (uint64_t u2 = u + 1; u2 < nu; ++u2) {
            const uint2 e2 = ld_upd<kCoh>(a.upd + u2);
            if (e2.x != e.x) break;
            if (ycsb_key(e2.y) == key && ycsb_field(e2.y) == fld) last = false;
        }
        if (last && u < a.vals_cap) a.rows[(uint64_t)key * LTPG_YCSB_FIELDS + fld] = __ldg(a.vals + u);
    }
}
template <int BS>
__global__ void __launch_bounds__(BS) ycsb_writeback_list(YcsbTunedArgs a) {
    writeback_list<false>(a);
    finish_batch(a.ctl);
}

// One cooperative kernel per batch: execute+register, grid barrier, check +
// write-back.  The barrier wait is bounded (grid_barrier); once a wait has
// run out, a block runs no further phase and calls no further barrier.
// With late reads (kLate, which needs a.lpt != 0): execute registers only,
// then check + reads, a second grid barrier, and the write-back.  Phases
// after the first load what earlier phases wrote with coherent loads
// (kCoh = true above; checkwb_tiles reads slots with ld.global.cg, at L2).
template <bool kStage, bool kLate>
__device__ __forceinline__ void ycsb_persistent_body(const YcsbTunedArgs &a) {
    extern __shared__ __align__(16) char smem[];
    const SmemPtrs p = carve(smem, a.tile);
    const uint32_t epoch = a.ctl->epoch;
    const uint64_t tag = slot_tag(epoch);
    if (kLate && !kStage && a.late == 3u) {  // write-first: five phases, four grid barriers
        wf_register_writes<true>(a, tag);
        bool ok = grid_barrier(a.ctl);
        if (ok) wf_register_reads<true, true>(a, epoch);
        ok = ok && grid_barrier(a.ctl);
        if (ok) wf_check_list<true>(a, epoch);
        ok = ok && grid_barrier(a.ctl);
        if (ok) late_read_loop<true>(a);
        ok = ok && grid_barrier(a.ctl);
        if (ok) writeback_list<true>(a);
        finish_batch(a.ctl);
        return;
    }
    if (kStage) {
        stage_init(p.tab, a.stage_entries);
        __syncthreads();
    }
    if (a.lpt) {
        if (a.filter) coop_exec_loop<kStage, true, true, !kLate>(a, p.tab, a.stage_bits, a.stage_rank, tag);
        else coop_exec_loop<kStage, false, true, !kLate>(a, p.tab, a.stage_bits, a.stage_rank, tag);
    } else if (!kLate) {
        exec_tiles<kStage>(a, p.dig, p.tab, tag);
    }
    if (kStage) {
        __syncthreads();
        const uint32_t ops = stage_flush(p.tab, a.stage_entries, a.reg, tag, a.bucket_counts);
        if (ops) red_add_u64(&a.st->staged_ops, ops);
    }
    bool ok = grid_barrier(a.ctl);
    if (ok) {
        if (!kLate) checkwb_tiles<0>(a, p.fl, epoch);
        else if (a.late == 2u) checkwb_tiles<2>(a, p.fl, epoch);
        else checkwb_tiles<1>(a, p.fl, epoch);
    }
    if (kLate) {
        if (a.late == 2u) {
            ok = ok && grid_barrier(a.ctl);
            if (ok) late_read_loop<true>(a);
        }
        ok = ok && grid_barrier(a.ctl);
        if (ok) writeback_late_loop<false, true>(a);
    }
    finish_batch(a.ctl);
}
template <bool kStage, bool kLate>
__global__ void __launch_bounds__(512) ycsb_persistent(YcsbTunedArgs a) { ycsb_persistent_body<kStage, kLate>(a); }
// Late reads on blocks of at most 256 threads with registers budgeted for six
// resident blocks per SM (40, with a few spills, against 59 and four): the row
// gathers of the late-read phase want the warps more than the other phases
// want the registers.
__global__ void __launch_bounds__(256, 6) ycsb_persistent_late_x6(YcsbTunedArgs a) {
    ycsb_persistent_body<false, true>(a);
}

// Static shared memory of a kernel, queried once per kernel.
static size_t static_smem(const void *k) {
    static std::mutex mu;
    static std::unordered_map<const void *, size_t> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(k);
    if (it != cache.end()) return it->second;
    cudaFuncAttributes fa{};
    const size_t v = cudaFuncGetAttributes(&fa, k) == cudaSuccess ? fa.sharedSizeBytes : 48 * 1024;
    cache.emplace(k, v);
    return v;
}

// Calls f with std::integral_constant<int, BS> for the launch's block size
// (128, 256 or 512; ltpg_set_launch admits no other).
template <class F>
static auto with_block(uint32_t block, F f) {
    switch (block) {
    case 128: return f(std::integral_constant<int, 128>());
    case 512: return f(std::integral_constant<int, 512>());
    default: return f(std::integral_constant<int, 256>());
    }
}

// Transactions per tile: as many whole transactions as the block reads with
// `per_thread` 16-byte vectors per thread, rounded down to a multiple of 32.
static uint32_t tuned_tile(uint32_t stride, uint32_t threads, uint32_t per_thread) {
    uint32_t t = threads * 4u * per_thread / stride;
    t = t / 32u * 32u;
    return t < 32u ? 32u : t;
}

// Launches the barrier-free execute kernel when stride / ops-per-thread is a
// power of two <= 32; returns false (nothing launched) otherwise.
template <int OPS, int BS>
static void launch_fast_t(ltpg_ctx *c, const YcsbTunedArgs &a, bool stage, uint32_t lpt) {
    const LaunchCfg &L = c->launch_y;
    const size_t smem = stage ? (size_t)a.stage_entries * sizeof(StageEnt) : 0;
    void (*k)(YcsbTunedArgs, uint32_t);
    const int sel = (stage ? 4 : 0) | (L.filter ? 2 : 0) | (L.dedupe ? 1 : 0);
    switch (sel) {
    case 0: k = ycsb_exec_fast<OPS, false, false, false, BS>; break;
    case 1: k = ycsb_exec_fast<OPS, false, false, true, BS>; break;
    case 2: k = ycsb_exec_fast<OPS, false, true, false, BS>; break;
    case 3: k = ycsb_exec_fast<OPS, false, true, true, BS>; break;
    case 4: k = ycsb_exec_fast<OPS, true, false, false, BS>; break;
    case 5: k = ycsb_exec_fast<OPS, true, false, true, BS>; break;
    case 6: k = ycsb_exec_fast<OPS, true, true, false, BS>; break;
    default: k = ycsb_exec_fast<OPS, true, true, true, BS>; break;
    }
    if (smem + static_smem((const void *)k) > 48 * 1024)
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint32_t threads = BS;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, (int)threads, smem);
    if (per_sm < 1) per_sm = 1;
    if (L.blocks_per_sm && (int)L.blocks_per_sm < per_sm) per_sm = (int)L.blocks_per_sm;
    const uint64_t nv = (uint64_t)a.B * lpt;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nv + threads - 1) / threads, (uint64_t)per_sm * c->sm_count);
    k<<<grid, threads, smem, c->stream>>>(a, lpt);
}

template <bool kReads, int BS>
static void (*coop_kernel(int sel))(YcsbTunedArgs) {
    switch (sel) {
    case 0: return ycsb_exec_coop<false, false, false, kReads, BS>;
    case 1: return ycsb_exec_coop<false, false, true, kReads, BS>;
    case 2: return ycsb_exec_coop<false, true, false, kReads, BS>;
    case 3: return ycsb_exec_coop<false, true, true, kReads, BS>;
    case 4: return ycsb_exec_coop<true, false, false, kReads, BS>;
    case 5: return ycsb_exec_coop<true, false, true, kReads, BS>;
    case 6: return ycsb_exec_coop<true, true, false, kReads, BS>;
    default: return ycsb_exec_coop<true, true, true, kReads, BS>;
    }
}

// reads = false: registration only (late reads)
static void launch_coop(ltpg_ctx *c, const YcsbTunedArgs &a, bool stage, bool reads) {
    const LaunchCfg &L = c->launch_y;
    const size_t smem = stage ? 2 * STAGE_WORDS * sizeof(uint32_t) + (size_t)a.stage_entries * sizeof(StageEnt) : 0;
    const int sel = (stage ? 4 : 0) | (L.filter ? 2 : 0) | (L.dedupe ? 1 : 0);
    void (*k)(YcsbTunedArgs) = with_block(L.block, [&](auto bs) {
        constexpr int BS = decltype(bs)::value;
        return reads ? coop_kernel<true, BS>(sel) : coop_kernel<false, BS>(sel);
    });
    if (smem + static_smem((const void *)k) > 48 * 1024)
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint32_t threads = L.block;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, (int)threads, smem);
    if (per_sm < 1) per_sm = 1;
    if (L.blocks_per_sm && (int)L.blocks_per_sm < per_sm) per_sm = (int)L.blocks_per_sm;
    const uint64_t nw = (uint64_t)a.B * a.lpt;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nw + threads - 1) / threads, (uint64_t)per_sm * c->sm_count);
    k<<<grid, threads, smem, c->stream>>>(a);
}

// Grid of a grid-stride kernel of block_threads threads over `items` lanes:
// at most the blocks that fit on the GPU at once (blocks_per_sm caps them
// when set).
static uint32_t stride_grid(ltpg_ctx *c, const void *k, uint64_t items) {
    const uint32_t threads = c->launch_y.block;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, (int)threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    if (c->launch_y.blocks_per_sm && (int)c->launch_y.blocks_per_sm < per_sm) per_sm = (int)c->launch_y.blocks_per_sm;
    const uint64_t g = std::min<uint64_t>((items + threads - 1) / threads, (uint64_t)per_sm * c->sm_count);
    return (uint32_t)std::max<uint64_t>(g, 1);
}

// Write-first registration (late_reads = 3): write registration, read
// registration + RAW, WAR / WAW, committed reads, commit decision +
// write-back.  Profiled as [registration (both), check, reads, write-back].
// The read registration also lists the updates (the list is allocated with
// the slots' batch arrays, so it exists for every YCSB batch), and the check
// and the write-back walk that list.
template <int BS>
static cudaError_t launch_write_first_t(ltpg_ctx *c, const YcsbTunedArgs &a) {
    const uint64_t lanes = (uint64_t)a.B * a.lpt, nvec = (uint64_t)a.B * a.stride / 4;
    prof_mark(c, 0);
    count_launch(c, 2);
    ycsb_wf_writes<BS><<<stride_grid(c, (const void *)ycsb_wf_writes<BS>, nvec), BS, 0, c->stream>>>(a);
    ycsb_wf_reads_list<BS><<<stride_grid(c, (const void *)ycsb_wf_reads_list<BS>, nvec), BS, 0, c->stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    prof_mark(c, 1);
    count_launch(c, 2);
    ycsb_wf_check_list<BS><<<stride_grid(c, (const void *)ycsb_wf_check_list<BS>, nvec), BS, 0, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 2);
    ycsb_read_late<BS><<<stride_grid(c, (const void *)ycsb_read_late<BS>, lanes), BS, 0, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 3);
    count_launch(c);
    ycsb_writeback_list<BS><<<stride_grid(c, (const void *)ycsb_writeback_list<BS>, std::max<uint64_t>(a.B, nvec)),
                              BS, 0, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 4);
    return predictor_after_batch(c);
}

static cudaError_t launch_write_first(ltpg_ctx *c, const YcsbTunedArgs &a) {
    return with_block(c->launch_y.block, [&](auto bs) { return launch_write_first_t<decltype(bs)::value>(c, a); });
}

// Launch shapes of the execute phase, by ops_per_thread: 1 = cooperative row
// reads (ycsb_exec_coop, any stride <= 32), 2 / 4 = per-thread row reads
// (ycsb_exec_fast, stride / ops a power of two); 8 = block tiles
// (ycsb_exec_tuned), which serve every stride.
static bool launch_fast_exec(ltpg_ctx *c, const YcsbTunedArgs &a, bool stage) {
    const uint32_t opt = c->launch_y.per_thread ? c->launch_y.per_thread : 4u;
    if (opt >= 8) return false;
    if (opt == 1 && a.lpt) {
        launch_coop(c, a, stage, true);
        return true;
    }
    const uint32_t ops = std::max<uint32_t>(2u, std::min<uint32_t>(opt, 4u));
    if (a.stride % ops) return false;
    const uint32_t lpt = a.stride / ops;
    if (lpt == 0 || lpt > 32 || (lpt & (lpt - 1))) return false;
    with_block(c->launch_y.block, [&](auto bs) {
        constexpr int BS = decltype(bs)::value;
        if (ops == 2) launch_fast_t<2, BS>(c, a, stage, lpt);
        else launch_fast_t<4, BS>(c, a, stage, lpt);
        return 0;
    });
    return true;
}

cudaError_t ycsb_run_tuned(ltpg_ctx *c, Slot &s, int mode) {
    if (s.n_txn == 0) return cudaSuccess;
    const LaunchCfg &L = c->launch_y;
    const uint32_t threads = L.block;
    const uint32_t per_thread = std::max<uint32_t>(1u, (L.per_thread ? L.per_thread : 4u) / 4u);
    YcsbTunedArgs a;
    a.ops = s.ops;
    a.val_off = s.val_off;
    a.vals = s.vals;
    a.B = s.n_txn;
    a.k = s.k;
    a.stride = s.stride;
    a.lpt = 0;
    if (s.stride <= 32) {
        a.lpt = 1;
        while (a.lpt < s.stride) a.lpt <<= 1;
    }
    a.tile = tuned_tile(s.stride, threads, per_thread);
    a.rows = c->ycsb.rows;
    a.n = c->ycsb.n;
    a.reg = c->ycsb.reg;
    a.results = s.results;
    a.flags = s.flags;
    a.bitmap = s.bitmap;
    a.st = s.stats;
    a.ctl = c->ctl;
    const bool stage = (c->stage_on || c->pred_on) && c->stage_map && c->bucket_counts;
    a.stage_map = c->stage_map;
    a.stage_bits = c->stage_bits;
    a.stage_rank = c->stage_rank;
    a.bucket_counts = c->bucket_counts;
    a.ways = L.ways ? L.ways : 4u;
    // with the predictor counting but staging off, the staging table is empty
    a.stage_entries = (stage && c->stage_on) ? STAGE_MAX_ENTRIES / a.ways * a.ways : 0u;
    // late reads need the one-op-per-lane layout (stride <= 32); write-first
    // registration has no staging path (with staging it reads late in a
    // kernel of their own)
    uint32_t late_mode = a.lpt ? L.late_reads : 0u;
    if (late_mode == 3u && stage) late_mode = 2u;
    const bool late = late_mode != 0u;
    a.filter = L.filter;
    a.late = late_mode;
    a.wbits = c->ycsb.wbits;
    a.upd = c->ycsb.upd;
    a.upd_cap = c->ycsb.upd_cap;
    a.vals_cap = s.cap_vals;
    const size_t smem = ycsb_smem_bytes(a.tile, threads, a.stage_entries);
    const size_t smem_cwb = ycsb_smem_bytes(a.tile, threads, 0);  // check + write-back needs no staging table
    cudaError_t e = cudaMemsetAsync(s.stats, 0, sizeof(DevStats), c->stream);
    if (e != cudaSuccess) return e;
    // write-first: the writer bitmap starts empty for every batch
    if (late_mode == 3u &&
        (e = cudaMemsetAsync(a.wbits, 0, (a.n + 31) / 32 * sizeof(uint32_t), c->stream)) != cudaSuccess)
        return e;
    auto exec_k = stage ? ycsb_exec_tuned<true> : ycsb_exec_tuned<false>;
    auto pers_k = stage ? (late ? ycsb_persistent<true, true> : ycsb_persistent<true, false>)
                        : (late ? (threads <= 256 ? ycsb_persistent_late_x6 : ycsb_persistent<false, true>)
                                : ycsb_persistent<false, false>);
    auto cwb_k = !late ? ycsb_checkwb_tuned<0> : late_mode == 1u ? ycsb_checkwb_tuned<1> : ycsb_checkwb_tuned<2>;
    // above 48 KB of static + dynamic shared memory a kernel must opt in
    for (const void *k : {(const void *)exec_k, (const void *)cwb_k, (const void *)pers_k})
        if (smem + static_smem(k) > 48 * 1024)
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mode == LTPG_MODE_PERSISTENT ? pers_k : exec_k,
                                                      (int)threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (L.blocks_per_sm && (int)L.blocks_per_sm < per_sm) per_sm = (int)L.blocks_per_sm;
    const uint32_t n_tiles = (a.B + a.tile - 1) / a.tile;
    const uint32_t grid = std::min<uint32_t>(n_tiles, (uint32_t)(per_sm * c->sm_count));
    if (mode == LTPG_MODE_PERSISTENT) {
        prof_mark(c, 0);
        void *args[] = {&a};
        count_launch(c);
        e = cudaLaunchCooperativeKernel((const void *)pers_k, dim3(grid), dim3(threads), args, smem, c->stream);
        if (e != cudaSuccess) return e;
        for (int m = 1; m < PROF_MARKS; ++m) prof_mark(c, m);
        return predictor_after_batch(c);
    }
    if (late_mode == 3u) return launch_write_first(c, a);
    prof_mark(c, 0);
    count_launch(c);
    if (late) launch_coop(c, a, stage, false);
    else if (!launch_fast_exec(c, a, stage)) exec_k<<<grid, threads, smem, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 1);
    count_launch(c);
    int per_sm_cwb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_cwb, cwb_k, (int)threads, smem_cwb);
    if (e != cudaSuccess) return e;
    if (per_sm_cwb < 1) per_sm_cwb = 1;
    const uint32_t grid_cwb = std::min<uint32_t>(n_tiles, (uint32_t)(per_sm_cwb * c->sm_count));
    cwb_k<<<grid_cwb, threads, smem_cwb, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 2);
    if (late_mode == 2u) {
        count_launch(c);
        with_block(threads, [&](auto bs) {
            constexpr int BS = decltype(bs)::value;
            ycsb_read_late<BS><<<stride_grid(c, (const void *)ycsb_read_late<BS>, (uint64_t)a.B * a.lpt), BS, 0,
                                 c->stream>>>(a);
            return 0;
        });
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    prof_mark(c, 3);
    if (late) {  // the write-back waits for every read of the batch
        count_launch(c);
        with_block(threads, [&](auto bs) {
            constexpr int BS = decltype(bs)::value;
            ycsb_writeback_late<BS>
                <<<stride_grid(c, (const void *)ycsb_writeback_late<BS>, a.B), BS, 0, c->stream>>>(a);
            return 0;
        });
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    prof_mark(c, 4);
    return predictor_after_batch(c);
}

}  // namespace ltpg
