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
//     made in shared memory and the tile's committed updates are compacted per
//     warp (ballot + prefix sum) before they are scattered.
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
    uint32_t *bucket_counts;
    uint32_t ways, stage_entries;
    uint32_t filter;
};

__device__ __forceinline__ uint64_t ld_ca_u64(const unsigned long long *p) {
    uint64_t v;
    asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
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
                    if (g != STAGE_NONE) {
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
                    const unsigned long long x =
                        r0.x ^ r0.y ^ r1.x ^ r1.y ^ r2.x ^ r2.y ^ r3.x ^ r3.y ^ r4.x ^ r4.y;
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

// ---- check + write-back over all tiles assigned to this block ------------------
// fl: tile flags; wbuf: per-warp compaction buffers of 128 (address, value) pairs.
__device__ __forceinline__ void checkwb_tiles(const YcsbTunedArgs &a, uint32_t *fl, ulonglong2 *wbuf,
                                              uint32_t epoch) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ulonglong2 *mybuf = wbuf + warp * 128;
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
                } else if (wmin < t) {
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
        // pass 3: committed updates, compacted per warp, then scattered
        for (uint32_t base = 0; base < nvec_tile; base += blockDim.x) {
            const uint32_t v = base + threadIdx.x;
            const bool act = v < nvec;
            uint4 w4 = make_uint4(LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD, LTPG_YCSB_OP_PAD);
            uint32_t lt = 0, j0 = 0;
            bool com = false;
            if (act) {
                lt = (v * 4) / a.stride;
                j0 = v * 4 - lt * a.stride;
                com = (fl[lt] & LTPG_FLAG_COMMIT) != 0u && a.val_off[t0 + lt + 1] != a.val_off[t0 + lt];
                if (com) w4 = ld_nc_u4(vp + v);
            }
            const uint32_t words[4] = {w4.x, w4.y, w4.z, w4.w};
            uint32_t mask = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (!ycsb_is_pad(words[q]) && ycsb_is_update(words[q])) mask |= 1u << q;
            const int cnt = __popc(mask);
            const int incl = warp_incl_scan(cnt);
            const int total = __shfl_sync(FULL, incl, 31);
            if (total == 0) continue;
            if (cnt) {
                // rank of this thread's first update among its transaction's updates
                const uint32_t t = t0 + lt;
                const uint32_t *tw = a.ops + (uint64_t)t * a.stride;
                uint32_t rank = 0;
                for (uint32_t j = 0; j < j0; ++j) {
                    const uint32_t x = tw[j];
                    rank += !ycsb_is_pad(x) && ycsb_is_update(x);
                }
                const uint32_t vb = a.val_off[t] + rank;
                int slot = incl - cnt, r = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (!(mask & (1u << q))) continue;
                    const uint32_t key = ycsb_key(words[q]), fld = ycsb_field(words[q]);
                    const bool ok = key < a.n && fld < LTPG_YCSB_FIELDS;
                    const uint64_t addr = ok ? (uint64_t)(a.rows + (uint64_t)key * LTPG_YCSB_FIELDS + fld) : 0ull;
                    mybuf[slot++] = make_ulonglong2(addr, a.vals[vb + r]);
                    ++r;
                }
            }
            __syncwarp();
            for (int e = lane; e < total; e += 32) {
                const ulonglong2 x = mybuf[e];
                if (x.x) *reinterpret_cast<uint64_t *>(x.x) = x.y;
            }
            __syncwarp();
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

// Shared memory layout: [dig: tile u64][fl: tile u32][wbuf: warps*128*16 B][stage table]
__host__ __device__ __forceinline__ size_t ycsb_smem_bytes(uint32_t tile, uint32_t threads, uint32_t stage_entries) {
    const size_t a = ((size_t)tile * 8 + 15) / 16 * 16;
    const size_t b = ((size_t)tile * 4 + 15) / 16 * 16;
    return a + b + (size_t)(threads / 32) * 128 * 16 + (size_t)stage_entries * sizeof(StageEnt);
}

struct SmemPtrs {
    unsigned long long *dig;
    uint32_t *fl;
    ulonglong2 *wbuf;
    StageEnt *tab;
};
__device__ __forceinline__ SmemPtrs carve(char *base, uint32_t tile) {
    SmemPtrs p;
    const size_t a = ((size_t)tile * 8 + 15) / 16 * 16;
    const size_t b = ((size_t)tile * 4 + 15) / 16 * 16;
    p.dig = reinterpret_cast<unsigned long long *>(base);
    p.fl = reinterpret_cast<uint32_t *>(base + a);
    p.wbuf = reinterpret_cast<ulonglong2 *>(base + a + b);
    p.tab = reinterpret_cast<StageEnt *>(base + a + b + (blockDim.x / 32) * 128 * 16);
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

__global__ void __launch_bounds__(512) ycsb_checkwb_tuned(YcsbTunedArgs a) {
    extern __shared__ __align__(16) char smem[];
    const SmemPtrs p = carve(smem, a.tile);
    checkwb_tiles(a, p.fl, p.wbuf, a.ctl->epoch);
    finish_batch(a.ctl);
}

// One cooperative kernel per batch: execute+register, grid barrier, check +
// write-back.  The barrier wait is bounded (2 s).
template <bool kStage>
__global__ void __launch_bounds__(512) ycsb_persistent(YcsbTunedArgs a) {
    extern __shared__ __align__(16) char smem[];
    const SmemPtrs p = carve(smem, a.tile);
    const uint32_t epoch = a.ctl->epoch;
    const uint64_t tag = slot_tag(epoch);
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
    if (grid_barrier(a.ctl, 2000000000ull)) checkwb_tiles(a, p.fl, p.wbuf, epoch);
    finish_batch(a.ctl);
}

// Transactions per tile: as many whole transactions as the block reads with
// `per_thread` 16-byte vectors per thread, rounded down to a multiple of 32.
static uint32_t tuned_tile(uint32_t stride, uint32_t threads, uint32_t per_thread) {
    uint32_t t = threads * 4u * per_thread / stride;
    t = t / 32u * 32u;
    return t < 32u ? 32u : t;
}

cudaError_t ycsb_run_tuned(ltpg_ctx *c, Slot &s, int mode) {
    if (s.n_txn == 0) return cudaSuccess;
    const LaunchCfg &L = c->launch_y;
    const uint32_t threads = L.block;
    const uint32_t per_thread = L.per_thread ? L.per_thread : 2u;
    YcsbTunedArgs a;
    a.ops = s.ops;
    a.val_off = s.val_off;
    a.vals = s.vals;
    a.B = s.n_txn;
    a.k = s.k;
    a.stride = s.stride;
    a.tile = tuned_tile(s.stride, threads, per_thread);
    a.rows = c->ycsb.rows;
    a.n = c->ycsb.n;
    a.reg = c->ycsb.reg;
    a.results = s.results;
    a.flags = s.flags;
    a.bitmap = s.bitmap;
    a.st = s.stats;
    a.ctl = c->ctl;
    const bool stage = c->stage_on && c->stage_map && c->bucket_counts;
    a.stage_map = c->stage_map;
    a.bucket_counts = c->bucket_counts;
    a.ways = L.ways ? L.ways : 4u;
    a.stage_entries = stage ? STAGE_MAX_ENTRIES / a.ways * a.ways : 0u;
    a.filter = L.filter;
    const size_t smem = ycsb_smem_bytes(a.tile, threads, a.stage_entries);
    cudaError_t e = cudaMemsetAsync(s.stats, 0, sizeof(DevStats), c->stream);
    if (e != cudaSuccess) return e;
    auto exec_k = stage ? ycsb_exec_tuned<true> : ycsb_exec_tuned<false>;
    auto pers_k = stage ? ycsb_persistent<true> : ycsb_persistent<false>;
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(exec_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ycsb_checkwb_tuned, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(pers_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
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
        prof_mark(c, 1);
        prof_mark(c, 2);
        prof_mark(c, 3);
        return cudaSuccess;
    }
    prof_mark(c, 0);
    count_launch(c);
    exec_k<<<grid, threads, smem, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 1);
    count_launch(c);
    ycsb_checkwb_tuned<<<grid, threads, smem, c->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_mark(c, 2);
    prof_mark(c, 3);
    return cudaSuccess;
}

}  // namespace ltpg
