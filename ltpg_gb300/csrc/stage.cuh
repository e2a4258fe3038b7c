// stage.cuh — shared-memory staging of hot registration slots, and the
// bounded grid barrier of the persistent kernels.
#pragma once
#include "devutil.cuh"

namespace ltpg {

// One staged row: its key, the minimum read / write TIDs seen by this block,
// the number of registrations it absorbed, and the row's checksum once some
// read of it in this block has loaded the row (dig_ok = 1).
struct __align__(16) StageEnt {
    uint32_t key, rmin, wmin, cnt;
    unsigned long long dig;
    uint32_t dig_ok, pad;
};
constexpr uint32_t STAGE_EMPTY = 0xFFFFFFFFu;
constexpr uint32_t STAGE_NONE = 0xFFFFu;     // stage_map value of an unstaged bucket
constexpr uint32_t STAGE_BUCKETS = LTPG_STAGE_BUCKETS;      // key-hash buckets seen by the predictor
constexpr uint32_t STAGE_MAX_ENTRIES = LTPG_STAGE_ENTRIES;  // 32 KB of shared memory per block
constexpr uint32_t COUNT_SAMPLE = 16u;       // unstaged ops are counted 1 in 16

__device__ __forceinline__ uint32_t key_bucket(uint32_t key) { return (key * 0x9E3779B1u) >> 16; }

// Staged-bucket set in compact form: one bit per bucket and, per 32-bucket
// word, the number of staged buckets before it.  The group of a staged bucket
// is its rank among the staged buckets.
constexpr uint32_t STAGE_WORDS = STAGE_BUCKETS / 32u;
__device__ __forceinline__ uint32_t stage_group(const uint32_t *bits, const uint32_t *rank, uint32_t b) {
    const uint32_t w = bits[b >> 5], bit = 1u << (b & 31u);
    return (w & bit) ? rank[b >> 5] + __popc(w & (bit - 1u)) : STAGE_NONE;
}

__device__ __forceinline__ void stage_init(StageEnt *tab, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        tab[i] = StageEnt{STAGE_EMPTY, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0ull, 0u, 0u};
}

// Finds or claims the entry of `key` among the `ways` entries of group g.
__device__ __forceinline__ StageEnt *stage_find(StageEnt *tab, uint32_t g, uint32_t ways, uint32_t key) {
    StageEnt *base = tab + g * ways;
    for (uint32_t w = 0; w < ways; ++w) {
        const uint32_t k0 = *reinterpret_cast<volatile uint32_t *>(&base[w].key);
        if (k0 == key) return &base[w];
        if (k0 == STAGE_EMPTY) {
            const uint32_t prev = atomicCAS(&base[w].key, STAGE_EMPTY, key);
            if (prev == STAGE_EMPTY || prev == key) return &base[w];
        }
    }
    return nullptr;
}

// Writes the block's staged minima to the global registration table (one
// atomic per staged row and kind instead of one per operation) and adds the
// staged access counts to the per-bucket counters.  Returns the number of
// operations this thread's entries absorbed.
__device__ __forceinline__ uint32_t stage_flush(const StageEnt *tab, uint32_t n, RegSlot *reg, uint64_t tag,
                                                uint32_t *bucket_counts) {
    uint32_t ops = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const StageEnt e = tab[i];
        if (e.key == STAGE_EMPTY) continue;
        if (e.rmin != 0xFFFFFFFFu) red_min(&reg[e.key].r, tag | e.rmin);
        if (e.wmin != 0xFFFFFFFFu) red_min(&reg[e.key].w, tag | e.wmin);
        if (bucket_counts && e.cnt) atomicAdd(&bucket_counts[key_bucket(e.key)], e.cnt);
        ops += e.cnt;
    }
    return ops;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The
// wait is bounded: after ctl->barrier_limit_ns (0: kBarrierLimitNs) a block
// records DERR_TIMEOUT and returns false, so a broken launch ends with an
// error status instead of a hang.  A wait that ran out anywhere in the grid
// makes every later arrival return false as well, so that no block runs a
// phase whose inputs some block did not finish.  Callers stop calling it
// once it has returned false.  Test hook: the block named by
// ctl->barrier_skip (index + 1) returns false without arriving, so the
// others' waits run out.
__device__ __forceinline__ bool grid_barrier(DevCtl *ctl) {
    __shared__ uint32_t ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile DevCtl *vc = ctl;
        const unsigned long long lim = vc->barrier_limit_ns;
        const uint64_t limit_ns = lim ? lim : kBarrierLimitNs;
        ok = 1u;
        if (vc->barrier_skip == blockIdx.x + 1u) {
            ok = 0u;
        } else {
            volatile uint32_t *gen = &ctl->barrier_gen;
            const uint32_t g0 = *gen;
            __threadfence();
            const uint32_t arrived = atomicAdd(&ctl->barrier_count, 1u) + 1u;
            if (arrived == gridDim.x) {
                ctl->barrier_count = 0u;
                __threadfence();
                atomicAdd(&ctl->barrier_gen, 1u);
            } else {
                const uint64_t t0 = global_ns();
                while (*gen == g0) {
                    __nanosleep(64);
                    if (global_ns() - t0 > limit_ns) {
                        report_error(ctl, DERR_TIMEOUT, blockIdx.x);
                        ok = 0u;
                        break;
                    }
                }
            }
            __threadfence();
            if (vc->error & DERR_TIMEOUT) ok = 0u;
        }
    }
    __syncthreads();
    return ok != 0u;
}

}  // namespace ltpg
