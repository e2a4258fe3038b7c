// devutil.cuh — small device helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace ltpg {

constexpr unsigned FULL = 0xFFFFFFFFu;

// 16-byte load of a registration slot that bypasses L1: slots are written by
// atomics at L2 in the previous phase.
__device__ __forceinline__ ulonglong2 ld_slot(const RegSlot *p) {
    ulonglong2 v;
    asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}
// Read-only 16-byte load through the non-coherent path (table rows, batches).
__device__ __forceinline__ ulonglong2 ld_nc16(const void *p) {
    ulonglong2 v;
    asm("ld.global.nc.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}
// Same load, kept in program order with the other volatile loads so that a
// thread's independent row reads are all issued before the first is consumed.
__device__ __forceinline__ ulonglong2 ld_nc16_issue(const void *p) {
    ulonglong2 v;
    asm volatile("ld.global.nc.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ uint4 ld_nc_u4(const void *p) {
    uint4 v;
    asm("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}
// Loads of words that other blocks of the same launch wrote before a grid
// barrier (the persistent kernels' later phases): relaxed at GPU scope, so
// they are served coherently by L2 and never by a stale L1 line or the
// read-only path, and the "memory" clobber keeps them after the barrier.
__device__ __forceinline__ uint32_t ld_gpu_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_gpu_u64(const unsigned long long *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_gpu_u8(const uint8_t *p) {
    uint16_t v;
    asm volatile("ld.relaxed.gpu.global.u8 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint2 ld_gpu_u2(const uint2 *p) {
    uint2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ ulonglong2 ld_gpu_slot(const RegSlot *p) {
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}
// Fire-and-forget atomic minimum (no return value, so it issues as a
// reduction at L2).
__device__ __forceinline__ void red_min(unsigned long long *p, unsigned long long v) {
    asm volatile("red.global.min.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// The same reduction without the compiler memory barrier, for the execute
// phases: it stays ordered with other volatile asm (the slot filter's load)
// and with barriers, but the compiler may move independent loads (rows, order
// lines, prices) across it, so they are in flight together.  Nothing in the
// execute phase reads back a slot it reduces into.
__device__ __forceinline__ void red_min_exec(unsigned long long *p, unsigned long long v) {
    asm volatile("red.global.min.u64 [%0], %1;" ::"l"(p), "l"(v));
}
__device__ __forceinline__ void red_add_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Xor of the 10 fields of a YCSB row (five 16-byte loads).
__device__ __forceinline__ unsigned long long row_xor(const uint64_t *__restrict__ rows, uint64_t key) {
    const char *p = reinterpret_cast<const char *>(rows + key * LTPG_YCSB_FIELDS);
    const ulonglong2 a = ld_nc16(p), b = ld_nc16(p + 16), c = ld_nc16(p + 32), d = ld_nc16(p + 48), e = ld_nc16(p + 64);
    return a.x ^ a.y ^ b.x ^ b.y ^ c.x ^ c.y ^ d.x ^ d.y ^ e.x ^ e.y;
}
// Last key a YCSB read covers (key + scan span, within the table).
__device__ __forceinline__ uint64_t scan_last(uint32_t w, uint64_t n) {
    const uint64_t last = (uint64_t)ycsb_key(w) + ycsb_span(w);
    return last < n ? last : n - 1;
}
// The keys of a range-scan read after its first (key + 1 .. last): each
// registered in its read slot (with `filter`, skipped when the slot already
// holds a smaller tag) and their rows xor-ed.  Point reads return 0.
__device__ __forceinline__ unsigned long long scan_rest(RegSlot *reg, const uint64_t *__restrict__ rows, uint64_t n,
                                                        uint32_t w, unsigned long long mine, bool filter) {
    unsigned long long x = 0;
    if (!ycsb_span(w)) return x;
    const uint64_t last = scan_last(w, n);
    for (uint64_t q = (uint64_t)ycsb_key(w) + 1; q <= last; ++q) {
        unsigned long long *p = &reg[q].r;
        bool go = true;
        if (filter) {
            unsigned long long cur;
            asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(cur) : "l"(p));
            go = cur > mine;
        }
        if (go) red_min(p, mine);
        x ^= row_xor(rows, q);
    }
    return x;
}
// RAW on the keys of a range-scan read after its first.
__device__ __forceinline__ bool scan_rest_raw(const RegSlot *reg, uint64_t n, uint32_t w, uint32_t t, uint32_t epoch) {
    if (!ycsb_span(w)) return false;
    const uint64_t last = scan_last(w, n);
    bool raw = false;
    for (uint64_t q = (uint64_t)ycsb_key(w) + 1; q <= last; ++q) raw |= slot_min(ld_slot(reg + q).y, epoch) < t;
    return raw;
}

__device__ __forceinline__ void report_error(DevCtl *ctl, uint32_t code, uint32_t index) {
    if (atomicOr(&ctl->error, code) == 0u) ctl->err_index = index;
}

// Called by every block at the very end of a batch's final kernel: the last
// block to finish advances the batch epoch.
__device__ __forceinline__ void finish_batch(DevCtl *ctl) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->done, 1u);
        if (prev == gridDim.x - 1u) {
            ctl->done = 0u;
            atomicAdd(&ctl->epoch, 1u);
            __threadfence();
        }
    }
}

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

}  // namespace ltpg
