// ycsb.cu — YCSB executor: table image, and the three-phase plain path.
//
// Follows YCSB_A_NAMESPACE of the reference (Y1/Execute.h:9-272): reads
// register in the read table and are checked for RAW, updates register in the
// write table and are checked for WAR and WAW (Y1/Execute.h:109-150), commit
// iff !WAW && (!RAW || !WAR) (Y1/Execute.h:187).  Unlike the reference, an
// update really writes its value into the table, and a read returns a checksum
// of the row it read.
#include "devutil.cuh"

namespace ltpg {

// ---- table image (YCSBDatabase::create_table, Y1/Database.h:348-375) --------
__global__ void ycsb_init_kernel(uint64_t *__restrict__ rows, uint64_t n, uint64_t seed) {
    const uint64_t total = n * LTPG_YCSB_FIELDS;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x)
        rows[i] = hash3(seed, i / LTPG_YCSB_FIELDS, i % LTPG_YCSB_FIELDS);
}

cudaError_t ycsb_init_table(ltpg_ctx *c) {
    const int blocks = c->sm_count * 8;
    ycsb_init_kernel<<<blocks, 256, 0, c->stream>>>(c->ycsb.rows, c->ycsb.n, c->ycsb_seed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(c->ycsb.reg, 0xFF, c->ycsb.n * sizeof(RegSlot), c->stream);
}


// ---- plain phase 1: execute + register (KERNEL_EXECUTE, Y1/ycsb.cu:9-24) -----
// One thread per operation; a block holds `tile` whole transactions.
__global__ void __launch_bounds__(256) ycsb_exec_plain(const uint32_t *__restrict__ ops, uint32_t B, uint32_t k,
                                                       uint32_t stride, uint32_t tile,
                                                       const uint64_t *__restrict__ rows, uint64_t n,
                                                       RegSlot *__restrict__ reg, int64_t *__restrict__ results,
                                                       DevCtl *ctl) {
    __shared__ unsigned long long dig[256];
    const uint64_t tag = slot_tag(ctl->epoch);
    const uint32_t lt = threadIdx.x / k, j = threadIdx.x % k;
    const uint32_t t = blockIdx.x * tile + lt;
    if (threadIdx.x < tile) dig[threadIdx.x] = 0ull;
    __syncthreads();
    if (lt < tile && t < B) {
        const uint32_t w = ops[(uint64_t)t * stride + j];
        if (!ycsb_is_pad(w)) {
            const uint32_t key = ycsb_key(w);
            if (key >= n) {
                report_error(ctl, DERR_BOUNDS, t);
            } else if (ycsb_is_update(w)) {
                red_min(&reg[key].w, tag | t);
            } else {
                // a point read, or a range scan of keys key .. key + span
                red_min(&reg[key].r, tag | t);
                const unsigned long long x = row_xor(rows, key) ^ scan_rest(reg, rows, n, w, tag | t, false);
                atomicAdd(&dig[lt], x * (2ull * j + 1ull));
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < tile) {
        const uint32_t tt = blockIdx.x * tile + threadIdx.x;
        if (tt < B) results[tt] = (int64_t)dig[threadIdx.x];
    }
}

// ---- plain phase 2: check (KERNEL_CHECK, Y1/ycsb.cu:25-40) -------------------
__global__ void __launch_bounds__(256) ycsb_check_plain(const uint32_t *__restrict__ ops, uint32_t B, uint32_t k,
                                                        uint32_t stride, uint32_t tile,
                                                        const RegSlot *__restrict__ reg, uint64_t n,
                                                        uint8_t *__restrict__ flags, DevCtl *ctl) {
    __shared__ uint32_t fl[256];
    const uint32_t epoch = ctl->epoch;
    const uint32_t lt = threadIdx.x / k, j = threadIdx.x % k;
    const uint32_t t = blockIdx.x * tile + lt;
    if (threadIdx.x < tile) fl[threadIdx.x] = 0u;
    __syncthreads();
    if (lt < tile && t < B) {
        const uint32_t w = ops[(uint64_t)t * stride + j];
        if (!ycsb_is_pad(w) && ycsb_key(w) < n) {
            const ulonglong2 s = ld_slot(reg + ycsb_key(w));
            const uint32_t rmin = slot_min(s.x, epoch), wmin = slot_min(s.y, epoch);
            uint32_t f = 0;
            if (ycsb_is_update(w)) {
                if (rmin < t) f |= LTPG_FLAG_WAR;
                if (wmin < t) f |= LTPG_FLAG_WAW;
            } else if (wmin < t || scan_rest_raw(reg, n, w, t, epoch)) {
                f |= LTPG_FLAG_RAW;
            }
            if (f) atomicOr(&fl[lt], f);
        }
    }
    __syncthreads();
    if (threadIdx.x < tile) {
        const uint32_t tt = blockIdx.x * tile + threadIdx.x;
        if (tt < B) {
            uint32_t f = fl[threadIdx.x];
            if (commits(f)) f |= LTPG_FLAG_COMMIT;
            flags[tt] = (uint8_t)f;
        }
    }
}

// ---- plain phase 3: write-back (KERNEL_WRITEBACK, Y1/ycsb.cu:41-58) ----------
// One thread per transaction.  The commit bitmap word of a warp is its ballot.
// A committed transaction's updates are stored by its own thread in op order,
// so one that updates a field twice leaves its later value (as a sequential
// replay does); no two committed transactions write one row (WAW).
__global__ void __launch_bounds__(256) ycsb_writeback_plain(const uint8_t *__restrict__ flags, uint32_t B,
                                                            const uint32_t *__restrict__ ops, uint32_t k,
                                                            uint32_t stride, const uint32_t *__restrict__ val_off,
                                                            const uint64_t *__restrict__ vals, uint64_t vals_cap,
                                                            uint64_t *__restrict__ rows, uint64_t n,
                                                            uint32_t *__restrict__ bitmap, DevStats *st,
                                                            DevCtl *ctl) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const uint32_t f = t < B ? flags[t] : 0u;
    const bool com = (f & LTPG_FLAG_COMMIT) != 0u;
    const unsigned bal = __ballot_sync(FULL, com);
    const unsigned braw = __ballot_sync(FULL, (f & LTPG_FLAG_RAW) != 0u);
    const unsigned bwar = __ballot_sync(FULL, (f & LTPG_FLAG_WAR) != 0u);
    const unsigned bwaw = __ballot_sync(FULL, (f & LTPG_FLAG_WAW) != 0u);
    if (lane == 0 && t < B) {
        bitmap[t >> 5] = bal;
        if (bal) {
            red_add_u64(&st->commits, __popc(bal));
            red_add_u64(&ctl->total_commits, __popc(bal));
        }
        if (braw) red_add_u64(&st->raw, __popc(braw));
        if (bwar) red_add_u64(&st->war, __popc(bwar));
        if (bwaw) red_add_u64(&st->waw, __popc(bwaw));
    }
    if (com && val_off[t + 1] != val_off[t]) {
        // value indices stay below the batch's value count and the buffer's
        // capacity: offsets that disagree with the op words (a malformed
        // batch) are reported, not followed out of bounds
        const uint64_t nv = min((uint64_t)val_off[B], vals_cap);
        uint32_t v = val_off[t];
        const uint32_t *w = ops + (uint64_t)t * stride;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t x = w[j];
            if (ycsb_is_pad(x) || !ycsb_is_update(x)) continue;
            const uint32_t key = ycsb_key(x), f = ycsb_field(x);
            if (v >= nv) {
                report_error(ctl, DERR_BOUNDS, t);
                break;
            }
            if (key < n && f < LTPG_YCSB_FIELDS) rows[(uint64_t)key * LTPG_YCSB_FIELDS + f] = vals[v];
            ++v;
        }
    }
    finish_batch(ctl);
}

// ---- value offsets made on the device -------------------------------------------
// A batch uploaded without val_off gets it here: the exclusive prefix over
// transactions of each one's update count, in three passes (per 1024
// transactions: counts and a block scan; one block: the scan of the block
// sums; every transaction: its block's offset).  The total must equal the
// batch's declared n_updates (the values it carries); a mismatch is reported
// as a range error.
__device__ __forceinline__ uint32_t block_excl_scan_1024(uint32_t v, uint32_t *total) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += x;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(FULL, w, o);
            if (lane >= o) w += x;
        }
        if (lane < nw) warp_sums[lane] = w;  // inclusive sums of the warps
    }
    __syncthreads();
    const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();  // warp_sums is reused by the next call
    return before + incl - v;
}

__global__ void __launch_bounds__(1024) ycsb_offsets_local(const uint32_t *__restrict__ ops, uint32_t B,
                                                           uint32_t stride, uint32_t *__restrict__ val_off,
                                                           uint32_t *__restrict__ blocks) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = 0;
    if (t < B) {
        const uint4 *p = reinterpret_cast<const uint4 *>(ops + (uint64_t)t * stride);
        for (uint32_t q = 0; q < stride / 4u; ++q) {
            const uint4 w = __ldg(p + q);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) n += (!ycsb_is_pad(ws[i]) && ycsb_is_update(ws[i])) ? 1u : 0u;
        }
    }
    uint32_t total;
    const uint32_t excl = block_excl_scan_1024(n, &total);
    if (t < B) val_off[t] = excl;
    if (threadIdx.x == 0) blocks[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) ycsb_offsets_blocks(uint32_t *blocks, uint32_t nb) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? blocks[i] : 0u;
        uint32_t total;
        const uint32_t excl = block_excl_scan_1024(v, &total);
        if (i < nb) blocks[i] = carry + excl;
        carry += total;
    }
    if (threadIdx.x == 0) blocks[nb] = carry;
}

__global__ void __launch_bounds__(1024) ycsb_offsets_add(uint32_t *__restrict__ val_off, uint32_t B,
                                                         const uint32_t *__restrict__ blocks, uint32_t nb,
                                                         uint32_t n_updates, DevCtl *ctl) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < B) val_off[t] += blocks[t / 1024u];
    if (t == 0) {
        val_off[B] = blocks[nb];
        if (blocks[nb] != n_updates) report_error(ctl, DERR_BOUNDS, 0u);
    }
}

cudaError_t ycsb_derive_offsets(ltpg_ctx *c, Slot &s, cudaStream_t st) {
    const uint32_t B = s.n_txn, nb = (B + 1023) / 1024;
    ycsb_offsets_local<<<nb, 1024, 0, st>>>(s.ops, B, s.stride, s.val_off, s.off_blocks);
    ycsb_offsets_blocks<<<1, 1024, 0, st>>>(s.off_blocks, nb);
    ycsb_offsets_add<<<nb, 1024, 0, st>>>(s.val_off, B, s.off_blocks, nb, s.n_updates, c->ctl);
    return cudaGetLastError();
}

static inline uint32_t plain_tile(uint32_t k) { return k >= 256 ? 1u : 256u / k; }

cudaError_t ycsb_phase(ltpg_ctx *c, Slot &s, int phase) {
    const uint32_t B = s.n_txn;
    if (B == 0) return cudaSuccess;
    const uint32_t tile = plain_tile(s.k);
    const uint32_t grid = (B + tile - 1) / tile;
    if (phase == 0) {
        cudaError_t e = cudaMemsetAsync(s.stats, 0, sizeof(DevStats), c->stream);
        if (e != cudaSuccess) return e;
        ycsb_exec_plain<<<grid, tile * s.k, 0, c->stream>>>(s.ops, B, s.k, s.stride, tile, c->ycsb.rows,
                                                            c->ycsb.n, c->ycsb.reg, s.results, c->ctl);
    } else if (phase == 1) {
        ycsb_check_plain<<<grid, tile * s.k, 0, c->stream>>>(s.ops, B, s.k, s.stride, tile, c->ycsb.reg,
                                                             c->ycsb.n, s.flags, c->ctl);
    } else {
        ycsb_writeback_plain<<<(B + 255) / 256, 256, 0, c->stream>>>(s.flags, B, s.ops, s.k, s.stride, s.val_off,
                                                                     s.vals, s.cap_vals, c->ycsb.rows, c->ycsb.n,
                                                                     s.bitmap,
                                                                     s.stats, c->ctl);
    }
    return cudaGetLastError();
}

}  // namespace ltpg

