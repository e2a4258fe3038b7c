// microbench.cu — access-pattern ceilings of this GPU for the engine's kernels.
//
// The execute / check kernels are made of four access patterns: random 80-byte
// row reads, random 16-byte slot reads, atomicMin reductions on random slots,
// and reductions that pile up on one hot slot.  Each kernel here runs one
// pattern alone over buffers as large as the real ones, so the measured rate
// is the practical roofline of that pattern (a streaming copy is included as
// the HBM reference).  Buffers are allocated per call.
#include <vector>

#include "devutil.cuh"

namespace ltpg {

__device__ __forceinline__ uint32_t mb_hash(uint64_t i, uint32_t salt) {
    return (uint32_t)(splitmix64(i ^ ((uint64_t)salt << 40)) >> 16);
}

__global__ void mb_copy(const ulonglong2 *__restrict__ src, ulonglong2 *__restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Per-thread row gather: each thread reads whole rows with five 16-byte loads.
__global__ void mb_gather_thread(const uint64_t *__restrict__ rows, uint64_t n_rows, uint64_t n_reads,
                                 unsigned long long *sink) {
    unsigned long long acc = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_reads;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = mb_hash(i, 1) % n_rows;
        const char *p = reinterpret_cast<const char *>(rows + r * 10);
        ulonglong2 a = ld_nc16_issue(p), b = ld_nc16_issue(p + 16), c = ld_nc16_issue(p + 32),
                   d = ld_nc16_issue(p + 48), e = ld_nc16_issue(p + 64);
        acc += a.x ^ a.y ^ b.x ^ b.y ^ c.x ^ c.y ^ d.x ^ d.y ^ e.x ^ e.y;
    }
    if (acc == 0x1234567ull) *sink = acc;
}

// Cooperative row gather: five lanes read one row, one 16-byte chunk each.
__global__ void mb_gather_coop(const uint64_t *__restrict__ rows, uint64_t n_rows, uint64_t n_reads,
                               unsigned long long *sink) {
    const uint32_t lane = threadIdx.x & 31, grp = lane / 5, chunk = lane % 5;
    unsigned long long acc = 0;
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t wi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; wi * 6 < n_reads; wi += warps) {
        const uint64_t i = wi * 6 + grp;
        if (grp < 6 && i < n_reads) {
            const uint64_t r = mb_hash(i, 1) % n_rows;
            const ulonglong2 v = ld_nc16_issue(reinterpret_cast<const char *>(rows + r * 10) + 16 * chunk);
            acc += v.x ^ v.y;
        }
    }
    if (acc == 0x1234567ull) *sink = acc;
}

__global__ void mb_slot_load(const RegSlot *__restrict__ slots, uint64_t n_slots, uint64_t n_ops,
                             unsigned long long *sink) {
    unsigned long long acc = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_ops; i += (uint64_t)gridDim.x * blockDim.x) {
        const ulonglong2 v = ld_slot(slots + mb_hash(i, 2) % n_slots);
        acc += v.x ^ v.y;
    }
    if (acc == 0x1234567ull) *sink = acc;
}

__global__ void mb_red_random(RegSlot *slots, uint64_t n_slots, uint64_t n_ops) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_ops; i += (uint64_t)gridDim.x * blockDim.x)
        red_min(&slots[mb_hash(i, 3) % n_slots].r, 0xFFFFFFFF00000000ull | (i & 0xFFFFFFFFull));
}

__global__ void mb_red_hot(RegSlot *slots, uint64_t n_ops) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_ops; i += (uint64_t)gridDim.x * blockDim.x)
        red_min(&slots[0].r, 0xFFFFFFFF00000000ull | (~i & 0xFFFFFFFFull));
}

}  // namespace ltpg

using namespace ltpg;

extern "C" int ltpg_microbench(ltpg_ctx *c, int kind, uint64_t n_items, uint32_t iters, double *rate) {
    if (!c || !rate || iters == 0 || n_items == 0) return LTPG_ERR_INVALID;
    if (cudaSetDevice(c->device) != cudaSuccess) return LTPG_ERR_CUDA;
    const uint64_t n_rows = 10000000ull, n_slots = 10000000ull;
    void *buf_a = nullptr, *buf_b = nullptr;
    unsigned long long *sink = nullptr;
    size_t bytes_a = 0, bytes_b = 0;
    if (kind == 0) bytes_a = bytes_b = n_items * 16;
    else if (kind == 1 || kind == 2) bytes_a = n_rows * 80;
    else bytes_a = n_slots * sizeof(RegSlot);
    cudaError_t e = cudaMalloc(&buf_a, bytes_a);
    if (e == cudaSuccess && bytes_b) e = cudaMalloc(&buf_b, bytes_b);
    if (e == cudaSuccess) e = cudaMalloc(&sink, 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf_a, 0x5A, bytes_a, c->stream);
    if (e != cudaSuccess) {
        cudaFree(buf_a);
        cudaFree(buf_b);
        cudaFree(sink);
        return LTPG_ERR_NOMEM;
    }
    const int grid = c->sm_count * 8, block = 256;
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    auto launch = [&]() {
        switch (kind) {
        case 0: mb_copy<<<grid, block, 0, c->stream>>>((const ulonglong2 *)buf_a, (ulonglong2 *)buf_b, n_items); break;
        case 1: mb_gather_thread<<<grid, block, 0, c->stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink); break;
        case 2: mb_gather_coop<<<grid, block, 0, c->stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink); break;
        case 3: mb_slot_load<<<grid, block, 0, c->stream>>>((const RegSlot *)buf_a, n_slots, n_items, sink); break;
        case 4: mb_red_random<<<grid, block, 0, c->stream>>>((RegSlot *)buf_a, n_slots, n_items); break;
        default: mb_red_hot<<<grid, block, 0, c->stream>>>((RegSlot *)buf_a, n_items); break;
        }
    };
    launch();  // warm
    cudaEventRecord(ev0, c->stream);
    for (uint32_t i = 0; i < iters; ++i) launch();
    cudaEventRecord(ev1, c->stream);
    e = cudaEventSynchronize(ev1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaFree(buf_a);
    cudaFree(buf_b);
    cudaFree(sink);
    if (e != cudaSuccess) return LTPG_ERR_CUDA;
    const double secs = ms / 1e3 / iters;
    // kind 0: bytes moved (read + write); 1, 2: useful row bytes; 3: slot loads; 4, 5: atomics
    const double units = kind == 0 ? 32.0 * n_items : (kind == 1 || kind == 2) ? 80.0 * n_items : (double)n_items;
    *rate = units / secs;
    return LTPG_OK;
}
