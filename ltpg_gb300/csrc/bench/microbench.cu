// microbench.cu — access-pattern ceilings of this GPU for the engine's kernels.
//
// The execute / check kernels are made of four access patterns: random 80-byte
// row reads, random 16-byte slot reads, atomicMin reductions on random slots,
// and reductions that pile up on one hot slot.  Each kernel here runs one
// pattern alone over buffers as large as the real ones, so the measured rate
// is the practical roofline of that pattern (a streaming copy is included as
// the HBM reference).  Buffers are allocated per call.
//
// Measurement only: built into libltpg_bench.so, which bench.py loads; the
// engine library (libltpg.so) does not contain it.
#include <cstring>
#include <vector>

#include "../../../include/ltpg_bench.h"
#include "../devutil.cuh"

namespace ltpg {

__device__ __forceinline__ uint32_t mb_hash(uint64_t i, uint32_t salt) {
    return (uint32_t)(splitmix64(i ^ ((uint64_t)salt << 40)) >> 16);
}

__global__ void mb_copy(const ulonglong2 *__restrict__ src, ulonglong2 *__restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// The load patterns are templated on U, the independent loads each thread
// keeps in flight (U items per iteration, all issued before any is used), and
// ltpg_microbench reports the best U: a ceiling must not be an artefact of too
// few loads in flight.

// Per-thread row gather: each thread reads whole rows with five 16-byte loads.
template <int U>
__global__ void mb_gather_thread(const uint64_t *__restrict__ rows, uint64_t n_rows, uint64_t n_reads,
                                 unsigned long long *sink) {
    unsigned long long acc = 0;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n_reads; i0 += step * U) {
        ulonglong2 v[U][5];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = i0 + step * u;
            const char *p = reinterpret_cast<const char *>(rows + (mb_hash(i, 1) % n_rows) * 10);
#pragma unroll
            for (int q = 0; q < 5; ++q)
                v[u][q] = i < n_reads ? ld_nc16_issue(p + 16 * q) : make_ulonglong2(0ull, 0ull);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 5; ++q) acc += v[u][q].x ^ v[u][q].y;
    }
    if (acc == 0x1234567ull) *sink = acc;
}

// Cooperative row gather: five lanes read one row, one 16-byte chunk each.
template <int U>
__global__ void mb_gather_coop(const uint64_t *__restrict__ rows, uint64_t n_rows, uint64_t n_reads,
                               unsigned long long *sink) {
    const uint32_t lane = threadIdx.x & 31, grp = lane / 5, chunk = lane % 5;
    unsigned long long acc = 0;
    const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t w0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; w0 * 6 < n_reads; w0 += warps * U) {
        ulonglong2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = (w0 + warps * u) * 6 + grp;
            v[u] = grp < 6 && i < n_reads
                       ? ld_nc16_issue(reinterpret_cast<const char *>(rows + (mb_hash(i, 1) % n_rows) * 10) + 16 * chunk)
                       : make_ulonglong2(0ull, 0ull);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc += v[u].x ^ v[u].y;
    }
    if (acc == 0x1234567ull) *sink = acc;
}

template <int U>
__global__ void mb_slot_load(const RegSlot *__restrict__ slots, uint64_t n_slots, uint64_t n_ops,
                             unsigned long long *sink) {
    unsigned long long acc = 0;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n_ops; i0 += step * U) {
        ulonglong2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = i0 + step * u;
            v[u] = i < n_ops ? ld_slot(slots + mb_hash(i, 2) % n_slots) : make_ulonglong2(0ull, 0ull);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc += v[u].x ^ v[u].y;
    }
    if (acc == 0x1234567ull) *sink = acc;
}

// Host-to-device transfer by a kernel: 16-byte loads straight from pinned host
// memory (addressable by the GPU), stores to device memory.
__global__ void mb_h2d_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
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

extern "C" int ltpg_microbench(int device, void *stream_ptr, int kind, uint64_t n_items, uint32_t iters,
                               double *rate) {
    if (!rate || iters == 0 || n_items == 0 || kind < 0 || kind > 7) return LTPG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LTPG_ERR_CUDA;
    int sm_count = 0;
    if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return LTPG_ERR_CUDA;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    const uint64_t n_rows = 10000000ull, n_slots = 10000000ull;
    void *buf_a = nullptr, *buf_b = nullptr;
    unsigned long long *sink = nullptr;
    size_t bytes_a = 0, bytes_b = 0;
    void *host = nullptr;
    if (kind == 6 || kind == 7) {  // host-to-device: pinned host source, device destination
        if (cudaMallocHost(&host, n_items * 16) != cudaSuccess) return LTPG_ERR_NOMEM;
        memset(host, 0x5A, n_items * 16);
        bytes_b = n_items * 16;
        bytes_a = 16;
    }
    if (kind == 0) bytes_a = bytes_b = n_items * 16;
    else if (kind == 1 || kind == 2) bytes_a = n_rows * 80;
    else if (kind != 6 && kind != 7) bytes_a = n_slots * sizeof(RegSlot);
    cudaError_t e = cudaMalloc(&buf_a, bytes_a);
    if (e == cudaSuccess && bytes_b) e = cudaMalloc(&buf_b, bytes_b);
    if (e == cudaSuccess) e = cudaMalloc(&sink, 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf_a, 0x5A, bytes_a, stream);
    if (e != cudaSuccess) {
        cudaFree(buf_a);
        cudaFree(buf_b);
        cudaFree(sink);
        return LTPG_ERR_NOMEM;
    }
    const int grid = sm_count * 8, block = 256;
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    // loads in flight per thread, for the load patterns (kinds 1-3)
    const int unrolls[3] = {1, 4, 8};
    const int n_unroll = (kind >= 1 && kind <= 3) ? 3 : 1;
    float best_ms = 0.f;
    for (int ui = 0; ui < n_unroll && e == cudaSuccess; ++ui) {
        const int U = unrolls[ui];
        auto launch = [&]() {
            switch (kind) {
            case 0: mb_copy<<<grid, block, 0, stream>>>((const ulonglong2 *)buf_a, (ulonglong2 *)buf_b, n_items); break;
            case 1:
                if (U == 1) mb_gather_thread<1><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                else if (U == 4) mb_gather_thread<4><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                else mb_gather_thread<8><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                break;
            case 2:
                if (U == 1) mb_gather_coop<1><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                else if (U == 4) mb_gather_coop<4><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                else mb_gather_coop<8><<<grid, block, 0, stream>>>((const uint64_t *)buf_a, n_rows, n_items, sink);
                break;
            case 3:
                if (U == 1) mb_slot_load<1><<<grid, block, 0, stream>>>((const RegSlot *)buf_a, n_slots, n_items, sink);
                else if (U == 4) mb_slot_load<4><<<grid, block, 0, stream>>>((const RegSlot *)buf_a, n_slots, n_items, sink);
                else mb_slot_load<8><<<grid, block, 0, stream>>>((const RegSlot *)buf_a, n_slots, n_items, sink);
                break;
            case 4: mb_red_random<<<grid, block, 0, stream>>>((RegSlot *)buf_a, n_slots, n_items); break;
            case 6: mb_h2d_kernel<<<grid, block, 0, stream>>>((const uint4 *)host, (uint4 *)buf_b, n_items); break;
            case 7: cudaMemcpyAsync(buf_b, host, n_items * 16, cudaMemcpyHostToDevice, stream); break;
            default: mb_red_hot<<<grid, block, 0, stream>>>((RegSlot *)buf_a, n_items); break;
            }
        };
        launch();  // warm
        cudaEventRecord(ev0, stream);
        for (uint32_t i = 0; i < iters; ++i) launch();
        cudaEventRecord(ev1, stream);
        e = cudaEventSynchronize(ev1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
        if (e == cudaSuccess && (best_ms == 0.f || ms < best_ms)) best_ms = ms;
    }
    const float ms = best_ms;
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaFree(buf_a);
    cudaFree(buf_b);
    cudaFree(sink);
    if (host) cudaFreeHost(host);
    if (e != cudaSuccess) return LTPG_ERR_CUDA;
    const double secs = ms / 1e3 / iters;
    // kind 0: bytes moved (read + write); 1, 2: useful row bytes; 3: slot loads; 4, 5: atomics;
    // 6, 7: bytes moved host to device (kernel, copy engine)
    const double units = kind == 0 ? 32.0 * n_items
                         : (kind == 1 || kind == 2) ? 80.0 * n_items
                         : (kind == 6 || kind == 7) ? 16.0 * n_items
                                                    : (double)n_items;
    *rate = units / secs;
    return LTPG_OK;
}
