// noalloc.cu — one YCSB batch on caller-owned device buffers, with no device
// memory allocation at all.
//
// Who needs it: a host program that embeds this engine inside a runtime that
// already owns all of the GPU's memory (a database server or serving process
// that carves every device buffer from its own fixed pool), or that drives
// batches from a latency-critical thread.  Such callers cannot call
// cudaMalloc / cudaFree: those calls can block, cudaFree synchronises the
// whole device, and memory taken outside the caller's pool breaks its budget.
// They allocate the table, the batch and the outputs themselves and pass
// device pointers; the only other memory this path touches is the scratch
// below, which lives in the library's static device data.
//
// Scratch: the per-key registration table (16 bytes per record) and a small
// control block, in file-scope __device__ arrays sized for at most
// LTPG_NOALLOC_MAX_RECORDS records (16 MiB + 128 bytes).  Every GPU that loads
// the library holds this memory until the process exits.
#include <mutex>

#include "engine.h"

namespace ltpg {
// The plain YCSB kernels (ycsb.cu), launched here on the static scratch.
__global__ void ycsb_exec_plain(const uint32_t *__restrict__ ops, uint32_t B, uint32_t k, uint32_t stride,
                                uint32_t tile, const uint64_t *__restrict__ rows, uint64_t n,
                                RegSlot *__restrict__ reg, int64_t *__restrict__ results, DevCtl *ctl);
__global__ void ycsb_check_plain(const uint32_t *__restrict__ ops, uint32_t B, uint32_t k, uint32_t stride,
                                 uint32_t tile, const RegSlot *__restrict__ reg, uint64_t n,
                                 uint8_t *__restrict__ flags, DevCtl *ctl);
__global__ void ycsb_writeback_plain(const uint8_t *__restrict__ flags, uint32_t B, const uint32_t *__restrict__ ops,
                                     uint32_t k, uint32_t stride, const uint32_t *__restrict__ val_off,
                                     const uint64_t *__restrict__ vals, uint64_t vals_cap,
                                     uint64_t *__restrict__ rows, uint64_t n,
                                     uint32_t *__restrict__ bitmap, DevStats *st, DevCtl *ctl);
}  // namespace ltpg

using namespace ltpg;

// Registration slots of the no-allocation path (epoch-tagged: each call runs
// with a newer epoch, see slot_tag in proto.h; they are set back to the
// cleared state only when the epoch would pass its last value).
static __device__ __align__(256) RegSlot g_noalloc_reg[LTPG_NOALLOC_MAX_RECORDS];
// Control block (epoch, error word, completion counter), and the batch
// counters the write-back kernel accumulates (not reported by this path).
static __device__ __align__(256) DevCtl g_noalloc_ctl;
static __device__ __align__(256) DevStats g_noalloc_stats;

namespace {
constexpr int kMaxDevices = 64;
struct NoallocDevice {
    bool ready = false;
    RegSlot *reg = nullptr;
    DevCtl *ctl = nullptr;
    DevStats *stats = nullptr;
    uint64_t epoch_next = 1;  // epoch of the next call (the device's never passes it)
};
NoallocDevice g_dev[kMaxDevices];
std::mutex g_mu;

// Once per device, with that device current: resolve the device addresses of
// the static arrays (their names are host-side stand-ins in host code) and
// initialise them.
int setup_device(int device, NoallocDevice **out) {
    std::lock_guard<std::mutex> lock(g_mu);
    NoallocDevice &d = g_dev[device];
    if (!d.ready) {
        void *reg = nullptr, *ctl = nullptr, *stats = nullptr;
        if (cudaGetSymbolAddress(&reg, g_noalloc_reg) != cudaSuccess) return LTPG_ERR_CUDA;
        if (cudaGetSymbolAddress(&ctl, g_noalloc_ctl) != cudaSuccess) return LTPG_ERR_CUDA;
        if (cudaGetSymbolAddress(&stats, g_noalloc_stats) != cudaSuccess) return LTPG_ERR_CUDA;
        if (cudaMemset(reg, 0xFF, sizeof(g_noalloc_reg)) != cudaSuccess) return LTPG_ERR_CUDA;
        DevCtl h{};
        h.epoch = 1;
        if (cudaMemcpy(ctl, &h, sizeof h, cudaMemcpyHostToDevice) != cudaSuccess) return LTPG_ERR_CUDA;
        if (cudaDeviceSynchronize() != cudaSuccess) return LTPG_ERR_CUDA;
        d.reg = static_cast<RegSlot *>(reg);
        d.ctl = static_cast<DevCtl *>(ctl);
        d.stats = static_cast<DevStats *>(stats);
        d.ready = true;
    }
    *out = &d;
    return LTPG_OK;
}

// Takes the epoch of one call; when it would pass the last epoch, enqueues on
// s the reset of the slots and of the epoch ahead of the call's kernels.
int reserve_epoch(NoallocDevice *d, cudaStream_t s) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (d->epoch_next <= kEpochLast) {
        ++d->epoch_next;
        return LTPG_OK;
    }
    if (cudaMemsetAsync(d->reg, 0xFF, sizeof(g_noalloc_reg), s) != cudaSuccess) return LTPG_ERR_CUDA;
    if (ctl_set_epoch(d->ctl, 1u, s) != cudaSuccess) return LTPG_ERR_CUDA;
    d->epoch_next = 2;
    return LTPG_OK;
}
}  // namespace

extern "C" int ltpg_ycsb_batch_noalloc(int device, uint64_t *rows, uint64_t n_records, const uint32_t *ops,
                                       const uint32_t *val_off, const uint64_t *vals, uint32_t n_txn,
                                       uint32_t ops_per_txn, uint8_t *flags, uint32_t *bitmap, int64_t *results,
                                       void *stream) {
    if (device < 0 || device >= kMaxDevices) return LTPG_ERR_INVALID;
    if (n_records == 0 || n_records > LTPG_NOALLOC_MAX_RECORDS) return LTPG_ERR_INVALID;
    if (n_txn == 0 || ops_per_txn == 0 || ops_per_txn > LTPG_YCSB_MAX_OPS) return LTPG_ERR_INVALID;
    if (!rows || !ops || !val_off || !flags || !bitmap || !results) return LTPG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LTPG_ERR_CUDA;
    NoallocDevice *d = nullptr;
    int r = setup_device(device, &d);
    if (r) return r;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t k = ops_per_txn, stride = ycsb_stride(k);
    const uint32_t tile = k >= 256 ? 1u : 256u / k;
    const uint32_t grid = (n_txn + tile - 1) / tile;
    // an earlier, unrelated launch error of this thread must not be taken
    // for one of this call's launches
    (void)cudaGetLastError();
    // the registration slots need no clearing between calls (older epochs
    // never match) except when the epoch would pass its last value
    if ((r = reserve_epoch(d, s)) != LTPG_OK) return r;
    ycsb_exec_plain<<<grid, tile * k, 0, s>>>(ops, n_txn, k, stride, tile, rows, n_records, d->reg, results, d->ctl);
    ycsb_check_plain<<<grid, tile * k, 0, s>>>(ops, n_txn, k, stride, tile, d->reg, n_records, flags, d->ctl);
    // the caller's vals hold val_off[n_txn] values, the bound the kernel reads
    ycsb_writeback_plain<<<(n_txn + 255) / 256, 256, 0, s>>>(flags, n_txn, ops, k, stride, val_off, vals, ~0ull,
                                                             rows, n_records, bitmap, d->stats, d->ctl);
    if (cudaGetLastError() != cudaSuccess) return LTPG_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LTPG_ERR_CUDA;
    uint32_t err = 0;
    if (cudaMemcpy(&err, &d->ctl->error, sizeof err, cudaMemcpyDeviceToHost) != cudaSuccess) return LTPG_ERR_CUDA;
    if (err) {
        DevCtl h{};
        if (cudaMemcpy(&h, d->ctl, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return LTPG_ERR_CUDA;
        h.error = 0;
        h.done = 0;
        if (cudaMemcpy(d->ctl, &h, sizeof h, cudaMemcpyHostToDevice) != cudaSuccess) return LTPG_ERR_CUDA;
        return LTPG_ERR_BOUNDS;
    }
    return LTPG_OK;
}

extern "C" int ltpg_debug_noalloc_set_epoch(int device, uint32_t epoch) {
    if (device < 0 || device >= kMaxDevices || epoch == 0u) return LTPG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LTPG_ERR_CUDA;
    NoallocDevice *d = nullptr;
    int r = setup_device(device, &d);
    if (r) return r;
    if (cudaDeviceSynchronize() != cudaSuccess) return LTPG_ERR_CUDA;
    if (ctl_set_epoch(d->ctl, epoch, nullptr) != cudaSuccess) return LTPG_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return LTPG_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    d->epoch_next = epoch;
    return LTPG_OK;
}

extern "C" int ltpg_debug_noalloc_get_epoch(int device, uint32_t *epoch) {
    if (device < 0 || device >= kMaxDevices || !epoch) return LTPG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LTPG_ERR_CUDA;
    NoallocDevice *d = nullptr;
    int r = setup_device(device, &d);
    if (r) return r;
    if (cudaDeviceSynchronize() != cudaSuccess) return LTPG_ERR_CUDA;
    if (cudaMemcpy(epoch, &d->ctl->epoch, sizeof *epoch, cudaMemcpyDeviceToHost) != cudaSuccess) return LTPG_ERR_CUDA;
    return LTPG_OK;
}
