// engine.h — context and device-side structures shared by the .cu files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "proto.h"

namespace ltpg {

// Device control block, one per context.
//  epoch        tag of the batch being run (see slot_tag in proto.h); bumped on
//               the device by the last block of a batch's final kernel, so a
//               captured CUDA graph can be replayed without host involvement.
//  done         completion counter of that final kernel.
//  error        OR of LTPG device error bits (bounds, timeouts).
//  err_index    first offending index, for the error message.
//  barrier      arrival count and generation of the persistent kernels' grid
//               barrier.
//  barrier_skip test hook: block index + 1 of a block that never arrives at a
//               grid barrier, so that the other blocks' bounded waits run out
//               (0 = none).
//  barrier_limit_ns  bound of one grid-barrier wait (0 = kBarrierLimitNs).
struct DevCtl {
    uint32_t epoch;
    uint32_t done;
    uint32_t error;
    uint32_t err_index;
    uint32_t barrier_count;
    uint32_t barrier_gen;
    uint32_t barrier_skip;
    uint32_t pad;
    unsigned long long total_commits;
    unsigned long long barrier_limit_ns;
};
constexpr uint32_t DERR_BOUNDS = 1u;
constexpr uint32_t DERR_TIMEOUT = 2u;
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // 2 s
// Batch epochs 1 .. kEpochLast tag the registration slots (slot_tag in
// proto.h: tag = 0xFFFFFFFF - epoch).  Epoch 0 would carry the tag of a
// cleared slot, and a wrapped epoch a tag larger than stale ones, so before a
// launch would run a batch past kEpochLast the host sets every slot back to
// the cleared state and the epoch to 1 (epoch_reserve in engine.cu).
constexpr uint32_t kEpochLast = 0xFFFFFFFFu;

// Per-batch counters accumulated on the device (ltpg_batch_stats).
struct DevStats {
    unsigned long long commits, raw, war, waw, staged_ops, total_ops, pad[2];
};

// A registration slot: minimum read and write TID of a row, epoch-tagged.
struct __align__(16) RegSlot {
    unsigned long long r, w;
};

struct YcsbDb {
    uint64_t n = 0;
    uint64_t *rows = nullptr;  // n * 10 u64
    RegSlot *reg = nullptr;    // n
    uint32_t *wbits = nullptr; // ceil(n / 32): keys with a writer in the batch (write-first registration)
    // write-first registration: entry u = {TID, op word} of a batch's u-th
    // update (u = its value index), so that the check and the write-back walk
    // the updates alone; as many entries as a slot has values
    uint2 *upd = nullptr;
    uint64_t upd_cap = 0;
};

struct TpccDb {
    uint32_t W = 0;
    uint64_t rows[LTPG_TPCC_TABLES] = {};
    uint64_t *tab[LTPG_TPCC_TABLES] = {};
    uint64_t n_slots = 0;
    RegSlot *reg = nullptr;  // flat over all tables
    uint64_t base[LTPG_TPCC_TABLES] = {};
    // Customer last-name index: per district its 3,000 keys
    // (min(C_LAST, 2^32 - 1) << 32 | C_ID) in ascending order.
    uint64_t *name_idx = nullptr;
};

// One device batch slot.
struct Slot {
    int workload = 0;
    uint32_t n_txn = 0;
    // YCSB
    uint32_t k = 0, stride = 0, n_updates = 0;
    uint32_t *ops = nullptr;
    uint32_t *val_off = nullptr;
    uint64_t *vals = nullptr;
    uint32_t *off_blocks = nullptr;  // value offsets made on the device: per-1024-transaction sums
    uint64_t cap_ops = 0, cap_vals = 0, cap_txn_y = 0;
    // TPC-C
    uint32_t n_lines = 0;
    uint64_t txn_base = 0;
    ltpg_tpcc_txn *txns = nullptr;
    ltpg_tpcc_line *lines = nullptr;
    uint32_t *packed_lines = nullptr;  // packed uploads land here before their unpacking
    // {n_lines, txn_base} of the batch in the slot, read by the kernels from
    // device memory so a captured graph stays valid when a new batch is
    // uploaded into the slot.
    uint64_t *dev_hdr = nullptr;
    uint64_t host_hdr[2] = {0, 0};
    uint64_t cap_txn_c = 0, cap_lines = 0;
    // outputs
    uint8_t *flags = nullptr;
    uint32_t *bitmap = nullptr;
    int64_t *results = nullptr;
    DevStats *stats = nullptr;
    uint64_t cap_out = 0;
    // pipelined host calls: the batch's copy is done / the slot's last use
    // (kernels and bitmap download) is done
    cudaEvent_t copied = nullptr, done = nullptr;
};

struct LaunchCfg {
    uint32_t block = 256;        // threads per block of the tuned kernels
    uint32_t per_thread = 1;     // YCSB op words per thread (1 = cooperative row reads, 2, 4, 8)
    uint32_t blocks_per_sm = 0;  // cap on resident blocks per SM (0 = occupancy)
    uint32_t ways = 4;           // shared-memory staging entries per hot bucket
    uint32_t filter = 1;         // read the slot before its atomicMin
    uint32_t dedupe = 0;         // one atomic per key per warp (measured slower on GB300 for both workloads)
    uint32_t late_reads = 0;     // YCSB: rows read after the check, by committed transactions only
};

}  // namespace ltpg

struct ltpg_predictor_state;

struct ltpg_ctx {
    int device = 0;
    ltpg_config cfg{};
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host-to-device copies of pipelined host calls
    cudaStream_t stream = nullptr;
    std::string err;
    ltpg::DevCtl *ctl = nullptr;
    ltpg::YcsbDb ycsb;
    ltpg::TpccDb tpcc;
    uint64_t ycsb_seed = 0, tpcc_seed = 0;
    std::vector<ltpg::Slot> slots;
    ltpg::LaunchCfg launch_y, launch_c;
    int sm_count = 0;
    // persistent-mode occupancy
    int persist_blocks_y = 0, persist_blocks_c = 0;
    // staging map (bucket -> way group), predictor output
    uint16_t *stage_map = nullptr;
    uint32_t *stage_bits = nullptr;  // staged-bucket bitmap (65536 bits)
    uint32_t *stage_rank = nullptr;  // staged buckets before each bitmap word
    uint32_t *bucket_counts = nullptr;  // per-batch access counts per bucket
    uint32_t stage_on = 0;
    // contention predictor (predictor.cu)
    ltpg_predictor_state *pred = nullptr;
    uint32_t pred_on = 0, pred_train = 0;
    // Epoch the next batch runs at, or more: every launch adds its batches
    // before it is enqueued, and the device adds one per batch it finishes,
    // so the device's epoch never passes this mirror.
    uint64_t epoch_next = 1;
    // measurement
    uint64_t launches = 0;
    bool profiling = false;
    bool capturing = false;
    uint32_t cur_slot = 0;
    std::vector<cudaEvent_t> prof_events;  // PROF_MARKS per slot
    // cached CUDA graphs keyed by (first, count, workload)
    struct GraphEntry {
        uint32_t first, count;
        int workload;
        cudaGraphExec_t exec;
        uint64_t kernels;
    };
    std::vector<GraphEntry> graphs;
};

// Kernel launchers implemented in ycsb.cu / tpcc.cu.
namespace ltpg {
// Records profiling event i (0..3) of the slot being run, if profiling is on.
// Profiling marks of a batch: 0 before the first kernel, then after the
// execute (1), check (2), read (3) and write-back (4) kernels; a phase a mode
// does not have (or runs inside another kernel) gets its mark at the same
// place as the one before, so its interval is 0.
constexpr int PROF_MARKS = 5;
void prof_mark(ltpg_ctx *c, int i);
// Drops the cached CUDA graphs (launch settings changed).
void drop_graphs_ctx(ltpg_ctx *c);
// Readies slot `slot` for a batch of the given shape (buffers, outputs, graph
// invalidation) and records the shape; the caller fills the batch buffers.
int slot_prepare_ycsb(ltpg_ctx *c, uint32_t slot, uint32_t n_txn, uint32_t k, uint32_t n_updates, Slot **out);
int slot_prepare_tpcc(ltpg_ctx *c, uint32_t slot, uint32_t n_txn, uint64_t n_lines, uint64_t txn_base, Slot **out);
// Makes generator g's batch batch_id in slot `slot` on stream st (gen_dev.cu).
int gen_device_batch(ltpg_ctx *c, ltpg_gen *g, uint64_t batch_id, uint32_t slot, cudaStream_t st);
// Makes room for `batches` more batch epochs before a launch (resets the
// registration slots and the epoch when the last epoch would be passed).
int epoch_reserve(ltpg_ctx *c, uint64_t batches);
// Sets the device epoch to `epoch`, in the order of stream `st`.
cudaError_t ctl_set_epoch(DevCtl *ctl, uint32_t epoch, cudaStream_t st);
// Record an error message on the context and return its code.
int ctx_fail(ltpg_ctx *c, int code, const char *msg);
int ctx_cuda_fail(ltpg_ctx *c, cudaError_t e, const char *what);
// Predictor step after a tuned YCSB batch (predictor.cu).
cudaError_t predictor_after_batch(ltpg_ctx *c);
void predictor_free(ltpg_ctx *c);
// Counts kernels launched by the engine.
inline void count_launch(ltpg_ctx *c, uint64_t n = 1) { c->launches += n; }
cudaError_t ycsb_init_table(ltpg_ctx *c);
cudaError_t ycsb_phase(ltpg_ctx *c, Slot &s, int phase);      // 0 exec, 1 check, 2 write-back
// Value offsets of the batch in s made on the device from its op words (the
// upload of a batch without val_off), on stream st.
cudaError_t ycsb_derive_offsets(ltpg_ctx *c, Slot &s, cudaStream_t st);
// Unpacks the slot's packed order lines into its lines, on stream st.
cudaError_t tpcc_unpack_lines(Slot &s, cudaStream_t st);
cudaError_t ycsb_run_tuned(ltpg_ctx *c, Slot &s, int mode);   // fused / persistent
cudaError_t tpcc_init_tables(ltpg_ctx *c);
cudaError_t tpcc_build_name_index(ltpg_ctx *c);
cudaError_t tpcc_phase(ltpg_ctx *c, Slot &s, int phase);
cudaError_t tpcc_run_tuned(ltpg_ctx *c, Slot &s, int mode);
}  // namespace ltpg
