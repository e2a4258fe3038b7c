/*
 * ltpg_bench.h — measurement entry points of libltpg_bench.so (bench-only;
 * not part of the engine library libltpg.so).  No counterpart in the
 * reference: they measure the access patterns the engine's kernels are made
 * of, as ceilings to read the kernels' rates against.
 */
#ifndef LTPG_BENCH_H
#define LTPG_BENCH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Runs one access pattern alone on `device` (on `stream`, a cudaStream_t or
 * NULL) and reports its rate: kind 0 streaming copy (bytes/s, read + write),
 * 1 random 80-byte row reads by one thread per row (useful bytes/s), 2 the
 * same with five lanes per row, 3 random 16-byte slot loads (loads/s),
 * 4 atomicMin on random slots (atomics/s), 5 atomicMin on one slot
 * (atomics/s), 6 host-to-device bytes read by a kernel from pinned memory,
 * 7 the same by the copy engine (bytes/s).  n_items = rows, loads, atomics
 * or 16-byte elements per launch; iters = timed launches.  Returns an
 * LTPG_* status (ltpg.h). */
int ltpg_microbench(int device, void *stream, int kind, uint64_t n_items, uint32_t iters, double *rate);

#ifdef __cplusplus
}
#endif
#endif /* LTPG_BENCH_H */
