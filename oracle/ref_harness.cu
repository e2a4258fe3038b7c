// ref_harness.cu — runs the reference's own kernels (from a cubin built by
// oracle/ref_build.py) on buffers prepared by the caller.
//
// TEST INFRASTRUCTURE ONLY: the GPU parity tests use it to pin the oracle to
// the reference itself.  It knows nothing about the reference's structs: the
// caller passes the bytes of every buffer (laid out from the reference's own
// headers), the kernel names and launch shapes; the harness copies the
// buffers to the device, launches the kernels in order with the buffers as
// their pointer arguments, and copies the requested buffers back.  ref_time
// repeats the launches with CUDA events around each kernel (the reference's
// own three-kernel batch time, measured on the device).
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

static int fail(char *err, int errlen, const char *what, CUresult r) {
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    snprintf(err, (size_t)errlen, "%s: %s", what, s ? s : "unknown");
    return 1;
}

#define DRV(call, what)                                       \
    do {                                                      \
        CUresult r_ = (call);                                 \
        if (r_ != CUDA_SUCCESS) {                             \
            rc = fail(err, errlen, what, r_);                 \
            goto done;                                        \
        }                                                     \
    } while (0)

// Runs the kernels `iters` times on one set of device buffers.  Before each
// iteration the listed byte ranges are reset (buffer, offset, length, value) —
// the reference's own per-batch clears — outside the timed span; each kernel is
// bracketed by CUDA events and its mean time written to ms[k].
static int run(const char *cubin, int n_kernels, const char *const *names, const unsigned *grids,
               const unsigned *blocks, int n_bufs, const uint64_t *sizes, void *const *host, const int *copy_back,
               int n_resets, const int *reset_buf, const uint64_t *reset_off, const uint64_t *reset_len,
               const unsigned char *reset_val, int iters, float *ms, char *err, int errlen) {
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    std::vector<CUdeviceptr> d((size_t)n_bufs, 0);
    std::vector<void *> params((size_t)n_bufs);
    std::vector<CUfunction> fn((size_t)n_kernels);
    std::vector<CUevent> ev((size_t)n_kernels + 1, nullptr);
    std::vector<double> acc((size_t)n_kernels, 0.0);
    DRV(cuInit(0), "cuInit");
    DRV(cuDeviceGet(&dev, 0), "cuDeviceGet");
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain");
    DRV(cuCtxSetCurrent(ctx), "cuCtxSetCurrent");
    DRV(cuModuleLoad(&mod, cubin), "cuModuleLoad");
    for (int i = 0; i < n_bufs; ++i) {
        DRV(cuMemAlloc(&d[i], sizes[i] ? sizes[i] : 16), "cuMemAlloc");
        if (sizes[i]) DRV(cuMemcpyHtoD(d[i], host[i], sizes[i]), "cuMemcpyHtoD");
        params[i] = &d[i];
    }
    for (int k = 0; k < n_kernels; ++k) DRV(cuModuleGetFunction(&fn[k], mod, names[k]), "cuModuleGetFunction");
    for (auto &e : ev) DRV(cuEventCreate(&e, CU_EVENT_DEFAULT), "cuEventCreate");
    for (int it = 0; it < iters; ++it) {
        for (int r = 0; r < n_resets; ++r) {
            if (reset_buf[r] < 0 || reset_buf[r] >= n_bufs || reset_off[r] + reset_len[r] > sizes[reset_buf[r]]) {
                snprintf(err, (size_t)errlen, "reset %d out of range", r);
                rc = 1;
                goto done;
            }
            DRV(cuMemsetD8(d[(size_t)reset_buf[r]] + reset_off[r], reset_val[r], reset_len[r]), "cuMemsetD8");
        }
        DRV(cuEventRecord(ev[0], nullptr), "cuEventRecord");
        for (int k = 0; k < n_kernels; ++k) {
            DRV(cuLaunchKernel(fn[k], grids[k], 1, 1, blocks[k], 1, 1, 0, nullptr, params.data(), nullptr),
                "cuLaunchKernel");
            DRV(cuEventRecord(ev[(size_t)k + 1], nullptr), "cuEventRecord");
        }
        DRV(cuEventSynchronize(ev[(size_t)n_kernels]), "kernel");
        for (int k = 0; k < n_kernels; ++k) {
            float t = 0.f;
            DRV(cuEventElapsedTime(&t, ev[(size_t)k], ev[(size_t)k + 1]), "cuEventElapsedTime");
            acc[(size_t)k] += t;
        }
    }
    if (ms)
        for (int k = 0; k < n_kernels; ++k) ms[k] = (float)(acc[(size_t)k] / (iters > 0 ? iters : 1));
    for (int i = 0; i < n_bufs; ++i)
        if (copy_back[i] && sizes[i]) DRV(cuMemcpyDtoH(host[i], d[i], sizes[i]), "cuMemcpyDtoH");
done:
    for (auto e : ev)
        if (e) cuEventDestroy(e);
    for (auto p : d)
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return rc;
}

extern "C" int ref_launch(const char *cubin, int n_kernels, const char *const *names, const unsigned *grids,
                          const unsigned *blocks, int n_bufs, const uint64_t *sizes, void *const *host,
                          const int *copy_back, char *err, int errlen) {
    return run(cubin, n_kernels, names, grids, blocks, n_bufs, sizes, host, copy_back, 0, nullptr, nullptr, nullptr,
               nullptr, 1, nullptr, err, errlen);
}

extern "C" int ref_time(const char *cubin, int n_kernels, const char *const *names, const unsigned *grids,
                        const unsigned *blocks, int n_bufs, const uint64_t *sizes, void *const *host,
                        const int *copy_back, int n_resets, const int *reset_buf, const uint64_t *reset_off,
                        const uint64_t *reset_len, const unsigned char *reset_val, int iters, float *ms, char *err,
                        int errlen) {
    return run(cubin, n_kernels, names, grids, blocks, n_bufs, sizes, host, copy_back, n_resets, reset_buf,
               reset_off, reset_len, reset_val, iters, ms, err, errlen);
}
