// ref_harness.cu — runs the reference's own kernels (from a cubin built by
// oracle/ref_build.py) on buffers prepared by the caller.
//
// TEST INFRASTRUCTURE ONLY: the GPU parity tests use it to pin the oracle to
// the reference itself.  It knows nothing about the reference's structs: the
// caller passes the bytes of every buffer (laid out from the reference's own
// headers), the kernel names and launch shapes; the harness copies the
// buffers to the device, launches the kernels in order with the buffers as
// their pointer arguments, and copies the requested buffers back.
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

extern "C" int ref_launch(const char *cubin, int n_kernels, const char *const *names, const unsigned *grids,
                          const unsigned *blocks, int n_bufs, const uint64_t *sizes, void *const *host,
                          const int *copy_back, char *err, int errlen) {
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    std::vector<CUdeviceptr> d((size_t)n_bufs, 0);
    std::vector<void *> params((size_t)n_bufs);
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
    for (int k = 0; k < n_kernels; ++k) {
        CUfunction f;
        DRV(cuModuleGetFunction(&f, mod, names[k]), "cuModuleGetFunction");
        DRV(cuLaunchKernel(f, grids[k], 1, 1, blocks[k], 1, 1, 0, nullptr, params.data(), nullptr), "cuLaunchKernel");
        DRV(cuCtxSynchronize(), "kernel");
    }
    for (int i = 0; i < n_bufs; ++i)
        if (copy_back[i] && sizes[i]) DRV(cuMemcpyDtoH(host[i], d[i], sizes[i]), "cuMemcpyDtoH");
done:
    for (auto p : d)
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return rc;
}
