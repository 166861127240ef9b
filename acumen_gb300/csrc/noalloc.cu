// Cross-correlation axis registration that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: an acquisition pipeline
// whose device memory was carved up in advance, or a host process whose
// framework allocator (a caching pool) already owns the whole device, or a
// time-critical thread that must not risk the implicit device
// synchronisation of cudaMalloc / cudaFree.  For them this entry point keeps
// its scratch -- the correlation sums of every lag, the argmax and the range
// flag -- in a fixed array in the library's own device memory, which exists on
// every GPU that has loaded the library's device code, until the process exits
// or the device is reset.  With CUDA's lazy loading (the default) that code is
// loaded on the first call on a device, and loading can allocate device
// memory: make the first call at start-up.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/acumen_gpu.h"
#include "ctx.h"
#include "prep.h"

namespace {

constexpr int kNoallocMaxLag = 2048;   // kmax limit

// Shared scratch: per-lag 128-bit correlation sums, the argmax index and the
// range flag (the layout of acu::xcorr_scratch_words), 8195 words = 64 KB.
constexpr int kNoallocWords = 2 * (2 * kNoallocMaxLag + 1) + 1;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoallocWords];

std::mutex g_noalloc_mu;
std::vector<void*> g_noalloc_addr;  // last resolved device address of g_noalloc_scratch, per device

// The array's device address on the current device.  The host symbol
// g_noalloc_scratch is only a stand-in and must never be passed to a kernel.
// Outside stream capture the address is looked up again on every call (a
// host-side table lookup), so a call after cudaDeviceReset, which reloads
// the library's device code and moves the array, gets the new address.
// During capture the last address resolved on this device is used: a first
// call outside capture must have resolved it.
int scratch_address(cudaStream_t st, unsigned long long** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "cudaStreamIsCapturing failed: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if ((int)g_noalloc_addr.size() <= dev) g_noalloc_addr.resize(dev + 1, nullptr);
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return acu::set_err(nullptr, ACU_ERR_CUDA, "cudaGetSymbolAddress of the registration scratch failed: %s",
                                cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    } else if (!g_noalloc_addr[dev]) {
        return acu::set_err(nullptr, ACU_ERR_INVALID,
                            "the first acu_xcorr_register_noalloc call on device %d is inside a stream capture; make "
                            "one call on this device before capturing",
                            dev);
    }
    *out = reinterpret_cast<unsigned long long*>(g_noalloc_addr[dev]);
    return ACU_OK;
}

}  // namespace

extern "C" int acu_xcorr_register_noalloc(int ndet, int nrows, const float* d_p0, const float* d_p180, int kmax,
                                          int64_t* corr_out, int* k_best, double* k_sub, void* stream)
{
    if (ndet < 2 || nrows < 1 || !d_p0 || !d_p180 || !k_best || !k_sub)
        return acu::set_err(nullptr, ACU_ERR_INVALID, "invalid cross-correlation arguments");
    if (kmax < 1 || kmax > kNoallocMaxLag)
        return acu::set_err(nullptr, ACU_ERR_INVALID,
                            "kmax=%d is outside 1..%d, the lag range of the fixed registration scratch", kmax,
                            kNoallocMaxLag);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* scratch = nullptr;
    int rc = scratch_address(st, &scratch);
    if (rc != ACU_OK) return rc;
    const size_t nw = acu::xcorr_scratch_words(kmax);
    // launch_xcorr clears the words this call uses before accumulating into them
    cudaError_t e = acu::launch_xcorr(ndet, nrows, kmax, d_p0, d_p180, scratch, st);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "cross-correlation launch failed: %s", cudaGetErrorString(e));
    unsigned long long h[kNoallocWords];
    e = cudaMemcpyAsync(h, scratch, sizeof(unsigned long long) * nw, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "reading the correlation back failed: %s", cudaGetErrorString(e));
    const char* why = "";
    rc = acu::xcorr_finish(kmax, h, corr_out, k_best, k_sub, &why);
    if (rc != ACU_OK) return acu::set_err(nullptr, rc, "cross-correlation registration: %s", why);
    return ACU_OK;
}
