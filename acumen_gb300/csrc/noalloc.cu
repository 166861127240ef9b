// Cross-correlation axis registration that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: an acquisition pipeline
// whose device memory was carved up in advance, or a host process whose
// framework allocator (a caching pool) already owns the whole device, or a
// time-critical thread that must not risk the implicit device
// synchronisation of cudaMalloc / cudaFree.  For them this entry point keeps
// its scratch -- the correlation sums of every lag and the argmax -- in a
// fixed array in the library's own device memory, which exists on every GPU
// that loads the library until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/acumen_gpu.h"
#include "ctx.h"
#include "prep.h"

namespace {

constexpr int kNoallocMaxLag = 2048;                      // kmax limit
constexpr int kNoallocSlots = 2 * kNoallocMaxLag + 1 + 2;  // lags + argmax word

// Shared scratch: per-lag correlation sums and the argmax index.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoallocSlots];

std::mutex g_noalloc_mu;
std::vector<void*> g_noalloc_addr;  // device address of g_noalloc_scratch, per device

// Resolves the array's device address on the current device once.  The host
// symbol g_noalloc_scratch is only a stand-in and must never be passed to a
// kernel.
int scratch_address(unsigned long long** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if ((int)g_noalloc_addr.size() <= dev) g_noalloc_addr.resize(dev + 1, nullptr);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return acu::set_err(nullptr, ACU_ERR_CUDA, "cudaGetSymbolAddress of the registration scratch failed: %s",
                                cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
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
    unsigned long long* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != ACU_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int nk = 2 * kmax + 1;
    unsigned long long* corr = scratch;
    int* best = reinterpret_cast<int*>(scratch + nk);
    // launch_xcorr zeroes the nk sums before accumulating into them
    acu::launch_xcorr(ndet, nrows, kmax, d_p0, d_p180, corr, best, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return acu::set_err(nullptr, ACU_ERR_CUDA, "xcorr launch failed: %s", cudaGetErrorString(e));
    long long h[2 * kNoallocMaxLag + 1];
    int bi = 0;
    e = cudaMemcpyAsync(h, corr, sizeof(long long) * nk, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bi, best, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return acu::set_err(nullptr, ACU_ERR_CUDA, "reading the correlation back failed: %s", cudaGetErrorString(e));
    double frac = 0.0;
    if (bi > 0 && bi < nk - 1) {
        const double cm = (double)h[bi - 1], c0 = (double)h[bi], cp = (double)h[bi + 1];
        const double den = cm - 2.0 * c0 + cp;
        if (den < 0.0) frac = 0.5 * (cm - cp) / den;
    }
    *k_best = bi - kmax;
    *k_sub = (double)(bi - kmax) + frac;
    if (corr_out)
        for (int i = 0; i < nk; ++i) corr_out[i] = h[i];
    return ACU_OK;
}
