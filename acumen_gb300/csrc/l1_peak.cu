// L1 load-bandwidth probe: the measured ceiling of the gather kernels
// (the projector and the backprojection run from L1 and L2, not from HBM).
//
// Every block reads the same 64 KB buffer over and over with 128-bit
// non-coherent loads (ld.global.nc.v4.f32, volatile inline PTX, so the
// compiler can neither merge nor hoist them): after the first pass the buffer
// sits in each SM's L1, so the loop measures the L1 data path alone.  A warp's
// load covers 512 consecutive bytes, four aligned 128-byte lines, the access
// pattern of the pixel-line projector; the eight loads of an iteration and
// consecutive iterations touch different lines.  Reports bytes per second over all
// SMs, bytes per SM clock (the clock taken from the SM's own cycle counter
// over the timed kernel) and that clock.  Prints one JSON line.
//
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 l1_peak.cu -o l1_peak
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

namespace {

constexpr int kWords = 4096;        // float4 words in the buffer: 64 KB
constexpr int kThreads = 256;
constexpr int kUnroll = 8;

__device__ __forceinline__ float4 ld_nc_v4(const float4* p)
{
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

__global__ void __launch_bounds__(kThreads, 4) k_l1_read(const float4* __restrict__ buf, int reps, float* out,
                                                      long long* cycles)
{
    const long long c0 = clock64();
    float a[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) a[u] = 0.f;
    // thread t starts at word t and strides by the block, so each warp reads
    // 32 consecutive words (512 bytes) per load; indices wrap inside 64 KB,
    // and an iteration advances by 8 x 256 words, half the buffer
    int idx = threadIdx.x;
#pragma unroll 1
    for (int r = 0; r < reps; ++r) {
        float4 v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) v[u] = ld_nc_v4(buf + ((idx + u * kThreads) & (kWords - 1)));
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) a[u] += (v[u].x + v[u].w) + (v[u].y + v[u].z);
        idx = (idx + kUnroll * kThreads) & (kWords - 1);
    }
    float s = 0.f;
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) s += a[u];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    const long long c1 = clock64();
    if (threadIdx.x == 0) cycles[blockIdx.x] = c1 - c0;
}

#define CHECK(x)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess) {                                                        \
            std::printf("{\"error\": \"%s: %s\"}\n", #x, cudaGetErrorString(e_));       \
            return 1;                                                                   \
        }                                                                               \
    } while (0)

}  // namespace

int main()
{
    int dev = 0, sms = 0;
    CHECK(cudaGetDevice(&dev));
    CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks_per_sm = 4, nblk = sms * blocks_per_sm, reps = 4096;
    float4* buf = nullptr;
    float* out = nullptr;
    long long* cyc = nullptr;
    CHECK(cudaMalloc(&buf, sizeof(float4) * kWords));
    CHECK(cudaMalloc(&out, sizeof(float) * nblk * kThreads));
    CHECK(cudaMalloc(&cyc, sizeof(long long) * nblk));
    std::vector<float4> h(kWords);
    for (int i = 0; i < kWords; ++i) h[i] = make_float4(1e-7f * i, 1e-7f, 0.f, 1e-8f);
    CHECK(cudaMemcpy(buf, h.data(), sizeof(float4) * kWords, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    CHECK(cudaEventCreate(&e0));
    CHECK(cudaEventCreate(&e1));
    for (int w = 0; w < 3; ++w) k_l1_read<<<nblk, kThreads>>>(buf, reps, out, cyc);
    CHECK(cudaGetLastError());
    CHECK(cudaDeviceSynchronize());
    float best_ms = 1e30f;
    double best_cyc = 0;
    for (int it = 0; it < 10; ++it) {
        CHECK(cudaEventRecord(e0));
        k_l1_read<<<nblk, kThreads>>>(buf, reps, out, cyc);
        CHECK(cudaEventRecord(e1));
        CHECK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CHECK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            std::vector<long long> hc(nblk);
            CHECK(cudaMemcpy(hc.data(), cyc, sizeof(long long) * nblk, cudaMemcpyDeviceToHost));
            best_ms = ms;
            best_cyc = (double)*std::max_element(hc.begin(), hc.end());
        }
    }
    const double bytes = (double)nblk * kThreads * reps * kUnroll * sizeof(float4);
    const double gbps = bytes / (best_ms * 1e-3) / 1e9;
    // one wave: the four blocks of an SM are resident together, so the longest
    // block's cycle count spans the kernel; the SM clock is cycles / time
    const double mhz = best_cyc / (best_ms * 1e-3) / 1e6;
    const double per_clk_sm = bytes / sms / best_cyc;
    std::printf("{\"l1_gbps\": %.1f, \"bytes_per_clk_per_sm\": %.2f, \"sm_mhz_from_cycles\": %.0f, \"sms\": %d, "
                "\"ms\": %.3f, \"bytes\": %.0f, \"how\": \"ld.global.nc.v4.f32 over a 64 KB L1-resident buffer, "
                "%d blocks x %d threads, %d x %d loads per thread, best of 10, CUDA events\"}\n",
                gbps, per_clk_sm, mhz, sms, best_ms, bytes, nblk, kThreads, reps, kUnroll);
    cudaFree(buf);
    cudaFree(out);
    cudaFree(cyc);
    return 0;
}
