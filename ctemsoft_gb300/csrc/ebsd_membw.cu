// Read-bandwidth probes of the memory hierarchy: the denominators of the
// pattern kernel's roofline, measured on the device it runs on.
//
// The pattern loop is a gather from a master pattern that stays resident in
// L2 (48 MB at 1001^2 x 11 bins) and whose neighbouring pixels hit the same
// nodes, so its algorithmic bytes are served mostly by L1 and L2 rather than
// HBM.  The copy-based HBM figure does not bound it; these probes measure
// the levels that do, with the loads the kernel uses (128-bit, read-only):
//
//   L1:  every CTA re-reads its own 16 KB block with L1-cached loads, so
//        after the first pass every request hits L1: the rate at which the
//        L1 data pipe returns 128-bit loads.
//   L2:  the grid sweeps a working set of the given size (48 MB: the
//        interleaved master) with loads that bypass L1 (ld.global.cg), after
//        one warming pass: the L2-to-SM rate, both dies' L2 included.
//   HBM: the same sweep over a working set several times the L2 size.
//
// Each probe is one launch of `passes` sweeps timed with CUDA events on a
// private stream; the best of `repeats` launches is returned.  Indices stay
// inside the buffer by construction (i < n4 in the sweeps, idx < 1024 within
// a CTA's block, blocks < n4 / 1024), and no loop waits on anything.
#include <cuda_runtime.h>

#include <algorithm>

#include "ebsd_internal.h"

namespace ebsd {

namespace {

constexpr int kProbeThreads = 256;
constexpr int kL1BlockFloat4 = 1024;  // 16 KB per CTA

__device__ __forceinline__ float4 ld_cg(const float4* p)
{
    float4 v;
    asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ float4 ld_ca(const float4* p)
{
    float4 v;
    asm volatile("ld.global.ca.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

// Sweep n4 float4 with L1-bypassing loads, `passes` times; four loads in
// flight per thread.  sink receives one value per thread (keeps the loads).
__global__ void __launch_bounds__(kProbeThreads) k_sweep_cg(const float4* __restrict__ buf,
                                                           long long n4, int passes,
                                                           float* __restrict__ sink)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    float acc = 0.0f;
    for (int r = 0; r < passes; ++r) {
        long long i = tid;
        for (; i + 3 * stride < n4; i += 4 * stride) {
            const float4 a = ld_cg(buf + i), b = ld_cg(buf + i + stride),
                         c = ld_cg(buf + i + 2 * stride), d = ld_cg(buf + i + 3 * stride);
            acc += (a.x + b.y) + (c.z + d.w);
        }
        for (; i < n4; i += stride) {
            const float4 a = ld_cg(buf + i);
            acc += a.x;
        }
    }
    sink[tid] = acc;
}

// Every CTA re-reads its own kL1BlockFloat4 float4 (blocks wrap around the
// buffer of n4 >= kL1BlockFloat4 float4) with L1-cached loads.
__global__ void __launch_bounds__(kProbeThreads) k_reread_ca(const float4* __restrict__ buf,
                                                            long long n4, int passes,
                                                            float* __restrict__ sink)
{
    const long long nblocks = n4 / kL1BlockFloat4;
    const float4* base = buf + (blockIdx.x % nblocks) * kL1BlockFloat4;
    float acc = 0.0f;
    for (int r = 0; r < passes; ++r) {
        // each pass maps the warps to other 512-byte runs of the block (an
        // XOR by a multiple of 32 float4 keeps every warp's 32 loads one
        // contiguous run), so no two passes load the same addresses in the
        // same order and the assembler cannot fold a pass into the previous
        const int swz = (r & 31) << 5;
#pragma unroll
        for (int k = 0; k < kL1BlockFloat4 / kProbeThreads; ++k) {
            const int idx = ((k * kProbeThreads + (int)threadIdx.x) ^ swz) & (kL1BlockFloat4 - 1);
            const float4 a = ld_ca(base + idx);
            acc += (a.x + a.y) + (a.z + a.w);
        }
    }
    sink[(long long)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

__global__ void k_fill(float4* buf, long long n4)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride)
        buf[i] = make_float4(1.0f, 2.0f, 3.0f, 4.0f);
}

}  // namespace

cudaError_t measure_read_bandwidth(int device, int level, long long bytes, int repeats,
                                   double* gbs, double* seconds)
{
    *gbs = 0.0;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    int sms = 0, per = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    const bool l1 = level == EBSD_BW_L1;
    if (l1)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_reread_ca, kProbeThreads, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_cg, kProbeThreads, 0);
    if (e != cudaSuccess) return e;
    const int grid = sms * std::max(per, 1);
    const long long n4 = std::max<long long>(bytes / 16, (long long)kL1BlockFloat4 * grid);
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    e = cudaMalloc(&buf, (size_t)n4 * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float) * (size_t)grid * kProbeThreads);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    if (e == cudaSuccess) {
        k_fill<<<grid, kProbeThreads, 0, s>>>(buf, n4);
        e = cudaGetLastError();
    }
    // passes per launch: 4096 re-reads of each CTA's block, 200 L2 sweeps,
    // 3 HBM sweeps (each launch a millisecond or more)
    const int passes = l1 ? 4096 : (level == EBSD_BW_L2 ? 200 : 3);
    const double moved = l1 ? (double)grid * kL1BlockFloat4 * 16.0 * passes
                            : (double)n4 * 16.0 * passes;
    double best = 1e30;
    for (int r = -1; r < std::max(repeats, 1) && e == cudaSuccess; ++r) {
        e = cudaEventRecord(a, s);
        if (e != cudaSuccess) break;
        if (l1)
            k_reread_ca<<<grid, kProbeThreads, 0, s>>>(buf, n4, passes, sink);
        else
            k_sweep_cg<<<grid, kProbeThreads, 0, s>>>(buf, n4, r < 0 ? 1 : passes, sink);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(b, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && r >= 0) best = std::min(best, (double)ms * 1e-3);
    }
    if (e == cudaSuccess && best < 1e30) {
        *gbs = moved / best / 1e9;
        if (seconds) *seconds = best;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (s) cudaStreamDestroy(s);
    cudaFree(sink);
    cudaFree(buf);
    return e;
}

}  // namespace ebsd
