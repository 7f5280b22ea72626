// mcrt_probe_l2_read: the L2 read bandwidth of the current GPU, the second roofline
// denominator of the traversal kernels (their node and triangle reads mostly hit L2).
//
// A buffer smaller than L2 is read once to make it resident, then `reps` times by one
// launch: every thread streams 16-B loads with the .cg hint (cached in L2, not in L1), so
// each pass reaches L2, not the SM caches.  bytes * reps over the launch's event time.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mcrt_gb300.h"
#include "wavefront.h"

namespace {

__global__ void __launch_bounds__(256) k_l2_read(const float4* __restrict__ buf, int64_t n, int reps,
                                                 unsigned* __restrict__ sink)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned      acc = 0u;
    for (int r = 0; r < reps; ++r)
    {
        int64_t i = t;
        for (; i + 3 * stride < n; i += 4 * stride)  // four independent loads in flight
        {
            const float4 v0 = __ldcg(buf + i), v1 = __ldcg(buf + i + stride);
            const float4 v2 = __ldcg(buf + i + 2 * stride), v3 = __ldcg(buf + i + 3 * stride);
            acc ^= __float_as_uint(v0.x) ^ __float_as_uint(v1.y) ^ __float_as_uint(v2.z) ^ __float_as_uint(v3.w);
            acc ^= __float_as_uint(v0.w) ^ __float_as_uint(v1.z) ^ __float_as_uint(v2.y) ^ __float_as_uint(v3.x);
            acc ^= __float_as_uint(v0.y) ^ __float_as_uint(v1.x) ^ __float_as_uint(v2.w) ^ __float_as_uint(v3.z);
            acc ^= __float_as_uint(v0.z) ^ __float_as_uint(v1.w) ^ __float_as_uint(v2.x) ^ __float_as_uint(v3.y);
        }
        for (; i < n; i += stride)
        {
            const float4 v = __ldcg(buf + i);
            acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^ __float_as_uint(v.w);
        }
    }
    if (acc == 0x9e3779b9u) sink[t & 255] = acc;  // keeps the loads; practically never stores
}

}  // namespace

extern "C" int mcrt_probe_l2_read(int64_t bytes, int32_t reps, float* gbs, void* stream)
{
    using namespace mcrt;
    if (!gbs || bytes < (int64_t(1) << 20) || bytes > (int64_t(96) << 20) || reps < 1 || reps > 1000)
        return set_error(MCRT_ERR_INVALID_ARGUMENT,
                         "mcrt_probe_l2_read: bytes must be in [1 MB, 96 MB], reps in [1, 1000]");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float4*      buf = nullptr;
    unsigned*    sink = nullptr;
    cudaEvent_t  e0 = nullptr, e1 = nullptr;
    auto         release = [&]() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(buf);
        cudaFree(sink);
    };
    const int64_t n = bytes / 16;
    if (cudaMalloc(&buf, n * 16) != cudaSuccess || cudaMalloc(&sink, 256 * sizeof(unsigned)) != cudaSuccess)
    {
        release();
        return set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_probe_l2_read: allocation failed");
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (sms > 0 ? sms : 1) * 8;
    cudaError_t e = cudaMemsetAsync(buf, 0x3c, n * 16, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess)
    {
        k_l2_read<<<grid, 256, 0, st>>>(buf, n, 1, sink);  // make the buffer L2-resident
        cudaEventRecord(e0, st);
        k_l2_read<<<grid, 256, 0, st>>>(buf, n, reps, sink);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
    }
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    release();
    if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("mcrt_probe_l2_read: ") + cudaGetErrorString(e));
    *gbs = ms > 0.f ? static_cast<float>(static_cast<double>(n) * 16.0 * reps / (ms * 1e-3) / 1e9) : 0.f;
    return MCRT_OK;
}
