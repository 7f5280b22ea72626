// mcrt_render_noalloc: the forward render for callers that cannot call cudaMalloc (or
// cudaFree) while they render:
//   - plug-ins living inside a host application that owns all device memory through its
//     own pool or arena and forbids allocations behind its back, so that its own
//     accounting and budget stay true;
//   - latency-bound render loops sharing the GPU with other streams: cudaMalloc and
//     cudaFree may synchronise the device and stall every stream on it;
//   - processes that reserve their memory at start-up under a hard budget and must not
//     grow afterwards.
//
// The wavefront needs scratch memory for its queues, its per-path ring and its counters.
// Here it lives in a file-scope static __device__ array of fixed size
// (kNoAllocScratchBytes, about 50 MB): no cudaMalloc, cudaFree, event, graph or library
// allocation happens in the call.  The array belongs to this file's module, so every GPU
// that loads it holds it until the process exits.  The render runs the wave schedule with
// waves of at most kNoAllocPaths paths and at most kNoAllocWaves waves; requests beyond
// either are rejected with MCRT_ERR_INVALID_ARGUMENT.
//
// Host code cannot use the array's name as a device address (on the host it is a
// stand-in).  The first call on a device takes the array's device address with
// cudaGetSymbolAddress while that device is current and caches it per device ordinal;
// make that first call before any stream capture begins.  The cached address does not
// survive cudaDeviceReset (the module is loaded again, possibly elsewhere): do not reset a
// device between calls.  Every call shares the one array, so two calls whose work
// overlaps on the GPU (different streams, or another host thread) race: serialise them.
// Everything that must start at zero is cleared at the start of each call.  The call
// leaves the calling thread's current device as it found it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mcrt_gb300.h"
#include "wavefront.h"

namespace mcrt {
namespace {

constexpr int64_t kNoAllocPaths = 65536;  // paths per wave (rays per queue)
constexpr int64_t kNoAllocWaves = 65536;  // waves per render
constexpr size_t  kHeaderBytes = 4096;    // Ctrl, stats, error word, one JobGPU
constexpr size_t  kChunkBytes = sizeof(int64_t) * (kNoAllocWaves + 1);
// queue_bytes(kNoAllocPaths) and ring_bytes(kNoAllocPaths), rounded up; checked at set-up
constexpr size_t kQueueBytes = (static_cast<size_t>(kNoAllocPaths) * 736 + 256 * 32 + 255) & ~size_t(255);
constexpr size_t kRingBytes = (static_cast<size_t>(kNoAllocPaths) * 20 + 512 + 255) & ~size_t(255);
constexpr size_t kNoAllocScratchBytes = kHeaderBytes + kChunkBytes + kQueueBytes + kRingBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mu;
void*         g_scratch_ptr[kMaxDevices] = {};

// restores the calling thread's current device on every return path
struct CurrentDeviceGuard
{
    int  saved = -1;
    CurrentDeviceGuard()
    {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
    }
    ~CurrentDeviceGuard()
    {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

struct Layout
{
    Ctrl*               ctrl;
    unsigned long long* stats;
    int*                err;
    JobGPU*             job;
    int64_t*            chunks;
    void*               queues;
    void*               ring;
};

Layout layout(void* base)
{
    char*  p = static_cast<char*>(base);
    Layout l;
    l.ctrl = reinterpret_cast<Ctrl*>(p);
    l.stats = reinterpret_cast<unsigned long long*>(p + 2048);
    l.err = reinterpret_cast<int*>(p + 2048 + 8 * sizeof(unsigned long long));
    l.job = reinterpret_cast<JobGPU*>(p + 2304);
    l.chunks = reinterpret_cast<int64_t*>(p + kHeaderBytes);
    l.queues = p + kHeaderBytes + kChunkBytes;
    l.ring = p + kHeaderBytes + kChunkBytes + kQueueBytes;
    return l;
}
static_assert(sizeof(Ctrl) <= 2048, "Ctrl must fit the scratch header");
static_assert(2304 + sizeof(JobGPU) <= kHeaderBytes, "JobGPU must fit the scratch header");

// writes the job and the wave boundaries (`per_wave` paths, the last one shorter)
__global__ void k_noalloc_setup(JobGPU job, JobGPU* dst, int64_t* chunks, int64_t total, int64_t per_wave,
                                int64_t waves)
{
    int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i == 0) *dst = job;
    for (; i <= waves; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        chunks[i] = i * per_wave < total ? i * per_wave : total;
}

}  // namespace
}  // namespace mcrt

using namespace mcrt;

extern "C" int mcrt_render_noalloc(mcrt_scene* scene, const mcrt_camera* camera, const mcrt_render_params* params,
                                   float* rgb_out_device, mcrt_render_stats* stats, void* stream)
{
    try
    {
        int rc = validate_job(scene, camera, params);
        if (rc) return rc;
        if (!rgb_out_device)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_render_noalloc: rgb_out must be a device pointer");
        if (params->ptr_mode != MCRT_PTR_DEVICE)
            return set_error(MCRT_ERR_INVALID_ARGUMENT,
                             "mcrt_render_noalloc takes device buffers only (ptr_mode = MCRT_PTR_DEVICE)");
        if (scene_stack_depth(scene, params->traverse) + 2 >= kStack)
            return set_error(MCRT_ERR_STACK_OVERFLOW, "BVH deeper than the traversal stack");
        if (params->spp > kNoAllocPaths)
            return set_error(MCRT_ERR_INVALID_ARGUMENT,
                             "mcrt_render_noalloc: spp " + std::to_string(params->spp) + " exceeds the " +
                                 std::to_string(kNoAllocPaths) + " path slots of its fixed scratch");
        const int64_t px = static_cast<int64_t>(camera->width) * camera->height;
        const int64_t total = px * params->spp;
        const int64_t per_wave = (kNoAllocPaths / params->spp) * params->spp;  // whole pixels per wave
        const int64_t waves = (total + per_wave - 1) / per_wave;
        if (waves > kNoAllocWaves)
            return set_error(MCRT_ERR_INVALID_ARGUMENT,
                             "mcrt_render_noalloc: " + std::to_string(total) + " paths need " +
                                 std::to_string(waves) + " waves, more than the " + std::to_string(kNoAllocWaves) +
                                 " its fixed scratch holds (at most " +
                                 std::to_string(kNoAllocWaves * per_wave) + " paths per call)");
        const int dev = scene_device(scene);
        if (dev < 0 || dev >= kMaxDevices) return set_error(MCRT_ERR_INVALID_ARGUMENT, "device index out of range");
        CurrentDeviceGuard keep_device;
        cudaError_t        e = cudaSetDevice(dev);
        if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        // a launch error left by the caller's earlier work is not this call's: clear it so
        // the check after the launches below sees only these launches
        (void)cudaGetLastError();
        void* base = nullptr;
        {
            std::lock_guard<std::mutex> lock(g_setup_mu);
            if (!g_scratch_ptr[dev])
            {
                if (queue_bytes(kNoAllocPaths) > kQueueBytes || ring_bytes(kNoAllocPaths) > kRingBytes)
                    return set_error(MCRT_ERR_INTERNAL, "no-alloc scratch smaller than one wave's state");
                void* p = nullptr;
                e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
                if (e != cudaSuccess || !p)
                    return set_error(MCRT_ERR_CUDA,
                                     std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
                g_scratch_ptr[dev] = p;
            }
            base = g_scratch_ptr[dev];
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        Layout       L = layout(base);
        JobGPU       J;
        J.scene = scene_view(scene);
        J.cam = make_camera(*camera);
        J.width = camera->width;
        J.height = camera->height;
        J.spp = params->spp;
        J.max_depth = params->max_depth;
        J.rr_depth = params->rr_depth;
        J.traverse = params->traverse;
        J.seed = params->seed;
        J.path_offset = 0;
        J.image = rgb_out_device;
        WaveArgs a{};
        carve_queues(a, L.queues, kNoAllocPaths);
        carve_ring(a, L.ring, kNoAllocPaths);  // a wave's paths finish before the next wave starts
        a.ctrl = L.ctrl;
        a.chunk_table = L.chunks;
        a.jobs = L.job;
        a.num_jobs = 1;
        a.stats = L.stats;
        a.err = L.err;
        a.batch_fetch = 1;
        // the array keeps the previous call's contents: clear what must start at zero
        e = cudaMemsetAsync(L.stats, 0, 8 * sizeof(unsigned long long), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(L.err, 0, sizeof(int), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(a.ring_cnt, 0, sizeof(int) * kNoAllocPaths, st);
        if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        k_noalloc_setup<<<static_cast<int>((waves + 256) / 256), 256, 0, st>>>(J, L.job, L.chunks, total, per_wave,
                                                                             waves);
        LaunchShape ls = launch_shape();
        // the shading build of mcrt_render for this scene, so both render the same image
        ls.lights = (J.scene.env_w > 0 ? 1 : 0) | (J.scene.light_area > 0.f ? 2 : 0);
        if (ls.lights == 0) ls.lights = 3;
        enqueue_render_begin(a, true, 0, st);
        for (int64_t k = 0; k < waves; ++k) enqueue_wave_plain(a, params->max_depth, ls, st);
        e = cudaGetLastError();
        if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
        unsigned long long hstats[8];
        int                herr = 0;
        e = cudaMemcpyAsync(hstats, L.stats, sizeof(hstats), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
        if (stats)
        {
            *stats = mcrt_render_stats{};
            stats->paths = total;
            stats->extension_rays = static_cast<int64_t>(hstats[0]);
            stats->shadow_rays = static_cast<int64_t>(hstats[1]);
            stats->waves = static_cast<int32_t>(waves);
            const int iters = wave_iterations(params->max_depth);
            stats->kernel_launches = static_cast<int32_t>(2 + waves * (1 + ((ls.lights & 2) ? 6 : 5) * iters));
            stats->extend_launches = static_cast<int32_t>(waves * iters);
            stats->d2h_bytes = static_cast<int64_t>(sizeof(hstats) + sizeof(herr));
        }
        if (herr & 1) return set_error(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
        if (herr & 2) return set_error(MCRT_ERR_QUEUE_OVERFLOW, "queue overflow");
        return MCRT_OK;
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_render_noalloc");
    }
}
