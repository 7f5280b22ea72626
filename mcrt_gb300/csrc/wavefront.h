// Wavefront state shared by the render entry points (kernels.cu, noalloc.cu): the control
// block, the SoA layout of the queues, and the host helpers that lay it out and enqueue
// iterations of stage kernels.
//
// Path state travels with its ray through the queues (no per-path slots): every stage
// reads and writes its items by queue position, so all per-path traffic is coalesced.
// One iteration (parity p = iteration & 1):
//   k_iter_begin  zero the counters this iteration appends to; admit new paths: the
//                 queue is topped up to its capacity from the path counter, bounded by
//                 the admission limit (the whole render when streaming, the current wave
//                 for the wave schedule)
//   k_regen       finish the paths that ended in the previous iteration (their
//                 next-event results are in): radiance into the ring, pixel resolved in
//                 sample order when its last path finished; start the admitted paths
//   k_extend      closest hit of every ray of queue p
//   k_shade       one vertex per ray: continuing paths to queue p ^ 1, ended paths to
//                 the finished list p ^ 1, next-event rays to the next-event queues
//   k_connect     trace the next-event rays; each result goes to the slot its path
//                 will read next (queue p ^ 1 position or finished-list position)
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mcrt_gb300.h"
#include "layout.h"

namespace mcrt {

constexpr int kTraceBlock = 128;
constexpr int kStack = 64;
// the smaller traversal stack, used when the tree is shallow enough (MCRT_VARIANT_STACK32)
constexpr int kSmallStack = 32;
// Traversal kernels under MCRT_VARIANT_REGCAP: __launch_bounds__(kTraceBlock, kTraceMinBlocks)
// caps them at 56 registers, so 9 blocks (36 warps) fit an SM.  Measured on the cfg1 frame:
// 8 blocks (64 registers) 52.6 / 59.9 ms extend / connect, 9 blocks 52.2 / 56.7, 10 blocks
// (48 registers, spills) 54.4 / 57.0.
#ifndef MCRT_TRACE_MIN_BLOCKS
#define MCRT_TRACE_MIN_BLOCKS 9
#endif
constexpr int kTraceMinBlocks = MCRT_TRACE_MIN_BLOCKS;
// The any-hit next-event kernel under MCRT_VARIANT_REGCAP: 40 registers, 12 blocks per SM
// (40 B of spills).  Next-event stage per cfg1 frame: 10 blocks (48 registers, no spills)
// 33.96 ms, 12 blocks 32.53 (an earlier build, with tmin read from the queue and more
// spills: 9 blocks 37.5, 10 blocks 36.5, 12 blocks 38.8).  Its adjoint build keeps 10.
#ifndef MCRT_ANYHIT_MIN_BLOCKS
#define MCRT_ANYHIT_MIN_BLOCKS 12
#endif
constexpr int kAnyHitMinBlocks = MCRT_ANYHIT_MIN_BLOCKS;
constexpr int kAnyHitMinBlocksAdj = 10;
constexpr int kMaxDepth = 62;
constexpr int64_t kMaxQueue = int64_t(1) << 27;     // rays per queue (result indices stay in int)
// Streaming schedule default: 64 M rays (49 GB of queues).  Per cfg1 frame (67 M paths):
// 1 / 2 / 4 / 8 / 16 / 32 / 64 M rays 184.6 / 146.9 / 128.1 / 118.3 / 113.4 / 111.4 /
// 109.5 ms -- fewer, longer launches amortise each launch's ramp and tail.  If its
// allocation fails the default halves itself, down to kMinDefaultQueue.
constexpr int64_t kDefaultQueue = int64_t(1) << 26;
constexpr int64_t kMinDefaultQueue = int64_t(1) << 20;

// counters of one render
struct Ctrl
{
    int                qcount[2];  // ray queues (by parity)
    int                dcount[2];  // lists of finished paths (by parity)
    int                scount[2];  // next-event queues of the current iteration: any-hit, closest-hit
    int                new_base;   // this iteration's admitted paths: first queue position
    int                new_count;  //   and how many
    int                chunk;      // wave schedule: index of the current wave
    int                fetch[3];   // rays taken so far by this iteration's k_extend, k_connect<0>, k_connect<1>
    unsigned long long next;      // index of the next path to admit
    unsigned long long limit;     // admission limit (exclusive)
    unsigned long long new_g;     // index of the first path admitted this iteration
    unsigned long long finished;  // paths whose radiance reached the ring
};

// device pointers of one render's state (SoA, `capacity` rays per queue)
struct WaveArgs
{
    Ctrl*          ctrl;
    const int64_t* chunk_table;  // wave schedule: wave boundaries (path indices)
    const JobGPU*  jobs;
    int            num_jobs;
    int64_t        capacity;
    // ray queues by parity.  o.w = job index, d.w = pixel index (int bits; extension rays
    // always span [kEpsRay, inf)); thr.w = flags | vertex << 8 | pending mask << 16;
    // rad.w = sample index (int bits)
    float4*   qo[2];
    float4*   qd[2];
    float4*   qthr[2];
    float4*   qrad[2];
    uint64_t* qrng[2];
    float4*   hits;  // by position of the current queue
    // finished paths by parity: radiance (w = sample), {pixel, job, pending mask, 0}
    float4* drad[2];
    int4*   dmeta[2];
    // next-event results by parity: [4 i + s] for queue position i, [4 capacity + 4 j + s]
    // for finished-list position j
    float4* nev[2];
    // next-event queues: [0] any-hit, [1] closest-hit; origin + stop distance (so.w: a
    // closest-hit ray stops at a nearer hit, emitter_span), direction + tmax, value,
    // meta = {result index, type | light << 2, pixel, job}; tmin is kEpsRay for all
    float4* so[2];
    float4* sd[2];
    float4* sv[2];
    int4*   sm[2];
    int64_t shadow_cap;
    // per-path radiance of path g at g % ring_size until its pixel resolves; per pixel
    // (at its first path's ring index) the count of its finished paths
    float4*             ring;
    int*                ring_cnt;
    int64_t             ring_size;
    unsigned long long* stats;  // [0] extension rays, [1] next-event rays, [2..5] work counters
    int*                err;
    // traversal kernels: each warp takes the next 32 queue entries from a counter until the
    // queue is empty (1), or every thread strides over the queue by the grid size (0)
    int batch_fetch;
    // adjoint (paths replayed through the same queues, JobGPU::image = dL/dimage): the
    // material ids of a path's parameterised Lambert vertices, 16 bits each, at most
    // kAdjLog per path (thr.w bits 20.. hold the count), two uint4 per queue position and
    // per finished-list position; gradients (in shared memory per block when grad_shared)
    uint4* qlog[2];
    uint4* dlog[2];
    float* g_albedo;
    float* g_emis;
    int    n_albedo;
    int    n_emis;
    int    grad_shared;
};

constexpr int kAdjLog = 16;

struct LaunchShape
{
    int grid_trace, grid_any, grid_connect, grid_shade, grid_regen, grid_small, block;  // grid_any: any-hit k_connect
    bool fast_only = false;  // every job traverses in FAST mode: kernels built without the REF traversal
    int  lights = 3;         // light kinds of the jobs (1 environment, 2 area, 3 both): the k_shade build
};

// sub-array allocator: consecutive 256-B aligned pieces of one block
struct Carver
{
    char* p;
    void* take(size_t n)
    {
        size_t off = (reinterpret_cast<uintptr_t>(p) + 255) & ~static_cast<uintptr_t>(255);
        char*  r = reinterpret_cast<char*>(off);
        p = r + n;
        return r;
    }
};

// bytes of the queues for `capacity` rays (256-B aligned sub-arrays)
size_t queue_bytes(int64_t capacity);
// lays the queues out in [base, base + queue_bytes(capacity))
void carve_queues(WaveArgs& a, void* base, int64_t capacity);
// bytes of a ring of `entries` paths (radiance + per-pixel counts)
size_t ring_bytes(int64_t entries);
void   carve_ring(WaveArgs& a, void* base, int64_t entries);
// ring entries the streaming schedule needs: paths admitted during the lifetime of one
// path (a path is finished at most max_depth + 2 iterations after admission, at most
// `capacity` paths are admitted per iteration) plus one pixel's samples
int64_t stream_ring_entries(int64_t capacity, int max_depth, int64_t max_spp, int64_t total);
// iterations of one wave of the wave schedule (even, so every wave starts on parity 0)
int wave_iterations(int max_depth);
// persistent grid sizes from the SM count and occupancy (queries only, no allocation)
LaunchShape launch_shape();
LaunchShape launch_shape_variant(bool stack32, bool regcap, bool fast_only = false);
// starts a render: zeroes the counters and sets the admission limit (`limit`; with `waves`
// nothing is admitted until the first wave's k_wave_next) -- one kernel, so it may run
// inside a stream capture; the per-pixel counts of the ring must be zero
void enqueue_render_begin(const WaveArgs& a, bool waves, int64_t limit, cudaStream_t st);
// one wave of the wave schedule with the plain kernels (no counters, 64-entry stacks)
void enqueue_wave_plain(const WaveArgs& a, int max_depth, const LaunchShape& ls, cudaStream_t st);
// Camera::Camera in float with the reference's operation order
CameraGPU make_camera(const mcrt_camera& c);
// argument checks shared by the render entry points; sets the last error
int validate_job(const mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p);
// records the calling thread's last error message and returns `code`
int set_error(int code, const std::string& msg);
// read-only facts about a scene handle
const SceneView& scene_view(const mcrt_scene* s);
int              scene_device(const mcrt_scene* s);
int              scene_stack_depth(const mcrt_scene* s, int traverse);  // see the stack checks

}  // namespace mcrt
