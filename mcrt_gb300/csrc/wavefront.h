// Wavefront state shared by the render entry points (kernels.cu, noalloc.cu): the per-
// wave control block, the SoA path-state layout, and the host helpers that lay it out
// and enqueue one wave of stage kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mcrt_gb300.h"
#include "layout.h"

namespace mcrt {

constexpr int kTraceBlock = 128;
constexpr int kStack = 64;
constexpr int kMaxDepth = 62;

// per-wave control block: the wave's path range and the queue counters of every depth
struct Ctrl
{
    int64_t base;
    int     count;
    int     chunk;
    int     qcount[kMaxDepth + 2];
    int     scount[kMaxDepth + 1][2];
};

// device pointers of one wave's state (SoA, `capacity` path slots)
struct WaveArgs
{
    Ctrl*               ctrl;
    const int64_t*      chunk_table;
    const JobGPU*       jobs;
    int                 num_jobs;
    int64_t             capacity;
    float4*             qo[2];  // ray queues (ping-pong by depth): origin + tmin
    float4*             qd[2];  //   direction + tmax
    int*                qp[2];  //   path slot of each queued ray
    float4*             hits;
    float4*             thr;      // throughput + flags
    float4*             rad;      // radiance gathered so far
    uint64_t*           rng;      // PCG32 state
    int*                pix;
    int*                job;
    float4*             nee_val;  // 4 next-event results per path slot (written by k_connect)
    int*                pend;     // per path slot: mask of next-event results not yet added
    float4*             so[2];    // next-event queues: [0] any-hit, [1] closest-hit
    float4*             sd[2];
    float4*             sv[2];
    int4*               sm[2];
    int64_t             shadow_cap;
    unsigned long long* stats;  // [0] extension rays, [1] next-event rays, [2..5] work counters
    int*                err;
};

// queues one k_shade launch reads and appends to (counts live in device memory)
struct QueueSel
{
    const int* count;       // rays in the input queue
    int        qs;          // input ray queue; continuing rays go to queue qs ^ 1
    int*       next_count;  // append counter of queue qs ^ 1
    int*       scount;      // [2] append counters of the next-event queues (any-hit, closest-hit)
    int*       dead_count;  // streaming: append counter of the list of slots whose path ended
    int*       dead;        //   and the list (nullptr for waves)
    int        depth;       // waves: the vertex index of every queued path; streaming: -1
                            // (each slot keeps its own in bits 8.. of thr.w)
};

// streaming schedule: counters of one render (iteration parity selects the queue pair)
struct StreamCtrl
{
    int                qcount[2];  // ray queues
    int                dcount[2];  // lists of slots whose path ended
    int                scount[2];  // next-event queues of the current iteration
    int                pad[2];
    unsigned long long next;       // index of the next path to start
    unsigned long long finished;   // paths whose radiance is in the ring
};

struct StreamArgs
{
    StreamCtrl* ctrl;
    int*        dead[2];    // slot lists by iteration parity
    int64_t*    gid;        // path index held by each slot, -1: none
    float4*     ring;       // radiance of path g at g % ring_size (until its pixel resolves)
    int*        ring_cnt;   // per pixel, at its first path's ring index: paths finished
    int64_t     ring_size;
    int64_t     total;      // paths of the render
};

struct LaunchShape
{
    int grid_trace, grid_shade, grid_small, block;
};

// bytes of the per-path arrays for `capacity` slots (256-B aligned sub-arrays)
size_t wave_bytes(int64_t capacity);
// lays the per-path arrays out in [base, base + wave_bytes(capacity))
void carve_wave(WaveArgs& a, void* base, int64_t capacity);
// persistent grid sizes from the SM count and occupancy (queries only, no allocation)
LaunchShape launch_shape();
LaunchShape launch_shape_variant(bool stack32, bool regcap);
// one wave of stage launches on `st`: begin, raygen, (extend, shade, connect) x depth, resolve
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
int              scene_bvh_depth(const mcrt_scene* s);

}  // namespace mcrt
