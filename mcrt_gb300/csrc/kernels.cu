// CUDA kernels (sm_103a) and the C ABI of mcrt_gb300.h.
//
// Kernels:
//   k_trace<ANY, MODE, STACK, MINB>  batch closest/any-hit queries (SceneBVH::intersect / occluded)
//   wavefront iterations (wavefront.h; all graph-capturable: every count is read from
//   device memory, grids are fixed):
//     k_render_begin, k_wave_next, k_iter_begin   counters and admission
//     k_regen            finish ended paths (ring, in-order pixel resolve) and start
//                        camera paths with the tent filter (demo_pt.cpp:689-708)
//     k_extend           closest hit of the ray queue
//     k_shade            one vertex of rayTrace (demo_pt.cpp:523-651): emission, NEE with
//                        MIS against the environment and the area lights, continuation,
//                        Russian roulette, over windows of queue entries sorted by
//                        material in shared memory; continuing paths, ended paths and
//                        next-event rays are appended to SoA queues by warp ballot /
//                        warp prefix sum + one atomic per warp
//     k_connect          next-event rays: any hit (environment) or bounded closest hit
//                        (area lights, which must hit the sampled emitter), MIS-weighted
//   k_adjoint            path-replay adjoint (one thread per path, replayed from its seed)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "device.cuh"
#include "estimator.cuh"
#include "host.h"
#include "wavefront.h"

namespace mcrt {


// ---------------------------------------------------------------------------
// batch trace
// ---------------------------------------------------------------------------
// Each warp takes the next 32 consecutive rays from a counter until the batch is done (the
// wavefront traversal kernels' warp batch fetch); STACK / MINB as the wavefront's builds:
// 32-entry stacks when the tree is shallow enough, registers capped for MINB blocks per SM
// in FAST mode (MODE 0, a build without the reference traversal), the general build in REF
// mode (MODE 1).
template <bool ANY, int MODE, int STACK, int MINB>
__global__ void __launch_bounds__(kTraceBlock, MINB)
    k_trace(SceneView s, const float4* __restrict__ rays, int64_t n, float4* __restrict__ hits, int* __restrict__ occ,
            int* err, unsigned long long* fetch)
{
    __shared__ int stack[STACK * kTraceBlock];
    int*           st = stack + threadIdx.x;
    const int      lane = threadIdx.x & 31;
    while (true)
    {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(fetch, 32ull);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= static_cast<unsigned long long>(n)) break;
        const int64_t i = static_cast<int64_t>(b) + lane;
        if (i >= n) continue;
        float4 a = rays[2 * i], d = rays[2 * i + 1];
        Hit    h;
        bool any = trace_ray<ANY, STACK, false, MODE == 1>(s, MODE, xyz(a), xyz(d), a.w, d.w, st, kTraceBlock, h, err);
        if (ANY)
            occ[i] = any ? 1 : 0;
        else
            hits[i] = any ? make_float4(h.t, h.u, h.v, __int_as_float(h.prim))
                          : make_float4(__int_as_float(0x7f800000), 0.f, 0.f, __int_as_float(-1));
    }
}

// ---------------------------------------------------------------------------
// wavefront stages (the iteration is described in wavefront.h)
// ---------------------------------------------------------------------------
// warp-reduced add of per-thread work counters into stats[slot], stats[slot + 1]
__device__ __forceinline__ void flush_count(unsigned long long* stats, int slot, const TraceCount& c)
{
    unsigned long long nn = c.nodes, tt = c.tris;
    for (int off = 16; off > 0; off >>= 1)
    {
        nn += __shfl_down_sync(0xffffffffu, nn, off);
        tt += __shfl_down_sync(0xffffffffu, tt, off);
    }
    if ((threadIdx.x & 31) == 0 && (nn | tt))
    {
        atomicAdd(&stats[slot], nn);
        atomicAdd(&stats[slot + 1], tt);
    }
}

__device__ __forceinline__ int find_job(const JobGPU* jobs, int num_jobs, int64_t g)
{
    int lo = 0, hi = num_jobs - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].path_offset <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// warp-aggregated append: returns this lane's first slot for `k` items
__device__ __forceinline__ int warp_append(int* counter, int k)
{
    const int lane = threadIdx.x & 31;
    int       incl = k;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
        int v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - k;
}

// adds a path's pending next-event results (slots[0..3], bits of `mask`) in slot order:
// the order in which rayTrace adds them (deterministic sum)
__device__ __forceinline__ float4 add_pending(const float4* slots, int mask, float4 r)
{
    for (int s = 0; s < 4; ++s)
        if (mask & (1 << s))
        {
            float4 v = slots[s];
            r.x += v.x;
            r.y += v.y;
            r.z += v.z;
        }
    return r;
}

// counters of a new render; the wave schedule admits nothing until k_wave_next
__global__ void k_render_begin(WaveArgs a, int waves, int64_t limit)
{
    Ctrl* c = a.ctrl;
    c->qcount[0] = c->qcount[1] = 0;
    c->dcount[0] = c->dcount[1] = 0;
    c->scount[0] = c->scount[1] = 0;
    c->new_base = c->new_count = 0;
    c->chunk = -1;
    c->fetch[0] = c->fetch[1] = c->fetch[2] = 0;
    c->next = 0;
    c->limit = waves ? 0ull : static_cast<unsigned long long>(limit);
    c->new_g = 0;
    c->finished = 0;
}

// wave schedule: admit the next wave's paths
__global__ void k_wave_next(WaveArgs a)
{
    Ctrl* c = a.ctrl;
    c->chunk += 1;
    c->limit = static_cast<unsigned long long>(a.chunk_table[c->chunk + 1]);
}

__global__ void k_iter_begin(WaveArgs a, int p)
{
    Ctrl* c = a.ctrl;
    c->qcount[p ^ 1] = 0;
    c->dcount[p ^ 1] = 0;
    c->scount[0] = 0;
    c->scount[1] = 0;
    c->fetch[0] = 0;
    c->fetch[1] = 0;
    c->fetch[2] = 0;
    // top the queue up with new paths (continuing rays are already in it)
    const int                q = c->qcount[p];
    const unsigned long long avail = c->limit > c->next ? c->limit - c->next : 0ull;
    const long long          room = a.capacity - static_cast<long long>(q);
    const int n = room > 0 ? static_cast<int>(avail < static_cast<unsigned long long>(room) ? avail : room) : 0;
    c->new_base = q;
    c->new_count = n;
    c->new_g = c->next;
    c->qcount[p] = q + n;
    c->next += static_cast<unsigned long long>(n);
}

// Gradient accumulators of an adjoint launch.  A kernel adds to the albedo gradients
// (GRAD_ALBEDO: k_regen, k_shade), to the emission gradients (GRAD_EMISSION: k_shade,
// k_connect) or both; each part it adds to is kept per block in shared memory when
// WaveArgs::grad_shared has that part's bit (flushed with one global atomic per nonzero
// entry when the block ends), and goes straight to the global vector otherwise.  A kernel's
// dynamic shared memory is the parts it uses (grad_smem_bytes), so the next-event kernels
// hold no albedo slice and keep their occupancy when there are thousands of albedos.
constexpr int GRAD_ALBEDO = 1, GRAD_EMISSION = 2;
// A part is kept per block while it fits 20 KB: then k_shade and k_regen keep their 9
// blocks per SM.  Few parameters need it (global atomics on cfg3's 256 albedos: adjoint
// 127 ms instead of 11.8); many do better in global memory at full occupancy (cfg4's 4096
// albedos, 48 KB: forward + adjoint 106.9 ms in global memory, 113.4 per block).
#ifndef MCRT_GRAD_SHARED_MAX
#define MCRT_GRAD_SHARED_MAX 20480
#endif
constexpr size_t kGradSharedMax = MCRT_GRAD_SHARED_MAX;  // bytes of one part kept per block

struct Grads
{
    float* ga;
    float* ge;
};

template <bool ADJ, int PARTS>
__device__ __forceinline__ Grads grads_begin(const WaveArgs& a, float* sgrad)
{
    Grads g{a.g_albedo, a.g_emis};
    if (!ADJ) return g;
    const bool sa = (PARTS & GRAD_ALBEDO) && (a.grad_shared & GRAD_ALBEDO);
    const bool se = (PARTS & GRAD_EMISSION) && (a.grad_shared & GRAD_EMISSION);
    if (!sa && !se) return g;  // uniform over the block: kernel arguments only
    const int ng = (sa ? 3 * a.n_albedo : 0) + (se ? 3 * a.n_emis : 0);
    for (int k = threadIdx.x; k < ng; k += blockDim.x) sgrad[k] = 0.f;
    __syncthreads();
    if (sa) g.ga = sgrad;
    if (se) g.ge = sgrad + (sa ? 3 * a.n_albedo : 0);
    return g;
}

template <bool ADJ, int PARTS>
__device__ __forceinline__ void grads_end(const WaveArgs& a, const float* sgrad)
{
    if (!ADJ) return;
    const bool sa = (PARTS & GRAD_ALBEDO) && (a.grad_shared & GRAD_ALBEDO);
    const bool se = (PARTS & GRAD_EMISSION) && (a.grad_shared & GRAD_EMISSION);
    if (!sa && !se) return;
    __syncthreads();
    const int na = sa ? 3 * a.n_albedo : 0, ng = na + (se ? 3 * a.n_emis : 0);
    for (int k = threadIdx.x; k < ng; k += blockDim.x)
    {
        const float v = sgrad[k];
        if (v != 0.f)
        {
            if (k < na)
                atomicAdd(&a.g_albedo[k], v);
            else
                atomicAdd(&a.g_emis[k - na], v);
        }
    }
}

// dynamic shared memory of a kernel that adds to the gradient parts PARTS
inline size_t grad_smem_bytes(const WaveArgs& a, int parts)
{
    size_t n = 0;
    if ((parts & GRAD_ALBEDO) && (a.grad_shared & GRAD_ALBEDO)) n += 3 * static_cast<size_t>(a.n_albedo);
    if ((parts & GRAD_EMISSION) && (a.grad_shared & GRAD_EMISSION)) n += 3 * static_cast<size_t>(a.n_emis);
    return n * sizeof(float);
}

__device__ __forceinline__ void add_grad3(float* g, int idx, float3 v)
{
    atomicAdd(&g[3 * idx + 0], v.x);
    atomicAdd(&g[3 * idx + 1], v.y);
    atomicAdd(&g[3 * idx + 2], v.z);
}

// dL/d(sample radiance) of a path: dL/dimage at its pixel / spp
__device__ __forceinline__ float3 path_dl(const JobGPU& J, int pixel)
{
    const float* g = J.image + 3 * static_cast<int64_t>(pixel);
    return mk(g[0], g[1], g[2]) * (1.0f / J.spp);
}

// the k-th 16-bit material id of a path's adjoint log (two uint4 = 8 words)
__device__ __forceinline__ int log_get(const unsigned* w, int k)
{
    unsigned v = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if (q == (k >> 1)) v = w[q];
    return static_cast<int>((v >> (16 * (k & 1))) & 0xffffu);
}

__device__ __forceinline__ void log_put(unsigned* w, int k, int matid)
{
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if (q == (k >> 1)) w[q] |= static_cast<unsigned>(matid & 0xffff) << (16 * (k & 1));
}

// starts camera path g (sample s of pixel x, y of its job) at position `pos` of ray
// queue p (demo_pt.cpp:689-700)
__device__ __forceinline__ void start_camera_path(const WaveArgs& a, int64_t g, int p, int pos)
{
    int           j = find_job(a.jobs, a.num_jobs, g);
    const JobGPU& J = a.jobs[j];
    int64_t       local = g - J.path_offset;
    int           pixel = static_cast<int>(local / J.spp);
    int           s = static_cast<int>(local - static_cast<int64_t>(pixel) * J.spp);
    int           x = pixel % J.width, y = pixel / J.width;
    Pcg           rng;
    rng.seed(J.seed, static_cast<uint32_t>(pixel), static_cast<uint32_t>(s));
    float r1 = 2.f * rng.uniform();
    float r2 = 2.f * rng.uniform();
    float dx = 0.f, dy = 0.f;
    if (J.spp > 1)
    {
        dx = tent(r1);
        dy = tent(r2);
    }
    float3 o, d;
    camera_ray(J.cam, (static_cast<float>(x) + 0.5f + dx) / static_cast<float>(J.width),
               (static_cast<float>(y) + 0.5f + dy) / static_cast<float>(J.height), o, d);
    a.qo[p][pos] = make_float4(o.x, o.y, o.z, __int_as_float(j));
    a.qd[p][pos] = make_float4(d.x, d.y, d.z, __int_as_float(pixel));
    a.qthr[p][pos] = make_float4(1.f, 1.f, 1.f, __int_as_float(0));  // vertex 0, nothing pending
    a.qrad[p][pos] = make_float4(0.f, 0.f, 0.f, __int_as_float(s));
    a.qrng[p][pos] = rng.state;
}

// Finishes the warp's ended paths (lanes with `valid`): radiance into the ring; a pixel
// whose last path this was is resolved by the whole warp from the ring in sample order,
// with the arithmetic of FrameBuffer::accumulatePixel / scale.  Called by all 32 lanes.
//
// Adjoint (ADJ): the path's radiance L is final here, so each logged Lambert vertex k
// gets + dL/dI * L / albedo_k; k_shade already added - dL/dI * L_before(k) / albedo_k.
// Together: (L - L_before(k)) / albedo_k, the path-replay albedo derivative.  A path
// whose L is NaN is scrubbed by the forward (demo_pt.cpp:653) and gets no + term.
template <bool ADJ>
__device__ __forceinline__ void finish_paths(const WaveArgs& a, const Grads& G, int p, int i, bool valid,
                                             unsigned long long& fin)
{
    if (ADJ)
    {
        if (!valid) return;
        const int4    m = a.dmeta[p][i];
        const float4 r = add_pending(a.nev[p] + 4 * a.capacity + 4 * static_cast<int64_t>(i), m.z, a.drad[p][i]);
        ++fin;
        if (isnan3(xyz(r)) || m.w == 0) return;
        const JobGPU&    J = a.jobs[m.y];
        const SceneView& S = J.scene;
        const float3     dl = path_dl(J, m.x);
        const uint4      l0 = a.dlog[p][2 * static_cast<int64_t>(i)], l1 = a.dlog[p][2 * static_cast<int64_t>(i) + 1];
        const unsigned   w[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
        for (int k = 0; k < m.w; ++k)
        {
            const MaterialGPU& M = S.materials[log_get(w, k)];
            const int          pk = M.albedo_param;
            if (M.r > 0.f) atomicAdd(&G.ga[3 * pk + 0], dl.x * r.x / M.r);
            if (M.g > 0.f) atomicAdd(&G.ga[3 * pk + 1], dl.y * r.y / M.g);
            if (M.b > 0.f) atomicAdd(&G.ga[3 * pk + 2], dl.z * r.z / M.b);
        }
        return;
    }
    const int     lane = threadIdx.x & 31;
    const int64_t R = a.ring_size;
    int64_t       cidx = 0;
    int           spp = 0, pixel = 0, job = 0;
    if (valid)
    {
        const int4    m = a.dmeta[p][i];
        const float4 r = add_pending(a.nev[p] + 4 * a.capacity + 4 * static_cast<int64_t>(i), m.z, a.drad[p][i]);
        pixel = m.x;
        job = m.y;
        const JobGPU& J = a.jobs[job];
        const int64_t first = J.path_offset + static_cast<int64_t>(pixel) * J.spp;
        a.ring[(first + __float_as_int(r.w)) % R] = make_float4(r.x, r.y, r.z, 0.f);
        cidx = first % R;
        spp = J.spp;
        ++fin;
    }
    __threadfence();  // ring entries visible before the counts that announce them
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    bool           resolve = false;
    if (valid)
    {
        // lanes finishing paths of the same pixel add to its count once
        const unsigned peers = __match_any_sync(vmask, static_cast<unsigned long long>(cidx));
        if (lane == __ffs(peers) - 1)
        {
            const int k = __popc(peers);
            resolve = atomicAdd(&a.ring_cnt[cidx], k) + k == spp;
        }
    }
    unsigned todo = __ballot_sync(0xffffffffu, resolve);
    if (!todo) return;
    __threadfence();
    while (todo)
    {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const int64_t c0 = __shfl_sync(0xffffffffu, cidx, src);
        const int     sp = __shfl_sync(0xffffffffu, spp, src);
        const int     px = __shfl_sync(0xffffffffu, pixel, src);
        const int     jb = __shfl_sync(0xffffffffu, job, src);
        float         s0 = 0.f, s1 = 0.f, s2 = 0.f;
        for (int k0 = 0; k0 < sp; k0 += 32)
        {
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k0 + lane < sp)
            {
                int64_t idx = c0 + k0 + lane;
                if (idx >= R) idx -= R;
                v = __ldcg(&a.ring[idx]);  // L2: written by other blocks of this launch
                if (isnan3(xyz(v))) v = make_float4(0.f, 0.f, 0.f, 0.f);  // demo_pt.cpp:653
                v.x = fmax_ref(0.f, v.x);                                   // demo_pt.cpp:703
                v.y = fmax_ref(0.f, v.y);
                v.z = fmax_ref(0.f, v.z);
            }
            const int m = min(32, sp - k0);
            for (int l = 0; l < m; ++l)  // sample order
            {
                s0 += __shfl_sync(0xffffffffu, v.x, l);
                s1 += __shfl_sync(0xffffffffu, v.y, l);
                s2 += __shfl_sync(0xffffffffu, v.z, l);
            }
        }
        if (lane == 0)
        {
            a.ring_cnt[c0] = 0;
            const JobGPU& J = a.jobs[jb];
            const float   scale = static_cast<float>(1.0 / J.spp);  // FrameBuffer::scale(1.0 / spp)
            float*        out = J.image + 3 * static_cast<int64_t>(px);
            out[0] = s0 * scale;
            out[1] = s1 * scale;
            out[2] = s2 * scale;
        }
    }
}

template <bool ADJ>
__global__ void __launch_bounds__(128) k_regen(WaveArgs a, int p)
{
    extern __shared__ float sgrad[];
    const Grads        G = grads_begin<ADJ, GRAD_ALBEDO>(a, sgrad);
    const Ctrl*        c = a.ctrl;
    const int          nd = min(c->dcount[p], static_cast<int>(a.capacity));
    const int          nn = c->new_count;
    const int          nb = c->new_base;
    const int64_t      g0 = static_cast<int64_t>(c->new_g);
    const int          n = max(nd, nn);
    const int          lane = threadIdx.x & 31;
    const int          warps_total = (gridDim.x * blockDim.x) >> 5;
    unsigned long long fin = 0;
    for (int wbase = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; wbase < n; wbase += warps_total * 32)
    {
        const int i = wbase + lane;
        if (wbase < nd) finish_paths<ADJ>(a, G, p, i, i < nd, fin);
        if (i < nn) start_camera_path(a, g0 + i, p, nb + i);
    }
    for (int off = 16; off > 0; off >>= 1) fin += __shfl_down_sync(0xffffffffu, fin, off);
    if (lane == 0 && fin) atomicAdd(&a.ctrl->finished, fin);
    grads_end<ADJ, GRAD_ALBEDO>(a, sgrad);
}

// Work distribution of the traversal kernels over a queue of n entries: with batch
// fetch each warp takes the next 32 consecutive entries from `counter` until the queue is
// exhausted (the launch ends within one batch of its slowest warp; consecutive entries
// are neighbouring paths, so a warp's rays stay coherent); otherwise a static grid
// stride.  Usage: for (QueueWalk w(...); w.valid(); w.next()) if (w.i < n) ...
struct QueueWalk
{
    int* counter;
    int  n, i, base;
    bool batch;
    __device__ __forceinline__ QueueWalk(int* c, int n_, bool batch_) : counter(c), n(n_), batch(batch_)
    {
        if (batch)
            fetch();
        else
            base = i = blockIdx.x * blockDim.x + threadIdx.x;
    }
    __device__ __forceinline__ void fetch()
    {
        int b = 0;
        if ((threadIdx.x & 31) == 0) b = atomicAdd(counter, 32);
        base = __shfl_sync(0xffffffffu, b, 0);
        i = base + (threadIdx.x & 31);
    }
    // batch: warp-uniform (the whole warp continues while its batch starts inside the queue)
    __device__ __forceinline__ bool valid() const { return batch ? base < n : i < n; }
    __device__ __forceinline__ void next()
    {
        if (batch)
            fetch();
        else
            base = i += gridDim.x * blockDim.x;
    }
};

__device__ __forceinline__ float4 hit_record(bool hit, const Hit& h)
{
    return hit ? make_float4(h.t, h.u, h.v, __int_as_float(h.prim)) : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
}

template <int STACK, bool COUNT, int MINB, bool REFM = true>
__global__ void __launch_bounds__(kTraceBlock, MINB) k_extend(WaveArgs a, int p)
{
    __shared__ int stack[STACK * kTraceBlock];
    int*           st = stack + threadIdx.x;
    const int      n = min(a.ctrl->qcount[p], static_cast<int>(a.capacity));
    const float    inf = __int_as_float(0x7f800000);
    TraceCount     cnt = {0u, 0u};
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stats[0], static_cast<unsigned long long>(n));
    for (QueueWalk w(&a.ctrl->fetch[0], n, a.batch_fetch != 0); w.valid(); w.next())
    {
        const int i = w.i;
        if (i >= n) continue;
        float4        o = a.qo[p][i], d = a.qd[p][i];
        const JobGPU& J = a.jobs[__float_as_int(o.w)];
        Hit           h;
        bool hit = trace_ray<false, STACK, COUNT, REFM>(J.scene, J.traverse, xyz(o), xyz(d), kEpsRay, inf, st,
                                                        kTraceBlock, h, a.err, &cnt);
        a.hits[i] = hit_record(hit, h);
    }
    if (COUNT) flush_count(a.stats, 2, cnt);
}

// Adjoint (ADJ): emission derivatives at emitter hits (the coefficient of E), and at a
// parameterised Lambert vertex k the - dL/dI * L_before(k) / albedo_k half of the albedo
// derivative; the vertex's material id goes to the path's log for the other half.
// Registers capped at 56 (9 blocks per SM).  Per cfg1 frame: uncapped (80 registers)
// 32.4 ms, 8 blocks 26.5, 9 blocks 25.0, 10 blocks 26.3.  One build only: builds under
// different register budgets contract multiply-adds differently, and every
// configuration must render the same image.
// k_shade sorts windows of kShadeWindow queue entries and shades them in rounds of 128.
constexpr int kShadeRounds = 4, kShadeWindow = 128 * kShadeRounds;

// Shading class of queue entry i: 0 a miss; else the hit material (light, Lambert, mirror,
// dielectric, Phong, GGX) and, with kShadeSide, the side of the surface the ray arrives
// from (by the first vertex normal): 1-12.  Entries of one class run the same code and
// continue in similar directions.
constexpr bool kShadeSide = true;

__device__ __forceinline__ int shade_class(const WaveArgs& a, int p, int i)
{
    const int prim = __float_as_int(a.hits[i].w);
    if (prim < 0) return 0;
    const SceneView& S = a.jobs[a.num_jobs == 1 ? 0 : __float_as_int(a.qo[p][i].w)].scene;
    const float4     na = __ldg(S.prim_shade + 3 * prim);
    const int        t = S.materials[__float_as_int(na.w)].type & 0xff;
    const int        c = t == MAT_GGX ? 6 : min(t, MAT_GLSY) + 1;
    if (!kShadeSide) return c;
    const float4 d = a.qd[p][i];
    return 2 * c - 1 + (d.x * na.x + d.y * na.y + d.z * na.z > 0.f ? 1 : 0);
}

// The block's kShadeWindow queue entries from `base` on, reordered by shading class (a
// counting sort in shared memory; entries past n last, class 15), so that a warp runs one
// material's code with all its lanes.  s_perm receives the entries in sorted order; the
// block then shades them in rounds of 128.  The order of the entries changes nothing a
// path computes: finished samples go to ring slots of their own.
__device__ __forceinline__ void shade_order(const WaveArgs& a, int p, int base, int n, int* s_base, int* s_perm)
{
    const int lane = threadIdx.x & 31;
    int       key[kShadeRounds], off[kShadeRounds];
#pragma unroll
    for (int r = 0; r < kShadeRounds; ++r)
    {
        const int i0 = base + r * 128 + threadIdx.x;
        key[r] = i0 < n ? shade_class(a, p, i0) : 15;
    }
    if (threadIdx.x < 16) s_base[threadIdx.x] = 0;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kShadeRounds; ++r)
    {
        const unsigned same = __match_any_sync(0xffffffffu, key[r]);
        const int      lead = __ffs(same) - 1;
        int            o = 0;
        if (lane == lead) o = atomicAdd(&s_base[key[r]], __popc(same));
        off[r] = __shfl_sync(0xffffffffu, o, lead) + __popc(same & lanemask_lt());
    }
    __syncthreads();
    if (threadIdx.x < 32)  // exclusive scan of the class counts
    {
        const int c = lane < 16 ? s_base[lane] : 0;
        int       incl = c;
        for (int d = 1; d < 16; d <<= 1)
        {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane < 16) s_base[lane] = incl - c;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kShadeRounds; ++r) s_perm[s_base[key[r]] + off[r]] = base + r * 128 + threadIdx.x;
    __syncthreads();
}

template <bool ADJ, int LIGHTS = 3>
__global__ void __launch_bounds__(128, 9) k_shade(WaveArgs a, int p)
{
    extern __shared__ float sgrad[];
    __shared__ int s_base[16], s_perm[kShadeWindow];
    const Grads G = grads_begin<ADJ, GRAD_ALBEDO | GRAD_EMISSION>(a, sgrad);
    const int n = min(a.ctrl->qcount[p], static_cast<int>(a.capacity));
    const int lane = threadIdx.x & 31;
    const int pn = p ^ 1;
    // pos: the first entry of this round; windows start at multiples of kShadeWindow, and a
    // window's valid entries fill its first rounds (the sort puts entries past n last)
    for (int pos = blockIdx.x * kShadeWindow; pos < n;)  // blocks of 128 threads
    {
        const int round = (pos % kShadeWindow) / 128;
        if (round == 0) shade_order(a, p, pos, n, s_base, s_perm);
        int      i = s_perm[round * 128 + threadIdx.x];
        bool     valid = i < n;
        bool     cont = false;
        float3   phit = mk(0.f, 0.f, 0.f), cdir = mk(0.f, 0.f, 1.f), T2 = mk(0.f, 0.f, 0.f);
        float4   rnew = make_float4(0.f, 0.f, 0.f, 0.f);
        int      flags2 = 0, n_nee = 0, job = 0, pixel = 0, nlog = 0;
        uint64_t rstate = 0;
        NeeRay   nee[4];
        unsigned lw[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        if (valid)
        {
            float4           o4 = a.qo[p][i], d4 = a.qd[p][i];
            float4           hh = a.hits[i];
            float4           t4 = a.qthr[p][i];
            float3           o = xyz(o4), d = xyz(d4);
            job = __float_as_int(o4.w);
            pixel = __float_as_int(d4.w);
            const JobGPU&    J = a.jobs[job];
            const SceneView& S = J.scene;
            float3           T = xyz(t4);
            const int        flags = __float_as_int(t4.w);
            const int        depth = (flags >> 8) & 0xff;
            bool             no_direct = depth == 0 || !(flags & 1);
            int              prim = __float_as_int(hh.w);
            float3           Ladd = mk(0.f, 0.f, 0.f);
            // results of the previous vertex's next-event rays first, then this vertex
            float4 rp = add_pending(a.nev[p] + 4 * static_cast<int64_t>(i), (flags >> 16) & 0xf, a.qrad[p][i]);
            float3 dl = mk(0.f, 0.f, 0.f);
            if (ADJ)
            {
                dl = path_dl(J, pixel);
                nlog = (flags >> 20) & 0x1f;
                if (nlog > 0)
                {
                    const uint4 l0 = a.qlog[p][2 * static_cast<int64_t>(i)];
                    const uint4 l1 = a.qlog[p][2 * static_cast<int64_t>(i) + 1];
                    lw[0] = l0.x, lw[1] = l0.y, lw[2] = l0.z, lw[3] = l0.w;
                    lw[4] = l1.x, lw[5] = l1.y, lw[6] = l1.z, lw[7] = l1.w;
                }
            }
            if (prim < 0)
            {
                Ladd = miss_emission<LIGHTS>(S, d, T, no_direct);
            }
            else
            {
                int    matid;
                float3 ns = shading_normal(S, prim, hh.y, hh.z, matid);
                Mat    m = load_mat(S, matid);
                if (m.consistent) ns = consistent_normal(S, prim, hh.y, hh.z, -d, ns);
                phit = o + d * hh.x;
                if (m.type == MAT_LGHT)
                {
                    if (no_direct && dot3(d, ns) < 0.f)
                    {
                        Ladd = T * m.color;
                        if (ADJ && m.emission_param >= 0 && m.emission_param < a.n_emis)
                            add_grad3(G.ge, m.emission_param, T * dl);
                    }
                }
                else
                {
                    if (ADJ && m.type == MAT_DIFF && m.albedo_param >= 0 && m.albedo_param < a.n_albedo)
                    {
                        if (!isnan3(xyz(rp)))
                        {
                            const int pk = m.albedo_param;
                            if (m.color.x > 0.f) atomicAdd(&G.ga[3 * pk + 0], -(dl.x * rp.x / m.color.x));
                            if (m.color.y > 0.f) atomicAdd(&G.ga[3 * pk + 1], -(dl.y * rp.y / m.color.y));
                            if (m.color.z > 0.f) atomicAdd(&G.ga[3 * pk + 2], -(dl.z * rp.z / m.color.z));
                        }
                        if (nlog < kAdjLog)
                            log_put(lw, nlog++, matid);
                        else
                            atomicOr(a.err, kErrQueue);
                    }
                    Pcg rng;
                    rng.state = a.qrng[p][i];
                    rng.inc = (static_cast<uint64_t>(pixel) << 1u) | 1u;
                    // the draws in a loop, not unrolled: smaller code (the kernel misses in
                    // the instruction cache) and fewer spills; 24.9 -> 24.4 ms per cfg1 frame
                    float u[NUM_DIMS];
#pragma unroll 1
                    for (int k = 0; k < NUM_DIMS; ++k) u[k] = rng.uniform();
                    rstate = rng.state;
                    float3 wi = -d;
                    bool   nee_here = does_nee(m.type);
                    if (nee_here) n_nee = make_nee<LIGHTS>(S, m, wi, ns, phit, T, u, nee);
                    cont = continue_path(m, wi, ns, T, u, depth, J.max_depth, J.rr_depth, T2, cdir);
                    flags2 = (nee_here ? 1 : 0) | ((depth + 1) << 8) | (nlog << 20);
                }
            }
            rnew = make_float4(rp.x + Ladd.x, rp.y + Ladd.y, rp.z + Ladd.z, rp.w);
        }
        const int pend = (1 << n_nee) - 1;
        // continuing paths -> queue p ^ 1, ended paths -> finished list p ^ 1 (ballot + popc,
        // one atomic per warp each); dest: where this vertex's next-event results go
        int      dest = -1;
        unsigned live = __ballot_sync(0xffffffffu, cont);
        if (live)
        {
            int base = 0;
            if (lane == 0) base = atomicAdd(&a.ctrl->qcount[pn], __popc(live));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (cont)
            {
                int k = base + __popc(live & lanemask_lt());
                if (k < a.capacity)
                {
                    a.qo[pn][k] = make_float4(phit.x, phit.y, phit.z, __int_as_float(job));
                    a.qd[pn][k] = make_float4(cdir.x, cdir.y, cdir.z, __int_as_float(pixel));
                    a.qthr[pn][k] = make_float4(T2.x, T2.y, T2.z, __int_as_float(flags2 | (pend << 16)));
                    a.qrad[pn][k] = rnew;
                    a.qrng[pn][k] = rstate;
                    if (ADJ && nlog > 0)
                    {
                        a.qlog[pn][2 * static_cast<int64_t>(k)] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                        a.qlog[pn][2 * static_cast<int64_t>(k) + 1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
                    }
                    dest = 4 * k;
                }
                else
                {
                    atomicOr(a.err, kErrQueue);
                }
            }
        }
        unsigned ended = __ballot_sync(0xffffffffu, valid && !cont);
        if (ended)
        {
            int base = 0;
            if (lane == 0) base = atomicAdd(&a.ctrl->dcount[pn], __popc(ended));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (valid && !cont)
            {
                int k = base + __popc(ended & lanemask_lt());
                if (k < a.capacity)
                {
                    a.drad[pn][k] = rnew;
                    a.dmeta[pn][k] = make_int4(pixel, job, pend, ADJ ? nlog : 0);
                    if (ADJ && nlog > 0)
                    {
                        a.dlog[pn][2 * static_cast<int64_t>(k)] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                        a.dlog[pn][2 * static_cast<int64_t>(k) + 1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
                    }
                    dest = static_cast<int>(4 * a.capacity) + 4 * k;
                }
                else
                {
                    atomicOr(a.err, kErrQueue);
                }
            }
        }
        if (dest < 0) n_nee = 0;  // no place for the results (queue overflow, reported)
        // next-event rays: any-hit queue [0], closest-hit queue [1] (warp prefix sums)
        int n_any = 0;
        for (int r = 0; r < n_nee; ++r) n_any += nee[r].type == NEE_ENV ? 1 : 0;
        int n_cl = n_nee - n_any;
        for (int qsel = 0; qsel < 2; ++qsel)
        {
            int k = qsel == 0 ? n_any : n_cl;
            int b = warp_append(&a.ctrl->scount[qsel], k);
            int w = 0;
            for (int r = 0; r < n_nee; ++r)
            {
                if ((nee[r].type == NEE_ENV) != (qsel == 0)) continue;
                int idx = b + w++;
                if (idx >= a.shadow_cap)
                {
                    atomicOr(a.err, kErrQueue);
                    break;
                }
                // .w: where a closest-hit ray stops at a nearer hit (tmin is kEpsRay for all)
                a.so[qsel][idx] = make_float4(phit.x, phit.y, phit.z, nee[r].tterm);
                a.sd[qsel][idx] = make_float4(nee[r].d.x, nee[r].d.y, nee[r].d.z, nee[r].tmax);
                a.sv[qsel][idx] = nee[r].val;
                a.sm[qsel][idx] = make_int4(dest + r, nee[r].type | (nee[r].light << 2), pixel, job);
            }
        }
        pos += 128;
        if (pos % kShadeWindow == 0) pos += (gridDim.x - 1) * kShadeWindow;
    }
    grads_end<ADJ, GRAD_ALBEDO | GRAD_EMISSION>(a, sgrad);
}

// Adjoint (ADJ): the emission derivative of each next-event contribution (the
// coefficient of the reached emitter's E)
template <bool ADJ>
__device__ __forceinline__ void connect_result(const WaveArgs& a, const Grads& G, int p, int q, int k, bool hit,
                                               const Hit& h)
{
    const float4     d = a.sd[q][k], v = a.sv[q][k];
    const int4       m = a.sm[q][k];
    const JobGPU&    J = a.jobs[m.w];
    const SceneView& S = J.scene;
    float3           coef;
    int              emat;
    float3           add = nee_contribution(S, m.y & 3, m.y >> 2, v, xyz(d), hit, h, coef, emat);
    a.nev[p ^ 1][m.x] = make_float4(add.x, add.y, add.z, 0.f);
    if (ADJ && emat >= 0)
    {
        const int ep = S.materials[emat].emission_param;
        if (ep >= 0 && ep < a.n_emis) add_grad3(G.ge, ep, coef * path_dl(J, m.z));
    }
}

// Q = 0: the any-hit queue (rays to the environment); Q = 1: the bounded closest-hit
// queue (rays to area lights).  One kernel per queue: the any-hit build needs no
// closest-hit state, so it fits 56 registers without spills (both in one kernel spilled
// 80 B; next-event stage 37.8 -> 37.5 ms per cfg1 frame) and runs capped at 40 registers
// for 12 blocks per SM (kAnyHitMinBlocks; its adjoint build at 10, kAnyHitMinBlocksAdj).
template <int STACK, bool COUNT, int MINB, bool ADJ, int Q, bool REFM = true>
__global__ void __launch_bounds__(kTraceBlock,
                                  (Q == 0 && MINB > 1) ? (ADJ ? kAnyHitMinBlocksAdj : kAnyHitMinBlocks) : MINB)
    k_connect(WaveArgs a, int p)
{
    extern __shared__ float sgrad[];
    __shared__ int stack[STACK * kTraceBlock];
    const Grads    G = grads_begin<ADJ, GRAD_EMISSION>(a, sgrad);
    int*           st = stack + threadIdx.x;
    TraceCount     cnt = {0u, 0u};
    const int      n = min(a.ctrl->scount[Q], static_cast<int>(a.shadow_cap));
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(&a.stats[1], static_cast<unsigned long long>(n));
    for (QueueWalk w(&a.ctrl->fetch[1 + Q], n, a.batch_fetch != 0); w.valid(); w.next())
    {
        const int k = w.i;
        if (k >= n) continue;
        float4        o = a.so[Q][k], d = a.sd[Q][k];
        const JobGPU& J = a.jobs[a.sm[Q][k].w];
        Hit           h;
        bool hit = trace_ray<Q == 0, STACK, COUNT, REFM, Q == 1>(J.scene, J.traverse, xyz(o), xyz(d), kEpsRay, d.w,
                                                                 st, kTraceBlock, h, a.err, &cnt, o.w);
        connect_result<ADJ>(a, G, p, Q, k, hit, h);
    }
    if (COUNT) flush_count(a.stats, 4, cnt);
    grads_end<ADJ, GRAD_EMISSION>(a, sgrad);
}

// ---------------------------------------------------------------------------
// MCRT_SCHEDULE_PATHS: the plain GPU path tracer.  One thread runs a path from the camera
// to its end (rayTrace's loop, demo_pt.cpp:523-651, in one kernel: no queues, no sorting,
// no compaction) and writes its radiance to ring[g - first]; k_resolve_paths then sums
// each pixel's samples in sample order.  The path arithmetic is the wavefront's, in the
// same order (each vertex adds its next-event results, the next its emission), so the
// image is the wavefront's up to the compiler's choice of fused multiply-adds in either
// kernel (a few ulp).
// ---------------------------------------------------------------------------
constexpr int kPathBlock = 64;

template <int STACK>
__global__ void __launch_bounds__(kPathBlock) k_paths(WaveArgs a, int64_t first, int64_t end)
{
    __shared__ int     stack[STACK * kPathBlock];
    int*               st = stack + threadIdx.x;
    const float        inf = __int_as_float(0x7f800000);
    unsigned long long ext = 0, nee_rays = 0;
    for (int64_t g = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < end;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const JobGPU&    J = a.jobs[find_job(a.jobs, a.num_jobs, g)];
        const SceneView& S = J.scene;
        const int64_t    local = g - J.path_offset;
        const int        pixel = static_cast<int>(local / J.spp);
        const int        s = static_cast<int>(local - static_cast<int64_t>(pixel) * J.spp);
        const int        x = pixel % J.width, y = pixel / J.width;
        Pcg              rng;
        rng.seed(J.seed, static_cast<uint32_t>(pixel), static_cast<uint32_t>(s));
        const float r1 = 2.f * rng.uniform();
        const float r2 = 2.f * rng.uniform();
        const float dx = J.spp > 1 ? tent(r1) : 0.f, dy = J.spp > 1 ? tent(r2) : 0.f;
        float3      o, d;
        camera_ray(J.cam, (static_cast<float>(x) + 0.5f + dx) / static_cast<float>(J.width),
                   (static_cast<float>(y) + 0.5f + dy) / static_cast<float>(J.height), o, d);
        float3 L = mk(0.f, 0.f, 0.f), T = mk(1.f, 1.f, 1.f);
        bool   last_nee = false;
        for (int depth = 0; depth <= J.max_depth; ++depth)
        {
            Hit        h;
            const bool hit = trace_ray<false, STACK>(S, J.traverse, o, d, kEpsRay, inf, st, kPathBlock, h, a.err);
            ++ext;
            const bool no_direct = depth == 0 || !last_nee;
            if (!hit)
            {
                L = L + miss_emission(S, d, T, no_direct);
                break;
            }
            int    matid;
            float3 ns = shading_normal(S, h.prim, h.u, h.v, matid);
            Mat    m = load_mat(S, matid);
            if (m.consistent) ns = consistent_normal(S, h.prim, h.u, h.v, -d, ns);
            const float3 phit = o + d * h.t;
            if (m.type == MAT_LGHT)
            {
                if (no_direct && dot3(d, ns) < 0.f) L = L + T * m.color;
                break;
            }
            float u[NUM_DIMS];
#pragma unroll 1
            for (int k = 0; k < NUM_DIMS; ++k) u[k] = rng.uniform();
            const float3 wi = -d;
            const bool   nee_here = does_nee(m.type);
            if (nee_here)
            {
                NeeRay    nee[4];
                const int nn = make_nee(S, m, wi, ns, phit, T, u, nee);
                for (int r = 0; r < nn; ++r)
                {
                    Hit        hs;
                    const bool any = nee[r].type == NEE_ENV;
                    const bool hh = any ? trace_ray<true, STACK>(S, J.traverse, phit, nee[r].d, kEpsRay, nee[r].tmax,
                                                                 st, kPathBlock, hs, a.err)
                                        : trace_ray<false, STACK, false, true, true>(S, J.traverse, phit, nee[r].d,
                                                                                   kEpsRay, nee[r].tmax, st,
                                                                                   kPathBlock, hs, a.err, nullptr,
                                                                                   nee[r].tterm);
                    ++nee_rays;
                    float3 coef;
                    int    emat;
                    L = L + nee_contribution(S, nee[r].type, nee[r].light, nee[r].val, nee[r].d, hh, hs, coef, emat);
                }
            }
            float3     T2, cdir;
            const bool cont = continue_path(m, wi, ns, T, u, depth, J.max_depth, J.rr_depth, T2, cdir);
            last_nee = nee_here;
            if (!cont) break;
            T = T2;
            o = phit;
            d = cdir;
        }
        a.ring[g - first] = make_float4(L.x, L.y, L.z, 0.f);
    }
    for (int off = 16; off > 0; off >>= 1)
    {
        ext += __shfl_down_sync(0xffffffffu, ext, off);
        nee_rays += __shfl_down_sync(0xffffffffu, nee_rays, off);
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicAdd(&a.stats[0], ext);
        atomicAdd(&a.stats[1], nee_rays);
    }
}

// the pixels whose samples are paths [first, end): the sum in sample order of each
// sample's radiance (NaN scrubbed, clamped at 0), times 1 / spp -- the arithmetic of the
// wavefront's resolve (FrameBuffer::accumulatePixel + scale, film.cpp:204-260)
__global__ void __launch_bounds__(128) k_resolve_paths(WaveArgs a, int64_t first, int64_t end)
{
    for (int64_t g = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < end;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const JobGPU& J = a.jobs[find_job(a.jobs, a.num_jobs, g)];
        const int64_t local = g - J.path_offset;
        if (local % J.spp != 0) continue;  // one thread per pixel: its first sample's
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        for (int k = 0; k < J.spp; ++k)
        {
            float4 v = a.ring[g - first + k];
            if (isnan3(xyz(v))) v = make_float4(0.f, 0.f, 0.f, 0.f);  // demo_pt.cpp:653
            s0 += fmax_ref(0.f, v.x);                                  // demo_pt.cpp:703
            s1 += fmax_ref(0.f, v.y);
            s2 += fmax_ref(0.f, v.z);
        }
        const float scale = static_cast<float>(1.0 / J.spp);
        float*      out = J.image + 3 * (local / J.spp);
        out[0] = s0 * scale;
        out[1] = s1 * scale;
        out[2] = s2 * scale;
    }
}

// ---------------------------------------------------------------------------
// path-replay adjoint (Vicini et al. 2021): each path is re-traced from its seed and
// differentiated on the fly; nothing is taped, memory is O(pixels + parameters).
// The radiance of a path is multilinear in the Lambert albedos and the emitter
// radiances of the vertices it visits:
//   d L / d albedo_k = (L - L_before(k)) / albedo_k, summed over the vertices k that use
//                      that albedo (L_before: radiance gathered before vertex k);
//   d L / d E        = the coefficient multiplying E in each emission term.
// Russian-roulette probabilities are held constant (their derivative has zero mean).
// ---------------------------------------------------------------------------
struct AdjointArgs
{
    const JobGPU* jobs;  // per job: scene, camera, params; .image = dL/dimage [H][W][3]
    int           num_jobs;
    float*       g_albedo;
    int          n_albedo;
    float*       g_emis;
    int          n_emis;
    int          shared_grads;  // accumulate in shared memory, flush once per block
    int64_t      total_paths;
    unsigned long long* stats;
    int*         err;
};

constexpr int kAdjBlock = 64;
constexpr int kMaxLog = kMaxDepth + 2;

template <int STACK>
__global__ void __launch_bounds__(kAdjBlock) k_adjoint(AdjointArgs a)
{
    extern __shared__ float sgrad[];  // (n_albedo + n_emis) * 3 when shared_grads
    __shared__ int          stack[STACK * kAdjBlock];
    int*                    st = stack + threadIdx.x;
    const int               ng = (a.n_albedo + a.n_emis) * 3;
    if (a.shared_grads)
        for (int k = threadIdx.x; k < ng; k += blockDim.x) sgrad[k] = 0.f;
    __syncthreads();
    float* ga = a.shared_grads ? sgrad : a.g_albedo;
    float* ge = a.shared_grads ? sgrad + 3 * a.n_albedo : a.g_emis;
    unsigned long long rays = 0;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < a.total_paths;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const JobGPU&    J = a.jobs[find_job(a.jobs, a.num_jobs, g)];
        const SceneView& S = J.scene;
        int64_t          local = g - J.path_offset;
        int pixel = static_cast<int>(local / J.spp);
        int s = static_cast<int>(local - static_cast<int64_t>(pixel) * J.spp);
        int x = pixel % J.width, y = pixel / J.width;
        Pcg rng;
        rng.seed(J.seed, static_cast<uint32_t>(pixel), static_cast<uint32_t>(s));
        float r1 = 2.f * rng.uniform();
        float r2 = 2.f * rng.uniform();
        float dx = J.spp > 1 ? tent(r1) : 0.f, dy = J.spp > 1 ? tent(r2) : 0.f;
        float3 o, d;
        camera_ray(J.cam, (static_cast<float>(x) + 0.5f + dx) / static_cast<float>(J.width),
                   (static_cast<float>(y) + 0.5f + dy) / static_cast<float>(J.height), o, d);
        const float* dLdI = J.image;
        float3       dl = mk(dLdI[3 * pixel], dLdI[3 * pixel + 1], dLdI[3 * pixel + 2]) * (1.0f / J.spp);
        float3 L = mk(0.f, 0.f, 0.f), T = mk(1.f, 1.f, 1.f);
        bool   last_nee = false;
        // per-vertex log for the albedo adjoint
        int    lparam[kMaxLog];
        float3 lalb[kMaxLog], lbefore[kMaxLog];
        int    nlog = 0;
        for (int depth = 0; depth <= J.max_depth; ++depth)
        {
            Hit  h;
            bool hit = trace_ray<false, STACK>(S, J.traverse, o, d, kEpsRay, __int_as_float(0x7f800000), st, kAdjBlock,
                                               h, a.err);
            ++rays;
            bool no_direct = depth == 0 || !last_nee;
            if (!hit)
            {
                L = L + miss_emission(S, d, T, no_direct);
                break;
            }
            int    matid;
            float3 ns = shading_normal(S, h.prim, h.u, h.v, matid);
            Mat    m = load_mat(S, matid);
            if (m.consistent) ns = consistent_normal(S, h.prim, h.u, h.v, -d, ns);
            float3 phit = o + d * h.t;
            if (m.type == MAT_LGHT)
            {
                if (no_direct && dot3(d, ns) < 0.f)
                {
                    L = L + T * m.color;
                    if (m.emission_param >= 0 && m.emission_param < a.n_emis)
                    {
                        float3 c = T * dl;
                        atomicAdd(&ge[3 * m.emission_param + 0], c.x);
                        atomicAdd(&ge[3 * m.emission_param + 1], c.y);
                        atomicAdd(&ge[3 * m.emission_param + 2], c.z);
                    }
                }
                break;
            }
            float u[NUM_DIMS];
#pragma unroll
            for (int k = 0; k < NUM_DIMS; ++k) u[k] = rng.uniform();
            float3 wi = -d;
            bool   nee_here = does_nee(m.type);
            float3 before = L;
            if (nee_here)
            {
                NeeRay nee[4];
                int    nn = make_nee(S, m, wi, ns, phit, T, u, nee);
                for (int r = 0; r < nn; ++r)
                {
                    Hit  hs;
                    bool any = nee[r].type == NEE_ENV;
                    bool hh = any ? trace_ray<true, STACK>(S, J.traverse, phit, nee[r].d, kEpsRay, nee[r].tmax, st,
                                                          kAdjBlock, hs, a.err)
                                  : trace_ray<false, STACK, false, true, true>(S, J.traverse, phit, nee[r].d, kEpsRay,
                                                                           nee[r].tmax, st, kAdjBlock, hs, a.err,
                                                                           nullptr, nee[r].tterm);
                    ++rays;
                    float3 coef;
                    int    emat;
                    float3 add = nee_contribution(S, nee[r].type, nee[r].light, nee[r].val, nee[r].d, hh, hs, coef, emat);
                    L = L + add;
                    if (emat >= 0)
                    {
                        int ep = S.materials[emat].emission_param;
                        if (ep >= 0 && ep < a.n_emis)
                        {
                            float3 c = coef * dl;
                            atomicAdd(&ge[3 * ep + 0], c.x);
                            atomicAdd(&ge[3 * ep + 1], c.y);
                            atomicAdd(&ge[3 * ep + 2], c.z);
                        }
                    }
                }
            }
            if (m.type == MAT_DIFF && m.albedo_param >= 0 && m.albedo_param < a.n_albedo && nlog < kMaxLog)
            {
                lparam[nlog] = m.albedo_param;
                lalb[nlog] = m.color;
                lbefore[nlog] = before;
                ++nlog;
            }
            float3 T2, cdir;
            bool   cont = continue_path(m, wi, ns, T, u, depth, J.max_depth, J.rr_depth, T2, cdir);
            last_nee = nee_here;
            if (!cont) break;
            T = T2;
            o = phit;
            d = cdir;
        }
        if (isnan3(L)) continue;  // demo_pt.cpp:653 scrubs the path to zero: no gradient
        for (int k = 0; k < nlog; ++k)
        {
            float3 Sk = L - lbefore[k];
            float3 al = lalb[k];
            int    pk = lparam[k];
            if (al.x > 0.f) atomicAdd(&ga[3 * pk + 0], dl.x * Sk.x / al.x);
            if (al.y > 0.f) atomicAdd(&ga[3 * pk + 1], dl.y * Sk.y / al.y);
            if (al.z > 0.f) atomicAdd(&ga[3 * pk + 2], dl.z * Sk.z / al.z);
        }
    }
    // warp-reduced ray count
    for (int off = 16; off > 0; off >>= 1) rays += __shfl_down_sync(0xffffffffu, rays, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&a.stats[0], rays);
    if (a.shared_grads)
    {
        __syncthreads();
        for (int k = threadIdx.x; k < ng; k += blockDim.x)
        {
            float v = sgrad[k];
            if (v != 0.f)
            {
                if (k < 3 * a.n_albedo)
                    atomicAdd(&a.g_albedo[k], v);
                else
                    atomicAdd(&a.g_emis[k - 3 * a.n_albedo], v);
            }
        }
    }
}

}  // namespace mcrt

// ===========================================================================
// host side: error handling, scene upload, render driver, C ABI
// ===========================================================================
using namespace mcrt;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

#define CK(x)                                                                                     \
    do                                                                                            \
    {                                                                                             \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess)                                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? MCRT_ERR_OUT_OF_MEMORY : MCRT_ERR_CUDA, \
                        std::string(#x) + ": " + cudaGetErrorString(e_));                         \
    } while (0)

struct Workspace
{
    int64_t             capacity = 0;  // rays per queue of `block`
    int64_t             ring = 0;      // entries of `ring_block`
    int                 jobs_cap = 0;
    int64_t             chunks_cap = 0;
    WaveArgs            args{};
    void*               block = nullptr;       // queues
    void*               ring_block = nullptr;  // ring + per-pixel counts
    JobGPU*             jobs = nullptr;
    int64_t*            chunk_table = nullptr;
    Ctrl*               ctrl = nullptr;
    unsigned long long* stats = nullptr;
    int*                err = nullptr;
    unsigned long long* h_poll = nullptr;  // pinned: completion polls of the streaming schedule
    int64_t             adj_capacity = 0;    // rays per queue of `adj_block`
    void*               adj_block = nullptr; // adjoint vertex logs
};

// One workspace per device, shared by every scene on it.  A render's queues and ring are
// its largest allocation (about 50 GB at the default 64 M-ray queue); kept per scene, they
// multiplied by the number of scenes a process holds (the 64-scene mix rendered scene by
// scene would have kept 412 GB).  A render takes its device's mutex (renders on one device
// share it anyway); the workspace grows to the largest render and lives until the process
// exits.
constexpr int kMaxDevices = 64;
struct DeviceWorkspace
{
    std::mutex mu;
    Workspace  ws;
};
DeviceWorkspace& device_workspace(int device)
{
    static DeviceWorkspace pool[kMaxDevices];
    return pool[device];
}

}  // namespace

struct TraceStatus
{
    int                err;
    int                pad;
    unsigned long long fetch;
};

struct mcrt_scene
{
    SceneView          view{};
    std::vector<void*> allocs;
    int64_t            fast_nodes = 0, ref_nodes = 0, refs = 0, bytes = 0;
    int                bvh_depth = 0;
    int                wide_depth = 0;  // levels of the eight-child tree
    int                device = 0;
    int                num_materials = 0;
    MaterialGPU*       d_materials = nullptr;
    std::vector<int32_t> mat_types;  // the uploaded materials' types (mcrt_scene_set_materials)
    std::vector<int64_t> array_bytes;  // bytes of each uploaded array, in upload order
    uint64_t             desc_hash = 0;  // of the description the scene was built from
    // error word and ray counter of the batch-trace calls on device buffers, one pair per
    // CUDA stream: calls on one stream run in order, and calls on different streams (from
    // different host threads) do not share one
    std::unordered_map<void*, TraceStatus*> err_by_stream;
    std::mutex         mu;
};

namespace {

// The traversal-stack depth a job needs, in the units of the "+ 2 < kStack" checks: the
// REF traversal walks the two-child tree (one int per level), the FAST traversal the
// eight-child tree (two ints per level).
int stack_depth(const mcrt_scene* s, int traverse)
{
#if MCRT_FAST_WIDE
    if (traverse != MCRT_TRAVERSE_REF) return 2 * s->wide_depth;
#endif
    return s->bvh_depth;
}

template <class T>
int upload(mcrt_scene* s, const std::vector<T>& v, const T** out)
{
    *out = nullptr;
    if (v.empty()) return MCRT_OK;
    void* p = nullptr;
    size_t bytes = v.size() * sizeof(T);
    CK(cudaMalloc(&p, bytes));
    s->allocs.push_back(p);
    s->bytes += static_cast<int64_t>(bytes);
    CK(cudaMemcpy(p, v.data(), bytes, cudaMemcpyHostToDevice));
    *out = static_cast<const T*>(p);
    return MCRT_OK;
}

int num_sms()
{
    static int sms = 0;
    if (!sms)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

CameraGPU make_camera_impl(const mcrt_camera& c)
{
    // Camera::Camera (camera.cpp:9-35), in float with the same operation order
    auto sub = [](const float* a, const float* b, float* o) {
        o[0] = a[0] - b[0];
        o[1] = a[1] - b[1];
        o[2] = a[2] - b[2];
    };
    auto norm = [](float* v) {
        float inv = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] *= inv;
        v[1] *= inv;
        v[2] *= inv;
    };
    auto cross = [](const float* a, const float* b, float* o) {
        o[0] = (a[1] * b[2]) - (a[2] * b[1]);
        o[1] = (a[2] * b[0]) - (a[0] * b[2]);
        o[2] = (a[0] * b[1]) - (a[1] * b[0]);
    };
    float fwd[3], fx[3], fy[3];
    sub(c.target, c.origin, fwd);
    norm(fwd);
    cross(fwd, c.up, fx);
    norm(fx);
    cross(fx, fwd, fy);
    CameraGPU g;
    g.ox = c.origin[0];
    g.oy = c.origin[1];
    g.oz = c.origin[2];
    g.fxx = fx[0];
    g.fxy = fx[1];
    g.fxz = fx[2];
    g.fyx = fy[0];
    g.fyy = fy[1];
    g.fyz = fy[2];
    g.wx = fwd[0];
    g.wy = fwd[1];
    g.wz = fwd[2];
    g.film_w = static_cast<float>(c.width) / static_cast<float>(c.height);
    g.film_h = 1.0f;
    float rad = c.fov_y * 0.5f / 180.0f * 3.14159265358979323846f;
    g.dist = g.film_h / (2.0f * std::tan(rad));
    return g;
}

// queues for `capacity` rays, a ring of `ring` entries, `num_jobs` jobs, `num_chunks` waves
int ensure_workspace(Workspace& w, int64_t capacity, int64_t ring, int num_jobs, int64_t num_chunks)
{
    if (w.capacity < capacity)
    {
        cudaFree(w.block);
        w.block = nullptr;
        w.capacity = 0;
        CK(cudaMalloc(&w.block, queue_bytes(capacity)));
        w.capacity = capacity;
    }
    if (w.ring < ring)
    {
        cudaFree(w.ring_block);
        w.ring_block = nullptr;
        w.ring = 0;
        CK(cudaMalloc(&w.ring_block, ring_bytes(ring)));
        w.ring = ring;
    }
    if (w.jobs_cap < num_jobs)
    {
        cudaFree(w.jobs);
        w.jobs = nullptr;
        w.jobs_cap = 0;
        CK(cudaMalloc(&w.jobs, sizeof(JobGPU) * num_jobs));
        w.jobs_cap = num_jobs;
    }
    if (w.chunks_cap < num_chunks + 1)
    {
        cudaFree(w.chunk_table);
        w.chunk_table = nullptr;
        w.chunks_cap = 0;
        CK(cudaMalloc(&w.chunk_table, sizeof(int64_t) * (num_chunks + 1)));
        w.chunks_cap = num_chunks + 1;
    }
    if (!w.ctrl)
    {
        CK(cudaMalloc(&w.ctrl, sizeof(Ctrl)));
        CK(cudaMalloc(&w.stats, sizeof(unsigned long long) * 8));
        CK(cudaMalloc(&w.err, sizeof(int)));
        CK(cudaMallocHost(&w.h_poll, 2 * sizeof(unsigned long long)));
    }
    if (w.block) carve_queues(w.args, w.block, w.capacity);
    if (w.ring_block) carve_ring(w.args, w.ring_block, w.ring);
    w.args.ctrl = w.ctrl;
    w.args.jobs = w.jobs;
    w.args.chunk_table = w.chunk_table;
    w.args.stats = w.stats;
    w.args.err = w.err;
    return MCRT_OK;
}

// Stage events: one pair per stage launch when profiling (never inside a graph).
struct StageTimer
{
    std::vector<cudaEvent_t> ev;  // pairs
    std::vector<int>         stage;
    void record(cudaStream_t st, int stg, bool begin)
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        ev.push_back(e);
        if (begin) stage.push_back(stg);
    }
    void sum(float* out)
    {
        for (size_t k = 0; k + 1 < ev.size(); k += 2)
        {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            out[stage[k / 2]] += ms;
        }
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        ev.clear();
        stage.clear();
    }
};

// one iteration of parity p (six launches); stage timer slots: 0 begin + regen,
// 1 extend, 2 shade, 3 connect
template <int STACK, bool COUNT, int MINB, bool ADJ = false, bool REFM = true>
void enqueue_iter(const WaveArgs& a, int p, const LaunchShape& ls, cudaStream_t st, StageTimer* tm)
{
    // adjoint: each kernel's shared gradient slices (0 for the forward)
    const size_t dr = ADJ ? grad_smem_bytes(a, GRAD_ALBEDO) : 0;
    const size_t ds = ADJ ? grad_smem_bytes(a, GRAD_ALBEDO | GRAD_EMISSION) : 0;
    const size_t dc = ADJ ? grad_smem_bytes(a, GRAD_EMISSION) : 0;
    auto beg = [&](int stg) {
        if (tm) tm->record(st, stg, true);
    };
    auto end = [&]() {
        if (tm) tm->record(st, 0, false);
    };
    beg(0);
    k_iter_begin<<<1, 1, 0, st>>>(a, p);
    k_regen<ADJ><<<ls.grid_regen, 128, dr, st>>>(a, p);
    end();
    beg(1);
    k_extend<STACK, COUNT, MINB, REFM><<<ls.grid_trace, kTraceBlock, 0, st>>>(a, p);
    end();
    beg(2);
    if (ls.lights == 1)
        k_shade<ADJ, 1><<<ls.grid_shade, 128, ds, st>>>(a, p);
    else if (ls.lights == 2)
        k_shade<ADJ, 2><<<ls.grid_shade, 128, ds, st>>>(a, p);
    else
        k_shade<ADJ, 3><<<ls.grid_shade, 128, ds, st>>>(a, p);
    end();
    beg(3);
    k_connect<STACK, COUNT, MINB, ADJ, 0, REFM><<<ls.grid_any, kTraceBlock, dc, st>>>(a, p);
    // closest-hit next-event rays exist only where a job has area lights
    if (ls.lights & 2) k_connect<STACK, COUNT, MINB, ADJ, 1, REFM><<<ls.grid_connect, kTraceBlock, dc, st>>>(a, p);
    end();
}

// one wave of the wave schedule: admit the wave, then iterate until its last path is
// finished (an even count, so the next wave starts on parity 0)
template <int STACK, bool COUNT, int MINB, bool REFM = true>
void enqueue_wave(const WaveArgs& a, int max_depth, const LaunchShape& ls, cudaStream_t st, StageTimer* tm)
{
    if (tm) tm->record(st, 0, true);
    k_wave_next<<<1, 1, 0, st>>>(a);
    if (tm) tm->record(st, 0, false);
    const int iters = wave_iterations(max_depth);
    for (int t = 0; t < iters; ++t) enqueue_iter<STACK, COUNT, MINB, false, REFM>(a, t & 1, ls, st, tm);
}

int validate_job_impl(const mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p)
{
    if (!s || !c || !p) return fail(MCRT_ERR_INVALID_ARGUMENT, "null scene, camera or params");
    if (c->width <= 0 || c->height <= 0 || p->spp <= 0)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "width, height and spp must be positive");
    if (p->max_depth < 0 || p->max_depth > kMaxDepth)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "max_depth must be in [0, 62]");
    if (p->traverse != MCRT_TRAVERSE_FAST && p->traverse != MCRT_TRAVERSE_REF)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "unknown traversal mode");
    if (static_cast<int64_t>(c->width) * c->height > (int64_t(1) << 31) / 2)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "image too large");
    if (p->schedule != MCRT_SCHEDULE_STREAM && p->schedule != MCRT_SCHEDULE_WAVES && p->schedule != MCRT_SCHEDULE_PATHS)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "unknown schedule");
    if (p->reserved != 0) return fail(MCRT_ERR_INVALID_ARGUMENT, "reserved field must be 0");
    if (p->path_chunk < 0 || p->path_chunk > kMaxQueue)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "path_chunk must be in [0, 2^27]");
    return MCRT_OK;
}

struct RunResult
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;  // around the kernels
    int64_t     waves = 0;                   // waves, or streaming iterations
    int64_t     launches = 0;
    int64_t     extend_launches = 0;
    int64_t     table_bytes = 0;  // host -> device besides the job table
    int         iter_launches = 6;  // launches per iteration (5 without area lights)
    int64_t     poll_bytes = 0;   // device -> host completion polls
};

struct WaveEnqueue
{
    const WaveArgs*    a;
    int                max_depth;
    const LaunchShape* ls;
    cudaStream_t       st;
    StageTimer*        tm;
    template <int S, bool C, int M, bool R>
    void run() const
    {
        enqueue_wave<S, C, M, R>(*a, max_depth, *ls, st, tm);
    }
};

struct IterEnqueue
{
    const WaveArgs*    a;
    int                p;
    const LaunchShape* ls;
    cudaStream_t       st;
    StageTimer*        tm;
    template <int S, bool C, int M, bool R>
    void run() const
    {
        enqueue_iter<S, C, M, false, R>(*a, p, *ls, st, tm);
    }
};

// dispatch of the traversal-kernel template variants.  Jobs that all traverse in FAST
// mode (f.ls->fast_only) get the builds without the REF traversal; any REF job runs the
// general build with 64-entry stacks and no register cap.
template <class F>
void with_variant(bool stack32, bool regcap, bool count, const F& f)
{
    constexpr int B = kTraceMinBlocks;
    if (!f.ls->fast_only)
        count ? f.template run<kStack, true, 1, true>() : f.template run<kStack, false, 1, true>();
    else if (stack32)
    {
        if (regcap)
            count ? f.template run<kSmallStack, true, B, false>()
                  : f.template run<kSmallStack, false, B, false>();
        else
            count ? f.template run<kSmallStack, true, 1, false>()
                  : f.template run<kSmallStack, false, 1, false>();
    }
    else
    {
        if (regcap)
            count ? f.template run<kStack, true, B, false>() : f.template run<kStack, false, B, false>();
        else
            count ? f.template run<kStack, true, 1, false>() : f.template run<kStack, false, 1, false>();
    }
}

// workspace, job table, zeroed statistics, pixel counts and counters; timing events
int begin_run(Workspace& w, const std::vector<JobGPU>& jobs, int64_t capacity, int64_t ring, int64_t num_chunks,
              cudaStream_t st, RunResult& run, WaveArgs& a)
{
    int rc = ensure_workspace(w, capacity, ring, static_cast<int>(jobs.size()), num_chunks);
    if (rc) return rc;
    a = w.args;  // sub-arrays sized for at least `capacity` / `ring`; use exactly those
    a.num_jobs = static_cast<int>(jobs.size());
    a.capacity = capacity;
    a.shadow_cap = 2 * capacity;
    a.ring_size = ring;
    CK(cudaMemcpyAsync(w.jobs, jobs.data(), sizeof(JobGPU) * jobs.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w.stats, 0, sizeof(unsigned long long) * 8, st));
    CK(cudaMemsetAsync(w.err, 0, sizeof(int), st));
    if (ring > 0) CK(cudaMemsetAsync(a.ring_cnt, 0, sizeof(int) * ring, st));
    CK(cudaEventCreate(&run.e0));
    CK(cudaEventCreate(&run.e1));
    return MCRT_OK;
}

// Boundaries of chunks of at most `capacity` paths on pixel boundaries (a pixel larger than
// the capacity gets a chunk of its own): table[k] .. table[k + 1] is chunk k.
std::vector<int64_t> pixel_chunks(const std::vector<JobGPU>& jobs, const std::vector<int64_t>& pix_spp,
                                  int64_t total, int64_t capacity)
{
    const int            num_jobs = static_cast<int>(jobs.size());
    std::vector<int64_t> table;
    table.push_back(0);
    int64_t pos = 0;
    int     j = 0;
    while (pos < total)
    {
        int64_t end = std::min(total, pos + capacity);
        while (j + 1 < num_jobs && jobs[j + 1].path_offset <= end - 1) ++j;
        // job containing `end` (exclusive bound): round down to its pixel boundary
        int jj = j;
        while (jj + 1 < num_jobs && jobs[jj + 1].path_offset <= end) ++jj;
        if (end < total)
        {
            int64_t local = end - jobs[jj].path_offset;
            int64_t rounded = jobs[jj].path_offset + (local / pix_spp[jj]) * pix_spp[jj];
            if (rounded <= pos)
            {
                // one pixel larger than the capacity: extend to its end
                rounded = jobs[jj].path_offset + ((local + pix_spp[jj] - 1) / pix_spp[jj]) * pix_spp[jj];
            }
            end = rounded;
        }
        table.push_back(end);
        pos = end;
    }
    return table;
}

// WAVES: waves of at most path_chunk paths, on pixel boundaries; each wave is admitted
// whole and runs until its last path is finished before the next is admitted
int run_waves(Workspace& w, const std::vector<JobGPU>& jobs, const std::vector<int64_t>& pix_spp, int64_t total,
              int max_depth, int64_t path_chunk, bool stack32, bool regcap, bool count, bool stages, bool graph,
              const LaunchShape& lsv, cudaStream_t st, StageTimer& timer, RunResult& run)
{
    int64_t capacity = path_chunk > 0 ? path_chunk : (int64_t(1) << 22);
    capacity = std::max<int64_t>(capacity, 64);
    const std::vector<int64_t> table = pixel_chunks(jobs, pix_spp, total, capacity);
    const int64_t num_chunks = static_cast<int64_t>(table.size()) - 1;
    int64_t       max_chunk = 0;
    for (int64_t k = 0; k < num_chunks; ++k) max_chunk = std::max(max_chunk, table[k + 1] - table[k]);
    if (max_chunk > kMaxQueue) return fail(MCRT_ERR_INVALID_ARGUMENT, "one pixel's samples exceed the queue limit");
    WaveArgs a;
    // a wave's paths are all finished before the next wave is admitted: a ring of one
    // wave never wraps onto a live entry
    int rc = begin_run(w, jobs, max_chunk, max_chunk, num_chunks, st, run, a);
    if (rc) return rc;
    CK(cudaMemcpyAsync(w.chunk_table, table.data(), sizeof(int64_t) * table.size(), cudaMemcpyHostToDevice, st));
    run.table_bytes = 8 * static_cast<int64_t>(table.size());
    const int iters = wave_iterations(max_depth);
    run.waves = num_chunks;
    run.launches = 1 + num_chunks * (1 + run.iter_launches * iters);
    run.extend_launches = num_chunks * iters;
    auto enqueue = [&](cudaStream_t s2, StageTimer* tm) {
        with_variant(stack32, regcap, count, WaveEnqueue{&a, max_depth, &lsv, s2, tm});
    };
    CK(cudaEventRecord(run.e0, st));
    k_render_begin<<<1, 1, 0, st>>>(a, 1, 0);
    if (graph)
    {
        cudaGraph_t     g;
        cudaGraphExec_t exec;
        cudaStream_t    cap;
        CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        enqueue(cap, nullptr);
        CK(cudaStreamEndCapture(cap, &g));
        CK(cudaGraphInstantiate(&exec, g, 0));
        for (int64_t k = 0; k < num_chunks; ++k) CK(cudaGraphLaunch(exec, st));
        CK(cudaEventRecord(run.e1, st));
        CK(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(g);
        cudaStreamDestroy(cap);
    }
    else
    {
        for (int64_t k = 0; k < num_chunks; ++k) enqueue(st, stages ? &timer : nullptr);
        CK(cudaGetLastError());
        CK(cudaEventRecord(run.e1, st));
    }
    return MCRT_OK;
}

// PATHS: the plain path tracer, one thread per path (k_paths), over chunks of at most
// path_chunk paths (default 64 M) on pixel boundaries, each chunk's pixels resolved by
// k_resolve_paths from the chunk's per-path radiance (the ring array)
int run_paths(Workspace& w, const std::vector<JobGPU>& jobs, const std::vector<int64_t>& pix_spp, int64_t total,
              int64_t path_chunk, int bvh_depth, cudaStream_t st, RunResult& run)
{
    int64_t capacity = path_chunk > 0 ? path_chunk : kDefaultQueue;
    capacity = std::max<int64_t>(capacity, 64);
    const std::vector<int64_t> table = pixel_chunks(jobs, pix_spp, total, capacity);
    const int64_t              num_chunks = static_cast<int64_t>(table.size()) - 1;
    int64_t                    max_chunk = 0;
    for (int64_t k = 0; k < num_chunks; ++k) max_chunk = std::max(max_chunk, table[k + 1] - table[k]);
    if (max_chunk > kMaxQueue) return fail(MCRT_ERR_INVALID_ARGUMENT, "one pixel's samples exceed the queue limit");
    WaveArgs a;
    int      rc = begin_run(w, jobs, 0, max_chunk, num_chunks, st, run, a);
    if (rc) return rc;
    const bool stack32 = bvh_depth + 2 < kSmallStack;
    int        occ = 0;
    if (stack32)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_paths<kSmallStack>, kPathBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_paths<kStack>, kPathBlock, 0);
    const int grid = num_sms() * std::max(occ, 1), grid_resolve = num_sms() * 8;
    run.waves = num_chunks;
    run.launches = 2 * num_chunks;
    run.extend_launches = num_chunks;
    CK(cudaEventRecord(run.e0, st));
    for (int64_t k = 0; k < num_chunks; ++k)
    {
        if (stack32)
            k_paths<kSmallStack><<<grid, kPathBlock, 0, st>>>(a, table[k], table[k + 1]);
        else
            k_paths<kStack><<<grid, kPathBlock, 0, st>>>(a, table[k], table[k + 1]);
        k_resolve_paths<<<grid_resolve, 128, 0, st>>>(a, table[k], table[k + 1]);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(run.e1, st));
    return MCRT_OK;
}

// Iterations in graph-launched pairs (parity 0, 1) until every path is finished, which
// the host learns from a device counter polled one batch behind the launches.
// iter(stream, parity, timer) enqueues one iteration.
template <class IterFn>
int stream_loop(Workspace& w, const WaveArgs& a, int64_t total, int max_depth, bool stages, bool graph,
                cudaStream_t st, StageTimer& timer, RunResult& run, const IterFn& iter)
{
    // while paths remain to be admitted every iteration traces a full queue, each path
    // has at most max_depth + 1 rays in queues, and a path is finished at most
    // max_depth + 2 iterations after admission
    const int64_t bound = (total * (max_depth + 1) + a.capacity - 1) / a.capacity + max_depth + 2;
    constexpr int kPairsPerPoll = 4;
    CK(cudaEventRecord(run.e0, st));
    k_render_begin<<<1, 1, 0, st>>>(a, 0, total);
    run.launches = 1;
    cudaGraph_t     g = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t    cap = nullptr;
    auto            release_graph = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (g) cudaGraphDestroy(g);
        if (cap) cudaStreamDestroy(cap);
    };
    if (graph)
    {
        CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        iter(cap, 0, nullptr);
        iter(cap, 1, nullptr);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (e != cudaSuccess)
        {
            release_graph();
            return fail(MCRT_ERR_CUDA, std::string("stream graph: ") + cudaGetErrorString(e));
        }
    }
    cudaEvent_t poll_ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaEventCreateWithFlags(&poll_ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&poll_ev[1], cudaEventDisableTiming);
    int64_t iters = 0;
    bool    done = false;
    for (int b = 0; !done && e == cudaSuccess; ++b)
    {
        for (int k = 0; k < kPairsPerPoll && e == cudaSuccess; ++k)
        {
            if (graph)
            {
                e = cudaGraphLaunch(exec, st);
            }
            else
            {
                iter(st, 0, stages ? &timer : nullptr);
                iter(st, 1, stages ? &timer : nullptr);
                e = cudaGetLastError();
            }
            iters += 2;
        }
        if (e != cudaSuccess) break;
        e = cudaMemcpyAsync(&w.h_poll[b & 1], &a.ctrl->finished, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            st);
        if (e == cudaSuccess) e = cudaEventRecord(poll_ev[b & 1], st);
        run.poll_bytes += sizeof(unsigned long long);
        if (e == cudaSuccess && b >= 1)
        {
            e = cudaEventSynchronize(poll_ev[(b - 1) & 1]);
            if (e == cudaSuccess && static_cast<int64_t>(w.h_poll[(b - 1) & 1]) >= total) done = true;
        }
        if (e == cudaSuccess && !done && iters > bound + 4 * kPairsPerPoll)
        {
            cudaStreamSynchronize(st);
            cudaEventDestroy(poll_ev[0]);
            cudaEventDestroy(poll_ev[1]);
            release_graph();
            return fail(MCRT_ERR_INTERNAL, "streaming render did not finish within its iteration bound");
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(run.e1, st);
    if (e == cudaSuccess && graph) e = cudaStreamSynchronize(st);  // before the graph is destroyed
    if (poll_ev[0]) cudaEventDestroy(poll_ev[0]);
    if (poll_ev[1]) cudaEventDestroy(poll_ev[1]);
    release_graph();
    if (e != cudaSuccess) return fail(MCRT_ERR_CUDA, std::string("streaming render: ") + cudaGetErrorString(e));
    run.waves = iters;
    run.launches += iters * run.iter_launches;
    run.extend_launches = iters;
    return MCRT_OK;
}

// STREAM: the queue is topped up with new camera paths every iteration
int run_stream(Workspace& w, const std::vector<JobGPU>& jobs, const std::vector<int64_t>& pix_spp, int64_t total,
               int max_depth, int64_t path_chunk, bool stack32, bool regcap, bool count, bool stages, bool graph,
               const LaunchShape& lsv, cudaStream_t st, StageTimer& timer, RunResult& run)
{
    int64_t capacity = path_chunk > 0 ? path_chunk : kDefaultQueue;
    capacity = std::min(capacity, (total + 31) / 32 * 32);
    capacity = std::max<int64_t>(capacity, 64);
    int64_t max_spp = 1;
    for (int64_t v : pix_spp) max_spp = std::max(max_spp, v);
    WaveArgs a;
    int      rc;
    for (;;)
    {
        const int64_t ring = stream_ring_entries(capacity, max_depth, max_spp, total);
        rc = begin_run(w, jobs, capacity, ring, 0, st, run, a);
        // the default capacity halves itself when the device has not the memory for it
        if (rc == MCRT_ERR_OUT_OF_MEMORY && path_chunk <= 0 && capacity > kMinDefaultQueue)
        {
            cudaGetLastError();
            capacity /= 2;
            continue;
        }
        break;
    }
    if (rc) return rc;
    auto iter = [&](cudaStream_t s2, int p, StageTimer* tm) {
        with_variant(stack32, regcap, count, IterEnqueue{&a, p, &lsv, s2, tm});
    };
    return stream_loop(w, a, total, max_depth, stages, graph, st, timer, run, iter);
}

// Path-replay adjoint on the streaming wavefront: the forward's stages with ADJ set (see
// k_shade, k_connect, finish_paths).  Needs max_depth < kAdjLog and material ids that fit
// the 16-bit log.
// REFM = false when every job traverses in FAST mode; the shading build follows ls.lights
// (the forward's specialisations)
template <int STACK, bool REFM>
void enqueue_adjoint_iter(const WaveArgs& a, int p, const LaunchShape& ls, cudaStream_t st)
{
    enqueue_iter<STACK, false, kTraceMinBlocks, true, REFM>(a, p, ls, st, nullptr);
}

template <int STACK, bool REFM>
int adjoint_launch_shape(const WaveArgs& a, LaunchShape& ls)
{
    const int dr = static_cast<int>(grad_smem_bytes(a, GRAD_ALBEDO));
    const int ds = static_cast<int>(grad_smem_bytes(a, GRAD_ALBEDO | GRAD_EMISSION));
    const int dc = static_cast<int>(grad_smem_bytes(a, GRAD_EMISSION));
    CK(cudaFuncSetAttribute(k_regen<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dr));
    CK(cudaFuncSetAttribute(k_shade<true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ds));
    CK(cudaFuncSetAttribute(k_shade<true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ds));
    CK(cudaFuncSetAttribute(k_shade<true, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, ds));
    constexpr int B = kTraceMinBlocks;
    CK(cudaFuncSetAttribute(k_connect<STACK, false, B, true, 0, REFM>, cudaFuncAttributeMaxDynamicSharedMemorySize, dc));
    CK(cudaFuncSetAttribute(k_connect<STACK, false, B, true, 1, REFM>, cudaFuncAttributeMaxDynamicSharedMemorySize, dc));
    const int sms = num_sms();
    int       occ_e = 0, occ_s = 0, occ_a = 0, occ_c = 0, occ_r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_extend<STACK, false, B, REFM>, kTraceBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_shade<true, 3>, 128, ds);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_r, k_regen<true>, 128, dr);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, k_connect<STACK, false, B, true, 0, REFM>, kTraceBlock, dc);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, k_connect<STACK, false, B, true, 1, REFM>, kTraceBlock, dc);
    ls.grid_trace = sms * std::max(occ_e, 1);
    ls.grid_any = sms * std::max(occ_a, 1);
    ls.grid_connect = sms * std::max(occ_c, 1);
    ls.grid_shade = sms * std::max(occ_s, 1);
    ls.grid_regen = sms * std::max(occ_r, 1);
    ls.grid_small = sms * 8;
    ls.block = 128;
    return MCRT_OK;
}

int adjoint_stream(Workspace& w, const std::vector<JobGPU>& jobs, int64_t total, int max_depth, int bvh_depth,
                   int64_t path_chunk, float* ga, int na, float* ge, int ne, cudaStream_t st, RunResult& run)
{
    int64_t capacity = path_chunk > 0 ? path_chunk : kDefaultQueue;
    capacity = std::min(capacity, (total + 31) / 32 * 32);
    capacity = std::max<int64_t>(capacity, 64);
    WaveArgs a;
    int      rc;
    for (;;)
    {
        rc = begin_run(w, jobs, capacity, 0, 0, st, run, a);
        if (rc == MCRT_OK && w.adj_capacity < capacity)
        {
            cudaFree(w.adj_block);
            w.adj_block = nullptr;
            w.adj_capacity = 0;
            if (cudaMalloc(&w.adj_block, 4 * (32 * static_cast<size_t>(capacity) + 256)) == cudaSuccess)
            {
                w.adj_capacity = capacity;
            }
            else
            {
                w.adj_block = nullptr;
                cudaEventDestroy(run.e0);
                cudaEventDestroy(run.e1);
                run.e0 = run.e1 = nullptr;
                rc = fail(MCRT_ERR_OUT_OF_MEMORY, "adjoint vertex log allocation failed");
            }
        }
        // the default capacity halves itself when the device has not the memory for it
        if (rc == MCRT_ERR_OUT_OF_MEMORY && path_chunk <= 0 && capacity > kMinDefaultQueue)
        {
            cudaGetLastError();
            capacity /= 2;
            continue;
        }
        break;
    }
    if (rc) return rc;
    Carver c{static_cast<char*>(w.adj_block)};
    for (int k = 0; k < 2; ++k)
    {
        a.qlog[k] = static_cast<uint4*>(c.take(32 * static_cast<size_t>(w.adj_capacity)));
        a.dlog[k] = static_cast<uint4*>(c.take(32 * static_cast<size_t>(w.adj_capacity)));
    }
    a.g_albedo = ga;
    a.g_emis = ge;
    a.n_albedo = na;
    a.n_emis = ne;
    // each gradient part per block in shared memory when it fits kGradSharedMax
    a.grad_shared = (sizeof(float) * 3 * static_cast<size_t>(na) <= kGradSharedMax ? GRAD_ALBEDO : 0) |
                    (sizeof(float) * 3 * static_cast<size_t>(ne) <= kGradSharedMax ? GRAD_EMISSION : 0);
    const bool   stack32 = bvh_depth + 2 < kSmallStack;
    bool         fast_only = true;
    int          lights = 0;
    for (const JobGPU& J : jobs)
    {
        fast_only = fast_only && J.traverse != MCRT_TRAVERSE_REF;
        lights |= (J.scene.env_w > 0 ? 1 : 0) | (J.scene.light_area > 0.f ? 2 : 0);
    }
    LaunchShape ls;
    rc = stack32 ? (fast_only ? adjoint_launch_shape<kSmallStack, false>(a, ls)
                              : adjoint_launch_shape<kSmallStack, true>(a, ls))
                 : (fast_only ? adjoint_launch_shape<kStack, false>(a, ls)
                              : adjoint_launch_shape<kStack, true>(a, ls));
    if (rc) return rc;
    ls.fast_only = fast_only;
    ls.lights = lights == 0 ? 3 : lights;
    run.iter_launches = (ls.lights & 2) ? 6 : 5;
    auto iter = [&](cudaStream_t s2, int p, StageTimer*) {
        if (stack32)
            fast_only ? enqueue_adjoint_iter<kSmallStack, false>(a, p, ls, s2)
                      : enqueue_adjoint_iter<kSmallStack, true>(a, p, ls, s2);
        else
            fast_only ? enqueue_adjoint_iter<kStack, false>(a, p, ls, s2)
                      : enqueue_adjoint_iter<kStack, true>(a, p, ls, s2);
    };
    StageTimer timer;
    return stream_loop(w, a, total, max_depth, false, true, st, timer, run, iter);
}

int render_jobs(int num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cams, const mcrt_render_params* params,
                float* const* outs, mcrt_render_stats* stats, cudaStream_t st)
{
    for (int j = 0; j < num_jobs; ++j)
    {
        int rc = validate_job_impl(scenes[j], &cams[j], &params[j]);
        if (rc) return rc;
        if (!outs[j]) return fail(MCRT_ERR_INVALID_ARGUMENT, "null image buffer");
    }
    mcrt_scene* owner = scenes[0];
    if (owner->device < 0 || owner->device >= kMaxDevices) return fail(MCRT_ERR_INVALID_ARGUMENT, "device index");
    std::lock_guard<std::mutex> lock(owner->mu);
    DeviceWorkspace&            dw = device_workspace(owner->device);
    std::lock_guard<std::mutex> wlock(dw.mu);
    CK(cudaSetDevice(owner->device));
    const mcrt_render_params& p0 = params[0];
    int                       ptr_mode = p0.ptr_mode;
    int                       bvh_depth = 0;
    int                       max_depth = 0;
    std::vector<JobGPU>       jobs(num_jobs);
    std::vector<int64_t>      pix_spp(num_jobs);
    int64_t                   total = 0;
    std::vector<float*>       dev_images(num_jobs, nullptr);
    std::vector<void*>        temp;
    auto cleanup = [&]() {
        for (void* t : temp) cudaFree(t);
    };
    for (int j = 0; j < num_jobs; ++j)
    {
        const mcrt_camera&        c = cams[j];
        const mcrt_render_params& p = params[j];
        JobGPU&                   J = jobs[j];
        J.scene = scenes[j]->view;
        J.cam = make_camera_impl(c);
        J.width = c.width;
        J.height = c.height;
        J.spp = p.spp;
        J.max_depth = p.max_depth;
        J.rr_depth = p.rr_depth;
        J.traverse = p.traverse;
        J.seed = p.seed;
        J.path_offset = total;
        int64_t px = static_cast<int64_t>(c.width) * c.height;
        total += px * p.spp;
        pix_spp[j] = p.spp;
        max_depth = std::max(max_depth, p.max_depth);
        bvh_depth = std::max(bvh_depth, stack_depth(scenes[j], p.traverse));
        if (ptr_mode == MCRT_PTR_DEVICE)
        {
            dev_images[j] = outs[j];
        }
        else
        {
            void* d = nullptr;
            cudaError_t e = cudaMalloc(&d, sizeof(float) * 3 * px);
            if (e != cudaSuccess)
            {
                cleanup();
                return fail(MCRT_ERR_OUT_OF_MEMORY, "image buffer allocation failed");
            }
            temp.push_back(d);
            dev_images[j] = static_cast<float*>(d);
        }
        J.image = dev_images[j];
    }
    if (bvh_depth + 2 >= kStack)
    {
        cleanup();
        return fail(MCRT_ERR_STACK_OVERFLOW, "BVH deeper than the traversal stack");
    }
    const bool count = (p0.profile & MCRT_PROFILE_COUNT) != 0;
    const bool stages = (p0.profile & MCRT_PROFILE_STAGES) != 0;
    const bool graph = p0.use_graph && !stages;
    // variant 0: the default policy (32-entry stacks when the tree is shallow enough,
    // traversal registers capped for kTraceMinBlocks blocks per SM);
    // MCRT_VARIANT_EXPLICIT: the given bits
    const int   vb = (p0.variant & MCRT_VARIANT_EXPLICIT) ? p0.variant : (MCRT_VARIANT_STACK32 | MCRT_VARIANT_REGCAP);
    const bool  stack32 = (vb & MCRT_VARIANT_STACK32) && bvh_depth + 2 < kSmallStack;
    const bool  regcap = (vb & MCRT_VARIANT_REGCAP) != 0;
    bool        fast_only = true;
    int         lights = 0;
    for (const JobGPU& J : jobs)
    {
        fast_only = fast_only && J.traverse != MCRT_TRAVERSE_REF;
        lights |= (J.scene.env_w > 0 ? 1 : 0) | (J.scene.light_area > 0.f ? 2 : 0);
    }
    LaunchShape lsv = launch_shape_variant(stack32, regcap, fast_only);
    lsv.lights = lights == 0 ? 3 : lights;
    Workspace&  w = dw.ws;
    w.args.batch_fetch = (vb & MCRT_VARIANT_GRIDSTRIDE) ? 0 : 1;
    StageTimer  timer;
    RunResult   run;
    run.iter_launches = (lsv.lights & 2) ? 6 : 5;
    int         rc = p0.schedule == MCRT_SCHEDULE_WAVES
                         ? run_waves(w, jobs, pix_spp, total, max_depth, p0.path_chunk, stack32, regcap, count, stages,
                                     graph, lsv, st, timer, run)
                     : p0.schedule == MCRT_SCHEDULE_PATHS
                         ? run_paths(w, jobs, pix_spp, total, p0.path_chunk, bvh_depth, st, run)
                         : run_stream(w, jobs, pix_spp, total, max_depth, p0.path_chunk, stack32, regcap, count,
                                      stages, graph, lsv, st, timer, run);
    if (rc)
    {
        cudaStreamSynchronize(st);
        cleanup();
        return rc;
    }
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        for (int j = 0; j < num_jobs; ++j)
            CK(cudaMemcpyAsync(outs[j], dev_images[j], sizeof(float) * 3 * cams[j].width * cams[j].height,
                               cudaMemcpyDeviceToHost, st));
    }
    unsigned long long hstats[8];
    int                herr = 0;
    CK(cudaMemcpyAsync(hstats, w.stats, sizeof(hstats), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, run.e0, run.e1);
    cudaEventDestroy(run.e0);
    cudaEventDestroy(run.e1);
    float stage_ms[4] = {0.f, 0.f, 0.f, 0.f};
    timer.sum(stage_ms);
    cleanup();
    if (stats)
    {
        stats->paths = total;
        stats->extension_rays = static_cast<int64_t>(hstats[0]);
        stats->shadow_rays = static_cast<int64_t>(hstats[1]);
        stats->waves = static_cast<int32_t>(run.waves);
        stats->kernel_launches = static_cast<int32_t>(run.launches);
        stats->device_ms = ms;
        for (int k = 0; k < 4; ++k) stats->stage_ms[k] = stage_ms[k];
        stats->extend_launches = static_cast<int32_t>(run.extend_launches);
        stats->ext_nodes = static_cast<int64_t>(hstats[2]);
        stats->ext_tris = static_cast<int64_t>(hstats[3]);
        stats->nee_nodes = static_cast<int64_t>(hstats[4]);
        stats->nee_tris = static_cast<int64_t>(hstats[5]);
        stats->node_bytes = MCRT_FAST_WIDE ? static_cast<int32_t>(sizeof(WideNode)) : static_cast<int32_t>(sizeof(FastNode));
        int64_t img_bytes = 0;
        for (int j = 0; j < num_jobs; ++j) img_bytes += 12 * static_cast<int64_t>(cams[j].width) * cams[j].height;
        stats->h2d_bytes = static_cast<int64_t>(sizeof(JobGPU)) * num_jobs + run.table_bytes;
        stats->d2h_bytes = static_cast<int64_t>(sizeof(hstats) + sizeof(herr)) + run.poll_bytes +
                           (ptr_mode != MCRT_PTR_DEVICE ? img_bytes : 0);
    }
    if (herr & kErrStack) return fail(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    if (herr & kErrQueue) return fail(MCRT_ERR_QUEUE_OVERFLOW, "queue overflow");
    return MCRT_OK;
}

}  // namespace

namespace mcrt {

size_t queue_bytes(int64_t capacity)
{
    const size_t C = static_cast<size_t>(capacity);
    // by parity: qo, qd, qthr, qrad (64 B) + qrng 8 + drad, dmeta 32 + nev 128; hits 16;
    // next-event queues: 2 x 2C x (so, sd, sv, sm) 64 B; 256-B alignment of 31 sub-arrays
    return 2 * C * (64 + 8 + 32 + 128) + C * 16 + 2 * (2 * C) * 64 + 256 * 32;
}

void carve_queues(WaveArgs& a, void* base, int64_t capacity)
{
    const int64_t C = capacity, S = 2 * capacity;
    Carver        c{static_cast<char*>(base)};
    for (int k = 0; k < 2; ++k)
    {
        a.qo[k] = static_cast<float4*>(c.take(16 * C));
        a.qd[k] = static_cast<float4*>(c.take(16 * C));
        a.qthr[k] = static_cast<float4*>(c.take(16 * C));
        a.qrad[k] = static_cast<float4*>(c.take(16 * C));
        a.qrng[k] = static_cast<uint64_t*>(c.take(8 * C));
        a.drad[k] = static_cast<float4*>(c.take(16 * C));
        a.dmeta[k] = static_cast<int4*>(c.take(16 * C));
        a.nev[k] = static_cast<float4*>(c.take(128 * C));
    }
    a.hits = static_cast<float4*>(c.take(16 * C));
    for (int k = 0; k < 2; ++k)
    {
        a.so[k] = static_cast<float4*>(c.take(16 * S));
        a.sd[k] = static_cast<float4*>(c.take(16 * S));
        a.sv[k] = static_cast<float4*>(c.take(16 * S));
        a.sm[k] = static_cast<int4*>(c.take(16 * S));
    }
    a.capacity = C;
    a.shadow_cap = S;
}

size_t ring_bytes(int64_t entries) { return 16 * static_cast<size_t>(entries) + 4 * static_cast<size_t>(entries) + 512; }

void carve_ring(WaveArgs& a, void* base, int64_t entries)
{
    Carver c{static_cast<char*>(base)};
    a.ring = static_cast<float4*>(c.take(16 * entries));
    a.ring_cnt = static_cast<int*>(c.take(4 * entries));
    a.ring_size = entries;
}

int64_t stream_ring_entries(int64_t capacity, int max_depth, int64_t max_spp, int64_t total)
{
    return std::min(total, (max_depth + 2) * capacity + max_spp);
}

int wave_iterations(int max_depth) { return (max_depth + 2 + 1) & ~1; }

void enqueue_render_begin(const WaveArgs& a, bool waves, int64_t limit, cudaStream_t st)
{
    k_render_begin<<<1, 1, 0, st>>>(a, waves ? 1 : 0, limit);
}

LaunchShape launch_shape() { return launch_shape_variant(false, false); }

LaunchShape launch_shape_variant(bool stack32, bool regcap, bool fast_only)
{
    LaunchShape ls;
    int         sms = num_sms();
    int         occ_t = 0, occ_s = 0, occ_a = 0;
    constexpr int B = kTraceMinBlocks;
    if (!fast_only)  // the general build (see with_variant)
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_t, k_extend<kStack, false, 1, true>, kTraceBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, k_connect<kStack, false, 1, false, 0, true>, kTraceBlock,
                                                      0);
    }
    else if (stack32)
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ_t, regcap ? k_extend<kSmallStack, false, B, false> : k_extend<kSmallStack, false, 1, false>,
            kTraceBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ_a,
            regcap ? k_connect<kSmallStack, false, B, false, 0, false> : k_connect<kSmallStack, false, 1, false, 0, false>,
            kTraceBlock, 0);
    }
    else
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ_t, regcap ? k_extend<kStack, false, B, false> : k_extend<kStack, false, 1, false>, kTraceBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ_a,
            regcap ? k_connect<kStack, false, B, false, 0, false> : k_connect<kStack, false, 1, false, 0, false>,
            kTraceBlock, 0);
    }
    ls.fast_only = fast_only;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_shade<false>, 128, 0);
    ls.grid_trace = sms * std::max(occ_t, 1);
    ls.grid_any = sms * std::max(occ_a, 1);
    ls.grid_connect = ls.grid_trace;
    ls.grid_shade = sms * std::max(occ_s, 1);
    ls.grid_regen = ls.grid_shade;
    ls.grid_small = sms * 8;
    ls.block = 128;
    return ls;
}

void enqueue_wave_plain(const WaveArgs& a, int max_depth, const LaunchShape& ls, cudaStream_t st)
{
    enqueue_wave<kStack, false, 1>(a, max_depth, ls, st, nullptr);
}

CameraGPU make_camera(const mcrt_camera& c) { return make_camera_impl(c); }

// uploads a prepared scene; the arrays are kept in upload order with their byte counts so
// the scene can be written to a cache file (scene_to_host)
// Bounding box of the emitter triangles and its margin: 1e-3 of the box diagonal plus its
// largest coordinate, far above the rounding of a triangle's hit distance (a few ulp of the
// vertex and origin coordinates); an empty box when the scene has no emitters.
static void emitter_box(const HostScene& hs, float3& lo, float3& hi, float& pad)
{
    const float inf = std::numeric_limits<float>::infinity();
    lo = make_float3(inf, inf, inf);
    hi = make_float3(-inf, -inf, -inf);
    pad = 0.f;
    for (const LightGPU& l : hs.lights)
        for (int c = 0; c < 3; ++c)
        {
            const float4 v = hs.prim_verts[3 * static_cast<size_t>(l.prim) + c];
            lo = make_float3(std::min(lo.x, v.x), std::min(lo.y, v.y), std::min(lo.z, v.z));
            hi = make_float3(std::max(hi.x, v.x), std::max(hi.y, v.y), std::max(hi.z, v.z));
        }
    if (hs.lights.empty()) return;
    const double dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    const double mag = std::max({std::fabs(lo.x), std::fabs(lo.y), std::fabs(lo.z), std::fabs(hi.x),
                                 std::fabs(hi.y), std::fabs(hi.z)});
    pad = static_cast<float>(1e-3 * (std::sqrt(dx * dx + dy * dy + dz * dz) + mag));
}

int scene_from_host(const HostScene& hs, int64_t num_tris, uint64_t desc_hash, mcrt_scene** out)
{
    mcrt_scene* s = new mcrt_scene();
    CK(cudaGetDevice(&s->device));
    int  rc = MCRT_OK;
    auto up = [&](auto& vec, auto** dst) {
        if (rc == MCRT_OK) rc = upload(s, vec, dst);
        s->array_bytes.push_back(static_cast<int64_t>(vec.size() * sizeof(vec[0])));
    };
    const FastNode*    fn;
    const float4*      ft;
    const RefNode*     rn;
    const RefPrim*     rp;
    const float4*      pv;
    const float4*      ps;
    const int*         lo;
    const LightGPU*    li;
    const MaterialGPU* mt;
    const float4*      er;
    const float*       em;
    const float*       ec;
    const int*         egm;
    const int*         egc;
    const float4*      pa;
    up(hs.bvh.fast_nodes, &fn);
    up(hs.bvh.fast_tris, &ft);
    up(hs.bvh.ref_nodes, &rn);
    up(hs.bvh.ref_prims, &rp);
    up(hs.prim_verts, &pv);
    up(hs.prim_shade, &ps);
    up(hs.light_of, &lo);
    up(hs.lights, &li);
    up(hs.materials, &mt);
    up(hs.env_rgb, &er);
    up(hs.env_marginal, &em);
    up(hs.env_cond, &ec);
    up(hs.env_guide_m, &egm);
    up(hs.env_guide_c, &egc);
    up(hs.prim_alpha, &pa);
    const WideNode* wn;
    const float4*   wt;
    up(hs.bvh.wide_nodes, &wn);
    up(hs.bvh.wide_tris, &wt);
    if (rc != MCRT_OK)
    {
        std::string msg = g_err;
        mcrt_scene_destroy(s);
        return fail(rc, msg);
    }
    SceneView& v = s->view;
    v.prim_alpha = pa;
    v.fast_nodes = fn;
    v.fast_tris = ft;
    v.wide_nodes = wn;
    v.wide_tris = wt;
    v.ref_nodes = rn;
    v.ref_prims = rp;
    v.prim_verts = pv;
    v.prim_shade = ps;
    v.light_of = lo;
    v.lights = li;
    v.materials = mt;
    v.env_rgb = er;
    v.env_marginal = em;
    v.env_cond = ec;
    v.env_guide_m = egm;
    v.env_guide_c = egc;
    v.num_lights = static_cast<int>(hs.lights.size());
    v.light_area = hs.light_area;
    emitter_box(hs, v.light_lo, v.light_hi, v.light_pad);
    v.env_w = hs.env_w;
    v.env_h = hs.env_h;
    v.env_norm = hs.env_norm;
    v.num_prims = static_cast<int>(num_tris);
    s->d_materials = const_cast<MaterialGPU*>(mt);
    s->num_materials = static_cast<int>(hs.materials.size());
    for (const MaterialGPU& g : hs.materials) s->mat_types.push_back(g.type);
    s->fast_nodes = static_cast<int64_t>(hs.bvh.fast_nodes.size());
    s->ref_nodes = static_cast<int64_t>(hs.bvh.ref_nodes.size());
    s->refs = static_cast<int64_t>(hs.bvh.ref_prims.size());
    s->bvh_depth = hs.bvh.max_depth;
    s->wide_depth = hs.bvh.wide_depth;
    s->desc_hash = desc_hash;
    *out = s;
    return MCRT_OK;
}

// downloads a scene's prepared arrays (the inverse of scene_from_host)
int scene_to_host(const mcrt_scene* s, HostScene& hs, int64_t& num_tris, uint64_t& desc_hash)
{
    if (s->array_bytes.size() != 17) return fail(MCRT_ERR_INTERNAL, "scene arrays not recorded");
    CK(cudaSetDevice(s->device));
    const SceneView& v = s->view;
    int              k = 0, rc = MCRT_OK;
    auto             down = [&](auto& vec, const void* src) {
        const int64_t bytes = s->array_bytes[k++];
        vec.resize(static_cast<size_t>(bytes) / sizeof(vec[0]));
        if (rc == MCRT_OK && bytes > 0)
        {
            cudaError_t e = cudaMemcpy(vec.data(), src, static_cast<size_t>(bytes), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = fail(MCRT_ERR_CUDA, std::string("scene download: ") + cudaGetErrorString(e));
        }
    };
    down(hs.bvh.fast_nodes, v.fast_nodes);
    down(hs.bvh.fast_tris, v.fast_tris);
    down(hs.bvh.ref_nodes, v.ref_nodes);
    down(hs.bvh.ref_prims, v.ref_prims);
    down(hs.prim_verts, v.prim_verts);
    down(hs.prim_shade, v.prim_shade);
    down(hs.light_of, v.light_of);
    down(hs.lights, v.lights);
    down(hs.materials, v.materials);
    down(hs.env_rgb, v.env_rgb);
    down(hs.env_marginal, v.env_marginal);
    down(hs.env_cond, v.env_cond);
    down(hs.env_guide_m, v.env_guide_m);
    down(hs.env_guide_c, v.env_guide_c);
    down(hs.prim_alpha, v.prim_alpha);
    down(hs.bvh.wide_nodes, v.wide_nodes);
    down(hs.bvh.wide_tris, v.wide_tris);
    hs.light_area = v.light_area;
    hs.env_w = v.env_w;
    hs.env_h = v.env_h;
    hs.env_norm = v.env_norm;
    hs.bvh.max_depth = s->bvh_depth;
    hs.bvh.wide_depth = s->wide_depth;
    num_tris = v.num_prims;
    desc_hash = s->desc_hash;
    return rc;
}

int validate_job(const mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p)
{
    return validate_job_impl(s, c, p);
}

int set_error(int code, const std::string& msg) { return fail(code, msg); }

bool fast_layout_wide() { return MCRT_FAST_WIDE != 0; }

const SceneView& scene_view(const mcrt_scene* s) { return s->view; }
int              scene_device(const mcrt_scene* s) { return s->device; }
int              scene_stack_depth(const mcrt_scene* s, int traverse) { return stack_depth(s, traverse); }

}  // namespace mcrt

extern "C" {

int mcrt_get_abi_version(void) { return MCRT_ABI_VERSION; }

const char* mcrt_last_error(void) { return g_err.c_str(); }

int mcrt_scene_destroy(mcrt_scene* s)
{
    if (!s) return MCRT_OK;
    cudaSetDevice(s->device);
    for (void* p : s->allocs) cudaFree(p);
    for (auto& e : s->err_by_stream) cudaFree(e.second);
    delete s;
    return MCRT_OK;
}

int mcrt_scene_create(const mcrt_scene_desc* desc, mcrt_scene** out)
{
    if (!desc || !out) return fail(MCRT_ERR_INVALID_ARGUMENT, "null desc or out");
    *out = nullptr;
    try
    {
        HostScene   hs;
        std::string err = prepare_scene(*desc, hs);
        if (!err.empty()) return fail(MCRT_ERR_INVALID_ARGUMENT, err);
        return mcrt::scene_from_host(hs, desc->num_triangles, mcrt::scene_desc_hash(*desc), out);
    }
    catch (const std::bad_alloc&)
    {
        return fail(MCRT_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_scene_create");
    }
}

int mcrt_scene_info(const mcrt_scene* s, int64_t* fast_nodes, int64_t* ref_nodes, int64_t* refs, int64_t* bytes)
{
    if (!s) return fail(MCRT_ERR_INVALID_ARGUMENT, "null scene");
    if (fast_nodes) *fast_nodes = s->fast_nodes;
    if (ref_nodes) *ref_nodes = s->ref_nodes;
    if (refs) *refs = s->refs;
    if (bytes) *bytes = s->bytes;
    return MCRT_OK;
}

int mcrt_scene_set_materials(mcrt_scene* s, int32_t n, const mcrt_material* m, void* stream)
{
    if (!s || !m) return fail(MCRT_ERR_INVALID_ARGUMENT, "null scene or materials");
    if (n != s->num_materials) return fail(MCRT_ERR_INVALID_ARGUMENT, "material count differs from the scene's");
    std::lock_guard<std::mutex> lock(s->mu);  // not while a render of this scene runs
    // the emitter table, its bounding box and the consistent-normal alphas are built with
    // the scene: a material may not become or stop being an emitter, nor ask for consistent
    // normals the scene was built without
    for (int k = 0; k < n; ++k)
    {
        const int t = m[k].type, base = t & 0xff;
        if ((t & ~(0xff | MCRT_MAT_CONSISTENT)) != 0 ||
            (base != MCRT_MAT_LGHT && base != MCRT_MAT_DIFF && base != MCRT_MAT_SPEC && base != MCRT_MAT_REFR &&
             base != MCRT_MAT_GLSY && base != MCRT_MAT_GGX))
            return fail(MCRT_ERR_INVALID_ARGUMENT, "unknown material type");
        if ((base == MCRT_MAT_LGHT) != ((s->mat_types[k] & 0xff) == MCRT_MAT_LGHT))
            return fail(MCRT_ERR_INVALID_ARGUMENT, "a material may not become or stop being an emitter (the emitter "
                                                   "table is built with the scene)");
        if ((t & MCRT_MAT_CONSISTENT) && !s->view.prim_alpha)
            return fail(MCRT_ERR_INVALID_ARGUMENT, "consistent normals need a scene built with them");
    }
    std::vector<MaterialGPU> g(n);
    for (int k = 0; k < n; ++k)
    {
        g[k].type = m[k].type;
        g[k].r = m[k].color[0];
        g[k].g = m[k].color[1];
        g[k].b = m[k].color[2];
        g[k].roughness = m[k].roughness;
        g[k].ior = m[k].ior;
        g[k].albedo_param = m[k].albedo_param;
        g[k].emission_param = m[k].emission_param;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(s->d_materials, g.data(), sizeof(MaterialGPU) * n, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    for (int k = 0; k < n; ++k) s->mat_types[k] = m[k].type;
    return MCRT_OK;
}

// Device buffer of the host-buffer trace calls of one host thread on one device, kept for
// the thread's life (1 MB: up to about 20,000 rays per call).
constexpr size_t kThreadTraceBufferMax = size_t(1) << 20;
struct ThreadTraceBuffer
{
    void*  ptr = nullptr;
    size_t bytes = 0;
    ~ThreadTraceBuffer()
    {
        if (ptr) cudaFree(ptr);  // at thread exit (an error after the runtime is gone is ignored)
    }
};

// this thread's buffer for `device`, or null (device index past the table: no reuse)
ThreadTraceBuffer* thread_trace_buffer(int device)
{
    constexpr int                  kDevices = 64;
    thread_local ThreadTraceBuffer buffers[kDevices];
    return device >= 0 && device < kDevices ? &buffers[device] : nullptr;
}

static int trace_impl(mcrt_scene* s, const mcrt_ray* rays, int64_t n, void* out, bool any, int32_t traverse,
                      int32_t ptr_mode, void* stream)
{
    if (!s || (!rays && n > 0) || (!out && n > 0)) return fail(MCRT_ERR_INVALID_ARGUMENT, "null argument");
    if (n < 0) return fail(MCRT_ERR_INVALID_ARGUMENT, "negative ray count");
    if (traverse != MCRT_TRAVERSE_FAST && traverse != MCRT_TRAVERSE_REF)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "unknown traversal mode");
    if (n == 0) return MCRT_OK;
    if (stack_depth(s, traverse) + 2 >= kStack)
        return fail(MCRT_ERR_STACK_OVERFLOW, "BVH deeper than the traversal stack");
    CK(cudaSetDevice(s->device));
    cudaStream_t  st = static_cast<cudaStream_t>(stream);
    const float4* d_rays = reinterpret_cast<const float4*>(rays);
    void*         d_out = out;
    void*         tmp_rays = nullptr;
    void*         tmp_out = nullptr;
    size_t        out_bytes = static_cast<size_t>(n) * (any ? sizeof(int) : sizeof(float4));
    // The kernel's error word and ray counter (TraceStatus): with host buffers, in the
    // call's own temporary allocation, so calls that share a stream from several host
    // threads (SceneBVH's one-ray queries from OpenMP threads on the default stream) never
    // share a counter; with device buffers, one per stream (one host thread per stream).
    const size_t  status_off = (out_bytes + 15) & ~static_cast<size_t>(15);
    TraceStatus*  d_status = nullptr;
    bool          owned = false;  // tmp_rays / tmp_out allocated by this call (freed at its end)
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        // small requests (the SceneBVH backend's one-ray queries) reuse a buffer kept per
        // host thread and device: no cudaMalloc / cudaFree (which synchronises the device)
        // per call
        const size_t rays_bytes = (sizeof(mcrt_ray) * n + 15) & ~static_cast<size_t>(15);
        const size_t need = rays_bytes + status_off + sizeof(TraceStatus);
        ThreadTraceBuffer* tb = thread_trace_buffer(s->device);
        if (tb && need <= kThreadTraceBufferMax)
        {
            if (tb->bytes < need)
            {
                if (cudaMalloc(&tb->ptr, kThreadTraceBufferMax) != cudaSuccess)
                {
                    tb->ptr = nullptr;
                    return fail(MCRT_ERR_OUT_OF_MEMORY, "trace buffer allocation failed");
                }
                tb->bytes = kThreadTraceBufferMax;
            }
            tmp_rays = tb->ptr;
            tmp_out = static_cast<char*>(tb->ptr) + rays_bytes;
        }
        else
        {
            CK(cudaMalloc(&tmp_rays, sizeof(mcrt_ray) * n));
            cudaError_t e = cudaMalloc(&tmp_out, status_off + sizeof(TraceStatus));
            if (e != cudaSuccess)
            {
                cudaFree(tmp_rays);
                return fail(MCRT_ERR_OUT_OF_MEMORY, "trace buffer allocation failed");
            }
            owned = true;
        }
        CK(cudaMemcpyAsync(tmp_rays, rays, sizeof(mcrt_ray) * n, cudaMemcpyHostToDevice, st));
        d_rays = static_cast<const float4*>(tmp_rays);
        d_out = tmp_out;
        d_status = reinterpret_cast<TraceStatus*>(static_cast<char*>(tmp_out) + status_off);
    }
    else
    {
        std::lock_guard<std::mutex> lock(s->mu);
        TraceStatus*&               slot = s->err_by_stream[stream];
        if (!slot)
        {
            cudaError_t e = cudaMalloc(&slot, sizeof(TraceStatus));
            if (e != cudaSuccess)
            {
                slot = nullptr;
                s->err_by_stream.erase(stream);
                return fail(MCRT_ERR_OUT_OF_MEMORY, "trace status allocation failed");
            }
        }
        d_status = slot;
    }
    CK(cudaMemsetAsync(d_status, 0, sizeof(TraceStatus), st));
    int*                d_err = &d_status->err;
    unsigned long long* d_fetch = &d_status->fetch;
    float4*             hits = static_cast<float4*>(d_out);
    int*                o = static_cast<int*>(d_out);
    const bool          small = stack_depth(s, traverse) + 2 < kSmallStack;
    auto launch = [&](auto kernel) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kTraceBlock, 0);
        const int64_t want = (n + kTraceBlock - 1) / kTraceBlock;
        const int grid = static_cast<int>(std::min<int64_t>(want, static_cast<int64_t>(num_sms()) * std::max(occ, 1)));
        kernel<<<grid, kTraceBlock, 0, st>>>(s->view, d_rays, n, hits, o, d_err, d_fetch);
    };
    if (traverse == MCRT_TRAVERSE_REF)
        any ? launch(k_trace<true, 1, kStack, 1>) : launch(k_trace<false, 1, kStack, 1>);
    else if (small)
        any ? launch(k_trace<true, 0, kSmallStack, kAnyHitMinBlocks>) : launch(k_trace<false, 0, kSmallStack, kTraceMinBlocks>);
    else
        any ? launch(k_trace<true, 0, kStack, kAnyHitMinBlocks>) : launch(k_trace<false, 0, kStack, kTraceMinBlocks>);
    CK(cudaGetLastError());
    int herr = 0;
    if (ptr_mode != MCRT_PTR_DEVICE) CK(cudaMemcpyAsync(out, tmp_out, out_bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (owned)
    {
        cudaFree(tmp_rays);
        cudaFree(tmp_out);
    }
    if (herr & kErrStack) return fail(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    return MCRT_OK;
}

int mcrt_trace_closest(mcrt_scene* s, const mcrt_ray* rays, int64_t n, mcrt_hit* hits, int32_t traverse,
                       int32_t ptr_mode, void* stream)
{
    try
    {
        return trace_impl(s, rays, n, hits, false, traverse, ptr_mode, stream);
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_trace_closest");
    }
}

int mcrt_trace_any(mcrt_scene* s, const mcrt_ray* rays, int64_t n, int32_t* occluded, int32_t traverse,
                   int32_t ptr_mode, void* stream)
{
    try
    {
        return trace_impl(s, rays, n, occluded, true, traverse, ptr_mode, stream);
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_trace_any");
    }
}

int mcrt_render(mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p, float* rgb, mcrt_render_stats* st,
                void* stream)
{
    try
    {
        float* outs[1] = {rgb};
        return render_jobs(1, &s, c, p, outs, st, static_cast<cudaStream_t>(stream));
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_render");
    }
}

int mcrt_render_batch(int32_t n, mcrt_scene* const* scenes, const mcrt_camera* cams, const mcrt_render_params* params,
                      float* const* outs, mcrt_render_stats* st, void* stream)
{
    if (n <= 0 || !scenes || !cams || !params || !outs) return fail(MCRT_ERR_INVALID_ARGUMENT, "empty batch");
    for (int j = 1; j < n; ++j)
        if (params[j].ptr_mode != params[0].ptr_mode)
            return fail(MCRT_ERR_INVALID_ARGUMENT, "all jobs of a batch share ptr_mode");
    try
    {
        return render_jobs(n, scenes, cams, params, outs, st, static_cast<cudaStream_t>(stream));
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_render_batch");
    }
}

static int adjoint_jobs(int num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cams,
                        const mcrt_render_params* params, const float* const* dLs, float* d_albedo, int32_t n_albedo,
                        float* d_emis, int32_t n_emis, mcrt_render_stats* stats, cudaStream_t st)
{
    if (num_jobs <= 0 || !scenes || !cams || !params || !dLs)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "empty adjoint batch");
    const int ptr_mode = params[0].ptr_mode;
    for (int j = 0; j < num_jobs; ++j)
    {
        int rc = validate_job_impl(scenes[j], &cams[j], &params[j]);
        if (rc) return rc;
        if (!dLs[j]) return fail(MCRT_ERR_INVALID_ARGUMENT, "null dL/dimage buffer");
        if (params[j].ptr_mode != ptr_mode) return fail(MCRT_ERR_INVALID_ARGUMENT, "all jobs share ptr_mode");
        if (stack_depth(scenes[j], params[j].traverse) + 2 >= kStack)
            return fail(MCRT_ERR_STACK_OVERFLOW, "BVH deeper than the stack");
    }
    if ((n_albedo > 0 && !d_albedo) || (n_emis > 0 && !d_emis) || n_albedo < 0 || n_emis < 0)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "null gradient buffer");
    mcrt_scene* owner = scenes[0];
    if (owner->device < 0 || owner->device >= kMaxDevices) return fail(MCRT_ERR_INVALID_ARGUMENT, "device index");
    std::lock_guard<std::mutex> lock(owner->mu);
    DeviceWorkspace&            dw = device_workspace(owner->device);
    std::lock_guard<std::mutex> wlock(dw.mu);
    CK(cudaSetDevice(owner->device));
    std::vector<void*> temp;
    auto               cleanup = [&]() {
        for (void* t : temp) cudaFree(t);
    };
    auto dev_alloc = [&](size_t bytes) -> void* {
        void* d = nullptr;
        if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
        temp.push_back(d);
        return d;
    };
    std::vector<JobGPU> jobs(num_jobs);
    int64_t             total = 0;
    int64_t             h2d = 0, d2h = 0;
    for (int j = 0; j < num_jobs; ++j)
    {
        const mcrt_camera&        c = cams[j];
        const mcrt_render_params& p = params[j];
        JobGPU&                   J = jobs[j];
        J.scene = scenes[j]->view;
        J.cam = make_camera_impl(c);
        J.width = c.width;
        J.height = c.height;
        J.spp = p.spp;
        J.max_depth = p.max_depth;
        J.rr_depth = p.rr_depth;
        J.traverse = p.traverse;
        J.seed = p.seed;
        J.path_offset = total;
        int64_t px = static_cast<int64_t>(c.width) * c.height;
        total += px * p.spp;
        if (ptr_mode == MCRT_PTR_DEVICE)
        {
            J.image = const_cast<float*>(dLs[j]);
        }
        else
        {
            void* d = dev_alloc(sizeof(float) * 3 * px);
            if (!d)
            {
                cleanup();
                return fail(MCRT_ERR_OUT_OF_MEMORY, "adjoint buffer allocation failed");
            }
            CK(cudaMemcpyAsync(d, dLs[j], sizeof(float) * 3 * px, cudaMemcpyHostToDevice, st));
            h2d += static_cast<int64_t>(sizeof(float) * 3 * px);
            J.image = static_cast<float*>(d);
        }
    }
    float* dga = d_albedo;
    float* dge = d_emis;
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        void* a2 = dev_alloc(sizeof(float) * 3 * std::max(n_albedo, 1));
        void* a3 = dev_alloc(sizeof(float) * 3 * std::max(n_emis, 1));
        if (!a2 || !a3)
        {
            cleanup();
            return fail(MCRT_ERR_OUT_OF_MEMORY, "adjoint buffer allocation failed");
        }
        if (n_albedo > 0) CK(cudaMemcpyAsync(a2, d_albedo, sizeof(float) * 3 * n_albedo, cudaMemcpyHostToDevice, st));
        if (n_emis > 0) CK(cudaMemcpyAsync(a3, d_emis, sizeof(float) * 3 * n_emis, cudaMemcpyHostToDevice, st));
        h2d += sizeof(float) * 3 * (n_albedo + n_emis);
        dga = static_cast<float*>(a2);
        dge = static_cast<float*>(a3);
    }
    Workspace& w = dw.ws;
    // the wavefront replay (default) needs the vertex log to hold every vertex and 16-bit
    // material ids; otherwise, or with MCRT_SCHEDULE_WAVES, one thread replays each path
    int  max_depth = 0, bvh_depth = 0;
    bool small_ids = true;
    for (int j = 0; j < num_jobs; ++j)
    {
        max_depth = std::max(max_depth, params[j].max_depth);
        bvh_depth = std::max(bvh_depth, stack_depth(scenes[j], params[j].traverse));
        small_ids = small_ids && scenes[j]->num_materials <= 65536;
    }
    if (params[0].schedule == MCRT_SCHEDULE_STREAM && max_depth < kAdjLog && small_ids)
    {
        w.args.batch_fetch = 1;
        RunResult run;
        int       rc = adjoint_stream(w, jobs, total, max_depth, bvh_depth, params[0].path_chunk, dga, n_albedo, dge,
                                      n_emis, st, run);
        if (rc)
        {
            cudaStreamSynchronize(st);
            cleanup();
            return rc;
        }
        h2d += static_cast<int64_t>(sizeof(JobGPU)) * num_jobs;
        if (ptr_mode != MCRT_PTR_DEVICE)
        {
            if (n_albedo > 0) CK(cudaMemcpyAsync(d_albedo, dga, sizeof(float) * 3 * n_albedo, cudaMemcpyDeviceToHost, st));
            if (n_emis > 0) CK(cudaMemcpyAsync(d_emis, dge, sizeof(float) * 3 * n_emis, cudaMemcpyDeviceToHost, st));
            d2h += sizeof(float) * 3 * (n_albedo + n_emis);
        }
        unsigned long long hstats[8];
        int                herr = 0;
        CK(cudaMemcpyAsync(hstats, w.stats, sizeof(hstats), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&herr, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        d2h += sizeof(hstats) + sizeof(herr) + run.poll_bytes;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, run.e0, run.e1);
        cudaEventDestroy(run.e0);
        cudaEventDestroy(run.e1);
        cleanup();
        if (stats)
        {
            *stats = mcrt_render_stats{};
            stats->paths = total;
            stats->extension_rays = static_cast<int64_t>(hstats[0]);
            stats->shadow_rays = static_cast<int64_t>(hstats[1]);
            stats->waves = static_cast<int32_t>(run.waves);
            stats->kernel_launches = static_cast<int32_t>(run.launches);
            stats->extend_launches = static_cast<int32_t>(run.extend_launches);
            stats->device_ms = ms;
            stats->h2d_bytes = h2d;
            stats->d2h_bytes = d2h;
        }
        if (herr & kErrStack) return fail(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
        if (herr & kErrQueue) return fail(MCRT_ERR_QUEUE_OVERFLOW, "queue overflow");
        return MCRT_OK;
    }
    int rc = ensure_workspace(w, 0, 0, num_jobs, 1);
    if (rc)
    {
        cleanup();
        return rc;
    }
    CK(cudaMemcpyAsync(w.jobs, jobs.data(), sizeof(JobGPU) * num_jobs, cudaMemcpyHostToDevice, st));
    h2d += static_cast<int64_t>(sizeof(JobGPU)) * num_jobs;
    CK(cudaMemsetAsync(w.stats, 0, sizeof(unsigned long long) * 8, st));
    CK(cudaMemsetAsync(w.err, 0, sizeof(int), st));
    AdjointArgs aa;
    aa.jobs = w.jobs;
    aa.num_jobs = num_jobs;
    aa.g_albedo = dga;
    aa.n_albedo = n_albedo;
    aa.g_emis = dge;
    aa.n_emis = n_emis;
    aa.total_paths = total;
    aa.stats = w.stats;
    aa.err = w.err;
    // the same bound as the wavefront's (one view of cfg4's scene with 4096 albedos, depth
    // 16: 5.8 ms in global memory, 11.1 ms per block; cfg3's 256: 7.0 per block, 20.3 global)
    size_t gbytes = sizeof(float) * 3 * static_cast<size_t>(n_albedo + n_emis);
    aa.shared_grads = gbytes <= kGradSharedMax ? 1 : 0;
    size_t dyn = aa.shared_grads ? gbytes : 0;
    // the static traversal stack plus the gradient accumulators may exceed the 48 KB default
    CK(cudaFuncSetAttribute(k_adjoint<kStack>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn)));
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adjoint<kStack>, kAdjBlock, dyn);
    int64_t want = (total + kAdjBlock - 1) / kAdjBlock;
    int     grid = static_cast<int>(std::min<int64_t>(want, static_cast<int64_t>(num_sms()) * std::max(occ, 1)));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    k_adjoint<kStack><<<grid, kAdjBlock, dyn, st>>>(aa);
    CK(cudaGetLastError());
    CK(cudaEventRecord(e1, st));
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        if (n_albedo > 0) CK(cudaMemcpyAsync(d_albedo, dga, sizeof(float) * 3 * n_albedo, cudaMemcpyDeviceToHost, st));
        if (n_emis > 0) CK(cudaMemcpyAsync(d_emis, dge, sizeof(float) * 3 * n_emis, cudaMemcpyDeviceToHost, st));
        d2h += sizeof(float) * 3 * (n_albedo + n_emis);
    }
    unsigned long long hstats[8];
    int                herr = 0;
    CK(cudaMemcpyAsync(hstats, w.stats, sizeof(hstats), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    d2h += sizeof(hstats) + sizeof(herr);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (stats)
    {
        *stats = mcrt_render_stats{};
        stats->paths = total;
        stats->extension_rays = static_cast<int64_t>(hstats[0]);
        stats->waves = 1;
        stats->kernel_launches = 1;
        stats->device_ms = ms;
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
    }
    if (herr & kErrStack) return fail(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    return MCRT_OK;
}

int mcrt_render_adjoint(mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p, const float* dL,
                        float* d_albedo, int32_t n_albedo, float* d_emis, int32_t n_emis, mcrt_render_stats* stats,
                        void* stream)
{
    try
    {
        if (!s || !c || !p) return fail(MCRT_ERR_INVALID_ARGUMENT, "null scene, camera or params");
        const float* dls[1] = {dL};
        return adjoint_jobs(1, &s, c, p, dls, d_albedo, n_albedo, d_emis, n_emis, stats,
                            static_cast<cudaStream_t>(stream));
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_render_adjoint");
    }
}

int mcrt_render_adjoint_batch(int32_t num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cameras,
                              const mcrt_render_params* params, const float* const* dL_dimages, float* d_albedo,
                              int32_t num_albedo_params, float* d_emission, int32_t num_emission_params,
                              mcrt_render_stats* stats, void* stream)
{
    try
    {
        return adjoint_jobs(num_jobs, scenes, cameras, params, dL_dimages, d_albedo, num_albedo_params, d_emission,
                            num_emission_params, stats, static_cast<cudaStream_t>(stream));
    }
    catch (...)
    {
        return fail(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_render_adjoint_batch");
    }
}

}  // extern "C"
