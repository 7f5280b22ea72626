// CUDA kernels (sm_103a) and the C ABI of mcrt_gb300.h.
//
// Kernels:
//   k_trace<ANY, MODE>   batch closest/any-hit queries (SceneBVH::intersect / occluded)
//   wavefront, one set of launches per wave of paths (all graph-capturable: every
//   count is read from device memory, grids are fixed):
//     k_begin_chunk      load the wave's path range from the chunk table
//     k_raygen           camera rays with the tent filter (demo_pt.cpp:689-700)
//     k_extend           closest hit of the live-path queue
//     k_shade            one vertex of rayTrace (demo_pt.cpp:523-651): emission, NEE with
//                        MIS against the environment and the area lights, continuation,
//                        Russian roulette; live paths and shadow rays are appended to
//                        SoA queues by warp ballot / warp prefix sum + one atomic per warp
//     k_connect          shadow rays: any hit (environment) or bounded closest hit (area
//                        lights, which must hit the sampled emitter), MIS-weighted add
//     k_resolve          per-pixel mean of the clamped per-sample radiance
//   k_adjoint            path-replay adjoint (one thread per path, replayed from its seed)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "device.cuh"
#include "host.h"

namespace mcrt {
std::string prepare_scene(const mcrt_scene_desc& d, HostScene& hs);

constexpr int kTraceBlock = 128;
constexpr int kStack = 64;
constexpr int kMaxDepth = 62;

// ---------------------------------------------------------------------------
// batch trace
// ---------------------------------------------------------------------------
template <bool ANY, int MODE>
__global__ void __launch_bounds__(kTraceBlock) k_trace(SceneView s, const float4* __restrict__ rays, int64_t n,
                                                       float4* __restrict__ hits, int* __restrict__ occ, int* err)
{
    __shared__ int stack[kStack * kTraceBlock];
    int*           st = stack + threadIdx.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        float4 a = rays[2 * i], b = rays[2 * i + 1];
        Hit    h;
        bool   any = trace_ray<ANY, kStack>(s, MODE, xyz(a), xyz(b), a.w, b.w, st, kTraceBlock, h, err);
        if (ANY)
            occ[i] = any ? 1 : 0;
        else
            hits[i] = any ? make_float4(h.t, h.u, h.v, __int_as_float(h.prim))
                          : make_float4(__int_as_float(0x7f800000), 0.f, 0.f, __int_as_float(-1));
    }
}

// ---------------------------------------------------------------------------
// wavefront state
// ---------------------------------------------------------------------------
struct Ctrl
{
    int64_t base;
    int     count;
    int     chunk;
    int     qcount[kMaxDepth + 2];
    int     scount[kMaxDepth + 1][2];
};

enum ShadowType
{
    SH_ENV = 0,
    SH_AREA_BSDF = 1,
    SH_AREA_LIGHT = 2
};

struct WaveArgs
{
    Ctrl*               ctrl;
    const int64_t*      chunk_table;
    const JobGPU*       jobs;
    int                 num_jobs;
    int64_t             capacity;
    float4*             qo[2];
    float4*             qd[2];
    int*                qp[2];
    float4*             hits;
    float4*             thr;
    float4*             rad;
    uint64_t*           rng;
    int*                pix;
    int*                job;
    float4*             so[2];  // [0] any-hit queue, [1] closest-hit queue
    float4*             sd[2];
    float4*             sv[2];
    int4*               sm[2];
    int64_t             shadow_cap;
    unsigned long long* stats;  // [0] extension rays, [1] shadow rays
    int*                err;
};

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

__global__ void k_begin_chunk(WaveArgs a)
{
    Ctrl* c = a.ctrl;
    int   idx = c->chunk;
    c->base = a.chunk_table[idx];
    c->count = static_cast<int>(a.chunk_table[idx + 1] - a.chunk_table[idx]);
    c->qcount[0] = c->count;
    for (int d = 1; d < kMaxDepth + 2; ++d) c->qcount[d] = 0;
    for (int d = 0; d < kMaxDepth + 1; ++d) c->scount[d][0] = c->scount[d][1] = 0;
    c->chunk = idx + 1;
}

__global__ void k_raygen(WaveArgs a)
{
    const int     count = a.ctrl->count;
    const int64_t base = a.ctrl->base;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x)
    {
        int64_t       g = base + p;
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
        a.qo[0][p] = make_float4(o.x, o.y, o.z, kEpsRay);
        a.qd[0][p] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
        a.qp[0][p] = p;
        a.thr[p] = make_float4(1.f, 1.f, 1.f, __int_as_float(0));
        a.rad[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.rng[p] = rng.state;
        a.pix[p] = pixel;
        a.job[p] = j;
    }
}

template <int STACK>
__global__ void __launch_bounds__(kTraceBlock) k_extend(WaveArgs a, int depth)
{
    __shared__ int stack[STACK * kTraceBlock];
    int*           st = stack + threadIdx.x;
    const int      n = a.ctrl->qcount[depth];
    const int      qs = depth & 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stats[0], static_cast<unsigned long long>(n));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        float4 o = a.qo[qs][i], d = a.qd[qs][i];
        int    p = a.qp[qs][i];
        int    j = a.job[p];
        Hit    h;
        bool   hit = trace_ray<false, STACK>(a.jobs[j].scene, a.jobs[j].traverse, xyz(o), xyz(d), o.w, d.w, st,
                                           kTraceBlock, h, a.err);
        a.hits[i] = hit ? make_float4(h.t, h.u, h.v, __int_as_float(h.prim))
                        : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    }
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

struct ShadowRay
{
    float3 d;
    float  tmax;
    float4 val;
    int    type, light;
};

__global__ void __launch_bounds__(128) k_shade(WaveArgs a, int depth)
{
    const int n = a.ctrl->qcount[depth];
    const int qs = depth & 1;
    const int lane = threadIdx.x & 31;
    const int warps_total = (gridDim.x * blockDim.x) >> 5;
    for (int wbase = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; wbase < n; wbase += warps_total * 32)
    {
        int  i = wbase + lane;
        bool valid = i < n;
        // outputs of this lane
        bool      cont = false;
        float3    phit = mk(0.f, 0.f, 0.f), cdir = mk(0.f, 0.f, 1.f);
        float3    T2 = mk(0.f, 0.f, 0.f);
        int       flags2 = 0;
        ShadowRay sh_any[2], sh_cl[2];
        int       n_any = 0, n_cl = 0;
        int       p = 0;
        uint64_t  rstate = 0;
        if (valid)
        {
            float4        o4 = a.qo[qs][i], d4 = a.qd[qs][i];
            float4        hh = a.hits[i];
            float3        o = xyz(o4), d = xyz(d4);
            p = a.qp[qs][i];
            const JobGPU& J = a.jobs[a.job[p]];
            const SceneView& S = J.scene;
            float4        t4 = a.thr[p];
            float3        T = xyz(t4);
            int           flags = __float_as_int(t4.w);
            bool          no_direct = depth == 0 || !(flags & 1);
            int           prim = __float_as_int(hh.w);
            float3        Ladd = mk(0.f, 0.f, 0.f);
            if (prim < 0)
            {
                if (no_direct && S.env_w > 0) Ladd = T * env_radiance(S, d);
            }
            else
            {
                int    matid;
                float3 ns = shading_normal(S, prim, hh.y, hh.z, matid);
                Mat    m = load_mat(S, matid);
                phit = o + d * hh.x;
                if (m.type == MAT_LGHT)
                {
                    if (no_direct && dot3(d, ns) < 0.f) Ladd = T * m.color;
                }
                else
                {
                    Pcg rng;
                    rng.state = a.rng[p];
                    rng.inc = (static_cast<uint64_t>(a.pix[p]) << 1u) | 1u;
                    float u[NUM_DIMS];
#pragma unroll
                    for (int k = 0; k < NUM_DIMS; ++k) u[k] = rng.uniform();
                    rstate = rng.state;
                    float3 wi = -d;
                    bool   nee = does_nee(m.type);
                    if (nee)
                    {
                        if (S.env_w > 0)
                        {
                            // sampleEnvmapUsingLightPDF (demo_pt.cpp:430-465)
                            float3 ldir, lrad;
                            float  lpdf;
                            env_sample(S, u[D_ENV_LIGHT_0], u[D_ENV_LIGHT_1], u[D_ENV_JITTER_U], u[D_ENV_JITTER_V],
                                       ldir, lrad, lpdf);
                            float g = fmax_ref(0.f, dot3(ldir, ns));
                            if (g > 0.f)
                            {
                                float  pe = env_pdf(S, ldir);
                                float  wE = pe / (pe + bsdf_pdf(m, wi, ns, ldir));
                                float3 irr = (bsdf_eval(m, wi, ns, ldir) * g * (1.0f / lpdf)) * lrad;
                                float3 val = T * (irr * wE);
                                if (!isnan3(val))
                                    sh_any[n_any++] = ShadowRay{ldir, __int_as_float(0x7f800000),
                                                                make_float4(val.x, val.y, val.z, 0.f), SH_ENV, 0};
                            }
                            // sampleEnvmapUsingSurfacePDF (demo_pt.cpp:466-507); GGX samples itself
                            if (m.type == MAT_DIFF)
                            {
                                float  r1 = 2.f * kPi * u[D_ENV_BSDF_0], r2 = u[D_ENV_BSDF_1], r2s = sqrtf(r2);
                                float3 w = ns;
                                float3 uu = normalize3(cross3(mk(0.3f, 0.4f, 0.5f), w));
                                float3 vv = cross3(w, uu);
                                float3 wo = normalize3(uu * (cosf(r1) * r2s) + vv * (sinf(r1) * r2s) + w * sqrtf(1.f - r2));
                                float  g2 = fmax_ref(0.f, dot3(wo, ns));
                                if (g2 > 0.f)
                                {
                                    float  pb = bsdf_pdf(m, wi, ns, wo);
                                    float  wB = pb / (pb + env_pdf(S, wo));
                                    float3 val = T * ((m.color * env_radiance(S, wo)) * wB);
                                    if (!isnan3(val))
                                        sh_any[n_any++] = ShadowRay{wo, __int_as_float(0x7f800000),
                                                                    make_float4(val.x, val.y, val.z, 0.f), SH_ENV, 0};
                                }
                            }
                            else
                            {
                                BsdfSample bs = bsdf_sample(m, wi, ns, u[D_ENV_BSDF_0], u[D_ENV_BSDF_1]);
                                if (maxc(bs.weight) > 0.f && bs.pdf > 0.f)
                                {
                                    float  wB = bs.pdf / (bs.pdf + env_pdf(S, bs.wo));
                                    float3 val = T * ((bs.weight * env_radiance(S, bs.wo)) * wB);
                                    if (!isnan3(val))
                                        sh_any[n_any++] = ShadowRay{bs.wo, __int_as_float(0x7f800000),
                                                                    make_float4(val.x, val.y, val.z, 0.f), SH_ENV, 0};
                                }
                            }
                        }
                        if (S.light_area > 0.f)
                        {
                            // BSDF sample with MIS (demo_pt.cpp:593-614)
                            BsdfSample bs = bsdf_sample(m, wi, ns, u[D_AREA_BSDF_0], u[D_AREA_BSDF_1]);
                            if (maxc(bs.weight) > 0.f)
                            {
                                float3 val = T * bs.weight;
                                sh_cl[n_cl++] = ShadowRay{bs.wo, __int_as_float(0x7f800000),
                                                          make_float4(val.x, val.y, val.z, bs.pdf), SH_AREA_BSDF, 0};
                            }
                            // light sample (demo_pt.cpp:618-641; scene.cpp:298-343)
                            int lo = 0, hi = S.num_lights - 1;
                            while (hi > lo)
                            {
                                int mid = lo + (hi - lo) / 2;
                                if (S.lights[mid].cdf >= u[D_LIGHT_PICK])
                                    hi = mid;
                                else
                                    lo = mid + 1;
                            }
                            LightGPU      L = S.lights[lo];
                            const float4* lv = S.prim_verts + 3 * L.prim;
                            float         r0 = sqrtf(u[D_LIGHT_U]);
                            float         lu = 1.f - r0, lvv = u[D_LIGHT_V] * r0;
                            float3 lp = xyz(lv[0]) * (1.f - lu - lvv) + xyz(lv[1]) * lu + xyz(lv[2]) * lvv;
                            int    lm;
                            float3 ln = shading_normal(S, L.prim, lu, lvv, lm);
                            float  pdfA = (1.f / L.area) * L.pdf;
                            float3 wo = lp - phit;
                            float  dist2 = dot3(wo, wo);
                            wo = normalize3(wo);
                            float cosl = dot3(ln, -wo);
                            float pdfW = pdfA * dist2 / fabsf(cosl);
                            if (cosl <= 0.f) pdfW = 0.f;
                            if (pdfW > 0.f)
                            {
                                float  pb = bsdf_pdf(m, wi, ns, wo);
                                float  mis = pdfW / (pdfW + pb);
                                float3 f = bsdf_eval(m, wi, ns, wo);
                                float  cs = fmaxf(dot3(ns, wo), 0.f);
                                if (maxc(f) > 0.f && cs > 0.f)
                                {
                                    float3 val = T * (f * (cs / pdfW * mis));
                                    sh_cl[n_cl++] = ShadowRay{wo, sqrtf(dist2) * 1.001f + kEpsRay,
                                                              make_float4(val.x, val.y, val.z, 0.f), SH_AREA_LIGHT, lo};
                                }
                            }
                        }
                    }
                    // continuation (demo_pt.cpp:647-650) and Russian roulette
                    BsdfSample cs = bsdf_sample(m, wi, ns, u[D_CONT_0], u[D_CONT_1]);
                    T2 = T * cs.weight;
                    cont = depth < J.max_depth;
                    if (J.rr_depth >= 0 && depth >= J.rr_depth)
                    {
                        float q = fminf(fmaxf(maxc(m.color), 0.f), 1.f);
                        if (u[D_RR] >= q)
                            cont = false;
                        else
                            T2 = T2 * (1.f / q);
                    }
                    if (!(maxc(T2) > 0.f)) cont = false;
                    cdir = cs.wo;
                    flags2 = nee ? 1 : 0;
                }
            }
            if (Ladd.x != 0.f || Ladd.y != 0.f || Ladd.z != 0.f)
            {
                float4 r = a.rad[p];
                a.rad[p] = make_float4(r.x + Ladd.x, r.y + Ladd.y, r.z + Ladd.z, r.w);
            }
        }
        // compaction of live paths into the next queue (ballot + popc)
        unsigned live = __ballot_sync(0xffffffffu, cont);
        if (live)
        {
            int base = 0;
            if (lane == 0) base = atomicAdd(&a.ctrl->qcount[depth + 1], __popc(live));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (cont)
            {
                int k = base + __popc(live & lanemask_lt());
                int qn = qs ^ 1;
                if (k < a.capacity)
                {
                    a.qo[qn][k] = make_float4(phit.x, phit.y, phit.z, kEpsRay);
                    a.qd[qn][k] = make_float4(cdir.x, cdir.y, cdir.z, __int_as_float(0x7f800000));
                    a.qp[qn][k] = p;
                    a.thr[p] = make_float4(T2.x, T2.y, T2.z, __int_as_float(flags2));
                    a.rng[p] = rstate;
                }
                else
                {
                    atomicOr(a.err, kErrQueue);
                }
            }
        }
        // shadow rays (warp prefix sum + one atomic per warp and queue)
        for (int qsel = 0; qsel < 2; ++qsel)
        {
            int k = qsel == 0 ? n_any : n_cl;
            int b = warp_append(&a.ctrl->scount[depth][qsel], k);
            for (int r = 0; r < 2; ++r)
            {
                if (r >= k) break;
                const ShadowRay& sr = qsel == 0 ? sh_any[r] : sh_cl[r];
                int              idx = b + r;
                if (idx >= a.shadow_cap)
                {
                    atomicOr(a.err, kErrQueue);
                    break;
                }
                a.so[qsel][idx] = make_float4(phit.x, phit.y, phit.z, kEpsRay);
                a.sd[qsel][idx] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.tmax);
                a.sv[qsel][idx] = sr.val;
                a.sm[qsel][idx] = make_int4(p, sr.type, sr.light, 0);
            }
        }
    }
}

template <int STACK>
__global__ void __launch_bounds__(kTraceBlock) k_connect(WaveArgs a, int depth)
{
    __shared__ int stack[STACK * kTraceBlock];
    int*           st = stack + threadIdx.x;
    const int      n0 = a.ctrl->scount[depth][0];
    const int      n1 = a.ctrl->scount[depth][1];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stats[1], static_cast<unsigned long long>(n0 + n1));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n0 + n1; i += gridDim.x * blockDim.x)
    {
        int    q = i < n0 ? 0 : 1;
        int    k = i < n0 ? i : i - n0;
        float4 o = a.so[q][k], d = a.sd[q][k], v = a.sv[q][k];
        int4   m = a.sm[q][k];
        int    p = m.x;
        const JobGPU&    J = a.jobs[a.job[p]];
        const SceneView& S = J.scene;
        Hit              h;
        float3           add = mk(0.f, 0.f, 0.f);
        if (q == 0)
        {
            if (!trace_ray<true, STACK>(S, J.traverse, xyz(o), xyz(d), o.w, d.w, st, kTraceBlock, h, a.err))
                add = xyz(v);
        }
        else if (trace_ray<false, STACK>(S, J.traverse, xyz(o), xyz(d), o.w, d.w, st, kTraceBlock, h, a.err))
        {
            int    matid;
            float3 dir = xyz(d);
            float3 ns = shading_normal(S, h.prim, h.u, h.v, matid);
            Mat    hm = load_mat(S, matid);
            if (hm.type == MAT_LGHT && !(dot3(ns, -dir) < 0.f))
            {
                if (m.y == SH_AREA_BSDF)
                {
                    // Scene::lightPdfW (scene.cpp:239-267) + lightRadiance (:345-366)
                    float cl = dot3(ns, -dir);
                    float pdfL = 0.f;
                    if (cl >= 1e-6f)
                    {
                        LightGPU L = S.lights[S.light_of[h.prim]];
                        float    pdfA = (1.f / L.area) * L.pdf;
                        pdfL = pdfA * (h.t * h.t) / cl;
                    }
                    float mis = v.w / (v.w + pdfL);
                    add = xyz(v) * hm.color * mis;
                }
                else if (S.light_of[h.prim] == m.z)
                {
                    add = xyz(v) * hm.color;
                }
            }
        }
        if (add.x != 0.f || add.y != 0.f || add.z != 0.f)
        {
            atomicAdd(&a.rad[p].x, add.x);
            atomicAdd(&a.rad[p].y, add.y);
            atomicAdd(&a.rad[p].z, add.z);
        }
    }
}

__global__ void k_resolve(WaveArgs a)
{
    const int     count = a.ctrl->count;
    const int64_t base = a.ctrl->base;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x)
    {
        int64_t       g = base + p;
        int           j = find_job(a.jobs, a.num_jobs, g);
        const JobGPU& J = a.jobs[j];
        int64_t       local = g - J.path_offset;
        if (local % J.spp != 0) continue;
        int   pixel = static_cast<int>(local / J.spp);
        float s[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < J.spp; ++k)
        {
            float4 r = a.rad[p + k];
            if (isnan3(xyz(r))) r = make_float4(0.f, 0.f, 0.f, 0.f);  // demo_pt.cpp:653
            s[0] += fmax_ref(0.f, r.x);                                // demo_pt.cpp:703
            s[1] += fmax_ref(0.f, r.y);
            s[2] += fmax_ref(0.f, r.z);
        }
        float scale = static_cast<float>(1.0 / J.spp);  // FrameBuffer::scale(1.0 / spp)
        float* px = J.image + 3 * static_cast<int64_t>(pixel);
        px[0] = s[0] * scale;
        px[1] = s[1] * scale;
        px[2] = s[2] * scale;
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
    int64_t  capacity = 0;
    int      jobs_cap = 0;
    int64_t  chunks_cap = 0;
    WaveArgs args{};
    void*    block = nullptr;  // one allocation for the per-path arrays
    JobGPU*  jobs = nullptr;
    int64_t* chunk_table = nullptr;
    Ctrl*    ctrl = nullptr;
    unsigned long long* stats = nullptr;
    int*     err = nullptr;
    void release()
    {
        cudaFree(block);
        cudaFree(jobs);
        cudaFree(chunk_table);
        cudaFree(ctrl);
        cudaFree(stats);
        cudaFree(err);
        block = nullptr;
        jobs = nullptr;
        chunk_table = nullptr;
        ctrl = nullptr;
        stats = nullptr;
        err = nullptr;
        capacity = 0;
        jobs_cap = 0;
        chunks_cap = 0;
    }
};

}  // namespace

struct mcrt_scene
{
    SceneView          view{};
    std::vector<void*> allocs;
    int64_t            fast_nodes = 0, ref_nodes = 0, refs = 0, bytes = 0;
    int                bvh_depth = 0;
    int                device = 0;
    int                num_materials = 0;
    MaterialGPU*       d_materials = nullptr;
    int*               d_err = nullptr;
    Workspace          ws;
    std::mutex         mu;
};

namespace {

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

CameraGPU make_camera(const mcrt_camera& c)
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

int ensure_workspace(Workspace& w, int64_t capacity, int num_jobs, int64_t num_chunks)
{
    if (w.capacity < capacity)
    {
        cudaFree(w.block);
        w.block = nullptr;
        int64_t C = capacity, S = 2 * capacity;
        // per-path: qo,qd x2 (64 B), qp x2 (8), hits 16, thr 16, rad 16, rng 8, pix 4, job 4
        // shadow: 2 queues x S x (so, sd, sv 48 B + sm 16 B)
        size_t bytes = static_cast<size_t>(C) * (64 + 8 + 16 + 16 + 16 + 8 + 4 + 4) + static_cast<size_t>(S) * 2 * 64 +
                       64 * 32;
        CK(cudaMalloc(&w.block, bytes));
        char* p = static_cast<char*>(w.block);
        auto take = [&](size_t n) {
            size_t off = (reinterpret_cast<uintptr_t>(p) + 255) & ~static_cast<uintptr_t>(255);
            char*  r = reinterpret_cast<char*>(off);
            p = r + n;
            return static_cast<void*>(r);
        };
        WaveArgs& a = w.args;
        for (int k = 0; k < 2; ++k)
        {
            a.qo[k] = static_cast<float4*>(take(16 * C));
            a.qd[k] = static_cast<float4*>(take(16 * C));
            a.qp[k] = static_cast<int*>(take(4 * C));
        }
        a.hits = static_cast<float4*>(take(16 * C));
        a.thr = static_cast<float4*>(take(16 * C));
        a.rad = static_cast<float4*>(take(16 * C));
        a.rng = static_cast<uint64_t*>(take(8 * C));
        a.pix = static_cast<int*>(take(4 * C));
        a.job = static_cast<int*>(take(4 * C));
        for (int k = 0; k < 2; ++k)
        {
            a.so[k] = static_cast<float4*>(take(16 * S));
            a.sd[k] = static_cast<float4*>(take(16 * S));
            a.sv[k] = static_cast<float4*>(take(16 * S));
            a.sm[k] = static_cast<int4*>(take(16 * S));
        }
        a.capacity = C;
        a.shadow_cap = S;
        w.capacity = capacity;
    }
    if (w.jobs_cap < num_jobs)
    {
        cudaFree(w.jobs);
        w.jobs = nullptr;
        CK(cudaMalloc(&w.jobs, sizeof(JobGPU) * num_jobs));
        w.jobs_cap = num_jobs;
    }
    if (w.chunks_cap < num_chunks + 1)
    {
        cudaFree(w.chunk_table);
        w.chunk_table = nullptr;
        CK(cudaMalloc(&w.chunk_table, sizeof(int64_t) * (num_chunks + 1)));
        w.chunks_cap = num_chunks + 1;
    }
    if (!w.ctrl)
    {
        CK(cudaMalloc(&w.ctrl, sizeof(Ctrl)));
        CK(cudaMalloc(&w.stats, sizeof(unsigned long long) * 4));
        CK(cudaMalloc(&w.err, sizeof(int)));
    }
    w.args.ctrl = w.ctrl;
    w.args.jobs = w.jobs;
    w.args.chunk_table = w.chunk_table;
    w.args.stats = w.stats;
    w.args.err = w.err;
    return MCRT_OK;
}

struct LaunchShape
{
    int grid_trace, grid_shade, grid_small, block;
};

template <int STACK>
void enqueue_wave(const WaveArgs& a, int max_depth, const LaunchShape& ls, cudaStream_t st)
{
    k_begin_chunk<<<1, 1, 0, st>>>(a);
    k_raygen<<<ls.grid_small, 256, 0, st>>>(a);
    for (int d = 0; d <= max_depth; ++d)
    {
        k_extend<STACK><<<ls.grid_trace, kTraceBlock, 0, st>>>(a, d);
        k_shade<<<ls.grid_shade, 128, 0, st>>>(a, d);
        k_connect<STACK><<<ls.grid_trace, kTraceBlock, 0, st>>>(a, d);
    }
    k_resolve<<<ls.grid_small, 256, 0, st>>>(a);
}

int validate_job(const mcrt_scene* s, const mcrt_camera* c, const mcrt_render_params* p)
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
    return MCRT_OK;
}

int render_jobs(int num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cams, const mcrt_render_params* params,
                float* const* outs, mcrt_render_stats* stats, cudaStream_t st)
{
    for (int j = 0; j < num_jobs; ++j)
    {
        int rc = validate_job(scenes[j], &cams[j], &params[j]);
        if (rc) return rc;
        if (!outs[j]) return fail(MCRT_ERR_INVALID_ARGUMENT, "null image buffer");
    }
    mcrt_scene* owner = scenes[0];
    std::lock_guard<std::mutex> lock(owner->mu);
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
        J.cam = make_camera(c);
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
        bvh_depth = std::max(bvh_depth, scenes[j]->bvh_depth);
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
    // wave boundaries on pixel boundaries so a pixel's samples resolve together
    int64_t capacity = p0.path_chunk > 0 ? p0.path_chunk : (int64_t(1) << 22);
    capacity = std::max<int64_t>(capacity, 64);
    std::vector<int64_t> table;
    table.push_back(0);
    {
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
    }
    int64_t num_chunks = static_cast<int64_t>(table.size()) - 1;
    int64_t max_chunk = 0;
    for (int64_t k = 0; k < num_chunks; ++k) max_chunk = std::max(max_chunk, table[k + 1] - table[k]);
    Workspace& w = owner->ws;
    int        rc = ensure_workspace(w, max_chunk, num_jobs, num_chunks);
    if (rc)
    {
        cleanup();
        return rc;
    }
    w.args.num_jobs = num_jobs;
    CK(cudaMemcpyAsync(w.jobs, jobs.data(), sizeof(JobGPU) * num_jobs, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w.chunk_table, table.data(), sizeof(int64_t) * table.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w.ctrl, 0, sizeof(Ctrl), st));
    CK(cudaMemsetAsync(w.stats, 0, sizeof(unsigned long long) * 4, st));
    CK(cudaMemsetAsync(w.err, 0, sizeof(int), st));

    LaunchShape ls;
    int         sms = num_sms();
    int         occ_t = 0, occ_s = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_t, k_extend<kStack>, kTraceBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_shade, 128, 0);
    ls.grid_trace = sms * std::max(occ_t, 1);
    ls.grid_shade = sms * std::max(occ_s, 1);
    ls.grid_small = sms * 8;
    ls.block = 128;

    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    int launches = 0;
    if (p0.use_graph)
    {
        cudaGraph_t     graph;
        cudaGraphExec_t exec;
        cudaStream_t    cap;
        CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        enqueue_wave<kStack>(w.args, max_depth, ls, cap);
        CK(cudaStreamEndCapture(cap, &graph));
        CK(cudaGraphInstantiate(&exec, graph, 0));
        for (int64_t k = 0; k < num_chunks; ++k)
        {
            CK(cudaGraphLaunch(exec, st));
            launches += 3 + 3 * (max_depth + 1);
        }
        CK(cudaEventRecord(e1, st));
        CK(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        cudaStreamDestroy(cap);
    }
    else
    {
        for (int64_t k = 0; k < num_chunks; ++k)
        {
            enqueue_wave<kStack>(w.args, max_depth, ls, st);
            launches += 3 + 3 * (max_depth + 1);
        }
        CK(cudaGetLastError());
        CK(cudaEventRecord(e1, st));
    }
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        for (int j = 0; j < num_jobs; ++j)
            CK(cudaMemcpyAsync(outs[j], dev_images[j], sizeof(float) * 3 * cams[j].width * cams[j].height,
                               cudaMemcpyDeviceToHost, st));
    }
    unsigned long long hstats[4];
    int                herr = 0;
    CK(cudaMemcpyAsync(hstats, w.stats, sizeof(hstats), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (stats)
    {
        stats->paths = total;
        stats->extension_rays = static_cast<int64_t>(hstats[0]);
        stats->shadow_rays = static_cast<int64_t>(hstats[1]);
        stats->waves = static_cast<int32_t>(num_chunks);
        stats->kernel_launches = launches;
        stats->device_ms = ms;
    }
    if (herr & kErrStack) return fail(MCRT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    if (herr & kErrQueue) return fail(MCRT_ERR_QUEUE_OVERFLOW, "queue overflow");
    return MCRT_OK;
}

}  // namespace

extern "C" {

int mcrt_get_abi_version(void) { return MCRT_ABI_VERSION; }

const char* mcrt_last_error(void) { return g_err.c_str(); }

int mcrt_scene_destroy(mcrt_scene* s)
{
    if (!s) return MCRT_OK;
    cudaSetDevice(s->device);
    for (void* p : s->allocs) cudaFree(p);
    s->ws.release();
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
        mcrt_scene* s = new mcrt_scene();
        CK(cudaGetDevice(&s->device));
        int rc = MCRT_OK;
        auto up = [&](auto& vec, auto** dst) {
            if (rc == MCRT_OK) rc = upload(s, vec, dst);
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
        if (rc != MCRT_OK)
        {
            std::string msg = g_err;
            mcrt_scene_destroy(s);
            return fail(rc, msg);
        }
        SceneView& v = s->view;
        v.fast_nodes = fn;
        v.fast_tris = ft;
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
        v.num_lights = static_cast<int>(hs.lights.size());
        v.light_area = hs.light_area;
        v.env_w = hs.env_w;
        v.env_h = hs.env_h;
        v.env_norm = hs.env_norm;
        v.num_prims = static_cast<int>(desc->num_triangles);
        s->d_materials = const_cast<MaterialGPU*>(mt);
        s->num_materials = static_cast<int>(hs.materials.size());
        s->fast_nodes = static_cast<int64_t>(hs.bvh.fast_nodes.size());
        s->ref_nodes = static_cast<int64_t>(hs.bvh.ref_nodes.size());
        s->refs = static_cast<int64_t>(hs.bvh.ref_prims.size());
        s->bvh_depth = hs.bvh.max_depth;
        *out = s;
        return MCRT_OK;
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
    return MCRT_OK;
}

static int trace_impl(mcrt_scene* s, const mcrt_ray* rays, int64_t n, void* out, bool any, int32_t traverse,
                      int32_t ptr_mode, void* stream)
{
    if (!s || (!rays && n > 0) || (!out && n > 0)) return fail(MCRT_ERR_INVALID_ARGUMENT, "null argument");
    if (n < 0) return fail(MCRT_ERR_INVALID_ARGUMENT, "negative ray count");
    if (traverse != MCRT_TRAVERSE_FAST && traverse != MCRT_TRAVERSE_REF)
        return fail(MCRT_ERR_INVALID_ARGUMENT, "unknown traversal mode");
    if (n == 0) return MCRT_OK;
    if (s->bvh_depth + 2 >= kStack) return fail(MCRT_ERR_STACK_OVERFLOW, "BVH deeper than the traversal stack");
    CK(cudaSetDevice(s->device));
    cudaStream_t  st = static_cast<cudaStream_t>(stream);
    const float4* d_rays = reinterpret_cast<const float4*>(rays);
    void*         d_out = out;
    void*         tmp_rays = nullptr;
    void*         tmp_out = nullptr;
    size_t        out_bytes = static_cast<size_t>(n) * (any ? sizeof(int) : sizeof(float4));
    if (ptr_mode != MCRT_PTR_DEVICE)
    {
        CK(cudaMalloc(&tmp_rays, sizeof(mcrt_ray) * n));
        cudaError_t e = cudaMalloc(&tmp_out, out_bytes);
        if (e != cudaSuccess)
        {
            cudaFree(tmp_rays);
            return fail(MCRT_ERR_OUT_OF_MEMORY, "trace buffer allocation failed");
        }
        CK(cudaMemcpyAsync(tmp_rays, rays, sizeof(mcrt_ray) * n, cudaMemcpyHostToDevice, st));
        d_rays = static_cast<const float4*>(tmp_rays);
        d_out = tmp_out;
    }
    if (!s->d_err) CK(cudaMalloc(&s->d_err, sizeof(int)));
    CK(cudaMemsetAsync(s->d_err, 0, sizeof(int), st));
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trace<false, 0>, kTraceBlock, 0);
    int64_t want = (n + kTraceBlock - 1) / kTraceBlock;
    int     grid = static_cast<int>(std::min<int64_t>(want, static_cast<int64_t>(num_sms()) * std::max(occ, 1)));
    float4* hits = static_cast<float4*>(d_out);
    int*    o = static_cast<int*>(d_out);
    if (any)
    {
        if (traverse == MCRT_TRAVERSE_REF)
            k_trace<true, 1><<<grid, kTraceBlock, 0, st>>>(s->view, d_rays, n, nullptr, o, s->d_err);
        else
            k_trace<true, 0><<<grid, kTraceBlock, 0, st>>>(s->view, d_rays, n, nullptr, o, s->d_err);
    }
    else
    {
        if (traverse == MCRT_TRAVERSE_REF)
            k_trace<false, 1><<<grid, kTraceBlock, 0, st>>>(s->view, d_rays, n, hits, nullptr, s->d_err);
        else
            k_trace<false, 0><<<grid, kTraceBlock, 0, st>>>(s->view, d_rays, n, hits, nullptr, s->d_err);
    }
    CK(cudaGetLastError());
    int herr = 0;
    if (ptr_mode != MCRT_PTR_DEVICE) CK(cudaMemcpyAsync(out, tmp_out, out_bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    cudaFree(tmp_rays);
    cudaFree(tmp_out);
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

int mcrt_render_adjoint(mcrt_scene*, const mcrt_camera*, const mcrt_render_params*, const float*, float*, int32_t,
                        float*, int32_t, mcrt_render_stats*, void*)
{
    return fail(MCRT_ERR_INTERNAL, "adjoint not built yet");
}

}  // extern "C"
