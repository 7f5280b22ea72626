// Device functions shared by every kernel: vector math, the per-path PCG32 stream,
// BVH traversal (fast watertight and reference-order), and the estimator's
// sampling/evaluation routines (restating src/examples/pt/demo_pt.cpp:416-655 and
// the src/core functions it calls, with the named extensions GGX, RR, IOR).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "layout.h"

// MCRT_NODE_V8: fetch a 64-B BVH node with two 256-bit loads (1) or four 128-bit loads (0).
#ifndef MCRT_NODE_V8
#define MCRT_NODE_V8 1
#endif

// MCRT_FAST_WIDE: the FAST traversal walks the eight-child compressed tree (1) or the
// two-child tree (0, the default).  Per cfg1 frame, extension / next-event kernels: two-child
// 45.3 / 33.5 ms, eight-child 60.1 / 54.4 ms (10.4 instead of 24.1 node visits per ray, but
// each visit costs about three times the instructions, and the kernels are bound by issue
// and divergence with the tree in L2, not by the node fetches).
#ifndef MCRT_FAST_WIDE
#define MCRT_FAST_WIDE 0
#endif

// MCRT_COLD: functions of materials the benchmark scenes do not use (Phong, consistent
// normals) are compiled out of line, which keeps them out of the shading kernel's
// instruction stream (that kernel misses in the instruction cache; 25.3 -> 25.1 ms per
// cfg1 frame).  Out-of-line copies of the hot BSDF and environment functions were
// measured slower: the calls spill more than the smaller code saves.
#ifndef MCRT_COLD
#define MCRT_COLD __noinline__
#endif

namespace mcrt {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kEpsRay = 1e-4f;   // NUM_EPS_RAY (constants.cpp:13)
constexpr float kEpsDet = 1e-6f;   // NUM_EPS_DET (constants.cpp:11)
constexpr float kEpsCos = 1e-6f;   // NUM_EPS_COSINE (constants.cpp:15)
constexpr int   kSentinel = 0x7fffffff;

// error bits written to the run's error word (never a trap)
constexpr int kErrStack = 1;
constexpr int kErrQueue = 2;

// Functions marked MCRT_HDI also compile for the host, where test harnesses run the same
// traversal code; these are the host forms of the device intrinsics they use.
#define MCRT_HDI __host__ __device__ __forceinline__
MCRT_HDI int ffs32(unsigned x)
{
#ifdef __CUDA_ARCH__
    return __ffs(static_cast<int>(x));
#else
    return __builtin_ffs(static_cast<int>(x));
#endif
}
MCRT_HDI int popc32(unsigned x)
{
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}
MCRT_HDI float bits_float(unsigned u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
MCRT_HDI int float_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_int(f);
#else
    int i;
    memcpy(&i, &f, 4);
    return i;
#endif
}
// byte permute with selector nibbles 0..7 (no sign replication)
MCRT_HDI unsigned byte_perm(unsigned a, unsigned b, unsigned sel)
{
#ifdef __CUDA_ARCH__
    return __byte_perm(a, b, sel);
#else
    const unsigned long long v = static_cast<unsigned long long>(b) << 32 | a;
    unsigned                 r = 0;
    for (int i = 0; i < 4; ++i) r |= static_cast<unsigned>((v >> (8 * ((sel >> (4 * i)) & 7u))) & 0xffu) << (8 * i);
    return r;
#endif
}
// round-to-nearest arithmetic without contraction (host code is compiled with
// -ffp-contract=off, so a plain operation is one rounding there)
MCRT_HDI float rn_add(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
MCRT_HDI float rn_sub(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
MCRT_HDI float rn_mul(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
MCRT_HDI float rn_div(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
MCRT_HDI float4 ldg4(const float4* p)
{
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}
MCRT_HDI void or_error(int* err, int bits)
{
#ifdef __CUDA_ARCH__
    atomicOr(err, bits);
#else
    *err |= bits;
#endif
}

// ---------------------------------------------------------------------------
// float3 helpers
// ---------------------------------------------------------------------------
MCRT_HDI float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
MCRT_HDI float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
MCRT_HDI float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
MCRT_HDI float3 operator*(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
MCRT_HDI float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
MCRT_HDI float3 operator-(float3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float  dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize3(float3 v)
{
    float inv = 1.0f / sqrtf(dot3(v, v));
    return v * inv;
}
__device__ __forceinline__ float  maxc(float3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
__device__ __forceinline__ bool   isnan3(float3 v) { return v.x != v.x || v.y != v.y || v.z != v.z; }
MCRT_HDI float3 xyz(float4 v) { return mk(v.x, v.y, v.z); }
MCRT_HDI float  comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ float  fmax_ref(float a, float b) { return a > b ? a : b; }  // numeric.cpp f_max

// ---------------------------------------------------------------------------
// PCG32 (O'Neill 2014): state per path slot, stream from the pixel index
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Pcg
{
    uint64_t state, inc;
    __device__ __forceinline__ uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xs = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    __device__ __forceinline__ float uniform() { return static_cast<float>(next() >> 8) * (1.0f / 16777216.0f); }
    __device__ __forceinline__ void seed(uint64_t seed, uint32_t pixel, uint32_t sample)
    {
        uint64_t initstate = splitmix64(seed ^ (static_cast<uint64_t>(sample) * 0xD1B54A32D192ED03ull));
        state = 0u;
        inc = (static_cast<uint64_t>(pixel) << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
};

// random numbers drawn per scattering vertex, in this order
enum Dim
{
    D_ENV_LIGHT_0 = 0, D_ENV_LIGHT_1, D_ENV_JITTER_U, D_ENV_JITTER_V, D_ENV_BSDF_0, D_ENV_BSDF_1,
    D_AREA_BSDF_0, D_AREA_BSDF_1, D_LIGHT_PICK, D_LIGHT_U, D_LIGHT_V, D_CONT_0, D_CONT_1, D_RR,
    NUM_DIMS
};

// ---------------------------------------------------------------------------
// traversal: fast layout (64-B two-child nodes, watertight triangle test)
// ---------------------------------------------------------------------------
struct Hit
{
    float t, u, v;
    int   prim;
};

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013) with the reference's
// acceptance rules: |det_MT| >= 1e-6 (triangle.cpp:33-35; det_MT = det * d[kz]) and
// tmin < t < tmax strictly.  u, v are the barycentrics of b and c as in M-T.
struct WatertightRay
{
    float3 o;
    int    kx, ky, kz;
    float  Sx, Sy, Sz;
    float  det_eps;
};

MCRT_HDI WatertightRay make_wray(float3 o, float3 d)
{
    WatertightRay r;
    r.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int   kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int   kx = kz == 2 ? 0 : kz + 1;
    int   ky = kx == 2 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.f)
    {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = comp(d, kx) / dz;
    r.Sy = comp(d, ky) / dz;
    r.Sz = 1.0f / dz;
    r.det_eps = kEpsDet * fabsf(r.Sz);
    return r;
}

MCRT_HDI bool watertight(const WatertightRay& r, float3 v0, float3 v1, float3 v2, float tmin,
                                           float tmax, float& t, float& u, float& v)
{
    float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float  Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float  Ax = comp(A, r.kx) - r.Sx * Akz, Ay = comp(A, r.ky) - r.Sy * Akz;
    float  Bx = comp(B, r.kx) - r.Sx * Bkz, By = comp(B, r.ky) - r.Sy * Bkz;
    float  Cx = comp(C, r.kx) - r.Sx * Ckz, Cy = comp(C, r.ky) - r.Sy * Ckz;
    float  U = Cx * By - Cy * Bx;
    float  V = Ax * Cy - Ay * Cx;
    float  W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f)
    {
        U = static_cast<float>(static_cast<double>(Cx) * By - static_cast<double>(Cy) * Bx);
        V = static_cast<float>(static_cast<double>(Ax) * Cy - static_cast<double>(Ay) * Cx);
        W = static_cast<float>(static_cast<double>(Bx) * Ay - static_cast<double>(By) * Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    float det = U + V + W;
    if (!(fabsf(det) >= r.det_eps)) return false;
    float T = U * (r.Sz * Akz) + V * (r.Sz * Bkz) + W * (r.Sz * Ckz);
    float inv = 1.0f / det;
    float tt = T * inv;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    u = V * inv;
    v = W * inv;
    return true;
}

// One 64-B node: two 32-B loads (ld.global.nc.v8, sm_100 and later) where 16-B loads take
// four.  FastNode arrays are 64-B aligned (cudaMalloc'd arrays of __align__(64) nodes).
__device__ __forceinline__ void ldg_node(const FastNode* p, float4& n0, float4& n1, float4& n2, int4& n3)
{
#if MCRT_NODE_V8
    unsigned a[8], b[8];
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]), "=r"(a[7])
        : "l"(p));
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8 + 32];"
        : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]), "=r"(b[5]), "=r"(b[6]), "=r"(b[7])
        : "l"(p));
    n0 = make_float4(__uint_as_float(a[0]), __uint_as_float(a[1]), __uint_as_float(a[2]), __uint_as_float(a[3]));
    n1 = make_float4(__uint_as_float(a[4]), __uint_as_float(a[5]), __uint_as_float(a[6]), __uint_as_float(a[7]));
    n2 = make_float4(__uint_as_float(b[0]), __uint_as_float(b[1]), __uint_as_float(b[2]), __uint_as_float(b[3]));
    n3 = make_int4(static_cast<int>(b[4]), static_cast<int>(b[5]), static_cast<int>(b[6]), static_cast<int>(b[7]));
#else
    const float4* q = reinterpret_cast<const float4*>(p);
    n0 = __ldg(q);
    n1 = __ldg(q + 1);
    n2 = __ldg(q + 2);
    n3 = __ldg(reinterpret_cast<const int4*>(q + 3));
#endif
}

// Work counters of a traversal (MCRT_PROFILE_COUNT): nodes fetched, triangles tested.
struct TraceCount
{
    unsigned nodes, tris;
};

// Two-child traversal over FastNode with a per-thread stack in shared memory
// (`stack` points at this thread's column, entries `stride` ints apart): closest-hit
// queries take the nearer child first, any-hit queries the one left last.  FastTrav holds the traversal state; fast_step descends to the next leaf, tests
// its triangles and pops.  Measured alternatives on this GPU (cfg1 frame, closest-hit
// traversal time): postponing leaves until the whole warp holds one (Aila & Laine 2009)
// 178 vs 132 ms; persistent lanes that take a new ray from the queue when 1-16 lanes of
// the warp are idle 153-161 vs 82 ms -- a ray pulled into a warp mid-traversal shares no
// nodes with its neighbours, and consecutive queue entries (neighbouring paths) do.
struct FastTrav
{
    float3        inv, ood;
    WatertightRay wr;
    float         tmin, best;
    float         tterm;  // TERM: a hit nearer than this ends the traversal
    Hit           hit;
    int           sp, cur;
};

__device__ __forceinline__ void fast_begin(FastTrav& r, float3 o, float3 d, float tmin, float tmax, int* stack)
{
    const float big = 1e30f;
    r.inv = mk(fabsf(d.x) > 1e-30f ? 1.0f / d.x : copysignf(big, d.x),
               fabsf(d.y) > 1e-30f ? 1.0f / d.y : copysignf(big, d.y),
               fabsf(d.z) > 1e-30f ? 1.0f / d.z : copysignf(big, d.z));
    r.ood = o * r.inv;
    r.wr = make_wray(o, d);
    r.tmin = tmin;
    r.best = tmax;
    r.hit.prim = -1;
    r.sp = 0;
    stack[0] = kSentinel;
    r.cur = 0;
}

// Inner nodes down to the next leaf, that leaf's triangles, then the next node from the
// stack.  Returns true when the traversal is over: stack empty, an any-hit query hit, a
// TERM query hit nearer than r.tterm, or the stack overflowed (error bit set, the hit so
// far kept).
template <int STACK, bool COUNT, bool TERM = false>
__device__ __forceinline__ bool fast_step(FastTrav& r, const FastNode* nodes, const float4* tris, bool any, int* stack,
                                          int stride, int* err, TraceCount* cnt)
{
    while (r.cur >= 0 && r.cur != kSentinel)
    {
        if (COUNT) cnt->nodes++;
        float4 n0, n1, n2;
        int4   n3;
        ldg_node(nodes + r.cur, n0, n1, n2, n3);
        float  c0lx = n0.x * r.inv.x - r.ood.x, c0hx = n0.y * r.inv.x - r.ood.x;
        float  c0ly = n0.z * r.inv.y - r.ood.y, c0hy = n0.w * r.inv.y - r.ood.y;
        float  c0lz = n2.x * r.inv.z - r.ood.z, c0hz = n2.y * r.inv.z - r.ood.z;
        float  c1lx = n1.x * r.inv.x - r.ood.x, c1hx = n1.y * r.inv.x - r.ood.x;
        float  c1ly = n1.z * r.inv.y - r.ood.y, c1hy = n1.w * r.inv.y - r.ood.y;
        float  c1lz = n2.z * r.inv.z - r.ood.z, c1hz = n2.w * r.inv.z - r.ood.z;
        float  t0n = fmaxf(fmaxf(fminf(c0lx, c0hx), fminf(c0ly, c0hy)), fmaxf(fminf(c0lz, c0hz), r.tmin));
        float  t0f = fminf(fminf(fmaxf(c0lx, c0hx), fmaxf(c0ly, c0hy)), fminf(fmaxf(c0lz, c0hz), r.best));
        float  t1n = fmaxf(fmaxf(fminf(c1lx, c1hx), fminf(c1ly, c1hy)), fmaxf(fminf(c1lz, c1hz), r.tmin));
        float  t1f = fminf(fminf(fmaxf(c1lx, c1hx), fmaxf(c1ly, c1hy)), fminf(fmaxf(c1lz, c1hz), r.best));
        // widen the far bound by a few ulp so boxes flat in one axis are not lost
        bool h0 = t0n <= t0f * 1.0000004f + 1e-30f;
        bool h1 = t1n <= t1f * 1.0000004f + 1e-30f;
        if (!h0 && !h1)
        {
            r.cur = stack[r.sp * stride];
            --r.sp;
        }
        else
        {
            int near = h0 ? n3.x : n3.y;
            if (h0 && h1)
            {
                int far = n3.y;
                // closest hit: nearer child first (cfg1 frame, extension rays: 50.4 ms;
                // farther first 80.3; nearer exit first 50.4).  Any hit: the child whose box
                // the ray leaves last first -- a next-event ray leaves the surface it starts
                // on, so an occluder, if there is one, lies away from the origin (next-event
                // rays: nearer first 57.1 ms, fixed left-first 46.5, farther entry first 39.7,
                // farther exit first 39.5, longer overlap first 48.8)
                if (any ? t1f > t0f : t1n < t0n)
                {
                    near = n3.y;
                    far = n3.x;
                }
                ++r.sp;
                if (r.sp >= STACK)
                {
                    atomicOr(err, kErrStack);
                    return true;
                }
                stack[r.sp * stride] = far;
            }
            r.cur = near;
        }
    }
    if (r.cur < 0)
    {
        int code = ~r.cur;
        int first = code >> 4, count = code & 15;
        if (COUNT) cnt->tris += count;
        for (int k = 0; k < count; ++k)
        {
            const float4* tp = tris + 3 * (first + k);
            float4        a = __ldg(tp + 0);
            float4        b = __ldg(tp + 1);
            float4        c = __ldg(tp + 2);
            float         t, u, v;
            if (watertight(r.wr, xyz(a), xyz(b), xyz(c), r.tmin, r.best, t, u, v))
            {
                r.best = t;
                r.hit.t = t;  // u, v: recomputed for the final hit only (refine_hit)
                r.hit.prim = __float_as_int(a.w);
                if (any || (TERM && t < r.tterm)) return true;
            }
        }
        r.cur = stack[r.sp * stride];
        --r.sp;
    }
    return r.cur == kSentinel;
}

template <bool ANY, int STACK, bool COUNT = false, bool TERM = false>
__device__ __forceinline__ bool trace_fast(const SceneView& s, float3 o, float3 d, float tmin, float tmax,
                                           int* stack, int stride, Hit& hit, int* err, TraceCount* cnt = nullptr,
                                           float tterm = 0.f)
{
    FastTrav r;
    fast_begin(r, o, d, tmin, tmax, stack);
    r.tterm = tterm;
    while (!fast_step<STACK, COUNT, TERM>(r, s.fast_nodes, s.fast_tris, ANY, stack, stride, err, cnt))
    {
    }
    hit = r.hit;
    return r.hit.prim >= 0;
}

// ---------------------------------------------------------------------------
// traversal: eight-child compressed nodes (WideNode, layout.h)
// ---------------------------------------------------------------------------
// One 96-B node: two 32-B loads, a 16-B load and the leaf mask (nodes are 32-B aligned:
// cudaMalloc'd arrays of __align__(32) 96-B nodes; the last 12 B are padding).
MCRT_HDI void ldg_wide(const WideNode* p, unsigned (&w)[21])
{
#ifndef __CUDA_ARCH__
    memcpy(w, p, sizeof(unsigned) * 21);
#else
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
        : "l"(p));
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8 + 32];"
        : "=r"(w[8]), "=r"(w[9]), "=r"(w[10]), "=r"(w[11]), "=r"(w[12]), "=r"(w[13]), "=r"(w[14]), "=r"(w[15])
        : "l"(p));
    asm("ld.global.nc.v4.b32 {%0, %1, %2, %3}, [%4 + 64];"
        : "=r"(w[16]), "=r"(w[17]), "=r"(w[18]), "=r"(w[19])
        : "l"(p));
    asm("ld.global.nc.b32 %0, [%1 + 80];" : "=r"(w[20]) : "l"(p));
#endif
}

// 8-bit plane q of byte k of `word` as the float 2^23 + q (exact): one byte permute
MCRT_HDI float qplane(unsigned word, int k)
{
    return bits_float(byte_perm(word, 0x4B000000u, 0x7650u | static_cast<unsigned>(k)));
}

// three-input minimum / maximum (one instruction on sm_100 and later)
#ifndef MCRT_WIDE_MAX3
#define MCRT_WIDE_MAX3 0
#endif
MCRT_HDI float fmax3f(float a, float b, float c)
{
#if defined(__CUDA_ARCH__) && MCRT_WIDE_MAX3
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
MCRT_HDI float fmin3f(float a, float b, float c)
{
#if defined(__CUDA_ARCH__) && MCRT_WIDE_MAX3
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}
#ifndef MCRT_WIDE_UNROLL
#define MCRT_WIDE_UNROLL 8
#endif
constexpr int kWideUnroll = MCRT_WIDE_UNROLL;

// the slot-indexed bits of m moved to positions slot ^ x (x in 0..7)
MCRT_HDI unsigned xor_permute8(unsigned m, unsigned x)
{
    if (x & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (x & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (x & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return m;
}

// Closest / any hit over the eight-child tree.  Each step visits one node: its eight child
// boxes are tested against [tmin, best] in the node's quantised frame (per axis
// t = (2^23 + q) a + b', a = cell / d, b' = (origin - o) / d - 2^23 a, the near plane the
// low one for a positive direction), the triangles of the hit leaf children are tested at
// once, and the hit inner children form a group (child block, pending bits in visiting
// order) from which the next node is taken; a group with children left goes to the
// per-thread stack (two ints per entry, `stack` with entries `stride` ints apart).
// Visiting order: slot ^ octant of the direction (near to far) for closest hits; the
// reverse for any-hit queries, whose occluders lie away from the surface the ray leaves.
template <bool ANY, int STACK, bool COUNT>
MCRT_HDI bool trace_wide(const SceneView& s, float3 o, float3 d, float tmin, float tmax, int* stack,
                                           int stride, Hit& hit, int* err, TraceCount* cnt)
{
    const float big = 1e20f;  // 1 / d for |d| below 1e-20 (keeps 2^23 a finite)
    const float3 inv = mk(fabsf(d.x) > 1e-20f ? 1.0f / d.x : copysignf(big, d.x),
                          fabsf(d.y) > 1e-20f ? 1.0f / d.y : copysignf(big, d.y),
                          fabsf(d.z) > 1e-20f ? 1.0f / d.z : copysignf(big, d.z));
    const unsigned      oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
    const unsigned      oxor = ANY ? (oct ^ 7u) : oct;
    const WatertightRay wr = make_wray(o, d);
    float               best = tmax;
    hit.prim = -1;
    int      sp = 0;
    int      node = 0;
    unsigned nbase = 0, nbits = 0;
    while (true)
    {
        if (COUNT) cnt->nodes++;
        unsigned w[21];
        ldg_wide(s.wide_nodes + node, w);
        // per axis: cell / d and the offset, with the near / far plane words by direction sign
        const float ax = bits_float((w[3] & 0xffu) << 23) * inv.x;
        const float ay = bits_float(((w[3] >> 8) & 0xffu) << 23) * inv.y;
        const float az = bits_float(((w[3] >> 16) & 0xffu) << 23) * inv.z;
        const float bx = (bits_float(w[0]) - o.x) * inv.x - 8388608.0f * ax;
        const float by = (bits_float(w[1]) - o.y) * inv.y - 8388608.0f * ay;
        const float bz = (bits_float(w[2]) - o.z) * inv.z - 8388608.0f * az;
        // w[8..9] lo.x, w[10..11] lo.y, w[12..13] lo.z, w[14..15] hi.x, w[16..17] hi.y, w[18..19] hi.z
        const bool     px = d.x >= 0.f, py = d.y >= 0.f, pz = d.z >= 0.f;
        const unsigned nx0 = px ? w[8] : w[14], nx1 = px ? w[9] : w[15];
        const unsigned fx0 = px ? w[14] : w[8], fx1 = px ? w[15] : w[9];
        const unsigned ny0 = py ? w[10] : w[16], ny1 = py ? w[11] : w[17];
        const unsigned fy0 = py ? w[16] : w[10], fy1 = py ? w[17] : w[11];
        const unsigned nz0 = pz ? w[12] : w[18], nz1 = pz ? w[13] : w[19];
        const unsigned fz0 = pz ? w[18] : w[12], fz1 = pz ? w[19] : w[13];
        unsigned hits = 0;
#pragma unroll kWideUnroll
        for (int k = 0; k < 8; ++k)
        {
            const int      b = k & 3;
            const unsigned wnx = k < 4 ? nx0 : nx1, wfx = k < 4 ? fx0 : fx1;
            const unsigned wny = k < 4 ? ny0 : ny1, wfy = k < 4 ? fy0 : fy1;
            const unsigned wnz = k < 4 ? nz0 : nz1, wfz = k < 4 ? fz0 : fz1;
            const float tnx = fmaf(qplane(wnx, b), ax, bx), tfx = fmaf(qplane(wfx, b), ax, bx);
            const float tny = fmaf(qplane(wny, b), ay, by), tfy = fmaf(qplane(wfy, b), ay, by);
            const float tnz = fmaf(qplane(wnz, b), az, bz), tfz = fmaf(qplane(wfz, b), az, bz);
            const float tn = fmax3f(tnx, tny, fmaxf(tnz, tmin));
            const float tf = fmin3f(tfx, tfy, fminf(tfz, best));
            if (tn <= tf * 1.0000004f + 1e-30f) hits |= 1u << k;
        }
        const unsigned imask = w[3] >> 24;
        // triangles of the hit leaf children: tri_base + first .. + count - 1
        unsigned lhit = hits & w[20];
        unsigned tbits = 0;
        while (lhit)
        {
            const int      sl = ffs32(lhit) - 1;
            lhit &= lhit - 1;
            const unsigned m = ((sl < 4 ? w[6] : w[7]) >> (8 * (sl & 3))) & 0xffu;
            const unsigned c = ((m >> 5) & 3u) + 1u;
            tbits |= ((1u << c) - 1u) << (m & 31u);
        }
        const unsigned tbase = w[5];
        const unsigned ihit = hits & imask;
        if (ihit)
        {
            nbase = w[4];
            nbits = (xor_permute8(ihit, oxor) << 24) | imask;
        }
        else
        {
            nbits = 0;
        }
        while (tbits)
        {
            const int k = ffs32(tbits) - 1;
            tbits &= tbits - 1;
            if (COUNT) cnt->tris++;
            const float4* tp = s.wide_tris + 3 * (tbase + k);
            const float4  ta = ldg4(tp + 0), tb = ldg4(tp + 1), tc = ldg4(tp + 2);
            float         t, u, v;
            if (watertight(wr, xyz(ta), xyz(tb), xyz(tc), tmin, best, t, u, v))
            {
                best = t;
                hit.t = t;  // u, v: recomputed for the final hit only (refine_hit)
                hit.prim = float_bits(ta.w);
                if (ANY) return true;
            }
        }
        if ((nbits >> 24) == 0)
        {
            if (sp == 0) break;
            --sp;
            nbase = static_cast<unsigned>(stack[(2 * sp) * stride]);
            nbits = static_cast<unsigned>(stack[(2 * sp + 1) * stride]);
        }
        const unsigned key = ffs32(nbits >> 24) - 1;
        nbits &= ~(1u << (24 + key));
        const unsigned slot = key ^ oxor;
        node = static_cast<int>(nbase + popc32(nbits & ((1u << slot) - 1u) & 0xffu));
        if (nbits >> 24)
        {
            if (2 * sp + 2 > STACK)
            {
                or_error(err, kErrStack);
                return hit.prim >= 0;
            }
            stack[(2 * sp) * stride] = static_cast<int>(nbase);
            stack[(2 * sp + 1) * stride] = static_cast<int>(nbits);
            ++sp;
        }
    }
    return hit.prim >= 0;
}

// ---------------------------------------------------------------------------
// traversal: reference order and arithmetic (MCRT_TRAVERSE_REF)
// ---------------------------------------------------------------------------
struct RefRay
{
    float3 o, d, inv;
    int    sx, sy, sz;  // dir_sign (ray.cpp:44-46)
    float  tmin, tmax;
};

__device__ __forceinline__ RefRay make_ref_ray(float3 o, float3 d, float tmin, float tmax)
{
    RefRay r;
    r.o = o;
    r.d = d;
    // inv_dir = 0 (not inf) for zero components (ray.cpp:39-42)
    r.inv = mk(d.x == 0.f ? 0.f : __fdiv_rn(1.0f, d.x), d.y == 0.f ? 0.f : __fdiv_rn(1.0f, d.y),
               d.z == 0.f ? 0.f : __fdiv_rn(1.0f, d.z));
    r.sx = d.x < 0.f;
    r.sy = d.y < 0.f;
    r.sz = d.z < 0.f;
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

// rayAABBOverlap (aabb.cpp:66-131), every operation rounded as the CPU does it
__device__ __forceinline__ bool ref_overlap(const RefRay& r, float3 lo, float3 hi)
{
    float tmin = __fmul_rn(__fsub_rn(r.sx ? hi.x : lo.x, r.o.x), r.inv.x);
    float tymin = __fmul_rn(__fsub_rn(r.sy ? hi.y : lo.y, r.o.y), r.inv.y);
    float tmax = __fmul_rn(__fsub_rn(r.sx ? lo.x : hi.x, r.o.x), r.inv.x);
    float tymax = __fmul_rn(__fsub_rn(r.sy ? lo.y : hi.y, r.o.y), r.inv.y);
    if ((tmin > tymax) || (tymin > tmax)) return false;
    if (tymin > tmin) tmin = tymin;
    if (tmin > r.tmax) return false;
    if (tymax < tmax) tmax = tymax;
    if (tmax < r.tmin) return false;
    float tzmin = __fmul_rn(__fsub_rn(r.sz ? hi.z : lo.z, r.o.z), r.inv.z);
    float tzmax = __fmul_rn(__fsub_rn(r.sz ? lo.z : hi.z, r.o.z), r.inv.z);
    if ((tmin > tzmax) || (tzmin > tmax)) return false;
    if (tzmin > tmin) tmin = tzmin;
    if (tmin > r.tmax) return false;
    if (tzmax < tmax) tmax = tzmax;
    if (tmax < r.tmin) return false;
    return true;
}

MCRT_HDI float3 sub_rn(float3 a, float3 b)
{
    return mk(rn_sub(a.x, b.x), rn_sub(a.y, b.y), rn_sub(a.z, b.z));
}
MCRT_HDI float3 cross_rn(float3 a, float3 b)
{
    return mk(rn_sub(rn_mul(a.y, b.z), rn_mul(a.z, b.y)), rn_sub(rn_mul(a.z, b.x), rn_mul(a.x, b.z)),
              rn_sub(rn_mul(a.x, b.y), rn_mul(a.y, b.x)));
}
MCRT_HDI float dot_rn(float3 a, float3 b)
{
    return rn_add(rn_add(rn_mul(a.x, b.x), rn_mul(a.y, b.y)), rn_mul(a.z, b.z));
}

// rayTriangleIntersect, MOLLER_TRUMBORE branch (triangle.cpp:13-51)
MCRT_HDI bool ref_mt(float3 orig, float3 dir, float3 v0, float3 v1, float3 v2, float& t, float& u,
                                       float& v)
{
    float3 v0v1 = sub_rn(v1, v0);
    float3 v0v2 = sub_rn(v2, v0);
    float3 pvec = cross_rn(dir, v0v2);
    float  det = dot_rn(v0v1, pvec);
    if (fabsf(det) < kEpsDet) return false;
    float  invDet = rn_div(1.0f, det);
    float3 tvec = sub_rn(orig, v0);
    u = rn_mul(dot_rn(tvec, pvec), invDet);
    if (u < 0.f || u > 1.f) return false;
    float3 qvec = cross_rn(tvec, v0v1);
    v = rn_mul(dot_rn(dir, qvec), invDet);
    if (v < 0.f || rn_add(u, v) > 1.f) return false;
    t = rn_mul(dot_rn(v0v2, qvec), invDet);
    return true;
}

// Iterative form of SplitBVHBranchNode/LeafNode::intersect (splitbvh.cpp:5-145):
// a node's own box is tested when it is visited (against the current tmax), leaf
// references are culled by their clipped bounds, children are visited left-first
// iff dir[split_axis] > 0, and ties keep the first hit found.
template <bool ANY, int STACK>
__device__ __forceinline__ bool trace_ref(const SceneView& s, float3 o, float3 d, float tmin, float tmax, int* stack,
                                          int stride, Hit& hit, int* err)
{
    RefRay r = make_ref_ray(o, d, tmin, tmax);
    hit.prim = -1;
    int sp = 0;
    stack[0] = 0;
    sp = 1;
    while (sp > 0)
    {
        --sp;
        int     n = stack[sp * stride];
        RefNode rn;
        rn.lo = __ldg(&s.ref_nodes[n].lo);
        rn.hi = __ldg(&s.ref_nodes[n].hi);
        if (!ref_overlap(r, xyz(rn.lo), xyz(rn.hi))) continue;
        int a = __float_as_int(rn.lo.w), b = __float_as_int(rn.hi.w);
        if (a < 0)
        {
            int first = ~a;
            for (int k = 0; k < b; ++k)
            {
                float4 plo = __ldg(&s.ref_prims[first + k].lo);
                float4 phi = __ldg(&s.ref_prims[first + k].hi);
                if (!ref_overlap(r, xyz(plo), xyz(phi))) continue;
                int           prim = __float_as_int(plo.w);
                const float4* pv = s.prim_verts + 3 * prim;
                float         t, u, v;
                if (ref_mt(r.o, r.d, xyz(__ldg(pv)), xyz(__ldg(pv + 1)), xyz(__ldg(pv + 2)), t, u, v) && t > r.tmin &&
                    t < r.tmax)
                {
                    r.tmax = t;
                    hit.t = t;
                    hit.u = u;
                    hit.v = v;
                    hit.prim = prim;
                    if (ANY) return true;
                }
            }
        }
        else
        {
            int  left = a, right = b >> 2, axis = b & 3;
            bool left_first = comp(r.d, axis) > 0.0f;
            if (sp + 2 > STACK)
            {
                atomicOr(err, kErrStack);
                return hit.prim >= 0;
            }
            stack[sp * stride] = left_first ? right : left;
            ++sp;
            stack[sp * stride] = left_first ? left : right;
            ++sp;
        }
    }
    return hit.prim >= 0;
}

// The watertight test decides which triangle is closest; the reported t, u, v of that
// one triangle are then recomputed with the reference's Moller-Trumbore arithmetic (each
// formula lands ~3 ulp from the exact t, on either side).
MCRT_HDI void refine_hit(const SceneView& s, float3 o, float3 d, float tmin, Hit& hit)
{
    const float4* pv = s.prim_verts + 3 * hit.prim;
    const float3  va = xyz(ldg4(pv)), vb = xyz(ldg4(pv + 1)), vc = xyz(ldg4(pv + 2));
    float         t, u, v;
    if (ref_mt(o, d, va, vb, vc, t, u, v) && t > tmin)
    {
        hit.t = t;
        hit.u = u;
        hit.v = v;
        return;
    }
    // the watertight test's own barycentrics: the traversal keeps only t and the primitive
    // (two registers fewer in its loop); the same inputs give the same result again
    hit.u = 0.f;
    hit.v = 0.f;
    if (watertight(make_wray(o, d), va, vb, vc, tmin, bits_float(0x7f800000u), t, u, v))
    {
        hit.u = u;
        hit.v = v;
    }
}

// REFM = false: a build for jobs that all traverse in FAST mode; without the reference
// traversal in the same kernel the fast one needs fewer registers (the any-hit kernel at
// 48 registers: 8 B of spills instead of 52).
// TERM: a closest-hit query that only asks whether the ray reaches an emitter, and `tterm`
// a distance no emitter hit can lie below (emitter_span): the FAST traversal stops at a
// nearer hit and reports no hit, which is the answer the full query gives the caller (its
// closest hit, nearer still, is no emitter).  The reference-order traversal and the wide
// one run the full query.
template <bool ANY, int STACK, bool COUNT = false, bool REFM = true, bool TERM = false>
__device__ __forceinline__ bool trace_ray(const SceneView& s, int mode, float3 o, float3 d, float tmin, float tmax,
                                          int* stack, int stride, Hit& hit, int* err, TraceCount* cnt = nullptr,
                                          float tterm = 0.f)
{
    if (REFM && mode == 1) return trace_ref<ANY, STACK>(s, o, d, tmin, tmax, stack, stride, hit, err);
#if MCRT_FAST_WIDE
    bool found = trace_wide<ANY, STACK, COUNT>(s, o, d, tmin, tmax, stack, stride, hit, err, cnt);
#else
    bool found = trace_fast<ANY, STACK, COUNT, TERM>(s, o, d, tmin, tmax, stack, stride, hit, err, cnt, tterm);
    if (TERM && found && hit.t < tterm) return false;
#endif
    if (!ANY && found) refine_hit(s, o, d, tmin, hit);
    return found;
}

// ---------------------------------------------------------------------------
// shading data
// ---------------------------------------------------------------------------
// TriangleObject::normal(u, v) (triangle.cpp:90-93); material id in .w of na
__device__ __forceinline__ float3 shading_normal(const SceneView& s, int prim, float u, float v, int& mat)
{
    const float4* p = s.prim_shade + 3 * prim;
    float4        na = __ldg(p), nb = __ldg(p + 1), nc = __ldg(p + 2);
    mat = __float_as_int(na.w);
    float w = 1.0f - u - v;
    return normalize3(xyz(na) * w + xyz(nb) * u + xyz(nc) * v);
}

struct Mat
{
    int    type;
    bool   consistent;  // MCRT_MAT_CONSISTENT: shade with the consistent normal
    float3 color;
    float  roughness, ior;
    int    albedo_param, emission_param;
};

__device__ __forceinline__ Mat load_mat(const SceneView& s, int m)
{
    MaterialGPU g = s.materials[m];
    Mat         r;
    r.type = g.type & 0xff;
    r.consistent = (g.type & 0x100) != 0;
    r.color = mk(g.r, g.g, g.b);
    r.roughness = g.roughness;
    r.ior = g.ior;
    r.albedo_param = g.albedo_param;
    r.emission_param = g.emission_param;
    return r;
}

constexpr int MAT_LGHT = 0, MAT_DIFF = 1, MAT_SPEC = 2, MAT_REFR = 3, MAT_GLSY = 4, MAT_GGX = 8;

// TriangleObject::consistentNormal (triangle.cpp:149-182; Reshetov, Soupikov, Kapustin
// 2010): from the interpolated normal np and the interpolated vertex alpha, the normal
// about which wi reflects to a direction that stays above the surface.  Float operations
// in the reference's order, no contraction.
__device__ MCRT_COLD float3 consistent_normal(const SceneView& s, int prim, float u, float v, float3 wi,
                                                    float3 np)
{
    const float4 al = __ldg(&s.prim_alpha[prim]);
    const float  w0 = __fsub_rn(__fsub_rn(1.0f, u), v);
    const float  alpha = __fadd_rn(__fadd_rn(__fmul_rn(w0, al.x), __fmul_rn(u, al.y)), __fmul_rn(v, al.z));
    const float  k = 2.0f / kPi;
    const float  t = __fsub_rn(1.0f, __fmul_rn(k, alpha));
    const float  q = __fdiv_rn(__fmul_rn(t, t),
                              __fadd_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, __fsub_rn(1.0f, k)), alpha)));
    const float  b = __fadd_rn(__fadd_rn(__fmul_rn(wi.x, np.x), __fmul_rn(wi.y, np.y)), __fmul_rn(wi.z, np.z));
    const float  g = __fadd_rn(1.0f, __fmul_rn(q, __fsub_rn(b, 1.0f)));
    const float  rho = __fsqrt_rn(__fdiv_rn(__fmul_rn(q, __fadd_rn(1.0f, g)), __fadd_rn(1.0f, b)));
    const float  c = __fadd_rn(g, __fmul_rn(rho, b));
    const float3 r = mk(__fsub_rn(__fmul_rn(c, np.x), __fmul_rn(rho, wi.x)),
                        __fsub_rn(__fmul_rn(c, np.y), __fmul_rn(rho, wi.y)),
                        __fsub_rn(__fmul_rn(c, np.z), __fmul_rn(rho, wi.z)));
    const float3 h = mk(__fadd_rn(wi.x, r.x), __fadd_rn(wi.y, r.y), __fadd_rn(wi.z, r.z));
    const float  inv = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(h.x, h.x), __fmul_rn(h.y, h.y)),
                                                             __fmul_rn(h.z, h.z))));
    return mk(__fmul_rn(h.x, inv), __fmul_rn(h.y, inv), __fmul_rn(h.z, inv));
}
__device__ __forceinline__ bool does_nee(int type) { return type == MAT_DIFF || type == MAT_GGX; }

// OrthonormalFrame::setFromNormal (geometry.cpp:74-105; Duff et al. 2017)
struct Frame
{
    float3 x, y, z;
    __device__ __forceinline__ explicit Frame(float3 n)
    {
        float       sign = copysignf(1.0f, n.z);
        const float a = -1.0f / (sign + n.z);
        const float b = n.x * n.y * a;
        x = mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
        y = mk(b, sign + n.y * n.y * a, -n.y);
        z = n;
    }
    __device__ __forceinline__ float3 to_world(float3 c) const { return x * c.x + y * c.y + z * c.z; }
    __device__ __forceinline__ float3 to_local(float3 v) const { return mk(dot3(v, x), dot3(v, y), dot3(v, z)); }
};

__device__ __forceinline__ float3 reflect_world(float3 wi, float3 n) { return n * (2.0f * dot3(n, wi)) - wi; }

// fresnelReflectance (geometry.cpp:14-43)
__device__ __forceinline__ float fresnel(float cos_i, float ior)
{
    if (ior < 0.f) return 1.f;
    float eta;
    if (cos_i < 0.f)
    {
        cos_i = -cos_i;
        eta = ior;
    }
    else
    {
        eta = 1.0f / ior;
    }
    float sin2t = fminf(1.0f, (eta * eta) * (1.0f - cos_i * cos_i));
    float cos_t = sqrtf(1.0f - sin2t);
    float t1 = eta * cos_t;
    float rs = (cos_i - t1) / (cos_i + t1);
    float t2 = eta * cos_i;
    float rp = (t2 - cos_t) / (t2 + cos_t);
    return (rs * rs + rp * rp) * 0.5f;
}

// GGX (Walter et al. 2007), local frame z = normal
__device__ __forceinline__ float ggx_D(float3 h, float a)
{
    float a2 = a * a;
    float d = h.z * h.z * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * d * d);
}
__device__ __forceinline__ float ggx_G1(float3 v, float a)
{
    float c2 = v.z * v.z;
    if (c2 <= 0.f) return 0.f;
    float t2 = (1.0f - c2) / c2;
    return 2.0f / (1.0f + sqrtf(1.0f + a * a * t2));
}
__device__ __forceinline__ float3 schlick(float3 f0, float c)
{
    float m = 1.0f - c;
    float m5 = m * m * m * m * m;
    return f0 + (mk(1.f, 1.f, 1.f) - f0) * m5;
}

struct BsdfSample
{
    float3 wo;
    float3 weight;
    float  pdf;
};

// GlossyBSDF (bsdf.cpp:209-301): Phong lobe of exponent 25 about the mirror direction.
__device__ MCRT_COLD BsdfSample phong_sample(float3 color, float3 wi, float3 nl, float r1, float r2)
{
    BsdfSample  s;
    const float g = 25.f;
    float       x = r1 * (2.f * kPi);
    float       r2p = powf(r2, 1.0f / (g + 1.0f));
    float       st = sqrtf(1.0f - r2p * r2p);
    float3      c = mk(sinf(x) * st, cosf(x) * st, r2p);
    float3      refl = reflect_world(wi, nl);
    Frame       onb(refl);
    float3      wo = onb.to_world(c);
    if (dot3(wo, nl) < 0.f) wo = mk(0.f, 0.f, 0.f);
    float c_o = fmax_ref(dot3(wo, nl), kEpsCos);
    s.pdf = (g + 1.f) / (2.f * kPi) * powf(fmax_ref(dot3(refl, wo), kEpsCos), g);
    float w = (g + 2.f) / (g + 1.f) * c_o / fmax_ref(fabsf(dot3(wi, nl)), fabsf(dot3(wo, nl)));
    if (w != w) w = 0.f;
    s.weight = color * w;
    s.wo = wo;
    return s;
}

__device__ MCRT_COLD float phong_pdf(float3 wi, float3 nl, float3 wo)
{
    float3 refl = reflect_world(wi, nl);
    return 26.f / (2.f * kPi) * powf(fmax_ref(dot3(refl, wo), kEpsCos), 25.f);
}

__device__ MCRT_COLD float3 phong_eval(float3 color, float3 wi, float3 nl, float3 wo)
{
    float3 refl = reflect_world(wi, nl);
    float  v = 27.f / (2.f * kPi) * powf(fmax_ref(dot3(refl, wo), kEpsCos), 25.f) /
              fmax_ref(fabsf(dot3(wi, nl)), fabsf(dot3(wo, nl)));
    return color * v;
}

// Material::sample (bsdf.cpp Lambert :51-87, Specular :134-162, Glossy :209-262,
// Refractive :319-418) plus the GGX conductor (Heitz 2018 visible normals)
__device__ __forceinline__ BsdfSample bsdf_sample(const Mat& m, float3 wi, float3 nl, float r1, float r2)
{
    BsdfSample s;
    s.pdf = 0.f;
    if (m.type == MAT_SPEC)
    {
        s.wo = reflect_world(wi, nl);
        s.weight = m.color;
        s.pdf = 1.f;
    }
    else if (m.type == MAT_REFR)
    {
        bool   outside = dot3(wi, nl) > 0.f;
        float3 n = outside ? nl : -nl;
        float3 refl = normalize3(reflect_world(wi, n));
        float  nc = 1.f, nt = m.ior;
        float  nnt = outside ? nc / nt : nt / nc;
        float  ddn = dot3(-wi, n);
        float  cos2t = 1.f - nnt * nnt * (1.f - ddn * ddn);
        if (cos2t < 0.f)
        {
            s.weight = m.color;
            s.pdf = 1.f;
            s.wo = refl;
        }
        else
        {
            float3 tdir = normalize3(-wi * nnt - n * (ddn * nnt + sqrtf(cos2t)));
            float  Re = fresnel(dot3(wi, nl), nt / nc);
            float  Tr = 1.f - Re;
            float  P = Re;
            if (r1 < P)
            {
                s.weight = m.color * (Re / P);
                s.pdf = P;
                s.wo = refl;
            }
            else
            {
                s.weight = m.color * (Tr / (1.f - P));
                s.pdf = 1.f - P;
                s.wo = tdir;
            }
        }
    }
    else if (m.type == MAT_GLSY)
    {
        s = phong_sample(m.color, wi, nl, r1, r2);
    }
    else if (m.type == MAT_GGX)
    {
        float3 n = dot3(wi, nl) < 0.f ? -nl : nl;
        Frame  fr(n);
        float3 wl = fr.to_local(wi);
        float  a = m.roughness;
        s.wo = n;
        s.weight = mk(0.f, 0.f, 0.f);
        if (wl.z > 0.f)
        {
            float3 vh = normalize3(mk(a * wl.x, a * wl.y, wl.z));
            float  lensq = vh.x * vh.x + vh.y * vh.y;
            float3 t1 = lensq > 0.f ? mk(-vh.y, vh.x, 0.f) * rsqrtf(lensq) : mk(1.f, 0.f, 0.f);
            float3 t2 = cross3(vh, t1);
            float  r = sqrtf(r1);
            float  phi = 2.f * kPi * r2;
            float  p1 = r * cosf(phi);
            float  p2 = r * sinf(phi);
            float  sh = 0.5f * (1.f + vh.z);
            p2 = (1.f - sh) * sqrtf(fmaxf(0.f, 1.f - p1 * p1)) + sh * p2;
            float3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.f, 1.f - p1 * p1 - p2 * p2));
            float3 h = normalize3(mk(a * nh.x, a * nh.y, fmaxf(0.f, nh.z)));
            float  wih = dot3(wl, h);
            float3 ol = h * (2.f * wih) - wl;
            s.wo = fr.to_world(ol);
            if (ol.z > 0.f && wih > 0.f)
            {
                s.pdf = ggx_G1(wl, a) * ggx_D(h, a) / (4.f * wl.z);
                s.weight = schlick(m.color, wih) * ggx_G1(ol, a);
            }
        }
    }
    else  // DIFF (and any other type, as Material's default)
    {
        float  x = r1 * (2.f * kPi);
        float  r2s = sqrtf(r2);
        float3 c = mk(cosf(x) * r2s, sinf(x) * r2s, sqrtf(1.f - r2));
        Frame  onb(nl);
        float3 wo = onb.to_world(c);
        float  c_o = fmax_ref(dot3(wo, nl), kEpsCos);
        s.pdf = c_o / kPi;
        s.weight = m.color;
        s.wo = wo;
    }
    return s;
}

// Material::pdfW
__device__ __forceinline__ float bsdf_pdf(const Mat& m, float3 wi, float3 nl, float3 wo)
{
    if (m.type == MAT_DIFF) return fmax_ref(dot3(wo, nl), kEpsCos) / kPi;
    if (m.type == MAT_GLSY) return phong_pdf(wi, nl, wo);
    if (m.type == MAT_GGX)
    {
        float3 n = dot3(wi, nl) < 0.f ? -nl : nl;
        Frame  fr(n);
        float3 wl = fr.to_local(wi), ol = fr.to_local(wo);
        if (wl.z <= 0.f || ol.z <= 0.f) return 0.f;
        float3 h = normalize3(wl + ol);
        return ggx_G1(wl, m.roughness) * ggx_D(h, m.roughness) / (4.f * wl.z);
    }
    return 0.f;
}

// Material::evaluate: the BSDF value without the cosine
__device__ __forceinline__ float3 bsdf_eval(const Mat& m, float3 wi, float3 nl, float3 wo)
{
    if (m.type == MAT_DIFF) return m.color * (1.0f / kPi);
    if (m.type == MAT_GLSY) return phong_eval(m.color, wi, nl, wo);
    if (m.type == MAT_GGX)
    {
        float3 n = dot3(wi, nl) < 0.f ? -nl : nl;
        Frame  fr(n);
        float3 wl = fr.to_local(wi), ol = fr.to_local(wo);
        if (wl.z <= 0.f || ol.z <= 0.f) return mk(0.f, 0.f, 0.f);
        float3 h = normalize3(wl + ol);
        float  a = m.roughness;
        float  v = ggx_D(h, a) * ggx_G1(wl, a) * ggx_G1(ol, a) / (4.f * wl.z * ol.z);
        return schlick(m.color, dot3(wl, h)) * v;
    }
    return mk(0.f, 0.f, 0.f);
}

// ---------------------------------------------------------------------------
// environment map (envmap.cpp:44-53, :333-506)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int clampi(int x, int a, int b) { return x < a ? a : (x > b ? b : x); }

__device__ __forceinline__ int lower_bound_cdf(const float* cdf, int n, float r)  // DiscreteSampler::sample
{
    int begin = 0, end = n - 1;
    while (end > begin)
    {
        int mid = begin + (end - begin) / 2;
        if (__ldg(cdf + mid) >= r)
            end = mid;
        else
            begin = mid + 1;
    }
    return begin;
}

// lower_bound_cdf with the search started from a guide table (guide[g] = the lower bound of
// g / G, G a power of two): the answer for r lies in [guide[g], guide[g + 1]] with
// g = floor(r * G), so the result is the full search's, in a few steps
__device__ __forceinline__ int lower_bound_guided(const float* cdf, const int* guide, int G, float r)
{
    const int g = clampi(static_cast<int>(r * static_cast<float>(G)), 0, G - 1);
    int       begin = __ldg(guide + g), end = __ldg(guide + g + 1);
    while (end > begin)
    {
        int mid = begin + (end - begin) / 2;
        if (__ldg(cdf + mid) >= r)
            end = mid;
        else
            begin = mid + 1;
    }
    return begin;
}

__device__ __forceinline__ float env_pdf_at(const SceneView& s, int ui, int vi)
{
    float lum = __ldg(&s.env_rgb[ui + vi * s.env_w].w);
    return s.env_norm * lum * static_cast<float>(s.env_w) * static_cast<float>(s.env_h) / (2.f * kPi * kPi);
}

__device__ __forceinline__ int2 env_texel(int env_w, int env_h, float3 d)
{
    float phi = acosf(d.y);
    float theta = atanf(d.z / d.x) + kPi * 0.5f;
    if (d.x < 0.f) theta += kPi;
    return make_int2(clampi(static_cast<int>(theta / (kPi * 2.f) * static_cast<float>(env_w)), 0, env_w - 1),
                     clampi(static_cast<int>(phi / kPi * static_cast<float>(env_h)), 0, env_h - 1));
}

__device__ __forceinline__ float env_pdf(const SceneView& s, float3 d)
{
    const int2 t = env_texel(s.env_w, s.env_h, d);
    return env_pdf_at(s, t.x, t.y);
}

__device__ __forceinline__ float3 env_radiance(const SceneView& s, float3 d)
{
    const int2 t = env_texel(s.env_w, s.env_h, d);
    return xyz(__ldg(&s.env_rgb[t.x + t.y * s.env_w]));
}

// EnvmapLoader::sample with the two texel-jitter numbers explicit
__device__ __forceinline__ void env_sample(const SceneView& s, float r1, float r2, float j1, float j2, float3& dir,
                                           float3& rad, float& pdf)
{
    int   W = s.env_w, H = s.env_h;
    int   ui0 = lower_bound_guided(s.env_marginal, s.env_guide_m, kEnvGuideM, r1);
    int   vi0 = lower_bound_guided(s.env_cond + static_cast<size_t>(ui0) * H,
                                   s.env_guide_c + static_cast<size_t>(ui0) * (kEnvGuideC + 1), kEnvGuideC, r2);
    float u = (static_cast<float>(ui0) + j1) / static_cast<float>(W);
    float v = (static_cast<float>(vi0) + j2) / static_cast<float>(H);
    int   ui = clampi(static_cast<int>(u * static_cast<float>(W)), 0, W - 1);
    int   vi = clampi(static_cast<int>(v * static_cast<float>(H)), 0, H - 1);
    float phi = v * kPi;
    float theta = u * 2.f * kPi;
    float sp = sinf(phi);
    dir = mk(sp * sinf(theta), cosf(phi), sp * -cosf(theta));
    pdf = env_pdf_at(s, ui, vi);
    rad = xyz(__ldg(&s.env_rgb[ui + vi * W]));
}

// Camera::makeRay (camera.cpp:37-43)
__device__ __forceinline__ void camera_ray(const CameraGPU& c, float mx, float my, float3& o, float3& d)
{
    float3 su = mk(c.fxx, c.fxy, c.fxz) * ((mx - 0.5f) * c.film_w);
    float3 sv = mk(c.fyx, c.fyy, c.fyz) * ((my - 0.5f) * c.film_h);
    float3 sw = mk(c.wx, c.wy, c.wz) * c.dist;
    o = mk(c.ox, c.oy, c.oz);
    d = normalize3(su + sv + sw);
}

// tent-filtered sample position (demo_pt.cpp:689-697)
__device__ __forceinline__ float tent(float r) { return r < 1.f ? sqrtf(r) - 1.f : 1.f - sqrtf(2.f - r); }

}  // namespace mcrt
