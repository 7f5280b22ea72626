// Device data layouts shared by the host builder/flattener and the CUDA kernels.
//
// HBM layout of one scene (all arrays 16-B aligned, nodes 64-B aligned):
//   FastNode  [num_fast_nodes]  64 B  two-child node, child boxes inline (binary tree of
//                                     the builder, children fetched with 4 x 16-B loads)
//   fast_tris [3 * num_refs]    48 B  per leaf reference, in leaf order:
//                                     {v0.xyz, prim}, {v1.xyz, -}, {v2.xyz, -}
//   RefNode   [num_ref_nodes]   32 B  the same binary tree with each node's OWN box, for the
//                                     reference-order traversal (MCRT_TRAVERSE_REF)
//   RefPrim   [num_refs]        32 B  clipped bound + primitive id per leaf reference
//   prim_verts[3 * num_prims]   48 B  original vertices a, b, c by primitive id (for the
//                                     reference Moller-Trumbore test)
//   prim_shade[3 * num_prims]   48 B  vertex normals na, nb, nc; .w of the first = material id
//   light_of  [num_prims]        4 B  emitter index or -1
//   lights    [num_lights]      16 B  {prim, area, pdf, cdf}
//   materials [num_materials]   32 B
//   envmap: rgb (float4 per texel), luminance, marginal + conditional CDFs
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define MCRT_HD __host__ __device__
#else
#define MCRT_HD
#include <vector_types.h>
#endif

namespace mcrt {

// children: c >= 0 inner node index; c < 0 leaf ~((first << 4) | count) into fast_tris
// (count <= 15; ~0 = empty); n3.z/w repeat the counts
struct __align__(64) FastNode
{
    float4 n0;  // c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y
    float4 n1;  // c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y
    float4 n2;  // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
    int4   n3;  // child0, child1, count0, count1
};

// Eight-child node of the FAST traversal (96 B, three 32-B loads), after the compressed
// wide BVH of Ylitie, Karras and Laine (HPG 2017): the children's boxes are quantised to
// 8 bits per plane on a per-node grid (origin p, power-of-two cell size 2^(e - 127) per
// axis, every child box rounded outwards), inner children are stored contiguously from
// child_base in slot order, and the leaf children's triangles contiguously from tri_base.
// Slots are assigned so that visiting them in the order slot ^ octant(ray direction)
// approximates front-to-back order for every octant.
//   w0: p.x, p.y, p.z, (e.x | e.y << 8 | e.z << 16 | imask << 24)
//   w1: child_base, tri_base, meta[0..3], meta[4..7]
//       meta[s] = leaf child: 0x80 | (count - 1) << 5 | first, its triangles tri_base + first
//       .. + count - 1 (count 1..4, first + count <= 32); 0 otherwise (inner children are
//       the bits of imask)
//   w2: lo.x[0..7], lo.y[0..7]            (8-bit quantised planes, byte s = slot s)
//   w3: lo.z[0..7], hi.x[0..7]
//   w4: hi.y[0..7], hi.z[0..7]
//   w5: unused
// An empty slot has lo = 255 > hi = 0 on every axis, so no ray enters it.
struct __align__(32) WideNode
{
    float4 w0;
    int4   w1;
    int4   w2, w3, w4;
    int4   w5;
};
#ifndef MCRT_WIDE_LEAF
#define MCRT_WIDE_LEAF 4
#endif
constexpr int kWideMaxLeafTris = MCRT_WIDE_LEAF;  // triangles per leaf child
constexpr int kWideMaxNodeTris = 32;  // triangles per node (the hit mask of a node's leaves)

// inner: a = left, b = (right << 2) | split_axis;  leaf: a = ~ref_begin, b = ref_count
struct __align__(32) RefNode
{
    float4 lo;  // bmin.xyz, a (int bits)
    float4 hi;  // bmax.xyz, b (int bits)
};

struct __align__(32) RefPrim
{
    float4 lo;  // clipped bmin.xyz, prim (int bits)
    float4 hi;  // clipped bmax.xyz, unused
};

struct __align__(32) MaterialGPU
{
    int   type;
    float r, g, b;
    float roughness;
    float ior;
    int   albedo_param;
    int   emission_param;
};

struct __align__(16) LightGPU
{
    int   prim;
    float area;
    float pdf;
    float cdf;
};

// Read-only view of one uploaded scene (device pointers).
// guide-table resolution of the environment-map CDF searches (powers of two)
constexpr int kEnvGuideM = 256;
constexpr int kEnvGuideC = 256;  // 64: 0.3 ms more shading per cfg1 frame

struct SceneView
{
    const FastNode*    fast_nodes;
    const float4*      fast_tris;
    const WideNode*    wide_nodes;  // the FAST traversal's eight-child tree
    const float4*      wide_tris;   // its leaf triangles {v0, prim}, {v1}, {v2} in node order
    const RefNode*     ref_nodes;
    const RefPrim*     ref_prims;
    const float4*      prim_verts;
    const float4*      prim_shade;
    const int*         light_of;
    const LightGPU*    lights;
    const MaterialGPU* materials;
    const float4*      env_rgb;       // W*H texels, .w = un-warped luminance
    const float*       env_marginal;  // W column CDF
    const float*       env_cond;      // W*H: per column, H-entry CDF (column-major)
    const int*         env_guide_m;   // kEnvGuideM + 1: lower bound of g / kEnvGuideM in env_marginal
    const int*         env_guide_c;   // W*(kEnvGuideC + 1): the same per column of env_cond
    const float4*      prim_alpha;    // per prim: consistent-normal alphas of a, b, c (or null)
    int                num_lights;
    float              light_area;
    // bounding box of the emitter triangles and the margin that keeps every hit the
    // traversal reports on an emitter inside it (emitter_span, estimator.cuh)
    float3             light_lo, light_hi;
    float              light_pad;
    int                env_w, env_h;
    float              env_norm;  // 1 / sum of sin-warped luminance
    int                num_prims;
    int                fast_root_is_leaf;  // unused: the flattener always emits a FastNode root
};

// Camera in the form Camera::makeRay uses (camera.cpp:9-43)
struct CameraGPU
{
    float ox, oy, oz;
    float fxx, fxy, fxz;  // m_frame_x
    float fyx, fyy, fyz;  // m_frame_y
    float wx, wy, wz;     // m_forward
    float film_w, film_h, dist;
};

struct JobGPU
{
    SceneView scene;
    CameraGPU cam;
    int       width, height, spp, max_depth, rr_depth, traverse;
    uint64_t  seed;
    int64_t   path_offset;  // first global path index of this job
    float*    image;        // device image (sum written by resolve)
};

}  // namespace mcrt
