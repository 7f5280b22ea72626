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
