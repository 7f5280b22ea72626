/*
 * mcrt_gb300.h -- C ABI of the GB300 (sm_103a) path-tracing library.
 *
 * Plain C: pointers, sizes and status codes; no C++ or torch types.  Every entry
 * point returns MCRT_OK (0) or a negative MCRT_ERR_* code and never throws across
 * the boundary; mcrt_last_error() returns the message of the calling thread's last
 * failure.  Device memory for a scene is owned by the library; the caller owns all
 * buffers it passes in.  A scene handle may be used from several host threads as
 * long as each thread uses its own CUDA stream.  Renders on one device share one
 * working-memory block (the ray queues, up to about 50 GB at the default 64 M-ray queue;
 * it grows to the largest render and is kept until the process exits), so they run one
 * after another.  Where that block cannot be allocated, the default queue halves itself.
 *
 * Reference interfaces replaced (paths are relative to the MCRT source tree):
 *   SceneBVH::SceneBVH            src/core/scenebvh.h:14, scenebvh.cpp:404-444 -> mcrt_scene_create
 *   SceneBVH::intersect           src/core/scenebvh.h:17, scenebvh.cpp:353-377 -> mcrt_trace_closest
 *   SceneBVH::occluded            src/core/scenebvh.h:18, scenebvh.cpp:379-396 -> mcrt_trace_any
 *   SceneBVH::~SceneBVH           src/core/scenebvh.cpp:398-402                -> mcrt_scene_destroy
 *   rayTrace + DemoSimple::run    src/examples/pt/demo_pt.cpp:512-720        -> mcrt_render
 *   FrameBuffer::dumpHDR/dumpPPM  src/core/film.cpp:9-108                    -> mcrt_film_encode
 *   FrameBuffer::tonemap*         src/core/film.cpp:110-203                  -> mcrt_film_tonemap
 *   (no reference counterpart: path-replay adjoint, batched launch, tuning)   -> mcrt_render_adjoint,
 *                                                                                mcrt_render_adjoint_batch,
 *                                                                                mcrt_render_batch,
 *                                                                                mcrt_autotune
 */
#ifndef MCRT_GB300_H
#define MCRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCRT_ABI_VERSION 4

/* status codes */
#define MCRT_OK 0
#define MCRT_ERR_INVALID_ARGUMENT (-1)
#define MCRT_ERR_CUDA (-2)
#define MCRT_ERR_OUT_OF_MEMORY (-3)
#define MCRT_ERR_QUEUE_OVERFLOW (-4)
#define MCRT_ERR_STACK_OVERFLOW (-5)
#define MCRT_ERR_INTERNAL (-6)
#define MCRT_ERR_IO (-7)

/* material types: the values of MaterialType in src/core/material.h:7, plus GGX */
#define MCRT_MAT_LGHT 0 /* emitter: radiance = color (Scene::lightRadiance, scene.cpp:345-366) */
#define MCRT_MAT_DIFF 1 /* Lambert (bsdf.cpp:51-116) */
#define MCRT_MAT_SPEC 2 /* mirror (bsdf.cpp:134-191) */
#define MCRT_MAT_REFR 3 /* smooth dielectric, exact Fresnel (bsdf.cpp:319-440) */
#define MCRT_MAT_GLSY 4 /* Phong lobe, exponent 25 (bsdf.cpp:209-301) */
#define MCRT_MAT_GGX 8  /* GGX conductor (new: Walter 2007, Heitz 2018, Schlick F0 = color) */
/* flag OR'd into a material type: the vertex shades with the consistent normal
 * (TriangleObject::consistentNormal, triangle.cpp:149-182; Reshetov et al. 2010) instead of
 * the interpolated vertex normal, so mirror reflections never leave through the surface;
 * needs the per-corner alphas of mcrt_scene_desc::vertex_alpha (or derived, see there) */
#define MCRT_MAT_CONSISTENT 0x100

typedef struct mcrt_material {
    int32_t type;           /* MCRT_MAT_* */
    float   color[3];       /* albedo / F0 / transmission tint / emitted radiance */
    float   roughness;      /* GGX alpha */
    float   ior;            /* REFR index of refraction (reference: fixed 1.33) */
    int32_t albedo_param;   /* adjoint parameter group of a DIFF albedo, -1 = none */
    int32_t emission_param; /* adjoint parameter group of an LGHT radiance, -1 = none */
} mcrt_material;

/* A binary BVH given by the caller (e.g. the reference SplitBVH tree,
 * splitbvh.h:32-58): node i is a leaf when node_info[6i] == 1.
 *   node_box[6i..6i+5]  = min xyz, max xyz of the node's bounding_box
 *   node_info[6i..6i+5] = is_leaf, left, right, split_axis, ref_begin, ref_count
 *   refs: ref_prim[k] primitive id, ref_box[6k..] its clipped bound
 * Children are visited left-first iff ray.dir[split_axis] > 0 (splitbvh.cpp:75). */
typedef struct mcrt_bvh_tree {
    int32_t        num_nodes;
    int32_t        num_refs;
    const float*   node_box;
    const int32_t* node_info;
    const int32_t* ref_prim;
    const float*   ref_box;
} mcrt_bvh_tree;

#define MCRT_BUILD_SAH 0       /* the library's own binned-SAH builder */
#define MCRT_BUILD_EXTERNAL 1  /* use desc->external_tree */
#define MCRT_BUILD_SAH_SPLIT 2 /* the library's builder with spatial splits (references straddling a
                                  split plane duplicated with clipped boxes, as the reference's
                                  SplitBVH, splitbvh.cpp:664-1408) */

typedef struct mcrt_scene_desc {
    int64_t              num_triangles;
    const float*         vertices;     /* [num_triangles][3][3] a, b, c (TriangleObject::a,b,c) */
    const float*         normals;      /* [num_triangles][3][3] na, nb, nc; NULL -> face normal */
    const int32_t*       material_ids; /* [num_triangles] */
    int32_t              num_materials;
    const mcrt_material* materials;
    int32_t              env_width; /* 0 -> no environment map */
    int32_t              env_height;
    const float*         env_rgb; /* [env_height][env_width][3], row-major, top row first (envmap.h:20-25) */
    int32_t              builder; /* MCRT_BUILD_* */
    int32_t              leaf_size; /* own builder: max triangles per leaf (0 -> 2) */
    const mcrt_bvh_tree* external_tree;
    /* [num_triangles][3] per-corner alpha for MCRT_MAT_CONSISTENT materials
     * (TriangleObject::m_vertex_alpha as Mesh::genNormals computes it, mesh.cpp:92-115);
     * NULL -> mcrt_vertex_alpha of the triangles (vertices welded by position) */
    const float*         vertex_alpha;
} mcrt_scene_desc;

typedef struct mcrt_scene mcrt_scene;

/* Rays and hits are structure-of-arrays-of-float4, 32 B per ray:
 *   rays[2i]   = {ox, oy, oz, tmin}, rays[2i+1] = {dx, dy, dz, tmax}
 * Hits: 16 B per ray {t, u, v, prim as int bits}; prim = -1 on a miss. */
typedef struct mcrt_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} mcrt_ray;

typedef struct mcrt_hit {
    float   t;
    float   u;
    float   v;
    int32_t prim;
} mcrt_hit;

/* traversal modes */
#define MCRT_TRAVERSE_FAST 0 /* 64-B two-child nodes, watertight FP32 test (Woop et al. 2013)
                                with the reference's absolute |det| < 1e-6 rejection */
#define MCRT_TRAVERSE_REF 1  /* the reference's own order and arithmetic: per-node box test at
                                visit time, clipped-bound test, Moller-Trumbore, inv_dir = 0
                                for zero direction components; bit-identical hits */

/* pointer-location flags for mcrt_trace_* and mcrt_render* */
#define MCRT_PTR_HOST 0   /* buffers are host memory: copied in/out inside the call */
#define MCRT_PTR_DEVICE 1 /* buffers are device memory */

typedef struct mcrt_camera {
    float   origin[3];
    float   target[3];
    float   up[3]; /* Scene::setCamera passes (0, 1, 0) */
    float   fov_y; /* degrees */
    int32_t width;
    int32_t height;
} mcrt_camera;

typedef struct mcrt_render_params {
    int32_t  spp;
    int32_t  max_depth;   /* bounces n = 0..max_depth, as demo_pt.cpp:520-523 */
    int32_t  rr_depth;    /* Russian roulette from this vertex index, -1 = off */
    uint64_t seed;
    int32_t  traverse;    /* MCRT_TRAVERSE_* for every ray of the render */
    int32_t  ptr_mode;    /* MCRT_PTR_* for image / gradient buffers */
    int64_t  path_chunk;  /* path slots in flight (both schedules), 0 -> library default */
    int32_t  block_size;  /* threads per block of the wavefront kernels, 0 -> default */
    int32_t  use_graph;   /* capture each wave's per-stage kernels in a CUDA graph */
    int32_t  profile;     /* MCRT_PROFILE_* bits (diagnostics; off for production renders) */
    int32_t  variant;     /* traversal kernel variant, MCRT_VARIANT_* bits (0: default) */
    int32_t  schedule;    /* MCRT_SCHEDULE_* (0: streaming) */
    int32_t  reserved;    /* must be 0 */
} mcrt_render_params;

/* How paths are fed to the stage kernels.  Both give bit-identical images.
 * STREAM: path_chunk slots; a slot whose path ended starts the next camera path in the
 *   following iteration, so the queues stay full until the last paths; per-path results
 *   go to a ring and each pixel is resolved (in sample order) when its last path ends.
 * WAVES:  path_chunk paths per wave, every wave runs depth 0..max_depth to completion
 *   before the next starts (the queues shrink with depth). */
#define MCRT_SCHEDULE_STREAM 0
#define MCRT_SCHEDULE_WAVES 1
/* the plain GPU path tracer: one thread runs each path from the camera to its end (no
 * queues); the wavefront's image up to a few ulp (the same paths, rays and arithmetic) */
#define MCRT_SCHEDULE_PATHS 2

/* variant 0 = default policy (STACK32 when the BVH is shallow enough, REGCAP);
 * MCRT_VARIANT_EXPLICIT | bits = exactly the given bits (for tuning) */
#define MCRT_VARIANT_STACK32 1  /* 32-entry shared-memory stacks (16 KB/block) when the BVH is shallow enough */
#define MCRT_VARIANT_REGCAP 2   /* cap registers at 56 so 9 blocks of 128 threads fit an SM */
#define MCRT_VARIANT_EXPLICIT 4 /* use the bits as given instead of the default policy */
#define MCRT_VARIANT_GRIDSTRIDE 8 /* traversal kernels: static grid stride instead of warps taking
                                     32-ray batches from a counter */


#define MCRT_PROFILE_STAGES 1 /* CUDA events around every stage launch -> stats.stage_ms */
#define MCRT_PROFILE_COUNT 2  /* count BVH nodes fetched / triangles tested per ray class */

typedef struct mcrt_render_stats {
    int64_t paths;
    int64_t extension_rays;
    int64_t shadow_rays;
    int32_t waves;       /* WAVES: waves; STREAM: iterations (regen + extend + shade + connect) */
    int32_t kernel_launches;
    float   device_ms;   /* CUDA-event time of the kernels (excludes host copies) */
    float   stage_ms[4]; /* MCRT_PROFILE_STAGES: begin+raygen+resolve, extend, shade, connect */
    int32_t extend_launches;
    int64_t ext_nodes;   /* MCRT_PROFILE_COUNT: nodes fetched / triangles tested by extension */
    int64_t ext_tris;    /* rays, and by next-event rays */
    int64_t nee_nodes;
    int64_t nee_tris;
    int64_t h2d_bytes;   /* host -> device bytes copied by the call (tables, host inputs) */
    int64_t d2h_bytes;   /* device -> host bytes copied by the call (host outputs, status) */
    int32_t node_bytes;  /* bytes of one node fetch of the traversal counted in ext_nodes / nee_nodes
                            (96: the FAST traversal's eight-child nodes; 64: two-child nodes) */
    int32_t reserved0;
} mcrt_render_stats;

int         mcrt_get_abi_version(void);
const char* mcrt_last_error(void);

/* Builds the BVH on the host (own SAH builder or the given tree), flattens it, builds
 * the emitter and environment-map sampling tables and uploads everything. */
int mcrt_scene_create(const mcrt_scene_desc* desc, mcrt_scene** out_scene);
int mcrt_scene_destroy(mcrt_scene* scene);
/* Per-corner alpha of consistent normals for a triangle soup: Mesh::genNormals
 * (mesh.cpp:66-116) with the corners welded by exact position: alpha = the angle of the
 * smallest cosine between the corner's vertex normal and the unit normals of the faces
 * sharing its position, times 1 + 0.03632 (1 - cos)^2.  out: [num_triangles][3]. */
int mcrt_vertex_alpha(const float* vertices, const float* normals, int64_t num_triangles, float* out);

/* The library's own BVH builder (binned SAH over object splits, multithreaded; host only,
 * no GPU needed), returned in the mcrt_bvh_tree form of the reference SplitBVH dump.  Call
 * with node_box == NULL to get *num_nodes / *num_refs, then with arrays of those sizes
 * (node_box [6 * nodes], node_info [6 * nodes], ref_prim [refs], ref_box [6 * refs]).
 * leaf_size: max references per leaf (1..15, 0 -> 2).  Replaces SplitBVH::SplitBVH
 * (splitbvh.cpp:1410-1625) for callers that build trees themselves. */
int mcrt_build_bvh(const float* vertices, int64_t num_triangles, int32_t leaf_size, int32_t* num_nodes,
                   int32_t* num_refs, float* node_box, int32_t* node_info, int32_t* ref_prim, float* ref_box);
/* The same with spatial splits (MCRT_BUILD_SAH_SPLIT): replaces SplitBVH::build
 * (splitbvh.cpp:1410-1625, spatial splitters :664-1408); refs may repeat a primitive. */
int mcrt_build_bvh_split(const float* vertices, int64_t num_triangles, int32_t leaf_size, int32_t* num_nodes,
                         int32_t* num_refs, float* node_box, int32_t* node_info, int32_t* ref_prim, float* ref_box);

/* Scene inputs from the reference's file formats (host only, no GPU needed).
 * mcrt_mesh_load_obj: the triangles Scene::loadModel(path, transform, mat) adds
 *   (scene.cpp:368-408): the OBJ read as Mesh::Mesh(filepath) does (mesh.cpp:24-60: "v"
 *   and "f" records, 1-based indices, the first three of a face), every vertex multiplied
 *   by `transform` (16 floats, column-major like glm::mat4; NULL = identity), then
 *   Mesh::genNormals (mesh.cpp:66-116): per-vertex normals and consistent-normal alphas.
 *   Call with vertices == NULL to get *num_triangles; then with arrays of that many
 *   triangles: vertices / normals [n][3][3] (a, b, c), vertex_alpha [n][3] (normals and
 *   vertex_alpha may be NULL) -- the mcrt_scene_desc fields of the same names.
 * mcrt_envmap_load_bin: the environment map file EnvmapLoader reads (envmap.cpp:98-119):
 *   {int32 width, int32 height} then width * height RGB floats, top row first.  Call with
 *   rgb == NULL to get the size; then with rgb [height][width][3] and the same size (the
 *   mcrt_scene_desc env_rgb layout). */
int mcrt_mesh_load_obj(const char* path, const float* transform, int64_t* num_triangles, float* vertices,
                       float* normals, float* vertex_alpha);
int mcrt_envmap_load_bin(const char* path, int32_t* width, int32_t* height, float* rgb);

/* Scene cache files (no reference counterpart: the reference rebuilds its SplitBVH, 58 s
 * at 1.3 M triangles, on every run).  mcrt_scene_save writes the prepared device scene
 * (node layouts, leaf triangles, shading, emitter and environment tables) with the hash of
 * the description it was built from; mcrt_scene_load uploads it again without building,
 * after checking the format version, a checksum and every stored index.  expected_hash:
 * the mcrt_scene_desc_hash of the description the caller wants (0 = accept any); a file
 * written for another description fails with MCRT_ERR_INVALID_ARGUMENT. */
int mcrt_scene_desc_hash(const mcrt_scene_desc* desc, uint64_t* hash);
int mcrt_scene_save(const mcrt_scene* scene, const char* path);
int mcrt_scene_load(const char* path, uint64_t expected_hash, mcrt_scene** out_scene);
/* Replace material colours (e.g. optimised albedos) without rebuilding the scene.  The
 * emitter set and consistent normals are fixed when the scene is built: a material that
 * would become or stop being MCRT_MAT_LGHT, or ask for MCRT_MAT_CONSISTENT in a scene built
 * without it, fails with MCRT_ERR_INVALID_ARGUMENT and changes nothing. */
int mcrt_scene_set_materials(mcrt_scene* scene, int32_t num_materials, const mcrt_material* materials,
                             void* stream);
/* Sizes of the device-resident scene: fast nodes, reference-layout nodes, triangle refs. */
int mcrt_scene_info(const mcrt_scene* scene, int64_t* fast_nodes, int64_t* ref_nodes, int64_t* refs,
                    int64_t* device_bytes);

/* Closest hit for n rays: SceneBVH::intersect / SplitBVH::intersect semantics with the
 * caller's [tmin, tmax]; ties keep the first hit in traversal order. */
int mcrt_trace_closest(mcrt_scene* scene, const mcrt_ray* rays, int64_t n, mcrt_hit* hits, int32_t traverse,
                       int32_t ptr_mode, void* stream);
/* Any hit: occluded[i] = 1 when some triangle is hit with tmin < t < tmax. */
int mcrt_trace_any(mcrt_scene* scene, const mcrt_ray* rays, int64_t n, int32_t* occluded, int32_t traverse,
                   int32_t ptr_mode, void* stream);

/* Forward render: rgb_out[height][width][3] = per-pixel mean of the clamped per-sample
 * radiance (row 0 = the camera's bottom row, as FrameBuffer::accumulatePixel). */
int mcrt_render(mcrt_scene* scene, const mcrt_camera* camera, const mcrt_render_params* params, float* rgb_out,
                mcrt_render_stats* stats, void* stream);

/* Path-replay adjoint of mcrt_render (same camera/params/seed): given dL/dimage
 * [height][width][3], ADDS dL/d(albedo) [num_albedo_params][3] and
 * dL/d(emission) [num_emission_params][3]; the caller zeroes them.  Memory is
 * O(pixels + parameters): paths are replayed from their seeds, nothing is taped. */
int mcrt_render_adjoint(mcrt_scene* scene, const mcrt_camera* camera, const mcrt_render_params* params,
                        const float* dL_dimage, float* d_albedo, int32_t num_albedo_params, float* d_emission,
                        int32_t num_emission_params, mcrt_render_stats* stats, void* stream);

/* The adjoint of mcrt_render_batch: every job's paths replayed in one launch, gradients
 * of all jobs summed into the same parameter vectors (e.g. many views of one scene).
 * dL_dimages[j] is job j's dL/dimage; ADDS into d_albedo / d_emission. */
int mcrt_render_adjoint_batch(int32_t num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cameras,
                              const mcrt_render_params* params, const float* const* dL_dimages, float* d_albedo,
                              int32_t num_albedo_params, float* d_emission, int32_t num_emission_params,
                              mcrt_render_stats* stats, void* stream);

/* Many (scene, camera, params) jobs of uneven size in one wavefront: jobs share every
 * stage launch.  rgb_out[j] receives job j's image. */
int mcrt_render_batch(int32_t num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cameras,
                      const mcrt_render_params* params, float* const* rgb_out, mcrt_render_stats* stats,
                      void* stream);

/* Film outputs (FrameBuffer, src/core/film.cpp) on an image in mcrt_render's layout
 * ([height][width][3] floats, row 0 the bottom row); ptr_mode says where rgb / out live.
 *   mcrt_film_encode: the bytes of FrameBuffer::dumpHDR (MCRT_FILM_HDR, film.cpp:35-108:
 *     Radiance header + RLE scanlines of literal runs) or dumpPPM (MCRT_FILM_PPM,
 *     film.cpp:9-33), byte for byte.  out = NULL: only *size is set (the file size).
 *   mcrt_film_tonemap: tonemapGamma(gamma) (MCRT_TONEMAP_GAMMA, film.cpp:196-203; the
 *     per-pixel powf is CUDA's, within its ulp bound of the C library's) or
 *     tonemapReinhard() (MCRT_TONEMAP_REINHARD, film.cpp:110-194, bit for bit), in place. */
#define MCRT_FILM_HDR 0
#define MCRT_FILM_PPM 1
#define MCRT_TONEMAP_GAMMA 0
#define MCRT_TONEMAP_REINHARD 1
int mcrt_film_encode(const float* rgb, int32_t width, int32_t height, int32_t format, uint8_t* out,
                     int64_t capacity, int64_t* size, int32_t ptr_mode, void* stream);
int mcrt_film_tonemap(float* rgb, int32_t width, int32_t height, int32_t op, float gamma, int32_t ptr_mode,
                      void* stream);

/* Autotuner (no reference counterpart).  Renders a reduced-spp probe of the jobs (the
 * same scenes, cameras and depths; about 4 queue capacities of paths in total) under
 * candidate launch configurations -- traversal kernel variants (stack depth, register
 * cap, work distribution) first, then queue capacities (path_chunk) with the best
 * variant -- times each by CUDA events (best of two) and writes the fastest to
 * tuned[0..num_jobs-1] (params with path_chunk and variant set, MCRT_VARIANT_EXPLICIT).
 * Every candidate renders the same image, so tuning never changes results.  report may
 * be NULL.  Allocates scratch images on the device; not for use inside a graph capture. */
#define MCRT_TUNE_MAX 16
typedef struct mcrt_tune_report {
    int32_t num_candidates;
    int32_t chosen;             /* index of the configuration written to tuned */
    int64_t probe_paths;        /* paths of one probe render */
    int64_t path_chunk[MCRT_TUNE_MAX];
    int32_t variant[MCRT_TUNE_MAX];
    float   ms[MCRT_TUNE_MAX];  /* kernel time of the probe render */
} mcrt_tune_report;

int mcrt_autotune(int32_t num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cameras,
                  const mcrt_render_params* params, mcrt_render_params* tuned, mcrt_tune_report* report,
                  void* stream);

/* Forward render that allocates nothing (no reference counterpart: MCRT has no GPU and no
 * allocation constraints).  For callers that cannot call cudaMalloc or cudaFree while they
 * render: plug-ins inside a host application that owns all device memory through its own
 * pool and forbids allocations behind its back; render loops sharing the GPU with other
 * streams, which cudaMalloc / cudaFree may stall by synchronising the device; processes
 * that reserve their memory at start-up under a hard budget.  Same image as mcrt_render
 * with ptr_mode = MCRT_PTR_DEVICE; rgb_out must be device memory.  It always runs the
 * WAVES schedule (params->schedule and params->path_chunk are not used).
 * Scratch: one fixed file-scope device array of about 50 MB, held by every GPU that loads
 * the library's module until the process exits; at most 65,536 path slots per wave
 * (spp <= 65,536) and 65,536 waves per call, larger requests fail with
 * MCRT_ERR_INVALID_ARGUMENT.  The first call on a device looks up the array's device
 * address and keeps it for the process (it does not survive cudaDeviceReset); make that
 * first call before any stream capture.  All calls share the array: calls whose work
 * overlaps on the GPU race, so serialise them.  The calling thread's current device is left
 * as it was.  stats->device_ms is not measured (timing would need events). */
int mcrt_render_noalloc(mcrt_scene* scene, const mcrt_camera* camera, const mcrt_render_params* params,
                        float* rgb_out_device, mcrt_render_stats* stats, void* stream);

/* L2 read bandwidth of the current GPU in GB/s (no reference counterpart: a roofline
 * denominator for the traversal kernels, whose node and triangle reads mostly hit L2).
 * Reads an L2-resident buffer of `bytes` (1 MB .. 96 MB) `reps` times (1 .. 1000) in one
 * launch with L1-bypassing 16-B loads; allocates and frees its buffer; blocks. */
int mcrt_probe_l2_read(int64_t bytes, int32_t reps, float* gbs, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MCRT_GB300_H */
