// One vertex of the radiance estimator (demo_pt.cpp:523-651), split into the pieces the
// wavefront kernels and the adjoint replay share:
//   vertex_emission  miss / emitter hit: passive emission (demo_pt.cpp:528-553)
//   make_nee         next-event rays at a Lambert or GGX vertex: environment light sample
//                    and BSDF sample (any-hit shadow rays, MIS-weighted, demo_pt.cpp:564-589),
//                    area-light BSDF sample and light sample (closest-hit rays whose result
//                    depends on which emitter they reach, demo_pt.cpp:591-642)
//   nee_contribution what a traced next-event ray adds (Scene::lightPdfW / lightRadiance,
//                    scene.cpp:239-267, :345-366)
//   continue_path    continuation sample (demo_pt.cpp:647-650) and Russian roulette
#pragma once
#include "device.cuh"

namespace mcrt {

enum NeeType
{
    NEE_ENV = 0,        // any hit: contributes `val` when unoccluded
    NEE_AREA_BSDF = 1,  // closest hit: emitter reached -> val * E * MIS(pdf_bsdf = val.w, pdf_light)
    NEE_AREA_LIGHT = 2  // closest hit, bounded: emitter `light` reached -> val * E
};

struct NeeRay
{
    float3 d;
    float  tmax;
    float4 val;
    int    type;
    int    light;
    float  tterm;  // closest-hit rays: a hit nearer than this cannot be an emitter (unused by any-hit rays)
};

// The part [t0, t1] of the ray o + t d (d unit length) inside the bounding box of the
// emitter triangles, widened by the scene's margin plus 1e-3 of the origin's largest
// coordinate so that every hit the traversal reports on an emitter lies inside it.  False
// when the ray cannot reach an emitter: then the closest hit, whatever it is, is not one.
__device__ __forceinline__ bool emitter_span(const SceneView& S, float3 o, float3 d, float& t0, float& t1)
{
    const float pad = S.light_pad + 1e-3f * fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    t0 = -__int_as_float(0x7f800000);
    t1 = __int_as_float(0x7f800000);
    const float lo[3] = {S.light_lo.x - pad, S.light_lo.y - pad, S.light_lo.z - pad};
    const float hi[3] = {S.light_hi.x + pad, S.light_hi.y + pad, S.light_hi.z + pad};
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        // an axis the ray moves along by less than 1e-20 per unit: parallel to the slab
        // (another axis bounds t by the box, so the drift stays far inside the margin)
        if (fabsf(dd[a]) < 1e-20f)
        {
            if (oo[a] < lo[a] || oo[a] > hi[a]) return false;
            continue;
        }
        const float inv = __fdividef(1.0f, dd[a]);  // within 2 ulp: far inside the margin
        const float ta = (lo[a] - oo[a]) * inv, tb = (hi[a] - oo[a]) * inv;
        t0 = fmaxf(t0, fminf(ta, tb));
        t1 = fminf(t1, fmaxf(ta, tb));
    }
    return t0 <= t1;
}

// emission picked up when the extension ray misses or hits an emitter
// LIGHTS: the light kinds a build handles (1 environment, 2 area lights, 3 both); the
// shading kernel is built per combination, so a render without one kind does not carry
// its code (the shading kernel misses in the instruction cache) or its registers
template <int LIGHTS = 3>
__device__ __forceinline__ float3 miss_emission(const SceneView& S, float3 d, float3 T, bool no_direct)
{
    if ((LIGHTS & 1) && no_direct && S.env_w > 0) return T * env_radiance(S, d);
    return mk(0.f, 0.f, 0.f);
}

// next-event rays of one scattering vertex (at most 2 any-hit + 2 closest-hit rays);
// u: the vertex's NUM_DIMS uniforms.  Returns the number written to out.
template <int LIGHTS = 3>
__device__ __forceinline__ int make_nee(const SceneView& S, const Mat& m, float3 wi, float3 ns, float3 phit, float3 T,
                                        const float* u, NeeRay* out)
{
    int k = 0;
    const float inf = __int_as_float(0x7f800000);
    if ((LIGHTS & 1) && S.env_w > 0)
    {
        // sampleEnvmapUsingLightPDF (demo_pt.cpp:430-465)
        float3 ldir, lrad;
        float  lpdf;
        env_sample(S, u[D_ENV_LIGHT_0], u[D_ENV_LIGHT_1], u[D_ENV_JITTER_U], u[D_ENV_JITTER_V], ldir, lrad, lpdf);
        float g = fmax_ref(0.f, dot3(ldir, ns));
        if (g > 0.f)
        {
            float  pe = env_pdf(S, ldir);
            float  wE = pe / (pe + bsdf_pdf(m, wi, ns, ldir));
            float3 irr = (bsdf_eval(m, wi, ns, ldir) * g * (1.0f / lpdf)) * lrad;
            float3 val = T * (irr * wE);
            if (!isnan3(val)) out[k++] = NeeRay{ldir, inf, make_float4(val.x, val.y, val.z, 0.f), NEE_ENV, 0};
        }
        // sampleEnvmapUsingSurfacePDF (demo_pt.cpp:466-507): the reference's own cosine
        // sample for Lambert; GGX samples its lobe
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
                if (!isnan3(val)) out[k++] = NeeRay{wo, inf, make_float4(val.x, val.y, val.z, 0.f), NEE_ENV, 0};
            }
        }
        else
        {
            BsdfSample bs = bsdf_sample(m, wi, ns, u[D_ENV_BSDF_0], u[D_ENV_BSDF_1]);
            if (maxc(bs.weight) > 0.f && bs.pdf > 0.f)
            {
                float  wB = bs.pdf / (bs.pdf + env_pdf(S, bs.wo));
                float3 val = T * ((bs.weight * env_radiance(S, bs.wo)) * wB);
                if (!isnan3(val)) out[k++] = NeeRay{bs.wo, inf, make_float4(val.x, val.y, val.z, 0.f), NEE_ENV, 0};
            }
        }
    }
    if ((LIGHTS & 2) && S.light_area > 0.f)
    {
        // BSDF sample, MIS against the area lights (demo_pt.cpp:593-614)
        // Only a ray that meets the emitters' box can contribute: the others are not traced,
        // and the traced ones end at the box (a farther hit is no emitter) and stop at a hit
        // before it (the closest hit is then no emitter either)
        BsdfSample bs = bsdf_sample(m, wi, ns, u[D_AREA_BSDF_0], u[D_AREA_BSDF_1]);
        float      e0, e1;
        if (maxc(bs.weight) > 0.f && emitter_span(S, phit, bs.wo, e0, e1) && e1 >= kEpsRay)
        {
            float3 val = T * bs.weight;
            out[k++] = NeeRay{bs.wo, e1, make_float4(val.x, val.y, val.z, bs.pdf), NEE_AREA_BSDF, 0, e0};
        }
        // light sample (demo_pt.cpp:618-641; Scene::sampleLightArea, scene.cpp:298-343)
        int lo = 0, hi = S.num_lights - 1;
        while (hi > lo)
        {
            int mid = lo + (hi - lo) / 2;
            if (__ldg(&S.lights[mid].cdf) >= u[D_LIGHT_PICK])
                hi = mid;
            else
                lo = mid + 1;
        }
        LightGPU      L = S.lights[lo];
        const float4* lv = S.prim_verts + 3 * L.prim;
        float         r0 = sqrtf(u[D_LIGHT_U]);
        float         lu = 1.f - r0, lvv = u[D_LIGHT_V] * r0;
        float3        lp = xyz(__ldg(lv)) * (1.f - lu - lvv) + xyz(__ldg(lv + 1)) * lu + xyz(__ldg(lv + 2)) * lvv;
        int           lm;
        float3        ln = shading_normal(S, L.prim, lu, lvv, lm);
        float         pdfA = (1.f / L.area) * L.pdf;
        float3        wo = lp - phit;
        float         dist2 = dot3(wo, wo);
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
            float e0, e1;
            if (maxc(f) > 0.f && cs > 0.f && emitter_span(S, phit, wo, e0, e1))
            {
                float3 val = T * (f * (cs / pdfW * mis));
                // closest hit bounded just past the sampled point: the same answer as the
                // reference's unbounded query for "did the ray reach emitter `lo`"; a hit
                // before the emitters' box ends the query (the ray is blocked)
                out[k++] = NeeRay{wo, sqrtf(dist2) * 1.001f + kEpsRay, make_float4(val.x, val.y, val.z, 0.f),
                                  NEE_AREA_LIGHT, lo, e0};
            }
        }
    }
    return k;
}

// Contribution of a traced next-event ray.  `coef` receives the factor that multiplies
// the emitter radiance (for the emission adjoint) and `emat` the emitter's material.
__device__ __forceinline__ float3 nee_contribution(const SceneView& S, int type, int light, float4 val, float3 dir,
                                                   bool hit, const Hit& h, float3& coef, int& emat)
{
    emat = -1;
    coef = mk(0.f, 0.f, 0.f);
    if (type == NEE_ENV) return hit ? mk(0.f, 0.f, 0.f) : xyz(val);
    if (!hit) return mk(0.f, 0.f, 0.f);
    int    matid;
    float3 ns = shading_normal(S, h.prim, h.u, h.v, matid);
    Mat    hm = load_mat(S, matid);
    if (hm.type != MAT_LGHT || dot3(ns, -dir) < 0.f) return mk(0.f, 0.f, 0.f);
    if (type == NEE_AREA_BSDF)
    {
        float cl = dot3(ns, -dir);
        float pdfL = 0.f;
        if (cl >= 1e-6f)
        {
            LightGPU L = S.lights[S.light_of[h.prim]];
            float    pdfA = (1.f / L.area) * L.pdf;
            pdfL = pdfA * (h.t * h.t) / cl;
        }
        float mis = val.w / (val.w + pdfL);
        coef = xyz(val) * mis;
    }
    else
    {
        if (S.light_of[h.prim] != light) return mk(0.f, 0.f, 0.f);
        coef = xyz(val);
    }
    emat = matid;
    return coef * hm.color;
}

// continuation sample + Russian roulette; returns whether the path goes on
__device__ __forceinline__ bool continue_path(const Mat& m, float3 wi, float3 ns, float3 T, const float* u, int depth,
                                              int max_depth, int rr_depth, float3& T2, float3& cdir)
{
    BsdfSample cs = bsdf_sample(m, wi, ns, u[D_CONT_0], u[D_CONT_1]);
    T2 = T * cs.weight;
    cdir = cs.wo;
    bool cont = depth < max_depth;
    if (rr_depth >= 0 && depth >= rr_depth)
    {
        // SmallVCM rule (vcm_material.h:632-641): q = max component of the reflectance
        float q = fminf(fmaxf(maxc(m.color), 0.f), 1.f);
        if (u[D_RR] >= q)
            cont = false;
        else
            T2 = T2 * (1.f / q);
    }
    if (!(maxc(T2) > 0.f)) cont = false;
    return cont;
}

}  // namespace mcrt
