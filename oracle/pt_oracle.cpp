// ============================================================================
// THE ORACLE — test infrastructure, never part of the product path.
//
// A CPU restatement of the reference renderer's unidirectional path tracer, used
// only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker.  Templated on the arithmetic type: `float` mode follows the reference's
// single-precision operation order (no FMA contraction: build with
// -ffp-contract=off) so per-function results can be compared bit-for-bit with the
// reference; `double` mode is the FP64 oracle that rendered images are checked
// against.
//
// What it restates (reference file:line):
//   rayTrace                          src/examples/pt/demo_pt.cpp:512-655
//   EnvmapSampler, MIS_weight         src/examples/pt/demo_pt.cpp:416-508
//   render loop + tent filter         src/examples/pt/demo_pt.cpp:680-710
//   Camera::Camera / makeRay          src/core/camera.cpp:9-43
//   rayTriangleIntersect (M-T)        src/core/triangle.cpp:13-51, :201-225
//   TriangleObject normal/area/sample src/core/triangle.cpp:71, :90-132
//   Scene::lightPdfW / sampleLightArea / lightRadiance  src/core/scene.cpp:239-366
//   DiscreteSampler                   src/core/sample.cpp:11-118
//   sampleHemisphereCosine            src/core/sample.cpp:132-137
//   Lambertian/Specular/Glossy/Refractive BSDFs  src/core/bsdf.cpp:51-440
//   fresnelReflectance, reflectWorld  src/core/geometry.cpp:14-55
//   OrthonormalFrame (Duff et al.)    src/core/geometry.cpp:74-110
//   EnvmapLoader buildCdf/sample/getPdf/sampleRadiance  src/core/envmap.cpp:44-53, :208-506
//   luminance                         src/core/numeric.cpp:62-66
//
// Named extensions (absent from demo_pt.cpp, specified here and in the CUDA path):
//   * per-path PCG32 random numbers (O'Neill 2014), keyed by (seed, pixel, sample),
//     drawn in a fixed block per vertex, instead of the global racy randf();
//   * max depth and Russian roulette as parameters (RR rule: continue with
//     q = clamp(maxComponent(colour), 0, 1), the SmallVCM rule of
//     src/examples/vcm/vcm_material.h:632-641);
//   * dielectric IOR as a material parameter (the reference fixes 1.33,
//     src/core/material.h:51);
//   * a GGX conductor: Walter et al. 2007 (D, separable Smith G), Heitz 2018
//     (visible-normal sampling), Schlick Fresnel with F0 = colour; next-event
//     estimation runs at GGX vertices as well as Lambert ones.
//   * the path-replay adjoint (Vicini et al. 2021) of the same estimator.
//
// Own BVH: a plain binned-SAH tree with conservative slab tests, independent of the
// product's builder; the closest hit it returns is the closest Moller-Trumbore hit
// accepted under the reference's rules (|det| >= 1e-6, tmin < t < tmax).
// ============================================================================
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace orc {

enum MatType { LGHT = 0, DIFF = 1, SPEC = 2, REFR = 3, GLSY = 4, GGX = 8 };

// ---------------------------------------------------------------------------
// vector type with the reference's operation order (src/core/vectors.cpp)
// ---------------------------------------------------------------------------
template <class T>
struct V3
{
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    V3 operator+(const V3& v) const { return V3(x + v.x, y + v.y, z + v.z); }
    V3 operator-(const V3& v) const { return V3(x - v.x, y - v.y, z - v.z); }
    V3 operator*(T f) const { return V3(x * f, y * f, z * f); }
    V3 operator*(const V3& v) const { return V3(x * v.x, y * v.y, z * v.z); }
    V3 operator/(T f) const
    {
        T r = T(1) / f;
        return V3(x * r, y * r, z * r);
    }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3& operator+=(const V3& v)
    {
        x += v.x;
        y += v.y;
        z += v.z;
        return *this;
    }
    V3& operator*=(const V3& v)
    {
        x *= v.x;
        y *= v.y;
        z *= v.z;
        return *this;
    }
    T  operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    T& at(int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator*(T a, const V3<T>& b) { return b * a; }
template <class T> T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(const V3<T>& a, const V3<T>& b)
{
    return V3<T>((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
template <class T> T length(const V3<T>& v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
template <class T> T lengthSquared(const V3<T>& v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
template <class T> V3<T> normalize(const V3<T>& v)
{
    T inv = T(1) / length(v);
    return V3<T>(v.x * inv, v.y * inv, v.z * inv);
}
template <class T> T fmaxr(T a, T b) { return a > b ? a : b; }  // numeric.cpp f_max
template <class T> T fminr(T a, T b) { return a < b ? a : b; }
template <class T> T maxComponent(const V3<T>& v) { return fmaxr(fmaxr(v.x, v.y), v.z); }
template <class T> V3<T> ld3(const float* p) { return V3<T>(T(p[0]), T(p[1]), T(p[2])); }

// The reference's translation units call cos/sin/acos/atan/tan/pow/fabs unqualified on
// float arguments; with its includes these resolve to the C library's double functions,
// so the result is computed in double and rounded where the reference stores a float
// (std::sqrt, written qualified, stays float).  These helpers make that explicit.
inline double dcos(double x) { return std::cos(x); }
inline double dsin(double x) { return std::sin(x); }
inline double dacos(double x) { return std::acos(x); }
inline double datan(double x) { return std::atan(x); }
inline double dtan(double x) { return std::tan(x); }
inline double dpow(double x, double y) { return std::pow(x, y); }
template <class T> bool isnan3(const V3<T>& v) { return v.x != v.x || v.y != v.y || v.z != v.z; }

template <class T> struct K;
template <> struct K<float>
{
    static constexpr float PI = 3.14159265358979323846f;  // static_cast<float>(const_pi)
    static constexpr float EPS_DET = 1e-6f;
    static constexpr float EPS_RAY = 1e-4f;
    static constexpr float EPS_COS = 1e-6f;
};
template <> struct K<double>
{
    static constexpr double PI = 3.14159265358979323846;
    static constexpr double EPS_DET = 1e-6;
    static constexpr double EPS_RAY = 1e-4;
    static constexpr double EPS_COS = 1e-6;
};

// ---------------------------------------------------------------------------
// PCG32 (O'Neill 2014, pcg32_random_r / pcg32_srandom_r), keyed per path
// ---------------------------------------------------------------------------
static inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Pcg32
{
    uint64_t state, inc;
    uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    float uniform() { return static_cast<float>(next() >> 8) * (1.0f / 16777216.0f); }
    // initstate from (seed, sample), stream from the pixel index
    void seed(uint64_t seed, uint32_t pixel, uint32_t sample)
    {
        uint64_t initstate = splitmix64(seed ^ (static_cast<uint64_t>(sample) * 0xD1B54A32D192ED03ull));
        state = 0u;
        inc = (static_cast<uint64_t>(pixel) << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
};

// The reference's own random numbers: std::default_random_engine (libstdc++: minstd_rand0,
// seed 1) through uniform_real_distribution<float> (generate_canonical<float, 24>: one
// engine call, (x - 1) / 2^31 in float, values >= 1 mapped to nextafter(1, 0)), one global
// stream as randf() (numeric.cpp:7-15).  Used single-threaded to replay the reference
// renderer draw for draw.
struct RefStream
{
    uint64_t  x = 1;
    long long count = 0;
    float     next()
    {
        ++count;
        x = (x * 16807ull) % 2147483647ull;
        float r = static_cast<float>(x - 1) / 2147483648.0f;
        if (r >= 1.0f) r = std::nextafter(1.0f, 0.0f);
        return r;
    }
};

// extension-ray log (debugging the replay): {path, n, ox, oy, oz, dx, dy, dz, prim, t}
static std::vector<double> g_ray_log;
static bool                g_ray_log_on = false;
static std::atomic<long long> g_ext_rays(0);  // extension rays of the last orc_render call
static long long           g_cur_path = 0;

// Random numbers consumed per scattering vertex, in this order.
enum Dim
{
    D_ENV_LIGHT_0 = 0, D_ENV_LIGHT_1, D_ENV_JITTER_U, D_ENV_JITTER_V, D_ENV_BSDF_0, D_ENV_BSDF_1,
    D_AREA_BSDF_0, D_AREA_BSDF_1, D_LIGHT_PICK, D_LIGHT_U, D_LIGHT_V, D_CONT_0, D_CONT_1, D_RR,
    NUM_DIMS
};

// ---------------------------------------------------------------------------
// discrete sampler (sample.cpp:11-118)
// ---------------------------------------------------------------------------
template <class T>
struct Discrete
{
    std::vector<T> pdf, cdf;
    void build(const std::vector<T>& data)
    {
        pdf = data;
        cdf.resize(data.size());
        T norm = T(0);
        for (T d : pdf) norm += d;
        T inv = T(1) / norm;
        for (auto& p : pdf) p = p * inv;
        T sum = T(0);
        for (size_t n = 0; n < pdf.size(); ++n)
        {
            sum += pdf[n];
            cdf[n] = sum;
        }
    }
    int sample(T r) const
    {
        int begin = 0, end = static_cast<int>(cdf.size()) - 1;
        while (end > begin)
        {
            int mid = begin + (end - begin) / 2;
            if (cdf[mid] >= r)
                end = mid;
            else
                begin = mid + 1;
        }
        return begin;
    }
};

// ---------------------------------------------------------------------------
// materials and BSDFs (bsdf.cpp, geometry.cpp; GGX new)
// ---------------------------------------------------------------------------
template <class T>
struct Material
{
    int   type;
    bool  consistent = false;  // type flag 0x100: shade with TriangleObject::consistentNormal
    V3<T> color;
    T     roughness;
    T     ior;
    int   albedo_param = -1;    // adjoint parameter group of a Lambert albedo
    int   emission_param = -1;  // adjoint parameter group of an emitter radiance
};

template <class T>
struct Frame
{
    V3<T> x, y, z;
    explicit Frame(const V3<T>& n)  // geometry.cpp:74-105 (Duff et al. 2017)
    {
        T       sign = std::copysign(T(1), n.z);
        const T a = T(-1) / (sign + n.z);
        const T b = n.x * n.y * a;
        x = V3<T>(T(1) + sign * n.x * n.x * a, sign * b, -sign * n.x);
        y = V3<T>(b, sign + n.y * n.y * a, -n.y);
        z = n;
    }
    V3<T> toWorld(const V3<T>& c) const { return x * c.x + y * c.y + z * c.z; }
    V3<T> toLocal(const V3<T>& v) const { return V3<T>(dot(v, x), dot(v, y), dot(v, z)); }
};

template <class T> V3<T> sampleHemisphereCosine(T x, T y)  // sample.cpp:132-137
{
    x *= 2 * K<T>::PI;
    T r2s = std::sqrt(y);
    return V3<T>(T(dcos(x) * r2s), T(dsin(x) * r2s), std::sqrt(1 - y));
}

template <class T> V3<T> reflectWorld(const V3<T>& wi, const V3<T>& nl)  // geometry.cpp:45-55
{
    return nl * (T(2) * dot(nl, wi)) - wi;
}

template <class T> T fresnelReflectance(T cos_theta_i, T ior)  // geometry.cpp:14-43
{
    if (ior < 0) return 1;
    T eta;
    if (cos_theta_i < 0)
    {
        cos_theta_i = -cos_theta_i;
        eta = ior;
    }
    else
    {
        eta = T(1) / ior;
    }
    const T sin_theta_t_sqr = fminr(T(1), (eta * eta) * (T(1) - cos_theta_i * cos_theta_i));
    const T cos_theta_t = std::sqrt(T(1) - sin_theta_t_sqr);
    T       t1 = eta * cos_theta_t;
    const T r_s = (cos_theta_i - t1) / (cos_theta_i + t1);
    T       t2 = eta * cos_theta_i;
    const T r_p = (t2 - cos_theta_t) / (t2 + cos_theta_t);
    return (r_s * r_s + r_p * r_p) * T(0.5);
}

// GGX microfacet helpers in the local frame (z = normal)
template <class T> T ggxD(const V3<T>& h, T a)
{
    T a2 = a * a;
    T c2 = h.z * h.z;
    T d = c2 * (a2 - T(1)) + T(1);
    return a2 / (K<T>::PI * d * d);
}
template <class T> T ggxG1(const V3<T>& v, T a)
{
    T c2 = v.z * v.z;
    if (c2 <= T(0)) return T(0);
    T t2 = (T(1) - c2) / c2;
    return T(2) / (T(1) + std::sqrt(T(1) + a * a * t2));
}
template <class T> V3<T> schlick(const V3<T>& f0, T c)
{
    T m = T(1) - c;
    T m5 = m * m * m * m * m;
    return f0 + (V3<T>(T(1)) - f0) * m5;
}

template <class T>
struct BsdfSample
{
    V3<T> wo;
    V3<T> weight;  // f * cos / pdf, as Material::sample's total_weight
    T     pdf;     // solid-angle pdf (or the reference's projected value for delta lobes)
};

// Material::sample (material.cpp:55-62 -> bsdf.cpp)
template <class T>
BsdfSample<T> bsdfSample(const Material<T>& m, const V3<T>& wi, const V3<T>& nl, T r1, T r2)
{
    BsdfSample<T> s;
    s.pdf = 0;
    switch (m.type)
    {
        case SPEC:  // bsdf.cpp:134-162
        {
            s.wo = reflectWorld(wi, nl);
            s.weight = m.color;
            s.pdf = 1;
            return s;
        }
        case REFR:  // bsdf.cpp:319-418
        {
            bool  outside = dot(wi, nl) > 0;
            V3<T> n = outside ? nl : -nl;
            V3<T> refl_dir = normalize(reflectWorld(wi, n));
            T     nc = 1, nt = m.ior;
            T     nnt = outside ? nc / nt : nt / nc;
            T     ddn = dot(-wi, n);
            T     cos2t = 1 - nnt * nnt * (1 - ddn * ddn);
            if (cos2t < 0)
            {
                s.weight = m.color;
                s.pdf = 1;
                s.wo = refl_dir;
                return s;
            }
            V3<T> tdir = normalize(-wi * nnt - n * (ddn * nnt + std::sqrt(cos2t)));
            T     Re = fresnelReflectance(dot(wi, nl), nt / nc);
            T     Tr = 1 - Re;
            T     P = Re;
            V3<T> tw(T(1));
            T     RP = Re / P;
            T     TP = Tr / (1 - P);
            if (r1 < P)
            {
                tw *= m.color * RP;
                s.weight = tw;
                s.pdf = P;
                s.wo = refl_dir;
            }
            else
            {
                tw *= m.color * TP;
                s.weight = tw;
                s.pdf = 1 - P;
                s.wo = tdir;
            }
            return s;
        }
        case GLSY:  // bsdf.cpp:209-262 (Phong lobe, glossiness 25)
        {
            T g = T(25);
            // sampleHemisphereCosinePower (sample.cpp:139-145)
            T     x = r1 * (2 * K<T>::PI);
            T     r2p = T(dpow(r2, 1.0 / (double(g) + 1.0)));
            T     sx = T(dsin(x)), cx = T(dcos(x)), st = T(std::sqrt(1.0 - double(r2p * r2p)));  // r2p * r2p is a float product
            V3<T> c(sx * st, cx * st, r2p);
            V3<T>    refl = reflectWorld(wi, nl);
            Frame<T> onb(refl);
            V3<T>    wo = onb.toWorld(c);
            if (dot(wo, nl) < 0) wo = V3<T>(T(0));
            T _cos = fmaxr(dot(wo, nl), K<T>::EPS_COS);
            s.pdf = T((g + T(1)) / (T(2) * K<T>::PI) * dpow(fmaxr(dot(refl, wo), K<T>::EPS_COS), g));
            T wo_n = dot(wo, nl);
            T wi_n = dot(wi, nl);
            T w = (g + T(2)) / (g + T(1)) * _cos / fmaxr(std::fabs(wi_n), std::fabs(wo_n));
            if (w != w) w = 0;
            s.weight = m.color * w;
            s.wo = wo;
            return s;
        }
        case GGX:  // Heitz 2018 visible-normal sampling of Walter et al. 2007 GGX
        {
            V3<T> n = dot(wi, nl) < 0 ? -nl : nl;  // two-sided conductor
            Frame<T> fr(n);
            V3<T>    wl = fr.toLocal(wi);
            T        a = m.roughness;
            if (wl.z <= T(0))
            {
                s.wo = n;
                s.weight = V3<T>(T(0));
                return s;
            }
            V3<T> vh = normalize(V3<T>(a * wl.x, a * wl.y, wl.z));
            T     lensq = vh.x * vh.x + vh.y * vh.y;
            V3<T> t1 = lensq > T(0) ? V3<T>(-vh.y, vh.x, T(0)) * (T(1) / std::sqrt(lensq)) : V3<T>(T(1), T(0), T(0));
            V3<T> t2 = cross(vh, t1);
            T     r = std::sqrt(r1);
            T     phi = T(2) * K<T>::PI * r2;
            T     p1 = r * std::cos(phi);
            T     p2 = r * std::sin(phi);
            T     sh = T(0.5) * (T(1) + vh.z);
            p2 = (T(1) - sh) * std::sqrt(fmaxr(T(0), T(1) - p1 * p1)) + sh * p2;
            V3<T> nh = t1 * p1 + t2 * p2 + vh * std::sqrt(fmaxr(T(0), T(1) - p1 * p1 - p2 * p2));
            V3<T> h = normalize(V3<T>(a * nh.x, a * nh.y, fmaxr(T(0), nh.z)));
            T     wih = dot(wl, h);
            V3<T> ol = h * (T(2) * wih) - wl;
            s.wo = fr.toWorld(ol);
            if (ol.z <= T(0) || wih <= T(0))
            {
                s.weight = V3<T>(T(0));
                return s;
            }
            s.pdf = ggxG1(wl, a) * ggxD(h, a) / (T(4) * wl.z);
            s.weight = schlick(m.color, wih) * ggxG1(ol, a);
            return s;
        }
        case DIFF:
        default:  // bsdf.cpp:51-87
        {
            V3<T>    c = sampleHemisphereCosine(r1, r2);
            Frame<T> onb(nl);
            V3<T>    wo = onb.toWorld(c);
            T        _cos = fmaxr(dot(wo, nl), K<T>::EPS_COS);
            s.pdf = _cos / K<T>::PI;
            s.weight = m.color;
            s.wo = wo;
            return s;
        }
    }
}

// Material::pdfW (bsdf.cpp calculatePdfW)
template <class T> T bsdfPdf(const Material<T>& m, const V3<T>& wi, const V3<T>& nl, const V3<T>& wo)
{
    switch (m.type)
    {
        case DIFF: return fmaxr(dot(wo, nl), K<T>::EPS_COS) / K<T>::PI;
        case GLSY:
        {
            T     g = T(25);
            V3<T> refl = reflectWorld(wi, nl);
            return T((g + T(1)) / (T(2) * K<T>::PI) * dpow(fmaxr(dot(refl, wo), K<T>::EPS_COS), g));
        }
        case GGX:
        {
            V3<T>    n = dot(wi, nl) < 0 ? -nl : nl;
            Frame<T> fr(n);
            V3<T>    wl = fr.toLocal(wi), ol = fr.toLocal(wo);
            if (wl.z <= T(0) || ol.z <= T(0)) return T(0);
            V3<T> h = normalize(wl + ol);
            return ggxG1(wl, m.roughness) * ggxD(h, m.roughness) / (T(4) * wl.z);
        }
        default: return T(0);
    }
}

// Material::evaluate (bsdf.cpp evaluate), BSDF value without the cosine
template <class T> V3<T> bsdfEval(const Material<T>& m, const V3<T>& wi, const V3<T>& nl, const V3<T>& wo)
{
    switch (m.type)
    {
        case DIFF: return V3<T>(T(1) / K<T>::PI) * m.color;
        case GLSY:
        {
            T     wo_n = dot(wo, nl), wi_n = dot(wi, nl);
            V3<T> refl = reflectWorld(wi, nl);
            T     g = T(25);
            return m.color * T((g + 2.0) / (2.0 * K<T>::PI) * dpow(fmaxr(dot(refl, wo), K<T>::EPS_COS), g) /
                               fmaxr(T(std::fabs(double(wi_n))), T(std::fabs(double(wo_n)))));
        }
        case GGX:
        {
            V3<T>    n = dot(wi, nl) < 0 ? -nl : nl;
            Frame<T> fr(n);
            V3<T>    wl = fr.toLocal(wi), ol = fr.toLocal(wo);
            if (wl.z <= T(0) || ol.z <= T(0)) return V3<T>(T(0));
            V3<T> h = normalize(wl + ol);
            T     a = m.roughness;
            T     s = ggxD(h, a) * ggxG1(wl, a) * ggxG1(ol, a) / (T(4) * wl.z * ol.z);
            return schlick(m.color, dot(wl, h)) * s;
        }
        default: return V3<T>(T(0));
    }
}

static inline bool doesNee(int type) { return type == DIFF || type == GGX; }

// ---------------------------------------------------------------------------
// environment map (envmap.cpp)
// ---------------------------------------------------------------------------
template <class T>
struct Envmap
{
    int              W = 0, H = 0;
    std::vector<T>   rgb;        // row-major, top-down
    std::vector<T>   luminance;  // un-warped (m_luminance)
    T                norm = 0;
    Discrete<T>              sampleU;
    std::vector<Discrete<T>> sampleUV;

    static T lum(T r, T g, T b)  // numeric.cpp:62-66 (computed in double, stored as T)
    {
        return static_cast<T>(0.299 * r + 0.587 * g + 0.114 * b);
    }

    void build(const float* data, int w, int h)  // envmap.cpp:208-331
    {
        W = w;
        H = h;
        rgb.assign(data, data + static_cast<size_t>(W) * H * 3);
        int            M = H, N = W;
        std::vector<T> l(static_cast<size_t>(M) * N);
        for (size_t n = 0; n < l.size(); ++n) l[n] = lum(rgb[3 * n], rgb[3 * n + 1], rgb[3 * n + 2]);
        luminance = l;
        for (int m = 0; m < M; ++m)
        {
            T phi = K<T>::PI * (T(m) + T(0.5)) / T(M);
            for (int n = 0; n < N; ++n) l[n + static_cast<size_t>(m) * N] = T(l[n + static_cast<size_t>(m) * N] * dsin(phi));
        }
        T acc = 0;
        for (T v : l) acc += v;
        norm = T(1) / acc;
        std::vector<T> colsum(N);
        sampleUV.resize(N);
        std::vector<T> col(M);
        for (int n = 0; n < N; ++n)
        {
            T s = 0;
            for (int m = 0; m < M; ++m)
            {
                col[m] = l[n + static_cast<size_t>(m) * N];
                s += col[m];
            }
            colsum[n] = s;
            sampleUV[n].build(col);
        }
        sampleU.build(colsum);
    }

    static int clampi(int x, int a, int b) { return x < a ? a : x > b ? b : x; }
    static int toInt(T x) { return x != x ? 0 : static_cast<int>(std::max(T(-2e9), std::min(T(2e9), x))); }

    static T dirToTheta(const V3<T>& d)  // envmap.cpp:44-53
    {
        T theta = T(datan(d.z / d.x) + double(T(K<T>::PI / 2)));  // + M_PI_2 (constants.cpp:20)
        if (d.x < 0) theta += K<T>::PI;
        return theta;
    }
    T pdfAt(int ui, int vi) const
    {
        return norm * luminance[ui + static_cast<size_t>(vi) * W] * T(W) * T(H) / (T(2) * K<T>::PI * K<T>::PI);
    }
    // sample(r1, r2) with the two texel-jitter numbers made explicit (envmap.cpp:333-459)
    void sample(T r1, T r2, T j1, T j2, V3<T>& dir, V3<T>& rad, T& pdf) const
    {
        int ui0 = sampleU.sample(r1);
        int vi0 = sampleUV[ui0].sample(r2);
        T   u = (T(ui0) + j1) / T(W);
        T   v = (T(vi0) + j2) / T(H);
        int ui = clampi(toInt(u * T(W)), 0, W - 1);
        int vi = clampi(toInt(v * T(H)), 0, H - 1);
        size_t off = (ui + static_cast<size_t>(vi) * W) * 3;
        T phi = v * K<T>::PI;
        T theta = u * 2 * K<T>::PI;
        dir = V3<T>(T(dsin(phi) * dsin(theta)), T(dcos(phi)), T(dsin(phi) * -dcos(theta)));
        pdf = pdfAt(ui, vi);
        rad = V3<T>(rgb[off], rgb[off + 1], rgb[off + 2]);
    }
    void texel(const V3<T>& d, int& ui, int& vi) const
    {
        T phi = T(dacos(d.y));
        T theta = dirToTheta(d);
        ui = clampi(toInt(theta / (K<T>::PI * 2) * T(W)), 0, W - 1);
        vi = clampi(toInt(phi / K<T>::PI * T(H)), 0, H - 1);
    }
    T pdf(const V3<T>& d) const  // envmap.cpp:461-480
    {
        int ui, vi;
        texel(d, ui, vi);
        return pdfAt(ui, vi);
    }
    V3<T> radiance(const V3<T>& d) const  // envmap.cpp:494-506
    {
        int ui, vi;
        texel(d, ui, vi);
        size_t off = (ui + static_cast<size_t>(vi) * W) * 3;
        return V3<T>(rgb[off], rgb[off + 1], rgb[off + 2]);
    }
};

// ---------------------------------------------------------------------------
// geometry and the oracle's own BVH
// ---------------------------------------------------------------------------
template <class T>
struct Tri
{
    V3<T> a, b, c, na, nb, nc, n;
    V3<T> alpha = V3<T>(T(1), T(1), T(1));  // TriangleObject::m_vertex_alpha
    T     area;
    int   mat;
};

// TriangleObject::consistentNormal (triangle.cpp:149-182): np = normal(u, v); the
// reference's float constant 2 / NUM_PI (NUM_PI = float(pi))
template <class T>
V3<T> consistentNormalOf(const Tri<T>& t, const V3<T>& np, T u, T v, const V3<T>& wi, V3<T>* refl = nullptr,
                         T* cos_wi = nullptr)
{
    const T k = T(2.0f / 3.14159265358979323846f);
    T       alpha = (T(1) - u - v) * t.alpha.x + u * t.alpha.y + v * t.alpha.z;
    T       s = T(1) - k * alpha;
    T       q = (s * s) / (T(1) + T(2) * (T(1) - k) * alpha);
    T       b = dot(wi, np);
    T       g = T(1) + q * (b - T(1));
    T       rho = std::sqrt(q * (T(1) + g) / (T(1) + b));
    V3<T>   r = (g + rho * b) * np - rho * wi;
    if (refl) *refl = r;
    if (cos_wi) *cos_wi = std::sqrt((T(1) + (g + rho * b) * b - rho) * T(0.5));
    return normalize(wi + r);
}

struct Node
{
    float bmin[3], bmax[3];
    int   left, right;  // inner: children; leaf: left = first, right = -(count)
};

template <class T>
struct Hit
{
    T   t = std::numeric_limits<T>::infinity();
    T   u = 0, v = 0;
    int prim = -1;
};

// Moller-Trumbore exactly as triangle.cpp:13-51 with the absolute det cull
template <class T>
static inline bool mtIntersect(const V3<T>& orig, const V3<T>& dir, const V3<T>& v0, const V3<T>& v1,
                               const V3<T>& v2, T& t, T& u, T& v)
{
    V3<T> v0v1 = v1 - v0;
    V3<T> v0v2 = v2 - v0;
    V3<T> pvec = cross(dir, v0v2);
    T     det = dot(v0v1, pvec);
    if (std::fabs(det) < K<T>::EPS_DET) return false;
    T     invDet = T(1) / det;
    V3<T> tvec = orig - v0;
    u = dot(tvec, pvec) * invDet;
    if (u < 0 || u > 1) return false;
    V3<T> qvec = cross(tvec, v0v1);
    v = dot(dir, qvec) * invDet;
    if (v < 0 || u + v > 1) return false;
    t = dot(v0v2, qvec) * invDet;
    return true;
}

template <class T>
struct Scene
{
    std::vector<Tri<T>>      tris;
    std::vector<Material<T>> mats;
    std::vector<Node>        nodes;
    std::vector<int>         order;  // leaf-ordered primitive ids
    std::vector<int>         lights;  // emissive triangle ids
    std::vector<int>         lightOf;  // per prim: light index or -1
    Discrete<T>              lightSampler;
    T                        lightArea = 0;
    Envmap<T>                env;
    bool                     hasEnv = false;

    // binned SAH over centroids, leaf <= 4
    void buildBVH()
    {
        int n = static_cast<int>(tris.size());
        order.resize(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::vector<float> bb(static_cast<size_t>(n) * 6), cen(static_cast<size_t>(n) * 3);
        for (int i = 0; i < n; ++i)
        {
            const Tri<T>& t = tris[i];
            for (int k = 0; k < 3; ++k)
            {
                float a = static_cast<float>(t.a[k]), b = static_cast<float>(t.b[k]), c = static_cast<float>(t.c[k]);
                bb[6 * i + k] = std::min(a, std::min(b, c));
                bb[6 * i + 3 + k] = std::max(a, std::max(b, c));
                cen[3 * i + k] = 0.5f * (bb[6 * i + k] + bb[6 * i + 3 + k]);
            }
        }
        nodes.clear();
        nodes.reserve(2 * static_cast<size_t>(n) / 2 + 2);
        struct Item { int node, begin, end; };
        std::vector<Item> stack;
        nodes.push_back(Node());
        stack.push_back({0, 0, n});
        const int B = 16;
        while (!stack.empty())
        {
            Item it = stack.back();
            stack.pop_back();
            Node nd;
            for (int k = 0; k < 3; ++k)
            {
                nd.bmin[k] = std::numeric_limits<float>::infinity();
                nd.bmax[k] = -std::numeric_limits<float>::infinity();
            }
            float cmin[3] = {1e30f, 1e30f, 1e30f}, cmax[3] = {-1e30f, -1e30f, -1e30f};
            for (int i = it.begin; i < it.end; ++i)
            {
                int p = order[i];
                for (int k = 0; k < 3; ++k)
                {
                    nd.bmin[k] = std::min(nd.bmin[k], bb[6 * p + k]);
                    nd.bmax[k] = std::max(nd.bmax[k], bb[6 * p + 3 + k]);
                    cmin[k] = std::min(cmin[k], cen[3 * p + k]);
                    cmax[k] = std::max(cmax[k], cen[3 * p + k]);
                }
            }
            int count = it.end - it.begin;
            int bestAxis = -1, bestSplit = -1;
            if (count > 4)
            {
                double bestCost = std::numeric_limits<double>::infinity();
                for (int ax = 0; ax < 3; ++ax)
                {
                    float ext = cmax[ax] - cmin[ax];
                    if (!(ext > 0)) continue;
                    int   cnt[B] = {0};
                    float lo[B][3], hi[B][3];
                    for (int b = 0; b < B; ++b)
                        for (int k = 0; k < 3; ++k)
                        {
                            lo[b][k] = 1e30f;
                            hi[b][k] = -1e30f;
                        }
                    for (int i = it.begin; i < it.end; ++i)
                    {
                        int p = order[i];
                        int b = std::min(B - 1, static_cast<int>((cen[3 * p + ax] - cmin[ax]) / ext * B));
                        cnt[b]++;
                        for (int k = 0; k < 3; ++k)
                        {
                            lo[b][k] = std::min(lo[b][k], bb[6 * p + k]);
                            hi[b][k] = std::max(hi[b][k], bb[6 * p + 3 + k]);
                        }
                    }
                    double rightArea[B];
                    int    rightCnt[B];
                    float  rl[3] = {1e30f, 1e30f, 1e30f}, rh[3] = {-1e30f, -1e30f, -1e30f};
                    int    rc = 0;
                    for (int b = B - 1; b > 0; --b)
                    {
                        rc += cnt[b];
                        for (int k = 0; k < 3; ++k)
                        {
                            rl[k] = std::min(rl[k], lo[b][k]);
                            rh[k] = std::max(rh[k], hi[b][k]);
                        }
                        double dx = rh[0] - rl[0], dy = rh[1] - rl[1], dz = rh[2] - rl[2];
                        rightArea[b] = rc ? dx * dy + dy * dz + dz * dx : 0;
                        rightCnt[b] = rc;
                    }
                    float ll[3] = {1e30f, 1e30f, 1e30f}, lh[3] = {-1e30f, -1e30f, -1e30f};
                    int   lc = 0;
                    for (int b = 0; b < B - 1; ++b)
                    {
                        lc += cnt[b];
                        for (int k = 0; k < 3; ++k)
                        {
                            ll[k] = std::min(ll[k], lo[b][k]);
                            lh[k] = std::max(lh[k], hi[b][k]);
                        }
                        if (lc == 0 || rightCnt[b + 1] == 0) continue;
                        double dx = lh[0] - ll[0], dy = lh[1] - ll[1], dz = lh[2] - ll[2];
                        double cost = (dx * dy + dy * dz + dz * dx) * lc + rightArea[b + 1] * rightCnt[b + 1];
                        if (cost < bestCost)
                        {
                            bestCost = cost;
                            bestAxis = ax;
                            bestSplit = b;
                        }
                    }
                }
            }
            if (count <= 4 || bestAxis < 0)
            {
                if (count > 4)
                {
                    // degenerate centroids: median split on index order
                    int mid = (it.begin + it.end) / 2;
                    nd.left = static_cast<int>(nodes.size());
                    nd.right = nd.left + 1;
                    nodes.push_back(Node());
                    nodes.push_back(Node());
                    nodes[it.node] = nd;
                    stack.push_back({nd.left, it.begin, mid});
                    stack.push_back({nd.right, mid, it.end});
                    continue;
                }
                nd.left = it.begin;
                nd.right = -count;
                nodes[it.node] = nd;
                continue;
            }
            float ext = cmax[bestAxis] - cmin[bestAxis];
            int*  mid = std::partition(order.data() + it.begin, order.data() + it.end, [&](int p) {
                int b = std::min(B - 1, static_cast<int>((cen[3 * p + bestAxis] - cmin[bestAxis]) / ext * B));
                return b <= bestSplit;
            });
            int m = static_cast<int>(mid - order.data());
            nd.left = static_cast<int>(nodes.size());
            nd.right = nd.left + 1;
            nodes.push_back(Node());
            nodes.push_back(Node());
            nodes[it.node] = nd;
            stack.push_back({nd.left, it.begin, m});
            stack.push_back({nd.right, m, it.end});
        }
    }

    // conservative slab test (bounds widened by a few ulp, Ize 2013); entry distance in tnear
    static bool boxHit(const Node& nd, const V3<T>& o, const V3<T>& inv, T tmin, T tmax, T* tnear = nullptr)
    {
        T t0 = tmin, t1 = tmax;
        for (int k = 0; k < 3; ++k)
        {
            T lo = (T(nd.bmin[k]) - o[k]) * inv[k];
            T hi = (T(nd.bmax[k]) - o[k]) * inv[k];
            if (lo > hi) std::swap(lo, hi);
            if (lo != lo) lo = -std::numeric_limits<T>::infinity();
            if (hi != hi) hi = std::numeric_limits<T>::infinity();
            hi *= T(1) + T(8) * std::numeric_limits<T>::epsilon();
            t0 = lo > t0 ? lo : t0;
            t1 = hi < t1 ? hi : t1;
            if (t0 > t1) return false;
        }
        if (tnear) *tnear = t0;
        return true;
    }

    Hit<T> trace(const V3<T>& o, const V3<T>& d, T tmin, T tmax, bool any) const
    {
        if (!rtInfo.empty()) return traceRefTree(o, d, tmin, tmax, any);
        Hit<T> h;
        if (nodes.empty()) return h;
        V3<T> inv(d.x != 0 ? T(1) / d.x : std::numeric_limits<T>::infinity(),
                  d.y != 0 ? T(1) / d.y : std::numeric_limits<T>::infinity(),
                  d.z != 0 ? T(1) / d.z : std::numeric_limits<T>::infinity());
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        T best = tmax;
        while (sp)
        {
            const Node& nd = nodes[stack[--sp]];
            if (!boxHit(nd, o, inv, tmin, best)) continue;
            if (nd.right < 0)
            {
                for (int i = nd.left; i < nd.left - nd.right; ++i)
                {
                    int           p = order[i];
                    const Tri<T>& tr = tris[p];
                    T             t, u, v;
                    if (mtIntersect(o, d, tr.a, tr.b, tr.c, t, u, v) && t > tmin && t < best)
                    {
                        best = t;
                        h.t = t;
                        h.u = u;
                        h.v = v;
                        h.prim = p;
                        if (any) return h;
                    }
                }
            }
            else
            {
                // front-to-back: push the farther child first (results do not depend on it)
                T    tl = 0, tr = 0;
                bool hl = boxHit(nodes[nd.left], o, inv, tmin, best, &tl);
                bool hr = boxHit(nodes[nd.right], o, inv, tmin, best, &tr);
                if (hl && hr)
                {
                    if (tl <= tr)
                    {
                        stack[sp++] = nd.right;
                        stack[sp++] = nd.left;
                    }
                    else
                    {
                        stack[sp++] = nd.left;
                        stack[sp++] = nd.right;
                    }
                }
                else if (hl)
                    stack[sp++] = nd.left;
                else if (hr)
                    stack[sp++] = nd.right;
            }
        }
        return h;
    }

    // Optional reference tree (e.g. the reference SplitBVH dumped node by node); when
    // present, trace() follows SplitBVH::intersect exactly (splitbvh.cpp:5-145): a node's
    // own box is tested at visit time against the current tmax with rayAABBOverlap
    // (aabb.cpp:66-131, inv_dir = 0 for zero components, ray.cpp:39-42), leaf references
    // are culled by their clipped bounds, children left-first iff dir[axis] > 0.
    std::vector<float> rtBox;   // 6 per node
    std::vector<int>   rtInfo;  // 6 per node: is_leaf, left, right, axis, ref_begin, ref_count
    std::vector<int>   rtPrim;
    std::vector<float> rtRefBox;  // 6 per reference

    static bool refOverlap(const float* b, const V3<T>& o, const V3<T>& inv, const int* sgn, T rtmin, T rtmax)
    {
        T tmin = (T(b[sgn[0] ? 3 : 0]) - o.x) * inv.x;
        T tymin = (T(b[sgn[1] ? 4 : 1]) - o.y) * inv.y;
        T tmax = (T(b[sgn[0] ? 0 : 3]) - o.x) * inv.x;
        T tymax = (T(b[sgn[1] ? 1 : 4]) - o.y) * inv.y;
        if ((tmin > tymax) || (tymin > tmax)) return false;
        if (tymin > tmin) tmin = tymin;
        if (tmin > rtmax) return false;
        if (tymax < tmax) tmax = tymax;
        if (tmax < rtmin) return false;
        T tzmin = (T(b[sgn[2] ? 5 : 2]) - o.z) * inv.z;
        T tzmax = (T(b[sgn[2] ? 2 : 5]) - o.z) * inv.z;
        if ((tmin > tzmax) || (tzmin > tmax)) return false;
        if (tzmin > tmin) tmin = tzmin;
        if (tmin > rtmax) return false;
        if (tzmax < tmax) tmax = tzmax;
        if (tmax < rtmin) return false;
        return true;
    }

    Hit<T> traceRefTree(const V3<T>& o, const V3<T>& d, T tmin, T tmax, bool any) const
    {
        Hit<T> h;
        V3<T>  inv(d.x == 0 ? T(0) : T(1) / d.x, d.y == 0 ? T(0) : T(1) / d.y, d.z == 0 ? T(0) : T(1) / d.z);
        int    sgn[3] = {d.x < 0, d.y < 0, d.z < 0};
        int    stack[256];
        int    sp = 0;
        stack[sp++] = 0;
        while (sp)
        {
            int        n = stack[--sp];
            const int* in = &rtInfo[6 * n];
            if (!refOverlap(&rtBox[6 * n], o, inv, sgn, tmin, tmax)) continue;
            if (in[0])
            {
                for (int k = 0; k < in[5]; ++k)
                {
                    int r = in[4] + k;
                    if (!refOverlap(&rtRefBox[6 * r], o, inv, sgn, tmin, tmax)) continue;
                    const Tri<T>& tr = tris[rtPrim[r]];
                    T             t, u, v;
                    if (mtIntersect(o, d, tr.a, tr.b, tr.c, t, u, v) && t > tmin && t < tmax)
                    {
                        tmax = t;
                        h.t = t;
                        h.u = u;
                        h.v = v;
                        h.prim = rtPrim[r];
                        if (any) return h;
                    }
                }
            }
            else if (sp + 2 <= 256)
            {
                bool leftFirst = d[in[3]] > 0;
                stack[sp++] = leftFirst ? in[2] : in[1];
                stack[sp++] = leftFirst ? in[1] : in[2];
            }
        }
        return h;
    }

    V3<T> shadingNormal(int p, T u, T v) const  // triangle.cpp:90-93
    {
        const Tri<T>& t = tris[p];
        return normalize((T(1) - u - v) * t.na + u * t.nb + v * t.nc);
    }

    V3<T> consistentNormal(int p, T u, T v, const V3<T>& wi) const
    {
        return consistentNormalOf(tris[p], shadingNormal(p, u, v), u, v, wi);
    }
};

// ---------------------------------------------------------------------------
// camera (camera.cpp:9-43)
// ---------------------------------------------------------------------------
template <class T>
struct Camera
{
    V3<T> origin, fx, fy, fwd;
    T     ww, wh, dist;
    Camera(const float* c /* origin3 target3 up3 fov */, int w, int h)
    {
        origin = ld3<T>(c);
        V3<T> target = ld3<T>(c + 3), up = ld3<T>(c + 6);
        T     fov = T(c[9]);
        ww = T(w) / T(h);
        wh = T(1);
        T rad = fov * T(0.5) / T(180) * K<T>::PI;  // toRadians(fov_y * 0.5f)
        dist = T(wh / (T(2) * dtan(rad)));
        fwd = normalize(target - origin);
        fx = normalize(cross(fwd, up));
        fy = cross(fx, fwd);
    }
    void makeRay(T mx, T my, V3<T>& o, V3<T>& d) const
    {
        V3<T> su = fx * (mx - T(0.5)) * ww;
        V3<T> sv = fy * (my - T(0.5)) * wh;
        V3<T> sw = fwd * dist;
        o = origin;
        d = normalize(su + sv + sw);
    }
};

// ---------------------------------------------------------------------------
// the integrator: rayTrace (demo_pt.cpp:512-655) with the named extensions
// ---------------------------------------------------------------------------
struct RenderParams
{
    int      width, height, spp, max_depth, rr_depth;
    uint64_t seed;
    int      ref_stream;  // 0: per-path PCG32; 1/2: the reference stream, call arguments
                          // evaluated right-to-left (GCC on x86-64 / aarch64) / left-to-right
};

template <class T>
struct PathLog  // per scattering vertex: what the adjoint needs
{
    int   param;
    V3<T> albedo;
    V3<T> before;
};

template <class T>
struct PathOut
{
    V3<T>     L;
    long long rays = 0;
    long long ext = 0;  // of which extension rays
};

// dL: adjoint seed for this path (dLoss/dI_px / spp); grads accumulate when non-null
template <class T>
PathOut<T> tracePath(const Scene<T>& sc, const V3<T>& o0, const V3<T>& d0, Pcg32& rng, const RenderParams& rp,
                     const V3<T>* dL, std::vector<double>* g_albedo, std::vector<double>* g_emis,
                     RefStream* rs = nullptr)
{
    const T eps = K<T>::EPS_RAY;
    const T inf = std::numeric_limits<T>::infinity();
    PathOut<T> out;
    V3<T>      L(T(0)), thr(T(1));
    V3<T>      ro = o0, rd = d0;
    bool       lastNee = false;
    PathLog<T> log[64];
    int        nlog = 0;
    auto emisGrad = [&](int mat, const V3<T>& coef) {
        if (!dL || !g_emis) return;
        int p = sc.mats[mat].emission_param;
        if (p < 0) return;
        (*g_emis)[3 * p + 0] += double(dL->x * coef.x);
        (*g_emis)[3 * p + 1] += double(dL->y * coef.y);
        (*g_emis)[3 * p + 2] += double(dL->z * coef.z);
    };

    for (int n = 0; n <= rp.max_depth; ++n)
    {
        Hit<T> hit = sc.trace(ro, rd, eps, inf, false);
        out.rays++;
        out.ext++;
        if (g_ray_log_on)
        {
            double rec[10] = {double(g_cur_path), double(n), double(ro.x), double(ro.y), double(ro.z),
                              double(rd.x), double(rd.y), double(rd.z), double(hit.prim), double(hit.t)};
            g_ray_log.insert(g_ray_log.end(), rec, rec + 10);
        }
        bool no_direct = n == 0 || !lastNee;
        if (hit.prim < 0)
        {
            if (no_direct && sc.hasEnv) L += thr * sc.env.radiance(rd);
            break;
        }
        const Tri<T>&      tri = sc.tris[hit.prim];
        const Material<T>& mat = sc.mats[tri.mat];
        V3<T>              phit = ro + rd * hit.t;
        V3<T>              nhit = sc.shadingNormal(hit.prim, hit.u, hit.v);
        if (mat.consistent) nhit = sc.consistentNormal(hit.prim, hit.u, hit.v, -rd);
        if (mat.type == LGHT)
        {
            if (no_direct && dot(rd, nhit) < 0)
            {
                L += thr * mat.color;
                emisGrad(tri.mat, thr);
            }
            break;
        }
        T u[NUM_DIMS];
        if (rs)
        {
            // the reference's draw order at this vertex (demo_pt.cpp:562-650): a pair passed
            // as two call arguments f(randf(), randf()) is drawn in argument-evaluation order
            for (int k = 0; k < NUM_DIMS; ++k) u[k] = T(0);
            auto pair = [&](int a, int b) {
                if (rp.ref_stream == 1)
                {
                    u[b] = T(rs->next());
                    u[a] = T(rs->next());
                }
                else
                {
                    u[a] = T(rs->next());
                    u[b] = T(rs->next());
                }
            };
            if (mat.type == DIFF)
            {
                if (sc.hasEnv)
                {
                    pair(D_ENV_LIGHT_0, D_ENV_LIGHT_1);       // envmap()->sample(randf(), randf())
                    u[D_ENV_JITTER_U] = T(rs->next());        // sampleByPdf (envmap.cpp:410-411)
                    u[D_ENV_JITTER_V] = T(rs->next());
                    u[D_ENV_BSDF_0] = T(rs->next());          // r1 = 2 pi randf(), r2 = randf()
                    u[D_ENV_BSDF_1] = T(rs->next());
                }
                if (sc.lightArea > 0)
                {
                    pair(D_AREA_BSDF_0, D_AREA_BSDF_1);       // mat.sample(..., randf(), randf(), ...)
                    u[D_LIGHT_PICK] = T(rs->next());          // DiscreteSampler::sample()
                    u[D_LIGHT_U] = T(rs->next());             // samplePoint: sqrt(randf()), randf()
                    u[D_LIGHT_V] = T(rs->next());
                }
            }
            pair(D_CONT_0, D_CONT_1);                         // continuation sample
            u[D_RR] = T(0);
        }
        else
        {
            for (int k = 0; k < NUM_DIMS; ++k) u[k] = T(rng.uniform());
        }
        V3<T> local(T(0));
        V3<T> wi = -rd;
        lastNee = doesNee(mat.type);
        V3<T> before = L;
        if (lastNee)
        {
            if (sc.hasEnv)
            {
                // sampleEnvmapUsingLightPDF (demo_pt.cpp:430-465)
                V3<T> irrL(T(0));
                T     pdfL = 1;
                V3<T> dirL(T(0));
                {
                    V3<T> ldir, lrad;
                    T     lpdf;
                    sc.env.sample(u[D_ENV_LIGHT_0], u[D_ENV_LIGHT_1], u[D_ENV_JITTER_U], u[D_ENV_JITTER_V], ldir, lrad,
                                  lpdf);
                    T g = fmaxr(T(0), dot(ldir, nhit));
                    if (g > 0)
                    {
                        out.rays++;
                        if (sc.trace(phit, ldir, eps, inf, true).prim < 0)
                        {
                            pdfL = sc.env.pdf(ldir);
                            dirL = ldir;
                            irrL += (bsdfEval(mat, wi, nhit, ldir) * g / lpdf) * lrad;
                        }
                    }
                    if (isnan3(irrL)) irrL = V3<T>(T(0));
                }
                // sampleEnvmapUsingSurfacePDF (demo_pt.cpp:466-507); GGX uses its own sampler
                V3<T> irrB(T(0));
                T     pdfB = 1;
                V3<T> dirB(T(0));
                if (mat.type == DIFF)
                {
                    T     r1 = 2 * K<T>::PI * u[D_ENV_BSDF_0], r2 = u[D_ENV_BSDF_1], r2s = std::sqrt(r2);
                    V3<T> w = nhit, uu = normalize(cross(V3<T>(T(0.3f), T(0.4f), T(0.5f)), w)), vv = cross(w, uu);
                    V3<T> wo = normalize(uu * T(dcos(r1) * r2s) + vv * T(dsin(r1) * r2s) + w * std::sqrt(1 - r2));
                    T     g = fmaxr(T(0), dot(wo, nhit));
                    if (g > 0)
                    {
                        out.rays++;
                        if (sc.trace(phit, wo, eps, inf, true).prim < 0)
                        {
                            pdfB = bsdfPdf(mat, wi, nhit, wo);
                            dirB = wo;
                            irrB += sc.env.radiance(wo);
                        }
                    }
                    if (isnan3(irrB)) irrB = V3<T>(T(0));
                    irrB = mat.color * irrB;
                }
                else
                {
                    BsdfSample<T> bs = bsdfSample(mat, wi, nhit, u[D_ENV_BSDF_0], u[D_ENV_BSDF_1]);
                    if (maxComponent(bs.weight) > 0 && bs.pdf > 0)
                    {
                        out.rays++;
                        if (sc.trace(phit, bs.wo, eps, inf, true).prim < 0)
                        {
                            pdfB = bs.pdf;
                            dirB = bs.wo;
                            irrB += bs.weight * sc.env.radiance(bs.wo);
                        }
                    }
                    if (isnan3(irrB)) irrB = V3<T>(T(0));
                }
                T wEnv = pdfL / (pdfL + bsdfPdf(mat, wi, nhit, dirL));
                T wBsdf = pdfB / (pdfB + sc.env.pdf(dirB));
                local += irrL * wEnv + irrB * wBsdf;
            }
            if (sc.lightArea > 0)
            {
                // BSDF sampling with MIS (demo_pt.cpp:593-614)
                BsdfSample<T> bs = bsdfSample(mat, wi, nhit, u[D_AREA_BSDF_0], u[D_AREA_BSDF_1]);
                if (maxComponent(bs.weight) > 0)
                {
                    out.rays++;
                    Hit<T> lh = sc.trace(phit, bs.wo, eps, inf, false);
                    if (lh.prim >= 0 && sc.mats[sc.tris[lh.prim].mat].type == LGHT)
                    {
                        V3<T> ln = sc.shadingNormal(lh.prim, lh.u, lh.v);
                        T     cl = dot(ln, -bs.wo);
                        T     pdfLight = 0;  // Scene::lightPdfW (scene.cpp:239-267)
                        if (cl >= T(1e-6f))
                        {
                            int li = sc.lightOf[lh.prim];
                            T   pdfA = (T(1) / sc.tris[lh.prim].area) * sc.lightSampler.pdf[li];
                            pdfLight = pdfA * (lh.t * lh.t) / cl;
                        }
                        if (!(dot(ln, -bs.wo) < 0))  // Scene::lightRadiance (scene.cpp:345-366)
                        {
                            T     mis = bs.pdf / (bs.pdf + pdfLight);
                            const Material<T>& lm = sc.mats[sc.tris[lh.prim].mat];
                            local += bs.weight * lm.color * mis;
                            emisGrad(sc.tris[lh.prim].mat, thr * bs.weight * mis);
                        }
                    }
                }
                // light sampling (demo_pt.cpp:618-641, scene.cpp:298-343)
                int           li = sc.lightSampler.sample(u[D_LIGHT_PICK]);
                const Tri<T>& lt = sc.tris[sc.lights[li]];
                T             r0 = std::sqrt(u[D_LIGHT_U]);
                T             lu = T(1) - r0;
                T             lv = u[D_LIGHT_V] * r0;
                V3<T>         lp = lt.a * (T(1) - lu - lv) + lt.b * lu + lt.c * lv;
                V3<T>         ln = normalize((T(1) - lu - lv) * lt.na + lu * lt.nb + lv * lt.nc);
                T             pdfA = (T(1) / lt.area) * sc.lightSampler.pdf[li];
                V3<T>         wo = lp - phit;
                T             dist2 = lengthSquared(wo);
                wo = normalize(wo);
                T cosl = dot(ln, -wo);
                // __pdfAtoW (geometry.cpp:222-225): its unqualified fabs(float) is the C
                // library's double fabs(double), so the division runs in double
                T pdfW = T(double(pdfA * dist2) / double(std::fabs(cosl)));
                if (cosl <= 0) pdfW = 0;
                if (pdfW > 0)
                {
                    T     pdfB = bsdfPdf(mat, wi, nhit, wo);
                    T     mis = pdfW / (pdfW + pdfB);
                    V3<T> f = bsdfEval(mat, wi, nhit, wo);
                    T     cosS = std::max(dot(nhit, wo), T(0));
                    if (maxComponent(f) > 0 && cosS > 0)
                    {
                        out.rays++;
                        // closest hit bounded just past the sampled point: same answer as the
                        // reference's unbounded query for the light-id test
                        Hit<T> lh = sc.trace(phit, wo, eps, std::sqrt(dist2) * T(1.001) + eps, false);
                        if (lh.prim >= 0 && sc.lightOf[lh.prim] == li &&
                            !(dot(sc.shadingNormal(lh.prim, lh.u, lh.v), -wo) < 0))
                        {
                            const Material<T>& lm = sc.mats[lt.mat];
                            local += f * lm.color * (cosS / pdfW * mis);
                            emisGrad(lt.mat, thr * f * (cosS / pdfW * mis));
                        }
                    }
                }
            }
        }
        L += thr * local;
        if (mat.type == DIFF && mat.albedo_param >= 0 && nlog < 64)
        {
            log[nlog].param = mat.albedo_param;
            log[nlog].albedo = mat.color;
            log[nlog].before = before;
            nlog++;
        }
        // continuation (demo_pt.cpp:647-650)
        BsdfSample<T> cs = bsdfSample(mat, wi, nhit, u[D_CONT_0], u[D_CONT_1]);
        thr *= cs.weight;
        ro = phit;
        rd = cs.wo;
        if (rp.rr_depth >= 0 && n >= rp.rr_depth)
        {
            T q = std::min(std::max(maxComponent(mat.color), T(0)), T(1));
            if (u[D_RR] >= q) break;
            thr = thr * (T(1) / q);
        }
        if (maxComponent(thr) <= T(0)) break;
    }
    if (isnan3(L)) L = V3<T>(T(0));
    out.L = L;
    if (dL && g_albedo)
    {
        for (int k = 0; k < nlog; ++k)
        {
            V3<T> S = L - log[k].before;
            for (int c = 0; c < 3; ++c)
            {
                T a = log[k].albedo[c];
                if (a > T(0)) (*g_albedo)[3 * log[k].param + c] += double((*dL)[c] * S[c] / a);
            }
        }
    }
    return out;
}

// reference-stream mode: stream position after each path (debugging the replay)
static long long* g_draw_log = nullptr;


template <class T>
struct RenderJob
{
    const Scene<T>*  sc;
    const Camera<T>* cam;
    RenderParams     rp;
    double*          sum;
    double*          sumsq;
    float*           paths;
    const float*     dLdI;
    int              n_albedo, n_emis;
};

template <class T>
long long renderRows(const RenderJob<T>& job, int row_begin, int row_end, int nthreads, std::vector<double>* ga,
                     std::vector<double>* ge)
{
    std::atomic<int>       next(row_begin);
    std::atomic<long long> rays(0);
    int                    nt = std::max(1, nthreads);
    RefStream              stream;
    RefStream*             rs = job.rp.ref_stream ? &stream : nullptr;
    if (rs) nt = 1;  // one global stream, consumed in the reference's pixel order
    std::vector<std::vector<double>> tga(nt), tge(nt);
    auto worker = [&](int tid) {
        long long myrays = 0, myext = 0;
        std::vector<double>* pa = nullptr;
        std::vector<double>* pe = nullptr;
        if (ga)
        {
            tga[tid].assign(ga->size(), 0.0);
            tge[tid].assign(ge->size(), 0.0);
            pa = &tga[tid];
            pe = &tge[tid];
        }
        const RenderParams& rp = job.rp;
        for (;;)
        {
            int y = next.fetch_add(1);
            if (y >= row_end) break;
            for (int x = 0; x < rp.width; ++x)
            {
                uint32_t pix = static_cast<uint32_t>(y) * rp.width + x;
                double   s[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
                V3<T>    dl;
                if (job.dLdI)
                    dl = V3<T>(T(job.dLdI[3 * pix]), T(job.dLdI[3 * pix + 1]), T(job.dLdI[3 * pix + 2])) *
                         (T(1) / T(rp.spp));
                for (int si = 0; si < rp.spp; ++si)
                {
                    Pcg32 rng;
                    rng.seed(rp.seed, pix, static_cast<uint32_t>(si));
                    T r1, r2;
                    if (rs)
                    {
                        r1 = rp.spp > 1 ? T(2) * T(rs->next()) : T(0);
                        r2 = rp.spp > 1 ? T(2) * T(rs->next()) : T(0);
                    }
                    else
                    {
                        r1 = T(2) * T(rng.uniform());
                        r2 = T(2) * T(rng.uniform());
                    }
                    T dx = 0, dy = 0;
                    if (rp.spp > 1)  // tent filter (demo_pt.cpp:689-697)
                    {
                        dx = r1 < 1 ? std::sqrt(r1) - 1 : 1 - std::sqrt(2 - r1);
                        dy = r2 < 1 ? std::sqrt(r2) - 1 : 1 - std::sqrt(2 - r2);
                    }
                    V3<T> o, d;
                    job.cam->makeRay((T(x) + T(0.5) + dx) / T(rp.width), (T(y) + T(0.5) + dy) / T(rp.height), o, d);
                    g_cur_path = static_cast<long long>(pix) * rp.spp + si;
                    PathOut<T> po = tracePath(*job.sc, o, d, rng, rp, job.dLdI ? &dl : nullptr, pa, pe, rs);
                    myrays += po.rays;
                    myext += po.ext;
                    V3<T> v(fmaxr(T(0), po.L.x), fmaxr(T(0), po.L.y), fmaxr(T(0), po.L.z));
                    for (int c = 0; c < 3; ++c)
                    {
                        s[c] += double(v[c]);
                        s2[c] += double(v[c]) * double(v[c]);
                    }
                    if (rs && g_draw_log) g_draw_log[static_cast<size_t>(pix) * rp.spp + si] = rs->count;
                    if (job.paths)
                    {
                        float* pp = job.paths + 3 * (static_cast<size_t>(pix) * rp.spp + si);
                        pp[0] = float(v.x);
                        pp[1] = float(v.y);
                        pp[2] = float(v.z);
                    }
                }
                for (int c = 0; c < 3; ++c)
                {
                    if (job.sum) job.sum[3 * pix + c] = s[c];
                    if (job.sumsq) job.sumsq[3 * pix + c] = s2[c];
                }
            }
        }
        rays += myrays;
        g_ext_rays += myext;
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker, i);
    worker(0);
    for (auto& t : th) t.join();
    if (ga)
    {
        for (int t = 0; t < nt; ++t)
        {
            for (size_t k = 0; k < ga->size(); ++k) (*ga)[k] += tga[t][k];
            for (size_t k = 0; k < ge->size(); ++k) (*ge)[k] += tge[t][k];
        }
    }
    return rays.load();
}

struct SceneAny
{
    int                            precision;
    std::unique_ptr<Scene<float>>  f;
    std::unique_ptr<Scene<double>> d;
};

template <class T>
void fillScene(Scene<T>& sc, const float* verts, const float* normals, const int* mat_ids, int n_tris,
               const int* mat_types, const float* mat_params, int n_mats, const float* env_rgb, int env_w,
               int env_h)
{
    sc.mats.resize(n_mats);
    for (int m = 0; m < n_mats; ++m)
    {
        const float* p = mat_params + 8 * m;  // color3, roughness, ior, albedo_param, emission_param, pad
        sc.mats[m].type = mat_types[m] & 0xff;
        sc.mats[m].consistent = (mat_types[m] & 0x100) != 0;
        sc.mats[m].color = ld3<T>(p);
        sc.mats[m].roughness = T(p[3]);
        sc.mats[m].ior = T(p[4]);
        sc.mats[m].albedo_param = static_cast<int>(p[5]);
        sc.mats[m].emission_param = static_cast<int>(p[6]);
    }
    sc.tris.resize(n_tris);
    sc.lightOf.assign(n_tris, -1);
    for (int i = 0; i < n_tris; ++i)
    {
        Tri<T>& t = sc.tris[i];
        t.a = ld3<T>(verts + 9 * i);
        t.b = ld3<T>(verts + 9 * i + 3);
        t.c = ld3<T>(verts + 9 * i + 6);
        t.n = normalize(cross(t.a - t.c, t.b - t.c));  // triangle.cpp:71
        if (normals)
        {
            t.na = ld3<T>(normals + 9 * i);
            t.nb = ld3<T>(normals + 9 * i + 3);
            t.nc = ld3<T>(normals + 9 * i + 6);
        }
        else
        {
            t.na = t.nb = t.nc = t.n;
        }
        t.area = length(cross(t.b - t.a, t.c - t.a)) * T(0.5);  // triangle.cpp:129-132
        t.mat = mat_ids[i];
        if (sc.mats[t.mat].type == LGHT)
        {
            sc.lightOf[i] = static_cast<int>(sc.lights.size());
            sc.lights.push_back(i);
        }
    }
    std::vector<T> areas;
    T              la = 0;
    for (int li : sc.lights)
    {
        areas.push_back(sc.tris[li].area);
        la += sc.tris[li].area;
    }
    sc.lightArea = la;
    if (!areas.empty()) sc.lightSampler.build(areas);
    if (env_rgb && env_w > 0 && env_h > 0)
    {
        sc.env.build(env_rgb, env_w, env_h);
        sc.hasEnv = true;
    }
    sc.buildBVH();
}

}  // namespace orc

using namespace orc;

extern "C" {

// mat_params: 8 floats per material {r, g, b, roughness, ior, albedo_param, emission_param, 0}
void* orc_scene_create(int precision, const float* verts, const float* normals, const int* mat_ids, int n_tris,
                       const int* mat_types, const float* mat_params, int n_mats, const float* env_rgb, int env_w,
                       int env_h)
{
    SceneAny* s = new SceneAny;
    s->precision = precision;
    if (precision == 64)
    {
        s->d.reset(new Scene<double>);
        fillScene(*s->d, verts, normals, mat_ids, n_tris, mat_types, mat_params, n_mats, env_rgb, env_w, env_h);
    }
    else
    {
        s->f.reset(new Scene<float>);
        fillScene(*s->f, verts, normals, mat_ids, n_tris, mat_types, mat_params, n_mats, env_rgb, env_w, env_h);
    }
    return s;
}

void orc_scene_destroy(void* h) { delete static_cast<SceneAny*>(h); }

// per-corner consistent-normal alphas, [n_tris][3]
void orc_scene_set_alpha(void* h, const float* alpha)
{
    SceneAny* s = static_cast<SceneAny*>(h);
    if (s->precision == 64)
        for (size_t i = 0; i < s->d->tris.size(); ++i) s->d->tris[i].alpha = ld3<double>(alpha + 3 * i);
    else
        for (size_t i = 0; i < s->f->tris.size(); ++i) s->f->tris[i].alpha = ld3<float>(alpha + 3 * i);
}

// TriangleObject::consistentNormal of one triangle (float): out = normal, reflection, cos
void orc_consistent_normal(const float* abc, const float* nabc, const float* alpha3, const float* wi, float u,
                           float v, float* out)
{
    Tri<float> t;
    t.a = ld3<float>(abc);
    t.b = ld3<float>(abc + 3);
    t.c = ld3<float>(abc + 6);
    t.na = ld3<float>(nabc);
    t.nb = ld3<float>(nabc + 3);
    t.nc = ld3<float>(nabc + 6);
    t.alpha = ld3<float>(alpha3);
    const V3<float> np = normalize((1.0f - u - v) * t.na + u * t.nb + v * t.nc);
    V3<float>       r;
    float           c = 0.f;
    const V3<float> n = consistentNormalOf(t, np, u, v, ld3<float>(wi), &r, &c);
    out[0] = n.x, out[1] = n.y, out[2] = n.z, out[3] = r.x, out[4] = r.y, out[5] = r.z, out[6] = c;
}

}  // extern "C"

template <class T>
static void setTree(Scene<T>& sc, const float* nb, const int* ni, int nn, const int* rp, const float* rb, int nr)
{
    sc.rtBox.assign(nb, nb + 6 * static_cast<size_t>(nn));
    sc.rtInfo.assign(ni, ni + 6 * static_cast<size_t>(nn));
    sc.rtPrim.assign(rp, rp + nr);
    sc.rtRefBox.assign(rb, rb + 6 * static_cast<size_t>(nr));
}

extern "C" {

// traverse the given binary tree with the reference's semantics from now on
void orc_scene_set_tree(void* h, const float* node_box, const int* node_info, int n_nodes, const int* ref_prim,
                        const float* ref_box, int n_refs)
{
    SceneAny* s = static_cast<SceneAny*>(h);
    if (s->precision == 64)
        setTree(*s->d, node_box, node_info, n_nodes, ref_prim, ref_box, n_refs);
    else
        setTree(*s->f, node_box, node_info, n_nodes, ref_prim, ref_box, n_refs);
}

}  // extern "C"

template <class T>
static long long renderT(const Scene<T>& sc, const float* cam, const int* ip, uint64_t seed, int row_begin,
                         int row_end, int nthreads, double* sum, double* sumsq, float* paths, const float* dLdI,
                         int n_albedo, double* g_albedo, int n_emis, double* g_emis)
{
    RenderParams rp{ip[0], ip[1], ip[2], ip[3], ip[4], seed, ip[5]};
    Camera<T>    c(cam, rp.width, rp.height);
    RenderJob<T> job{&sc, &c, rp, sum, sumsq, paths, dLdI, n_albedo, n_emis};
    if (dLdI)
    {
        std::vector<double> ga(3 * static_cast<size_t>(std::max(n_albedo, 0)), 0.0),
            ge(3 * static_cast<size_t>(std::max(n_emis, 0)), 0.0);
        long long r = renderRows(job, row_begin, row_end, nthreads, &ga, &ge);
        for (size_t k = 0; k < ga.size(); ++k) g_albedo[k] += ga[k];
        for (size_t k = 0; k < ge.size(); ++k) g_emis[k] += ge[k];
        return r;
    }
    return renderRows(job, row_begin, row_end, nthreads, nullptr, nullptr);
}

extern "C" {

// cam: origin3 target3 up3 fov_y; ip: width, height, spp, max_depth, rr_depth (-1 = off),
// ref_stream (0: per-path PCG32; 1/2: the reference's global stream, single-threaded).
// Writes per-pixel sums (and sums of squares) of the clamped per-sample radiance over
// rows [row_begin, row_end); paths (optional) receives every sample's radiance.
// With dLdI non-null it also runs the path-replay adjoint and accumulates gradients.
long long orc_render(void* h, const float* cam, const int* ip, unsigned long long seed, int row_begin, int row_end,
                     int nthreads, double* sum, double* sumsq, float* paths, const float* dLdI, int n_albedo,
                     double* g_albedo, int n_emis, double* g_emis)
{
    SceneAny* s = static_cast<SceneAny*>(h);
    g_ext_rays = 0;
    if (s->precision == 64)
        return renderT(*s->d, cam, ip, seed, row_begin, row_end, nthreads, sum, sumsq, paths, dLdI, n_albedo,
                       g_albedo, n_emis, g_emis);
    return renderT(*s->f, cam, ip, seed, row_begin, row_end, nthreads, sum, sumsq, paths, dLdI, n_albedo, g_albedo,
                   n_emis, g_emis);
}

// the oracle's own closest/any hit with the reference's acceptance rules
void orc_trace(void* h, const float* rays, long long n, int any, float* t_out, int* prim_out)
{
    SceneAny* s = static_cast<SceneAny*>(h);
    for (long long i = 0; i < n; ++i)
    {
        const float* r = rays + 8 * i;
        if (s->precision == 64)
        {
            Hit<double> hh = s->d->trace(ld3<double>(r), ld3<double>(r + 4), r[3], r[7], any != 0);
            t_out[i] = float(hh.t);
            prim_out[i] = hh.prim;
        }
        else
        {
            Hit<float> hh = s->f->trace(ld3<float>(r), ld3<float>(r + 4), r[3], r[7], any != 0);
            t_out[i] = hh.t;
            prim_out[i] = hh.prim;
        }
    }
}

// Closest hit by testing every triangle (no tree): DebugMesh::intersect
// (splitbvh/debug_mesh.cpp:780-809), the linear-scan oracle of the reference's one
// known-answer check (demo_splitbvh.cpp:194-238).  The reference's Moller-Trumbore
// acceptance; a tie keeps the lower primitive index (the first found).  Rays as orc_trace;
// `threads` host threads over the rays.
void orc_linear_trace(void* h, const float* rays, long long n, float* t_out, int* prim_out, int threads)
{
    SceneAny* s = static_cast<SceneAny*>(h);
    if (!s->f)  // a double-precision scene: nothing traced
    {
        for (long long i = 0; i < n; ++i)
        {
            t_out[i] = std::numeric_limits<float>::infinity();
            prim_out[i] = -1;
        }
        return;
    }
    const auto&     tris = s->f->tris;
    const long long nt = static_cast<long long>(tris.size());
    auto            work = [&](long long begin, long long end) {
        for (long long i = begin; i < end; ++i)
        {
            const float*    r = rays + 8 * i;
            const V3<float> o = ld3<float>(r), d = ld3<float>(r + 4);
            float           best = r[7];
            int             prim = -1;
            for (long long p = 0; p < nt; ++p)
            {
                float t, u, v;
                if (mtIntersect(o, d, tris[p].a, tris[p].b, tris[p].c, t, u, v) && t > r[3] && t < best)
                {
                    best = t;
                    prim = static_cast<int>(p);
                }
            }
            t_out[i] = prim >= 0 ? best : std::numeric_limits<float>::infinity();
            prim_out[i] = prim;
        }
    };
    const int                nth = std::max(1, threads);
    std::vector<std::thread> th;
    const long long          chunk = (n + nth - 1) / nth;
    for (int k = 0; k < nth; ++k)
    {
        const long long b = k * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back(work, b, e);
    }
    for (auto& t : th) t.join();
}

// ---- per-function entry points (float arithmetic, for pins against the reference)
void orc_material_sample(int type, const float* color, float roughness, float ior, const float* wi, const float* nl,
                         float r1, float r2, float* wo, float* weight, float* pdf)
{
    Material<float> m;
    m.type = type;
    m.color = ld3<float>(color);
    m.roughness = roughness;
    m.ior = ior;
    BsdfSample<float> s = bsdfSample(m, ld3<float>(wi), ld3<float>(nl), r1, r2);
    wo[0] = s.wo.x, wo[1] = s.wo.y, wo[2] = s.wo.z;
    weight[0] = s.weight.x, weight[1] = s.weight.y, weight[2] = s.weight.z;
    *pdf = s.pdf;
}

void orc_material_evaluate(int type, const float* color, float roughness, float ior, const float* wi,
                           const float* nl, const float* wo, float* f, float* pdf)
{
    Material<float> m;
    m.type = type;
    m.color = ld3<float>(color);
    m.roughness = roughness;
    m.ior = ior;
    V3<float> v = bsdfEval(m, ld3<float>(wi), ld3<float>(nl), ld3<float>(wo));
    f[0] = v.x, f[1] = v.y, f[2] = v.z;
    *pdf = bsdfPdf(m, ld3<float>(wi), ld3<float>(nl), ld3<float>(wo));
}

float orc_fresnel(float c, float ior) { return fresnelReflectance(c, ior); }

void orc_onb_to_world(const float* n, const float* c, float* out)
{
    Frame<float> f(ld3<float>(n));
    V3<float>    v = f.toWorld(ld3<float>(c));
    out[0] = v.x, out[1] = v.y, out[2] = v.z;
}

void orc_sample_hemisphere_cosine(float x, float y, float* out)
{
    V3<float> v = sampleHemisphereCosine(x, y);
    out[0] = v.x, out[1] = v.y, out[2] = v.z;
}

void orc_camera_ray(const float* cam, int w, int h, float mx, float my, float* o, float* d)
{
    Camera<float> c(cam, w, h);
    V3<float>     oo, dd;
    c.makeRay(mx, my, oo, dd);
    o[0] = oo.x, o[1] = oo.y, o[2] = oo.z;
    d[0] = dd.x, d[1] = dd.y, d[2] = dd.z;
}

int orc_discrete_sample(const float* w, int n, float r, float* pdf)
{
    Discrete<float>    s;
    std::vector<float> data(w, w + n);
    s.build(data);
    int i = s.sample(r);
    if (pdf) *pdf = s.pdf[i];
    return i;
}

void* orc_envmap_create(const float* rgb, int w, int h)
{
    Envmap<float>* e = new Envmap<float>;
    e->build(rgb, w, h);
    return e;
}
void orc_envmap_destroy(void* h) { delete static_cast<Envmap<float>*>(h); }
void orc_envmap_sample(void* h, float r1, float r2, float j1, float j2, float* dir, float* rad, float* pdf)
{
    V3<float> d, r;
    static_cast<Envmap<float>*>(h)->sample(r1, r2, j1, j2, d, r, *pdf);
    dir[0] = d.x, dir[1] = d.y, dir[2] = d.z;
    rad[0] = r.x, rad[1] = r.y, rad[2] = r.z;
}
float orc_envmap_pdf(void* h, const float* dir) { return static_cast<Envmap<float>*>(h)->pdf(ld3<float>(dir)); }
void  orc_envmap_radiance(void* h, const float* dir, float* rad)
{
    V3<float> r = static_cast<Envmap<float>*>(h)->radiance(ld3<float>(dir));
    rad[0] = r.x, rad[1] = r.y, rad[2] = r.z;
}
// (u_i, v_i) of the sampled texel before jitter, for pins against the reference
void orc_envmap_sample_texel(void* h, float r1, float r2, int* ui, int* vi)
{
    Envmap<float>* e = static_cast<Envmap<float>*>(h);
    *ui = e->sampleU.sample(r1);
    *vi = e->sampleUV[*ui].sample(r2);
}

void orc_set_draw_log(long long* log) { g_draw_log = log; }
long long orc_last_extension_rays() { return g_ext_rays.load(); }
void orc_ray_log(int on) { g_ray_log_on = on != 0; g_ray_log.clear(); }
long long orc_ray_log_size() { return static_cast<long long>(g_ray_log.size() / 10); }
void orc_ray_log_read(double* out) { std::memcpy(out, g_ray_log.data(), sizeof(double) * g_ray_log.size()); }

void orc_pcg32(unsigned long long seed, unsigned pixel, unsigned sample, int n, float* out)
{
    Pcg32 r;
    r.seed(seed, pixel, sample);
    for (int i = 0; i < n; ++i) out[i] = r.uniform();
}

// ---------------------------------------------------------------------------
// Film outputs, restated from film.cpp.  Images are [h][w][3] floats with row 0 the
// bottom row (FrameBuffer's layout); both writers emit rows top to bottom.
// ---------------------------------------------------------------------------

// FrameBuffer::dumpHDR (film.cpp:35-108): Radiance header, then per row the new-style
// RLE scanline marker and four channel blocks of literal runs (<= 127 bytes, no repeats).
// Returns the file size; writes it to out when capacity allows.
long long orc_film_hdr(int w, int h, const float* rgb, unsigned char* out, long long capacity)
{
    std::string head = "#?RADIANCE\n# Made with custom writer\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n-Y " +
                       std::to_string(h) + " +X " + std::to_string(w) + "\n";
    std::vector<unsigned char> f(head.begin(), head.end());
    std::vector<unsigned char> line(4 * static_cast<size_t>(w));
    for (int j = h - 1; j >= 0; --j)
    {
        for (int i = 0; i < w; ++i)
        {
            const float* c = rgb + 3 * (static_cast<size_t>(j) * w + i);
            // toRGBE (film.cpp:49-64): d = m 2^e, scale = m * 256 / d = 2^(8 - e)
            float d = c[0] > c[1] ? c[0] : c[1];
            d = d > c[2] ? d : c[2];
            unsigned char* q = &line[4 * static_cast<size_t>(i)];
            if (d <= 1e-32)
            {
                q[0] = q[1] = q[2] = q[3] = 0;
                continue;
            }
            int   e;
            float m = static_cast<float>(std::frexp(static_cast<double>(d), &e));
            float s = m * 256.0f / d;
            q[0] = static_cast<unsigned char>(c[0] * s);
            q[1] = static_cast<unsigned char>(c[1] * s);
            q[2] = static_cast<unsigned char>(c[2] * s);
            q[3] = static_cast<unsigned char>(e + 128);
        }
        f.push_back(2);
        f.push_back(2);
        f.push_back(static_cast<unsigned char>((w >> 8) & 0xFF));
        f.push_back(static_cast<unsigned char>(w & 0xFF));
        for (int k = 0; k < 4; ++k)
            for (int cursor = 0; cursor < w;)
            {
                const int run = std::min(127, w - cursor);
                f.push_back(static_cast<unsigned char>(run));
                for (int i = cursor; i < cursor + run; ++i) f.push_back(line[4 * static_cast<size_t>(i) + k]);
                cursor += run;
            }
    }
    if (out && capacity >= static_cast<long long>(f.size())) std::memcpy(out, f.data(), f.size());
    return static_cast<long long>(f.size());
}

// FrameBuffer::dumpPPM (film.cpp:9-33): "P6 w h 255", bytes (unsigned char)(min(1, v) * 255)
long long orc_film_ppm(int w, int h, const float* rgb, unsigned char* out, long long capacity)
{
    std::string head = "P6\n" + std::to_string(w) + " " + std::to_string(h) + "\n255\n";
    std::vector<unsigned char> f(head.begin(), head.end());
    for (int j = h - 1; j >= 0; --j)
        for (int i = 0; i < w; ++i)
            for (int k = 0; k < 3; ++k)
            {
                float v = rgb[3 * (static_cast<size_t>(j) * w + i) + k];
                f.push_back(static_cast<unsigned char>((1.0f < v ? 1.0f : v) * 255));
            }
    if (out && capacity >= static_cast<long long>(f.size())) std::memcpy(out, f.data(), f.size());
    return static_cast<long long>(f.size());
}

// FrameBuffer::tonemapGamma (mode 0, film.cpp:196-203) and tonemapReinhard (mode 1,
// film.cpp:110-194; its contrast is fixed at 0.77 and light adaptation at 0, so every
// pixel maps x -> x / (x + (c * mean_x + (1 - c) * mean_lum)^0.77), c = 0.5, with the
// means accumulated in float in pixel order), in place
void orc_film_tonemap(int w, int h, float* rgb, int mode, float gamma)
{
    const size_t n = static_cast<size_t>(w) * h;
    if (mode == 0)
    {
        const float inv = 1.0f / gamma;
        for (size_t k = 0; k < 3 * n; ++k)
        {
            float x = rgb[k];
            x = x < 0.0f ? 0.0f : x > 1.0f ? 1.0f : x;
            rgb[k] = powf(x, inv);
        }
        return;
    }
    std::vector<float> lum(n);
    float              l_mean = 0, r_mean = 0, g_mean = 0, b_mean = 0;
    for (size_t p = 0; p < n; ++p)
    {
        const float* c = rgb + 3 * p;
        // luminance (numeric.cpp:62-66) in double
        lum[p] = static_cast<float>(0.299 * c[0] + 0.587 * c[1] + 0.114 * c[2]);
        if (lum[p] < 1e-7f) lum[p] = 1e-7f;
    }
    for (size_t p = 0; p < n; ++p)
    {
        l_mean += lum[p];
        r_mean += rgb[3 * p];
        g_mean += rgb[3 * p + 1];
        b_mean += rgb[3 * p + 2];
    }
    l_mean /= n;
    r_mean /= n;
    g_mean /= n;
    b_mean /= n;
    const float c = 0.5f, m = 0.77f, f = expf(-0.0f);
    const float kr = powf(f * (c * r_mean + (1.0f - c) * l_mean), m);
    const float kg = powf(f * (c * g_mean + (1.0f - c) * l_mean), m);
    const float kb = powf(f * (c * b_mean + (1.0f - c) * l_mean), m);
    for (size_t p = 0; p < n; ++p)
    {
        float* x = rgb + 3 * p;
        x[0] = x[0] / (x[0] + kr);
        x[1] = x[1] / (x[1] + kg);
        x[2] = x[2] / (x[2] + kb);
    }
}

}  // extern "C"
