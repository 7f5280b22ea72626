// Film outputs on the device: FrameBuffer's writers and tone mappers (film.cpp) for an
// image in the layout mcrt_render writes ([height][width][3] floats, row 0 the bottom).
//
//   k_film_hdr    FrameBuffer::dumpHDR (film.cpp:35-108): every pixel's RGBE bytes go
//                 straight to their place in the file (rows top to bottom, per row the
//                 scanline marker and four channel blocks of literal runs of <= 127 bytes),
//                 so the file is one pass over the image
//   k_film_ppm    FrameBuffer::dumpPPM (film.cpp:9-33)
//   k_film_gamma  FrameBuffer::tonemapGamma (film.cpp:196-203), in place
//   Reinhard      FrameBuffer::tonemapReinhard (film.cpp:110-194): its contrast is fixed at
//                 0.77 and its light adaptation at 0, so each pixel maps x -> x / (x + K_c)
//                 with K_c = (0.5 mean_c + 0.5 mean_lum)^0.77 per channel; the means are
//                 float sums in pixel order (one thread, the reference's rounding), K_c is
//                 evaluated on the host with the C library's powf as the reference does
//
// Byte- and bit-exact against the reference except tonemapGamma, whose per-pixel powf is
// CUDA's (within its documented ulp bound of the C library's).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "wavefront.h"

namespace mcrt {
namespace {

std::string hdr_header(int w, int h)
{
    return "#?RADIANCE\n# Made with custom writer\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n-Y " + std::to_string(h) +
           " +X " + std::to_string(w) + "\n";
}

std::string ppm_header(int w, int h) { return "P6\n" + std::to_string(w) + " " + std::to_string(h) + "\n255\n"; }

int64_t hdr_runs(int w) { return (w + 126) / 127; }
int64_t hdr_line_bytes(int w) { return 4 + 4 * (w + hdr_runs(w)); }

__global__ void k_film_hdr(const float* __restrict__ rgb, int w, int h, uint8_t* __restrict__ out, int64_t head)
{
    const int64_t n = static_cast<int64_t>(w) * h;
    const int64_t runs = (w + 126) / 127;
    const int64_t line = 4 + 4 * (w + runs);
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const int j = static_cast<int>(p / w), i = static_cast<int>(p - static_cast<int64_t>(j) * w);
        const float* c = rgb + 3 * p;
        // toRGBE (film.cpp:49-64): d = m 2^e; m * 256 / d = 2^(8 - e) exactly
        float   d = c[0] > c[1] ? c[0] : c[1];
        d = d > c[2] ? d : c[2];
        uint8_t q[4] = {0, 0, 0, 0};
        if (!(static_cast<double>(d) <= 1e-32))
        {
            int         e;
            const float m = frexpf(d, &e);
            const float s = __fdiv_rn(__fmul_rn(m, 256.0f), d);
            q[0] = static_cast<uint8_t>(__fmul_rn(c[0], s));
            q[1] = static_cast<uint8_t>(__fmul_rn(c[1], s));
            q[2] = static_cast<uint8_t>(__fmul_rn(c[2], s));
            q[3] = static_cast<uint8_t>(e + 128);
        }
        uint8_t* row = out + head + static_cast<int64_t>(h - 1 - j) * line;
        if (i == 0)
        {
            row[0] = 2;
            row[1] = 2;
            row[2] = static_cast<uint8_t>((w >> 8) & 0xFF);
            row[3] = static_cast<uint8_t>(w & 0xFF);
        }
        const int64_t run = i / 127, in_run = i - run * 127;
        for (int k = 0; k < 4; ++k)
        {
            uint8_t* chan = row + 4 + k * (w + runs);
            if (in_run == 0) chan[run * 128] = static_cast<uint8_t>(min(127, w - i));
            chan[run * 128 + 1 + in_run] = q[k];
        }
    }
}

__global__ void k_film_ppm(const float* __restrict__ rgb, int w, int h, uint8_t* __restrict__ out, int64_t head)
{
    const int64_t n = 3 * static_cast<int64_t>(w) * h;
    for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < n;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const int64_t p = q / 3;
        const int     k = static_cast<int>(q - 3 * p);
        const int     j = static_cast<int>(p / w), i = static_cast<int>(p - static_cast<int64_t>(j) * w);
        const float   v = rgb[q];
        const float   c = 1.0f < v ? 1.0f : v;  // f_min(1, v)
        out[head + (static_cast<int64_t>(h - 1 - j) * w + i) * 3 + k] = static_cast<uint8_t>(__fmul_rn(c, 255.0f));
    }
}

__global__ void k_film_gamma(float* rgb, int64_t n, float inv_gamma)
{
    for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < n;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        float x = rgb[q];
        x = x < 0.0f ? 0.0f : x > 1.0f ? 1.0f : x;  // clampf
        rgb[q] = powf(x, inv_gamma);
    }
}

// luminance (numeric.cpp:62-66): in double, then clamped at 1e-7 (film.cpp:118-120)
__global__ void k_film_lum(const float* __restrict__ rgb, int64_t n, float* __restrict__ lum)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const float* c = rgb + 3 * p;
        double       l = __dadd_rn(__dadd_rn(__dmul_rn(0.299, c[0]), __dmul_rn(0.587, c[1])), __dmul_rn(0.114, c[2]));
        float        f = static_cast<float>(l);
        lum[p] = f < 1e-7f ? 1e-7f : f;
    }
}

// the four means of tonemapReinhard, summed in float in pixel order (one thread)
__global__ void k_film_means(const float* __restrict__ rgb, const float* __restrict__ lum, int64_t n,
                             float* __restrict__ means)
{
    float l = 0.f, r = 0.f, g = 0.f, b = 0.f;
    for (int64_t p = 0; p < n; ++p)
    {
        l = __fadd_rn(l, lum[p]);
        r = __fadd_rn(r, rgb[3 * p]);
        g = __fadd_rn(g, rgb[3 * p + 1]);
        b = __fadd_rn(b, rgb[3 * p + 2]);
    }
    const float fn = static_cast<float>(n);
    means[0] = __fdiv_rn(l, fn);
    means[1] = __fdiv_rn(r, fn);
    means[2] = __fdiv_rn(g, fn);
    means[3] = __fdiv_rn(b, fn);
}

__global__ void k_film_reinhard(float* rgb, int64_t n, float kr, float kg, float kb)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        float* x = rgb + 3 * p;
        x[0] = __fdiv_rn(x[0], __fadd_rn(x[0], kr));
        x[1] = __fdiv_rn(x[1], __fadd_rn(x[1], kg));
        x[2] = __fdiv_rn(x[2], __fadd_rn(x[2], kb));
    }
}

int grid_for(int64_t n) { return static_cast<int>(std::min<int64_t>((n + 255) / 256, 152 * 16)); }

#define FCK(x)                                                                                             \
    do                                                                                                     \
    {                                                                                                      \
        cudaError_t e_ = (x);                                                                              \
        if (e_ != cudaSuccess)                                                                             \
        {                                                                                                  \
            release();                                                                                     \
            return set_error(e_ == cudaErrorMemoryAllocation ? MCRT_ERR_OUT_OF_MEMORY : MCRT_ERR_CUDA,     \
                             std::string(#x) + ": " + cudaGetErrorString(e_));                             \
        }                                                                                                  \
    } while (0)

}  // namespace
}  // namespace mcrt

using namespace mcrt;

extern "C" int mcrt_film_encode(const float* rgb, int32_t width, int32_t height, int32_t format, uint8_t* out,
                                int64_t capacity, int64_t* size, int32_t ptr_mode, void* stream)
{
    try
    {
        if (!rgb || !size || width <= 0 || height <= 0)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_film_encode: null image or size, or empty image");
        if (format != MCRT_FILM_HDR && format != MCRT_FILM_PPM)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_film_encode: unknown format");
        const std::string head = format == MCRT_FILM_HDR ? hdr_header(width, height) : ppm_header(width, height);
        const int64_t     body = format == MCRT_FILM_HDR ? hdr_line_bytes(width) * height
                                                         : 3 * static_cast<int64_t>(width) * height;
        *size = static_cast<int64_t>(head.size()) + body;
        if (!out) return MCRT_OK;  // size query
        if (capacity < *size) return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_film_encode: output buffer too small");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const float* d_rgb = rgb;
        uint8_t*     d_out = out;
        void*        tmp_in = nullptr;
        void*        tmp_out = nullptr;
        auto         release = [&]() {
            cudaFree(tmp_in);
            cudaFree(tmp_out);
        };
        const size_t img_bytes = sizeof(float) * 3 * static_cast<size_t>(width) * height;
        if (ptr_mode != MCRT_PTR_DEVICE)
        {
            FCK(cudaMalloc(&tmp_in, img_bytes));
            FCK(cudaMalloc(&tmp_out, static_cast<size_t>(*size)));
            FCK(cudaMemcpyAsync(tmp_in, rgb, img_bytes, cudaMemcpyHostToDevice, st));
            d_rgb = static_cast<const float*>(tmp_in);
            d_out = static_cast<uint8_t*>(tmp_out);
        }
        FCK(cudaMemcpyAsync(d_out, head.data(), head.size(), cudaMemcpyHostToDevice, st));
        const int64_t n = static_cast<int64_t>(width) * height;
        if (format == MCRT_FILM_HDR)
            k_film_hdr<<<grid_for(n), 256, 0, st>>>(d_rgb, width, height, d_out, static_cast<int64_t>(head.size()));
        else
            k_film_ppm<<<grid_for(3 * n), 256, 0, st>>>(d_rgb, width, height, d_out,
                                                         static_cast<int64_t>(head.size()));
        FCK(cudaGetLastError());
        if (ptr_mode != MCRT_PTR_DEVICE)
            FCK(cudaMemcpyAsync(out, d_out, static_cast<size_t>(*size), cudaMemcpyDeviceToHost, st));
        FCK(cudaStreamSynchronize(st));
        release();
        return MCRT_OK;
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_film_encode");
    }
}

extern "C" int mcrt_film_tonemap(float* rgb, int32_t width, int32_t height, int32_t op, float gamma, int32_t ptr_mode,
                                 void* stream)
{
    try
    {
        if (!rgb || width <= 0 || height <= 0)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_film_tonemap: null or empty image");
        if (op != MCRT_TONEMAP_GAMMA && op != MCRT_TONEMAP_REINHARD)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_film_tonemap: unknown operator");
        cudaStream_t  st = static_cast<cudaStream_t>(stream);
        const int64_t n = static_cast<int64_t>(width) * height;
        const size_t  img_bytes = sizeof(float) * 3 * static_cast<size_t>(n);
        float*        d_rgb = rgb;
        void*         tmp = nullptr;
        void*         lum = nullptr;
        auto          release = [&]() {
            cudaFree(tmp);
            cudaFree(lum);
        };
        if (ptr_mode != MCRT_PTR_DEVICE)
        {
            FCK(cudaMalloc(&tmp, img_bytes));
            FCK(cudaMemcpyAsync(tmp, rgb, img_bytes, cudaMemcpyHostToDevice, st));
            d_rgb = static_cast<float*>(tmp);
        }
        if (op == MCRT_TONEMAP_GAMMA)
        {
            k_film_gamma<<<grid_for(3 * n), 256, 0, st>>>(d_rgb, 3 * n, 1.0f / gamma);
        }
        else
        {
            FCK(cudaMalloc(&lum, sizeof(float) * (n + 4)));
            float* d_lum = static_cast<float*>(lum);
            float* d_means = d_lum + n;
            k_film_lum<<<grid_for(n), 256, 0, st>>>(d_rgb, n, d_lum);
            k_film_means<<<1, 1, 0, st>>>(d_rgb, d_lum, n, d_means);
            float means[4];
            FCK(cudaMemcpyAsync(means, d_means, sizeof(means), cudaMemcpyDeviceToHost, st));
            FCK(cudaStreamSynchronize(st));
            // film.cpp:149-186 with c = 0.5, a = 0, f = exp(-0) = 1, m = 0.77
            const float c = 0.5f, m = 0.77f, f = std::exp(-0.0f);
            const float kr = std::pow(f * (c * means[1] + (1.0f - c) * means[0]), m);
            const float kg = std::pow(f * (c * means[2] + (1.0f - c) * means[0]), m);
            const float kb = std::pow(f * (c * means[3] + (1.0f - c) * means[0]), m);
            k_film_reinhard<<<grid_for(n), 256, 0, st>>>(d_rgb, n, kr, kg, kb);
        }
        FCK(cudaGetLastError());
        if (ptr_mode != MCRT_PTR_DEVICE) FCK(cudaMemcpyAsync(rgb, d_rgb, img_bytes, cudaMemcpyDeviceToHost, st));
        FCK(cudaStreamSynchronize(st));
        release();
        return MCRT_OK;
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_film_tonemap");
    }
}
