// mcrt_autotune: picks the launch configuration of a render (or batch of renders) by
// timing a reduced-spp probe of the same jobs through the public render entry point.
//
// The search is two-stage, so it costs about eight probe renders (each best of two):
//   1. traversal kernel variants at the default queue capacity: 32-entry or 64-entry
//      shared-memory stacks, 56-register cap or none, warp batch fetch or grid stride;
//   2. queue capacities (2^21 .. 2^26 rays) with the best variant.
// Every configuration renders the same image (the schedule never changes a path's
// arithmetic), so only the time is compared.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "wavefront.h"

namespace {

struct Candidate
{
    int64_t path_chunk;
    int32_t variant;
    float   ms;
};

}  // namespace

extern "C" int mcrt_autotune(int32_t num_jobs, mcrt_scene* const* scenes, const mcrt_camera* cameras,
                             const mcrt_render_params* params, mcrt_render_params* tuned, mcrt_tune_report* report,
                             void* stream)
{
    using namespace mcrt;
    if (num_jobs <= 0 || !scenes || !cameras || !params || !tuned)
        return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_autotune: empty job list or null output");
    try
    {
        for (int j = 0; j < num_jobs; ++j)
        {
            int rc = validate_job(scenes[j], &cameras[j], &params[j]);
            if (rc) return rc;
        }
        // probe: the same jobs with spp scaled so that the probe holds about two of the
        // largest candidate queues of paths (or the whole render if it is smaller)
        constexpr int64_t kMaxCapacity = int64_t(1) << 26;
        int64_t           total = 0;
        for (int j = 0; j < num_jobs; ++j)
            total += static_cast<int64_t>(cameras[j].width) * cameras[j].height * params[j].spp;
        const double                    scale = std::min(1.0, 2.0 * kMaxCapacity / static_cast<double>(total));
        std::vector<mcrt_render_params> probe(params, params + num_jobs);
        int64_t                         probe_paths = 0;
        for (int j = 0; j < num_jobs; ++j)
        {
            probe[j].spp = std::max(1, static_cast<int>(std::lround(params[j].spp * scale)));
            probe[j].ptr_mode = MCRT_PTR_DEVICE;
            probe[j].profile = 0;
            probe[j].use_graph = 1;
            probe[j].schedule = MCRT_SCHEDULE_STREAM;
            probe_paths += static_cast<int64_t>(cameras[j].width) * cameras[j].height * probe[j].spp;
        }
        if (params[0].schedule != MCRT_SCHEDULE_STREAM)
            for (auto& p : probe) p.schedule = params[0].schedule;
        cudaError_t e = cudaSetDevice(scene_device(scenes[0]));
        if (e != cudaSuccess) return set_error(MCRT_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        std::vector<float*> images(num_jobs, nullptr);
        auto                release = [&]() {
            for (float* p : images) cudaFree(p);
        };
        for (int j = 0; j < num_jobs; ++j)
        {
            e = cudaMalloc(&images[j], sizeof(float) * 3 * cameras[j].width * cameras[j].height);
            if (e != cudaSuccess)
            {
                release();
                return set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_autotune: scratch image allocation failed");
            }
        }
        std::vector<Candidate> tried;
        auto                   time_config = [&](int64_t chunk, int32_t variant, float& best) -> int {
            for (auto& p : probe)
            {
                p.path_chunk = chunk;
                p.variant = variant;
            }
            best = 1e30f;
            for (int rep = 0; rep < 2; ++rep)
            {
                mcrt_render_stats st{};
                int rc = mcrt_render_batch(num_jobs, scenes, cameras, probe.data(), images.data(), &st, stream);
                if (rc) return rc;
                best = std::min(best, st.device_ms);
            }
            tried.push_back({chunk, variant, best});
            return MCRT_OK;
        };
        // warm-up: module load, workspace allocation
        {
            float ms;
            int   rc = time_config(0, 0, ms);
            if (rc)
            {
                release();
                return rc;
            }
            tried.clear();
        }
        const int32_t X = MCRT_VARIANT_EXPLICIT;
        const int32_t variants[] = {X | MCRT_VARIANT_STACK32 | MCRT_VARIANT_REGCAP, X | MCRT_VARIANT_REGCAP,
                                    X | MCRT_VARIANT_STACK32, X,
                                    X | MCRT_VARIANT_STACK32 | MCRT_VARIANT_REGCAP | MCRT_VARIANT_GRIDSTRIDE};
        int32_t       best_variant = variants[0];
        float         best_ms = 1e30f;
        for (int32_t v : variants)
        {
            float ms;
            int   rc = time_config(0, v, ms);
            if (rc)
            {
                release();
                return rc;
            }
            if (ms < best_ms)
            {
                best_ms = ms;
                best_variant = v;
            }
        }
        int64_t best_chunk = 0;
        for (int64_t chunk = int64_t(1) << 21; chunk <= kMaxCapacity; chunk <<= 1)
        {
            if (chunk > 2 * probe_paths) break;
            float ms;
            int   rc = time_config(chunk, best_variant, ms);
            if (rc)
            {
                release();
                return rc;
            }
            if (ms < best_ms)
            {
                best_ms = ms;
                best_chunk = chunk;
            }
        }
        release();
        int chosen = 0;
        for (size_t k = 0; k < tried.size(); ++k)
            if (tried[k].path_chunk == best_chunk && tried[k].variant == best_variant) chosen = static_cast<int>(k);
        for (int j = 0; j < num_jobs; ++j)
        {
            tuned[j] = params[j];
            tuned[j].path_chunk = best_chunk;
            tuned[j].variant = best_variant;
        }
        if (report)
        {
            *report = mcrt_tune_report{};
            report->num_candidates = static_cast<int32_t>(std::min<size_t>(tried.size(), MCRT_TUNE_MAX));
            report->chosen = chosen < MCRT_TUNE_MAX ? chosen : 0;
            report->probe_paths = probe_paths;
            for (int k = 0; k < report->num_candidates; ++k)
            {
                report->path_chunk[k] = tried[k].path_chunk;
                report->variant[k] = tried[k].variant;
                report->ms[k] = tried[k].ms;
            }
        }
        return MCRT_OK;
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_autotune");
    }
}
