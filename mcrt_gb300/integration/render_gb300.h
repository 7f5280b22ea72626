// The integrator seam of MCRT on the GB300 library: a finalized MCRT Scene (built through
// its own API: Scene::add / loadModel, todo_addMaterial, Scene::setEnvmap) rendered by
// mcrt_render in place of rayTrace + DemoSimple::run (src/examples/pt/demo_pt.cpp:512-720).
// Compile render_gb300.cpp into the application with MCRT's src/core headers and this
// repository's include/ on the include path, and link libmcrt_gb300.so.
#pragma once
#include <cstdint>

#include "mcrt_gb300.h"

class Scene;
class FrameBuffer;

// The library's scene for an MCRT Scene: its triangles (vertices and vertex normals), one
// library material per MCRT material the triangles use (type, colour, roughness, IOR), and
// the environment map read from `envmap_bin` (the file given to Scene::setEnvmap; NULL for
// none).  Returns MCRT_OK or an MCRT_ERR_* code (mcrt_last_error() has the message).
int gb300_scene_from_mcrt(const Scene& scene, const char* envmap_bin, mcrt_scene** out);

// Renders `camera` (the arguments given to Scene::setCamera) with `params` into `fb`, which
// is resized to the camera's film and holds per-pixel means afterwards: what
// DemoSimple::run leaves in its FrameBuffer after accumulatePixel and scale(1 / spp), ready
// for dumpHDR / tonemapGamma / dumpPPM.  params->ptr_mode is ignored (host memory).
int gb300_render_into(mcrt_scene* scene, const mcrt_camera& camera, const mcrt_render_params& params,
                      FrameBuffer& fb, mcrt_render_stats* stats);
