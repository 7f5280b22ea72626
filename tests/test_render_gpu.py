"""Rendered images of the CUDA wavefront against the oracle (same seeds) and the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cfg0(res=32):
    from mcrt_gb300 import scenes
    return scenes.cfg0_scene(), scenes.cfg0_camera(res, res)


def _crn_compare(gpu, cpu, name):
    """Same seed, same random-number schedule: most pixels agree to float noise.
    A path diverges only where float rounding flips a sampling decision."""
    rel = np.abs(gpu - cpu) / (np.abs(cpu) + 1e-3)
    frac_close = np.mean(rel < 1e-3)
    mre = np.abs(gpu.mean() - cpu.mean()) / max(cpu.mean(), 1e-9)
    assert frac_close > 0.9, f"{name}: only {frac_close:.3f} of pixels match the oracle"
    assert mre < 5e-3, f"{name}: mean relative error {mre:.2e}"


def _ray_counts_agree(st, ref):
    """Same estimator, same random numbers: the same extension rays to within a few paths.
    The oracle traces every next-event ray of the reference; the GPU skips the area-light
    rays that cannot reach the emitters' box, so it traces at most as many."""
    assert abs(st["extension_rays"] - ref["extension_rays"]) <= 0.01 * ref["extension_rays"]
    ref_nee = ref["rays"] - ref["extension_rays"]
    assert st["shadow_rays"] <= 1.01 * ref_nee


@pytest.mark.parametrize("traverse", [0, 1])
def test_cfg0_crn_matches_float_oracle(traverse, cuda_device):
    from mcrt_gb300 import GpuScene
    from oracle.oracle import OracleScene
    desc, cam = _cfg0(32)
    gpu, st = GpuScene(desc).render(cam, spp=16, max_depth=8, rr_depth=3, seed=7, traverse=traverse)
    ref = OracleScene(desc, 32).render(cam.as_array(), 32, 32, 16, 8, 3, seed=7)
    _crn_compare(gpu, ref["mean"].astype(np.float32), "cfg0")
    _ray_counts_agree(st, ref)


def test_cfg1_small_crn_matches_float_oracle(cuda_device):
    """Environment map + GGX + dielectric patches (level-5 sphere, 256x128 map)."""
    from mcrt_gb300 import GpuScene, scenes
    from oracle.oracle import OracleScene
    desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
    cam = scenes.cfg1_camera(32, 32)
    gpu, st = GpuScene(desc).render(cam, spp=8, max_depth=6, seed=3)
    ref = OracleScene(desc, 32).render(cam.as_array(), 32, 32, 8, 6, -1, seed=3)
    _crn_compare(gpu, ref["mean"].astype(np.float32), "cfg1-small")


def test_cfg0_ztest_vs_fp64_oracle(cuda_device):
    """Independent seeds: per-pixel z-test of the GPU mean against the FP64 oracle."""
    from mcrt_gb300 import GpuScene
    from oracle.oracle import OracleScene
    desc, cam = _cfg0(24)
    sc = GpuScene(desc)
    batches = [sc.render(cam, spp=256, max_depth=8, rr_depth=3, seed=100 + b)[0] for b in range(8)]
    g = np.mean(batches, axis=0)
    gvar = np.var(batches, axis=0, ddof=1) / len(batches)
    ref = OracleScene(desc, 64).render(cam.as_array(), 24, 24, 1024, 8, 3, seed=999)
    z = (g - ref["mean"]) / np.sqrt(gvar + ref["var_of_mean"] + 1e-12)
    assert np.mean(np.abs(z) > 4) < 0.01, f"{np.mean(np.abs(z) > 4):.3f} of pixels beyond 4 sigma"
    for c in range(3):
        rel = abs(g[..., c].mean() - ref["mean"][..., c].mean()) / ref["mean"][..., c].mean()
        assert rel < 0.01, f"channel {c}: mean relative error {rel:.4f}"


@pytest.mark.parametrize("schedule", [0, 1])
def test_graph_and_direct_launches_agree(schedule, cuda_device):
    from mcrt_gb300 import GpuScene
    desc, cam = _cfg0(32)
    sc = GpuScene(desc)
    kw = dict(spp=8, max_depth=8, rr_depth=3, seed=5, path_chunk=3000, schedule=schedule)
    a, sa = sc.render(cam, use_graph=False, **kw)
    b, sb = sc.render(cam, use_graph=True, **kw)
    assert sa["waves"] > 1
    np.testing.assert_array_equal(a, b)
    assert sa["rays"] == sb["rays"]


@pytest.mark.parametrize("path_chunk", [64, 256, 3000, 0])
def test_streaming_equals_waves_bit_exactly(path_chunk, cuda_device):
    """Path regeneration changes which slot and iteration a path runs in, never its
    arithmetic: the images are identical.  Small slot counts make the per-path ring wrap
    (ring = (max_depth + 2) * slots + spp < paths)."""
    from mcrt_gb300 import GpuScene
    desc, cam = _cfg0(32)
    sc = GpuScene(desc)
    kw = dict(spp=4, max_depth=8, rr_depth=3, seed=13, path_chunk=path_chunk)
    w, sw = sc.render(cam, schedule=1, **kw)
    s, ss = sc.render(cam, schedule=0, use_graph=True, **kw)
    np.testing.assert_array_equal(s, w)
    assert ss["rays"] == sw["rays"] and ss["paths"] == sw["paths"] == 32 * 32 * 4
    if path_chunk:
        assert ss["waves"] > 8


def test_streaming_batch_of_uneven_jobs_equals_waves(cuda_device):
    """Jobs of different spp / depth in one streaming render: each pixel resolves from
    its own job's samples."""
    from mcrt_gb300 import GpuScene, render_batch, scenes
    jobs = scenes.cfg2_jobs(n_scenes=4, seed=5, max_level=4)
    gs = [GpuScene(d) for d, _, _ in jobs]
    cams = [c for _, c, _ in jobs]
    for k, c in enumerate(cams):
        c.width, c.height = 24 + 8 * k, 16 + 4 * k
    params = [dict(p, spp=1 + 3 * k, path_chunk=512) for k, (_, _, p) in enumerate(jobs)]
    outs_s, st_s = render_batch(gs, cams, [dict(p, schedule=0) for p in params])
    outs_w, st_w = render_batch(gs, cams, [dict(p, schedule=1) for p in params])
    for a, b in zip(outs_s, outs_w):
        np.testing.assert_array_equal(a, b)
    assert st_s["rays"] == st_w["rays"]


def test_unknown_schedule_is_rejected(cuda_device):
    from mcrt_gb300 import GpuScene
    desc, cam = _cfg0(8)
    from mcrt_gb300._native import McrtError
    with pytest.raises(McrtError, match="schedule"):
        GpuScene(desc).render(cam, spp=1, max_depth=2, schedule=7)


@pytest.mark.parametrize("schedule", [0, 2])
def test_batch_equals_individual_renders(schedule, cuda_device):
    """A batch of uneven jobs renders each job's own image, in the streaming wavefront and
    in the plain one-thread-per-path tracer (chunks of 300 paths that straddle jobs)."""
    from mcrt_gb300 import GpuScene, render_batch, scenes
    jobs = scenes.cfg2_jobs(n_scenes=3, seed=11, max_level=4)
    gs = [GpuScene(d) for d, _, _ in jobs]
    cams = [c for _, c, _ in jobs]
    for c in cams:
        c.width = c.height = 32
    params = [dict(p, schedule=schedule, path_chunk=300 if schedule == 2 else 0) for _, _, p in jobs]
    outs, st = render_batch(gs, cams, params)
    for s, c, p, o in zip(gs, cams, params, outs):
        single, _ = s.render(c, **p)
        if schedule == 2:
            np.testing.assert_array_equal(o, single)
        else:
            np.testing.assert_allclose(o, single, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("schedule", [0, 1])
def test_chunking_is_invisible(schedule, cuda_device):
    """Waves or slot pools of any size give the same image (waves end on pixel
    boundaries; streamed pixels resolve from the ring in sample order)."""
    from mcrt_gb300 import GpuScene
    desc, cam = _cfg0(20)
    sc = GpuScene(desc)
    a, _ = sc.render(cam, spp=5, max_depth=8, rr_depth=3, seed=9, path_chunk=0, schedule=schedule)
    b, sb = sc.render(cam, spp=5, max_depth=8, rr_depth=3, seed=9, path_chunk=777, schedule=schedule)
    assert sb["waves"] > 2
    np.testing.assert_array_equal(a, b)


def test_render_into_device_tensor(cuda_device):
    import torch
    from mcrt_gb300 import GpuScene
    desc, cam = _cfg0(16)
    sc = GpuScene(desc)
    host, _ = sc.render(cam, spp=4, max_depth=4, seed=1)
    out = torch.zeros((16, 16, 3), dtype=torch.float32, device=cuda_device)
    sc.render(cam, spp=4, max_depth=4, seed=1, out=out)
    np.testing.assert_allclose(out.cpu().numpy(), host, rtol=1e-5, atol=1e-6)


def test_autotune_picks_a_timed_configuration_with_identical_image(cuda_device):
    """The autotuner times kernel variants and queue capacities on a probe and returns
    params that render the same image as the defaults."""
    from mcrt_gb300 import GpuScene, autotune, render_batch, scenes
    jobs = scenes.cfg2_jobs(n_scenes=3, seed=7, max_level=4)
    gs = [GpuScene(d) for d, _, _ in jobs]
    cams = [c for _, c, _ in jobs]
    for c in cams:
        c.width, c.height = 48, 40
    params = [dict(p, spp=4) for _, _, p in jobs]
    tuned, rep = autotune(gs, cams, params)
    assert len(rep["candidates"]) >= 5
    assert all(c["ms"] > 0 for c in rep["candidates"])
    best = rep["candidates"][rep["chosen"]]
    assert best["ms"] == min(c["ms"] for c in rep["candidates"])
    assert all(t["variant"] == best["variant"] and t["path_chunk"] == best["path_chunk"] for t in tuned)
    a, _ = render_batch(gs, cams, params)
    b, _ = render_batch(gs, cams, tuned)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("variant", [4 | 1 | 2 | 8, 4, 4 | 1, 4 | 2])
def test_kernel_variants_render_identical_images(variant, cuda_device):
    """Stack depth, register cap and work distribution change only how rays
    are traced, never a path's result."""
    from mcrt_gb300 import GpuScene, scenes
    desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
    cam = scenes.cfg1_camera(48, 40)
    sc = GpuScene(desc)
    kw = dict(spp=4, max_depth=6, seed=3, path_chunk=1024)
    a, sa = sc.render(cam, **kw)
    b, sb = sc.render(cam, variant=variant, **kw)
    np.testing.assert_array_equal(a, b)
    assert sa["rays"] == sb["rays"]


def test_consistent_normals_match_oracle(cuda_device):
    """A coarse mirror sphere shaded with consistent normals (MCRT_MAT_CONSISTENT; alphas from
    mcrt_vertex_alpha, pinned to Mesh::genNormals): the GPU render against the float oracle
    with the same alphas and random numbers, and visibly different from interpolated normals."""
    from mcrt_gb300 import GpuScene, scenes
    from mcrt_gb300.scene import CONSISTENT, SPEC, vertex_alpha
    from oracle.oracle import OracleScene
    desc = scenes.cfg0_scene(sphere_level=1)
    plain = scenes.cfg0_scene(sphere_level=1)
    desc.materials[-1].type = SPEC | CONSISTENT
    plain.materials[-1].type = SPEC
    desc.vertex_alpha = vertex_alpha(desc.vertices, desc.normals)
    cam = scenes.cfg0_camera(32, 32)
    kw = dict(spp=16, max_depth=8, rr_depth=3, seed=7)
    gpu, _ = GpuScene(desc).render(cam, **kw)
    ref = OracleScene(desc, 32).render(cam.as_array(), 32, 32, 16, 8, 3, seed=7)
    _crn_compare(gpu, ref["mean"].astype(np.float32), "consistent")
    other, _ = GpuScene(plain).render(cam, **kw)
    assert np.mean(np.abs(other - gpu) > 1e-3) > 0.01
    # derived alphas (desc.vertex_alpha None) equal the explicit ones
    desc2 = scenes.cfg0_scene(sphere_level=1)
    desc2.materials[-1].type = SPEC | CONSISTENT
    np.testing.assert_array_equal(GpuScene(desc2).render(cam, **kw)[0], gpu)


def test_area_and_environment_lights_in_one_scene(cuda_device):
    """Both light kinds in one render (the shading build for both): the Cornell box, open
    towards the camera, under a sky with a sun, against the float oracle with the same
    random numbers; then batched with an area-light-only job (both jobs run the build for
    both kinds), each image as that job renders alone."""
    from mcrt_gb300 import GpuScene, render_batch, scenes
    from oracle.oracle import OracleScene
    desc, cam = _cfg0(32)
    desc.envmap = scenes.sky_envmap(64, 32, sun_radiance=50.0, sun_diameter_deg=8.0)
    kw = dict(spp=16, max_depth=6, rr_depth=3, seed=9)
    both = GpuScene(desc)
    gpu, _ = both.render(cam, **kw)
    ref = OracleScene(desc, 32).render(cam.as_array(), 32, 32, 16, 6, 3, seed=9)
    _crn_compare(gpu, ref["mean"].astype(np.float32), "area+env")
    area_desc, area_cam = _cfg0(16)
    area = GpuScene(area_desc)
    outs, _ = render_batch([area, both], [area_cam, cam], [kw, kw])
    for o, alone in zip(outs, [area.render(area_cam, **kw)[0], gpu]):
        close = np.mean(np.abs(o - alone) / (np.abs(alone) + 1e-3) < 1e-3)
        assert close > 0.98, close


def test_fast_only_builds_render_the_general_builds_image(cuda_device):
    """A render whose jobs all traverse in FAST mode runs traversal kernels built without the
    reference-order traversal; batched with a REF job, the same FAST job runs the general
    build (64-entry stacks, no register cap).  Its image is the same bit for bit."""
    from mcrt_gb300 import TRAVERSE_FAST, TRAVERSE_REF, GpuScene, render_batch, scenes
    desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
    cam = scenes.cfg1_camera(32, 32)
    fast, ref = GpuScene(desc), GpuScene(desc)  # same light kinds: the same shading build
    kw = dict(spp=8, max_depth=6, seed=5)
    alone, _ = fast.render(cam, traverse=TRAVERSE_FAST, **kw)
    outs, _ = render_batch([fast, ref], [cam, cam],
                           [dict(kw, traverse=TRAVERSE_FAST), dict(kw, traverse=TRAVERSE_REF)])
    np.testing.assert_array_equal(outs[0], alone)


def _reference_cornell_scene():
    """The reference's own Cornell box (demo_pt.cpp:83-414: diffuse walls, an emitter,
    12 mirror and 12 dielectric triangles, IOR 1.33) as exported into the fixtures, with
    the reference SplitBVH tree of the same triangles and demo_pt's camera."""
    from conftest import golden
    from mcrt_gb300 import CameraDesc
    from mcrt_gb300.scene import Material, SceneDesc
    from parity import fixture_tree
    fx = golden("ref_image_cornell.npz")
    verts = fx["verts"]
    mats = [Material(int(t), tuple(float(x) for x in c), ior=1.33) for t, c in zip(fx["mat_types"], fx["mat_colors"])]
    desc = SceneDesc(verts, np.arange(verts.shape[0], dtype=np.int32), mats)
    tfx = golden("ref_traverse_cornell.npz")
    assert np.array_equal(tfx["verts"], verts)
    c = fx["camera"]
    res = fx["batch_means"].shape[1]
    cam = CameraDesc(origin=tuple(float(x) for x in c[0:3]), target=tuple(float(x) for x in c[3:6]), width=res,
                     height=res, fov_y=float(c[6]))
    return fx, desc, cam, fixture_tree(tfx)


@pytest.mark.parametrize("mode", ["ref-tree-REF", "own-tree-FAST"])
def test_reference_cornell_matches_reference_path_tracer(mode, cuda_device):
    """The GPU against the reference's own demo_pt rayTrace image (16 batches of per-pixel
    means stored by the fixture generator), in the reference's semantics: depth 10, no
    Russian roulette, mirror and dielectric (IOR 1.33) boxes.  Independent random numbers:
    per-pixel z-test and image-mean z-test of 8 GPU renders of 256 spp each.

    With the reference tree and its traversal order the coplanar box bottoms and floor
    resolve as in the reference, and the image-mean test is strict.  On the library's own
    tree a ray hitting the floor where a box bottom coincides with it may report the other
    (coplanar) face; that moves the image mean by about 1 %, so the own-tree check bounds
    the image mean to 2 % and keeps the pixel z-test."""
    from mcrt_gb300 import GpuScene, TRAVERSE_FAST, TRAVERSE_REF
    fx, desc, cam, tree = _reference_cornell_scene()
    if mode == "ref-tree-REF":
        sc, traverse = GpuScene(desc, builder="external", external_tree=tree), TRAVERSE_REF
    else:
        sc, traverse = GpuScene(desc), TRAVERSE_FAST
    b = np.stack([sc.render(cam, spp=256, max_depth=10, rr_depth=-1, seed=300 + k, traverse=traverse)[0]
                  for k in range(8)]).astype(np.float64)
    g, gvar = b.mean(axis=0), b.var(axis=0, ddof=1) / b.shape[0]
    ref_b = fx["batch_means"].astype(np.float64)
    ref_mean, ref_var = ref_b.mean(axis=0), ref_b.var(axis=0, ddof=1) / ref_b.shape[0]
    z = (g - ref_mean) / np.sqrt(gvar + ref_var + 1e-12)
    assert np.mean(np.abs(z) > 4) < 0.01, f"{mode}: {np.mean(np.abs(z) > 4):.3f} of pixels beyond 4 sigma"
    res = g.shape[0]
    for c in range(3):
        d = g[..., c].mean() - ref_mean[..., c].mean()
        se = np.sqrt(gvar[..., c].sum() + ref_var[..., c].sum()) / (res * res)
        if mode == "ref-tree-REF":
            assert abs(d / se) < 4.0, f"{mode}: channel {c}: image-mean z = {d / se:.2f}"
        else:
            assert abs(d) < 0.02 * ref_mean[..., c].mean(), f"{mode}: channel {c}: image mean off by {d:.4g}"


def test_phong_crn_matches_float_oracle(cuda_device):
    """GlossyBSDF (the reference's Phong lobe, exponent 25; bsdf.cpp:209-301) on the GPU
    against the oracle's restatement with the same seed: the cfg0 box with a Phong sphere
    and a Phong floor."""
    from mcrt_gb300 import scenes
    from mcrt_gb300 import GpuScene
    from mcrt_gb300.scene import GLSY
    from oracle.oracle import OracleScene
    desc = scenes.cfg0_scene()
    desc.materials[-1].type = GLSY              # the sphere
    desc.materials[-1].color = (0.85, 0.7, 0.5)
    floor = int(desc.material_ids[0])
    desc.materials[floor].type = GLSY
    cam = scenes.cfg0_camera(32, 32)
    gpu, st = GpuScene(desc).render(cam, spp=16, max_depth=8, rr_depth=3, seed=9)
    ref = OracleScene(desc, 32).render(cam.as_array(), 32, 32, 16, 8, 3, seed=9)
    _crn_compare(gpu, ref["mean"].astype(np.float32), "phong")
    _ray_counts_agree(st, ref)


def test_scene_built_through_the_mcrt_api_renders_the_same_image(cuda_device):
    """The reference's Cornell box built with MCRT's calls (mcrt_gb300.mcrt_scene: Scene::add,
    todo_addMaterial, setCamera, finalize) renders bit for bit the image of the same scene
    described directly."""
    from conftest import golden
    from mcrt_gb300.mcrt_scene import Material, Scene, TriangleObject, todo_addMaterial
    fx, desc, cam, _ = _reference_cornell_scene()
    sc = Scene()
    for v, t, c in zip(fx["verts"], fx["mat_types"], fx["mat_colors"]):
        m = todo_addMaterial(Material(tuple(float(x) for x in c), 0.0, int(t)))
        sc.add(TriangleObject(tuple(v[0:3]), tuple(v[3:6]), tuple(v[6:9])), m)
    sc.setCamera(cam.origin, cam.target, cam.width, cam.height, cam.fov_y)
    from mcrt_gb300 import GpuScene
    a, _ = sc.finalize().render(sc.camera(), spp=8, max_depth=10, seed=5)
    b, _ = GpuScene(desc).render(cam, spp=8, max_depth=10, seed=5)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("schedule", [0, 1])
def test_emitter_box_culling_changes_no_pixel(schedule, cuda_device):
    """Next-event rays toward the area lights are culled, bounded and cut short by the box
    of the emitter triangles.  Two point-sized emitters far outside the scene widen that box
    over everything, so nothing is culled, without changing how the lights are sampled:
    they come first in the emitter CDF with probability 0 and are never hit.  The image is
    the same to the bit; only the number of traced next-event rays differs."""
    from mcrt_gb300 import TRAVERSE_FAST, TRAVERSE_REF, GpuScene, scenes
    from mcrt_gb300.scene import LGHT, Material, SceneDesc
    desc = scenes.cfg0_scene()
    cam = scenes.cfg0_camera(48, 48)
    mats = list(desc.materials) + [Material(LGHT, (0.0, 0.0, 0.0))]
    far = np.array([[-50.0] * 9, [50.0] * 9], np.float32)
    up = np.tile(np.array([0.0, 1.0, 0.0], np.float32), (2, 3))
    wide = SceneDesc(np.concatenate([far, desc.vertices]),
                     np.concatenate([np.full(2, len(mats) - 1), desc.material_ids]).astype(np.int32), mats,
                     normals=np.concatenate([up, desc.normals]))
    kw = dict(spp=32, max_depth=8, rr_depth=3, seed=21, schedule=schedule)
    tight, loose = GpuScene(desc), GpuScene(wide)
    for traverse in (TRAVERSE_FAST, TRAVERSE_REF):
        a, sa = tight.render(cam, traverse=traverse, **kw)
        b, sb = loose.render(cam, traverse=traverse, **kw)
        np.testing.assert_array_equal(a, b)
        assert sa["extension_rays"] == sb["extension_rays"]
        assert sa["shadow_rays"] < 0.8 * sb["shadow_rays"], (sa["shadow_rays"], sb["shadow_rays"])


def test_set_materials_keeps_the_emitter_set(cuda_device):
    """New colours are taken without a rebuild; a change of the emitter set (built into the
    light table and the emitter box) or a request for consistent normals the scene was built
    without is refused and changes nothing."""
    import copy
    from mcrt_gb300 import GpuScene, McrtError, scenes
    from mcrt_gb300.scene import CONSISTENT, DIFF, LGHT
    desc = scenes.cfg0_scene()
    sc = GpuScene(desc)
    cam = scenes.cfg0_camera(16, 16)
    before, _ = sc.render(cam, spp=4, max_depth=4, seed=1)
    light = next(i for i, m in enumerate(desc.materials) if m.type == LGHT)
    wall = next(i for i, m in enumerate(desc.materials) if m.type == DIFF)
    for k, t in ((light, DIFF), (wall, LGHT), (wall, DIFF | CONSISTENT), (wall, 77)):
        mats = copy.deepcopy(desc.materials)
        mats[k].type = t
        with pytest.raises(McrtError):
            sc.set_materials(mats)
    after, _ = sc.render(cam, spp=4, max_depth=4, seed=1)
    np.testing.assert_array_equal(before, after)
    mats = copy.deepcopy(desc.materials)
    mats[wall].color = (0.2, 0.3, 0.4)
    sc.set_materials(mats)
    changed, _ = sc.render(cam, spp=4, max_depth=4, seed=1)
    assert not np.array_equal(before, changed)


@pytest.mark.parametrize("w,h,spp,depth", [(1, 1, 1, 0), (3, 2, 1, 1), (7, 5, 3, 0), (16, 9, 2, 3)])
def test_small_and_odd_frames_match_the_oracle(w, h, spp, depth, cuda_device):
    """Frame edges: one pixel, odd sizes, one sample (no tent filter), depth 0 (the camera
    hit and its next-event rays only).  Same random numbers: per pixel the same value up to
    float rounding, and the same extension rays."""
    from mcrt_gb300 import CameraDesc, GpuScene, scenes
    from oracle.oracle import OracleScene
    desc = scenes.cfg0_scene()
    cam = CameraDesc(width=w, height=h, **scenes.CORNELL_CAMERA)
    gpu, st = GpuScene(desc).render(cam, spp=spp, max_depth=depth, rr_depth=-1, seed=5)
    ref = OracleScene(desc, 32).render(cam.as_array(), w, h, spp, depth, -1, seed=5)
    assert gpu.shape == (h, w, 3)
    close = np.isclose(gpu, ref["mean"], rtol=2e-3, atol=1e-4).all(axis=-1)
    assert close.mean() >= (1.0 if w * h < 10 else 0.9), (gpu, ref["mean"])
    assert st["paths"] == w * h * spp
    assert abs(st["extension_rays"] - ref["extension_rays"]) <= max(1, 0.01 * ref["extension_rays"])


@pytest.mark.parametrize("with_env", [False, True])
def test_single_emitter_triangle_and_empty_background(with_env, cuda_device):
    """The smallest scene: one emitter triangle.  Camera rays that hit its front face see
    its radiance, rays that hit its back see nothing, and missed rays see black or, with
    an environment map, the map; the GPU and the oracle agree pixel by pixel."""
    from mcrt_gb300 import CameraDesc, GpuScene, scenes
    from mcrt_gb300.scene import LGHT, Material, SceneDesc
    from oracle.oracle import OracleScene
    v = np.array([[-1.0, -1.0, 0.0, 1.0, -1.0, 0.0, 0.0, 1.0, 0.0]], np.float32)
    env = scenes.sky_envmap(64, 32) if with_env else None
    desc = SceneDesc(v, np.zeros(1, np.int32), [Material(LGHT, (2.0, 3.0, 4.0))], envmap=env)
    for z in (3.0, -3.0):  # the face the camera sees: front, then back
        cam = CameraDesc(origin=(0.0, 0.0, z), target=(0.0, 0.0, 0.0), width=12, height=12, fov_y=50.0)
        gpu, _ = GpuScene(desc).render(cam, spp=2, max_depth=2, seed=3)
        ref = OracleScene(desc, 32).render(cam.as_array(), 12, 12, 2, 2, -1, seed=3)
        np.testing.assert_allclose(gpu, ref["mean"], rtol=2e-3, atol=1e-4)
        lit = np.isclose(gpu, [2.0, 3.0, 4.0], rtol=1e-5).all(axis=-1)
        assert lit.any() == (z > 0)
        if not with_env:  # each of the 2 samples sees the radiance or nothing
            frac = gpu / np.array([2.0, 3.0, 4.0], np.float32)
            np.testing.assert_allclose(frac, np.round(frac * 2) / 2, atol=1e-6)


def _paths_scenes(name):
    from mcrt_gb300 import scenes
    from mcrt_gb300.scene import CONSISTENT, GLSY, SPEC
    if name == "cfg0":
        return scenes.cfg0_scene(), scenes.cfg0_camera(40, 24), dict(spp=6, max_depth=8, rr_depth=3)
    if name == "cfg1-small":  # environment map, GGX and dielectric patches
        desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
        return desc, scenes.cfg1_camera(32, 32), dict(spp=5, max_depth=6)
    desc = scenes.cfg0_scene()  # Phong sphere, consistent-normal mirror floor
    desc.materials[-1].type = GLSY
    desc.materials[int(desc.material_ids[0])].type = SPEC | CONSISTENT
    return desc, scenes.cfg0_camera(32, 32), dict(spp=4, max_depth=8, rr_depth=3)


@pytest.mark.parametrize("name", ["cfg0", "cfg1-small", "phong-mirror"])
def test_plain_path_tracer_renders_the_wavefront_image(name, cuda_device):
    """MCRT_SCHEDULE_PATHS (one thread per path, no queues; chunks of 777 paths rounded to
    pixels) renders the streaming wavefront's image with the same rays.  The two kernels
    run the same arithmetic in the same order, but the compiler may fuse a multiply-add in
    one and not the other: the Cornell box comes out identical to the bit, the environment
    and GGX scene within a few ulp on a few pixels (4e-6 relative at most)."""
    from mcrt_gb300 import TRAVERSE_FAST, TRAVERSE_REF, GpuScene
    desc, cam, kw = _paths_scenes(name)
    sc = GpuScene(desc)
    for traverse in (TRAVERSE_FAST, TRAVERSE_REF) if name == "cfg0" else (TRAVERSE_FAST,):
        a, sa = sc.render(cam, seed=11, traverse=traverse, **kw)
        b, sb = sc.render(cam, seed=11, traverse=traverse, schedule=2, path_chunk=777, **kw)
        if name == "cfg0":
            np.testing.assert_array_equal(a, b)
        close = np.isclose(a, b, rtol=1e-5, atol=1e-6).all(axis=-1)
        assert close.mean() >= 0.995, f"{(~close).sum()} pixels differ"
        for key in ("extension_rays", "shadow_rays"):
            assert abs(sa[key] - sb[key]) <= 1e-3 * sa[key], (key, sa[key], sb[key])
        assert sb["paths"] == cam.width * cam.height * kw["spp"]
