"""The oracle (CPU restatement) pinned against the reference's own outputs (golden
fixtures generated from the compiled reference), and against the reference library
directly where it is available."""
import os
import numpy as np
import pytest

from conftest import golden
from parity import TRAVERSE_SETS, classify


@pytest.fixture(scope="module")
def orc():
    from oracle.oracle import load_restatement
    return load_restatement()


def _f(x):
    return np.ascontiguousarray(x, np.float32)


def test_material_sample_and_evaluate_match_reference(orc):
    import ctypes
    fx = golden("ref_functions.npz")
    wi, nl, r, col = fx["mat_wi"], fx["mat_nl"], fx["mat_r"], fx["mat_color"]
    for ty in (1, 2, 3, 4):
        wo = np.zeros(3, np.float32)
        w = np.zeros(3, np.float32)
        f = np.zeros(3, np.float32)
        pdf = ctypes.c_float()
        got_wo, got_w, got_pdf, got_f, got_epdf = [], [], [], [], []
        ewo = _f(fx[f"mat{ty}_eval_wo"])  # keep alive: ctypes takes a raw pointer
        for i in range(wi.shape[0]):
            orc.orc_material_sample(ty, col[i].ctypes.data, 1.0, 1.33, wi[i].ctypes.data, nl[i].ctypes.data,
                                    float(r[i, 0]), float(r[i, 1]), wo.ctypes.data, w.ctypes.data, ctypes.byref(pdf))
            got_wo.append(wo.copy())
            got_w.append(w.copy())
            got_pdf.append(pdf.value)
            orc.orc_material_evaluate(ty, col[i].ctypes.data, 1.0, 1.33, wi[i].ctypes.data, nl[i].ctypes.data,
                                      ewo[i].ctypes.data, f.ctypes.data, ctypes.byref(pdf))
            got_f.append(f.copy())
            got_epdf.append(pdf.value)
        # the sampled directions and weights only involve sqrt and the platform's sinf/cosf/powf
        np.testing.assert_allclose(np.array(got_wo), fx[f"mat{ty}_wo"], rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(np.array(got_w), fx[f"mat{ty}_weight"], rtol=2e-5, atol=1e-6)
        np.testing.assert_allclose(np.array(got_pdf), fx[f"mat{ty}_pdf"], rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(np.array(got_f), fx[f"mat{ty}_eval_f"], rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(np.array(got_epdf), fx[f"mat{ty}_eval_pdf"], rtol=2e-5, atol=1e-7)
        # the restatement follows the reference's float/double evaluation: bit-exact
        assert np.array_equal(np.array(got_wo, np.float32), fx[f"mat{ty}_wo"])
        assert np.array_equal(np.array(got_w, np.float32), fx[f"mat{ty}_weight"])
        assert np.array_equal(np.array(got_pdf, np.float32), fx[f"mat{ty}_pdf"])


def test_fresnel_frame_warp_camera_exact(orc):
    fx = golden("ref_functions.npz")
    got = np.array([orc.orc_fresnel(float(c), float(i)) for c, i in zip(fx["fresnel_cos"], fx["fresnel_ior"])],
                   np.float32)
    assert np.array_equal(got, fx["fresnel"])
    n, c = fx["onb_n"], fx["onb_c"]
    out = np.zeros(3, np.float32)
    world = []
    for i in range(n.shape[0]):
        orc.orc_onb_to_world(_f(n[i]).ctypes.data, _f(c[i]).ctypes.data, out.ctypes.data)
        world.append(out.copy())
    assert np.array_equal(np.array(world), fx["onb_world"])
    hs = []
    for x, y in fx["mat_r"]:
        orc.orc_sample_hemisphere_cosine(float(x), float(y), out.ctypes.data)
        hs.append(out.copy())
    assert np.array_equal(np.array(hs), fx["cosine_hemisphere"])
    cam = fx["camera"]
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    ds = []
    for mx, my in fx["camera_m"]:
        orc.orc_camera_ray(_f(cam).ctypes.data, 320, 240, float(mx), float(my), o.ctypes.data, d.ctypes.data)
        ds.append(d.copy())
    assert np.array_equal(np.array(ds), fx["camera_d"])


def test_discrete_sampler_and_triangle_sampling_exact(orc):
    import ctypes
    fx = golden("ref_functions.npz")
    w = _f(fx["discrete_w"])
    pdf = ctypes.c_float()
    idx, pd = [], []
    for r in fx["discrete_r"]:
        idx.append(orc.orc_discrete_sample(w.ctypes.data, w.size, float(r), ctypes.byref(pdf)))
        pd.append(pdf.value)
    assert np.array_equal(np.array(idx), fx["discrete_idx"])
    assert np.array_equal(np.array(pd, np.float32), fx["discrete_pdf"])
    # the zero-weight bin is never chosen
    assert 5 not in set(idx)


def test_envmap_pdf_radiance_and_sample_texel(orc):
    fx = golden("ref_functions.npz")
    env = _f(fx["env"])
    h = orc.orc_envmap_create(env.ctypes.data, env.shape[1], env.shape[0])
    try:
        pdf = np.array([orc.orc_envmap_pdf(h, _f(d).ctypes.data) for d in fx["env_dirs"]], np.float32)
        assert np.array_equal(pdf, fx["env_pdf"])
        rad = np.zeros(3, np.float32)
        rads = []
        for d in fx["env_dirs"]:
            orc.orc_envmap_radiance(h, _f(d).ctypes.data, rad.ctypes.data)
            rads.append(rad.copy())
        assert np.array_equal(np.array(rads), fx["env_rad"])
        # EnvmapLoader::sample draws two hidden randf() for the texel jitter: the chosen texel,
        # its pdf and radiance are determined by (r1, r2); the direction lies inside it
        import ctypes
        W, H = env.shape[1], env.shape[0]
        ui, vi = ctypes.c_int(), ctypes.c_int()
        for i, (r1, r2) in enumerate(fx["mat_r"]):
            orc.orc_envmap_sample_texel(h, float(r1), float(r2), ctypes.byref(ui), ctypes.byref(vi))
            d = fx["env_sample_dir"][i].astype(np.float64)
            phi = np.arccos(np.clip(d[1], -1, 1))
            th = np.arctan2(d[0], -d[2]) % (2 * np.pi)
            assert abs(phi / np.pi * H - (vi.value + 0.5)) <= 0.5 + 1e-3
            du = (th / (2 * np.pi) * W - (ui.value + 0.5) + W / 2) % W - W / 2
            assert abs(du) <= 0.5 + 1e-3
            assert fx["env_sample_pdf"][i] > 0
    finally:
        orc.orc_envmap_destroy(h)


@pytest.mark.parametrize("name", ["cornell", "cfg0", "sphere5", "debugmesh", "debugmesh_diag"])
def test_oracle_closest_hits_match_reference(name):
    from oracle.oracle import OracleScene
    from parity import fixture_scene
    fx = golden(f"ref_traverse_{name}.npz")
    osc = OracleScene(fixture_scene(fx), 32)
    for k in TRAVERSE_SETS:
        if f"rays_{k}" not in fx.files:
            continue
        rays = fx[f"rays_{k}"]
        t, p = osc.trace(rays)
        bad, _ = classify(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], t, p)
        assert not bad.any(), f"{name}/{k}: {bad.sum()} mismatches"


def _reference_cornell():
    """The reference's Cornell box (demo_pt.cpp:83-414) as exported into the fixtures,
    with the reference SplitBVH tree of the same triangles."""
    from oracle.oracle import OracleScene
    from mcrt_gb300.scene import Material, SceneDesc
    from parity import fixture_tree
    fx = golden("ref_image_cornell.npz")
    verts = fx["verts"]
    mt, mc = fx["mat_types"], fx["mat_colors"]
    mats = [Material(int(t), tuple(float(x) for x in c)) for t, c in zip(mt, mc)]
    desc = SceneDesc(verts, np.arange(verts.shape[0], dtype=np.int32), mats)
    cam7 = fx["camera"]
    cam = np.concatenate([cam7[:6], [0, 1, 0], cam7[6:]]).astype(np.float32)
    tfx = golden("ref_traverse_cornell.npz")
    assert np.array_equal(tfx["verts"], verts)
    return desc, cam, fixture_tree(tfx), OracleScene


def test_oracle_replays_reference_path_tracer_bit_exactly():
    """Fed the reference's own random stream (std::default_random_engine through
    uniform_real_distribution<float>, drawn in demo_pt's order) and traversing the
    reference's own tree, the float restatement reproduces every sample of the
    reference rayTrace bit for bit."""
    desc, cam, tree, OracleScene = _reference_cornell()
    px = golden("ref_paths_cornell.npz")
    res, spp = int(px["res"]), int(px["spp"])
    out = OracleScene(desc, 32).set_reference_tree(tree).render(cam, res, res, spp, 10, -1, ref_stream=1,
                                                                keep_paths=True)
    assert np.array_equal(out["paths"], px["paths"])


def test_oracle_image_matches_reference_path_tracer():
    """The float restatement in reference semantics (depth 10, no RR, IOR 1.33, NEE at
    Lambert vertices only, the reference tree) on the reference's own Cornell box vs the
    reference's demo_pt rayTrace, independent random numbers: z-test on batch means."""
    desc, cam, tree, OracleScene = _reference_cornell()
    fx = golden("ref_image_cornell.npz")
    res = fx["batch_means"].shape[1]
    ref_b = fx["batch_means"].astype(np.float64)
    ref_mean = ref_b.mean(axis=0)
    ref_var = ref_b.var(axis=0, ddof=1) / ref_b.shape[0]
    out = OracleScene(desc, 32).set_reference_tree(tree).render(cam, res, res, 2048, 10, -1, seed=5)
    z = (out["mean"] - ref_mean) / np.sqrt(out["var_of_mean"] + ref_var + 1e-12)
    assert np.mean(np.abs(z) > 4) < 0.01, f"{np.mean(np.abs(z) > 4):.3f} beyond 4 sigma"
    for c in range(3):
        d = out["mean"][..., c].mean() - ref_mean[..., c].mean()
        se = np.sqrt(out["var_of_mean"][..., c].sum() + ref_var[..., c].sum()) / (res * res)
        assert abs(d / se) < 4.0, f"channel {c}: image-mean z = {d / se:.2f}"


def test_fp64_and_fp32_oracles_agree_path_by_path():
    from mcrt_gb300 import scenes
    from oracle.oracle import OracleScene
    desc = scenes.cfg0_scene()
    cam = scenes.cfg0_camera(16, 16).as_array()
    a = OracleScene(desc, 32).render(cam, 16, 16, 8, 8, 3, seed=2, keep_paths=True)["paths"]
    b = OracleScene(desc, 64).render(cam, 16, 16, 8, 8, 3, seed=2, keep_paths=True)["paths"]
    rel = np.abs(a - b) / (np.abs(b) + 1e-3)
    assert np.mean(rel < 1e-4) > 0.97


def test_oracle_against_reference_library_directly():
    """Where the reference is compiled here, call it directly on fresh random inputs."""
    from oracle.oracle import load_reference
    ref = load_reference()
    if ref is None:
        pytest.skip("reference sources not present on this machine (fixtures cover it)")
    import ctypes
    from oracle.oracle import load_restatement
    orc = load_restatement()
    rng = np.random.default_rng(99)
    for _ in range(500):
        wi = _f(rng.normal(size=3))
        wi /= np.linalg.norm(wi)
        nl = _f(rng.normal(size=3))
        nl /= np.linalg.norm(nl)
        col = _f(rng.uniform(0, 1, 3))
        r1, r2 = rng.uniform(size=2)
        for ty in (1, 2, 3):
            a_wo, a_w, b_wo, b_w = (np.zeros(3, np.float32) for _ in range(4))
            p1, p2, c1 = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
            ref.ref_material_sample(ty, col.ctypes.data, wi.ctypes.data, nl.ctypes.data, float(r1), float(r2),
                                    a_wo.ctypes.data, a_w.ctypes.data, ctypes.byref(p1), ctypes.byref(c1))
            orc.orc_material_sample(ty, col.ctypes.data, 1.0, 1.33, wi.ctypes.data, nl.ctypes.data, float(r1),
                                    float(r2), b_wo.ctypes.data, b_w.ctypes.data, ctypes.byref(p2))
            assert np.array_equal(a_w, b_w)
            np.testing.assert_allclose(a_wo, b_wo, rtol=1e-6, atol=1e-7)


def test_film_writers_and_tonemaps_match_reference():
    """The oracle's restatement of film.cpp against the reference's own FrameBuffer:
    dumpHDR / dumpPPM byte for byte, tonemapGamma / tonemapReinhard bit for bit."""
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_film.npz"))
    k = 0
    while f"img{k}" in g:
        img = g[f"img{k}"]
        assert O.film_encode(img, True) == g[f"hdr{k}"].tobytes(), f"hdr {k}"
        assert O.film_encode(img, False) == g[f"ppm{k}"].tobytes(), f"ppm {k}"
        np.testing.assert_array_equal(O.film_tonemap(img, False, 2.2), g[f"gamma{k}"])
        np.testing.assert_array_equal(O.film_tonemap(img, True), g[f"reinhard{k}"])
        k += 1
    assert k == 5


def test_consistent_normal_matches_reference():
    """TriangleObject::consistentNormal (triangle.cpp:149-182) restated by the oracle: the
    normal, the consistent reflection and its cosine, bit for bit on 2,000 random cases."""
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_consistent.npz"))
    lib = O.load_restatement()
    abc, nabc, alpha, wi, u, v, want = (np.ascontiguousarray(g[k]) for k in ("abc", "nabc", "alpha", "wi", "u", "v",
                                                                             "out"))
    got = np.zeros_like(want)
    for i in range(want.shape[0]):
        o = np.zeros(7, np.float32)
        rows = [np.ascontiguousarray(x[i]) for x in (abc, nabc, alpha, wi)]
        lib.orc_consistent_normal(*[O.ptr(r) for r in rows], float(u[i]), float(v[i]), O.ptr(o))
        got[i] = o
    np.testing.assert_array_equal(got, want)


def test_linear_scan_matches_the_oracle_tree():
    """The oracle's linear scan (the reference's DebugMesh rule) and its tree traversal give
    the same closest hits on 20,000 random rays against 1000 random triangles."""
    from mcrt_gb300.scene import DIFF, Material, SceneDesc
    from oracle.oracle import OracleScene
    rng = np.random.default_rng(3)
    verts = rng.uniform(-1, 1, (1000, 9)).astype(np.float32)
    orc = OracleScene(SceneDesc(verts, np.zeros(1000, np.int32), [Material(DIFF, (0.5, 0.5, 0.5))]), 32)
    n = 20000
    d = rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    rays[:, 3] = 1e-4
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    t_lin, p_lin = orc.linear_trace(rays, threads=4)
    t_bvh, p_bvh = orc.trace(rays)
    assert np.array_equal(p_lin, p_bvh)
    hit = p_lin >= 0
    assert np.array_equal(t_lin[hit], t_bvh[hit]) and hit.mean() > 0.5
