"""Hit parity of the CUDA traversal against the reference SplitBVH, through the C ABI."""
import os
import numpy as np
import pytest

from conftest import golden
from parity import TRAVERSE_SETS, classify, fixture_scene, fixture_tree, mt_terms

FIXTURES = ["cornell", "cfg0", "sphere5", "debugmesh", "debugmesh_diag"]

pytestmark = pytest.mark.gpu


def _scene(fx, builder):
    from mcrt_gb300 import GpuScene
    desc = fixture_scene(fx)
    if builder == "external":
        return GpuScene(desc, builder="external", external_tree=fixture_tree(fx))
    return GpuScene(desc, builder=builder)


def _sets(fx):
    return [k for k in TRAVERSE_SETS if f"rays_{k}" in fx.files]


@pytest.mark.parametrize("name", FIXTURES)
def test_ref_mode_bit_exact_on_reference_tree(name, cuda_device):
    """Same BVH (the reference's own SplitBVH tree), same rays: identical prim, t, u, v."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, "external")
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_REF)
        prim = out[:, 3].view(np.int32)
        ref_p = fx[f"prim_{k}"]
        assert np.array_equal(prim, ref_p), f"{name}/{k}: {np.sum(prim != ref_p)} prim mismatches"
        hit = ref_p >= 0
        assert np.array_equal(out[hit, 0].view(np.int32), fx[f"t_{k}"][hit].view(np.int32)), f"{name}/{k}: t"
        assert np.array_equal(out[hit, 1].view(np.int32), fx[f"u_{k}"][hit].view(np.int32)), f"{name}/{k}: u"
        assert np.array_equal(out[hit, 2].view(np.int32), fx[f"v_{k}"][hit].view(np.int32)), f"{name}/{k}: v"


@pytest.mark.parametrize("name", FIXTURES)
def test_ref_mode_occluded_matches_scenebvh(name, cuda_device):
    """SceneBVH::occluded(ray, tfar) = a hit in [1e-4, tfar - 1e-4] (scenebvh.cpp:379-396)."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, "external")
    for k in _sets(fx):
        rays = fx[f"rays_{k}"].copy()
        rays[:, 3] = np.float32(1e-4)
        rays[:, 7] = (rays[:, 7] - np.float32(1e-4)).astype(np.float32)
        occ = sc.trace_any(rays, TRAVERSE_REF)
        assert np.array_equal(occ, fx[f"occ_{k}"]), f"{name}/{k}: {np.sum(occ != fx[f'occ_{k}'])} mismatches"


@pytest.mark.parametrize("builder", ["external", "sah", "sah_split"])
@pytest.mark.parametrize("name", FIXTURES)
def test_fast_mode_nonmarginal(name, builder, cuda_device):
    """Watertight FP32 traversal: same prim and t within 4 ulp on every non-marginal ray."""
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden(f"ref_traverse_{name}.npz")
    sc = _scene(fx, builder)
    total = 0
    marginal_total = 0
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_FAST)
        bad, marginal = classify(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], out[:, 0],
                                 out[:, 3].view(np.int32))
        assert not bad.any(), f"{name}/{k}/{builder}: {bad.sum()} non-marginal mismatches, e.g. ray {np.argmax(bad)}"
        total += rays.shape[0]
        if k != "axis":
            marginal_total += int(marginal.sum())
    # marginal disagreements stay rare apart from the zero-direction rays
    assert marginal_total <= max(8, total // 200), f"{marginal_total} marginal disagreements of {total}"


@pytest.mark.parametrize("builder", ["external", "sah"])
def test_ref_mode_own_builder_closest_hit(builder, cuda_device):
    """Reference arithmetic on the library's own tree: the closest hit is tree-independent."""
    from mcrt_gb300 import TRAVERSE_REF
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, builder)
    for k in _sets(fx):
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_REF)
        bad, _ = classify(fx["verts"], rays, fx[f"t_{k}"], fx[f"prim_{k}"], out[:, 0], out[:, 3].view(np.int32))
        assert not bad.any()


def test_fast_any_hit_matches_occluded(cuda_device):
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, "sah")
    for k in ["primary", "incoherent", "segment"]:
        rays = fx[f"rays_{k}"].copy()
        rays[:, 3] = np.float32(1e-4)
        rays[:, 7] = (rays[:, 7] - np.float32(1e-4)).astype(np.float32)
        occ = sc.trace_any(rays, TRAVERSE_FAST)
        diff = occ != fx[f"occ_{k}"]
        # disagreements only on rays whose reference closest hit is marginal
        assert diff.sum() <= max(2, rays.shape[0] // 1000), f"{k}: {diff.sum()}"


def test_device_pointer_path(cuda_device):
    """Rays and hits resident in device memory (torch tensors) give the same answer."""
    import torch
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, "sah")
    rays = fx["rays_incoherent"]
    host = sc.trace_closest(rays, TRAVERSE_FAST)
    dev = sc.trace_closest(torch.from_numpy(rays).to(cuda_device), TRAVERSE_FAST).cpu().numpy()
    assert np.array_equal(host.view(np.int32), dev.view(np.int32))


def test_empty_and_single_ray(cuda_device):
    from mcrt_gb300 import TRAVERSE_FAST, TRAVERSE_REF
    fx = golden("ref_traverse_cornell.npz")
    sc = _scene(fx, "external")
    assert sc.trace_closest(np.zeros((0, 8), np.float32)).shape == (0, 4)
    r = fx["rays_primary"][:1]
    for mode in (TRAVERSE_FAST, TRAVERSE_REF):
        out = sc.trace_closest(r, mode)
        assert out[0, 3].view(np.int32) == fx["prim_primary"][0]


def test_l2_read_probe(cuda_device):
    """The L2 roofline denominator: a plausible bandwidth, above the HBM copy rate of this
    class of GPU (several TB/s) and below any L2's (100 TB/s)."""
    import ctypes
    from mcrt_gb300 import _native as N
    lib = N.load()
    g = ctypes.c_float(0.0)
    N.check(lib.mcrt_probe_l2_read(48 << 20, 20, ctypes.byref(g), None), "mcrt_probe_l2_read")
    assert 3000.0 < g.value < 100000.0, g.value


def _chain_tree(n):
    """A chain-shaped binary tree over n triangles: inner node i holds triangle i's leaf on
    the left and inner node i + 1 on the right, so the tree is n - 1 levels deep."""
    v = np.zeros((n, 3, 3), np.float32)
    x = np.arange(n, dtype=np.float32)
    v[:, 0, 0], v[:, 1, 0], v[:, 2, 0] = x, x + 0.5, x
    v[:, 1, 1], v[:, 2, 2] = 0.5, 0.5
    lo, hi = v.min(axis=1), v.max(axis=1)
    inner, leaves = n - 1, n
    node_box = np.zeros((inner + leaves, 6), np.float32)
    node_info = np.zeros((inner + leaves, 6), np.int32)
    for i in range(inner):
        right = i + 1 if i + 1 < inner else inner + n - 1
        node_box[i] = np.concatenate([lo[i:].min(axis=0), hi[i:].max(axis=0)])
        node_info[i] = (0, inner + i, right, 0, 0, 0)
    for k in range(leaves):
        node_box[inner + k] = np.concatenate([lo[k], hi[k]])
        node_info[inner + k] = (1, -1, -1, 0, k, 1)
    tree = dict(node_box=node_box, node_info=node_info, ref_prim=np.arange(n, dtype=np.int32),
                ref_box=np.concatenate([lo, hi], axis=1))
    return v, tree


def test_tree_deeper_than_the_stack_is_refused_before_any_launch(cuda_device):
    """An external tree deeper than the 64-entry traversal stack: trace and render calls fail
    on the host with MCRT_ERR_STACK_OVERFLOW before any kernel is launched, and the scene is
    destroyed cleanly."""
    from mcrt_gb300 import GpuScene, scenes
    from mcrt_gb300 import _native as N
    from mcrt_gb300.scene import DIFF, Material, SceneDesc
    v, tree = _chain_tree(80)
    sc = GpuScene(SceneDesc(v, np.zeros(80, np.int32), [Material(DIFF)]), builder="external", external_tree=tree)
    rays = np.zeros((4, 8), np.float32)
    rays[:, 0:3] = (0.25, 0.1, -1.0)
    rays[:, 3] = 1e-4
    rays[:, 6] = 1.0
    rays[:, 7] = np.inf
    for call in (lambda: sc.trace_closest(rays), lambda: sc.trace_any(rays),
                 lambda: sc.render(scenes.cfg0_camera(8, 8), spp=1, max_depth=2)):
        with pytest.raises(N.McrtError) as e:
            call()
        assert "stack overflow" in str(e.value) and "deeper" in str(e.value), str(e.value)
    sc.close()


@pytest.fixture(scope="module")
def cfg1_hits():
    """The 1.31 M-triangle geometry of the large configuration (regenerated here and checked
    against the fixture's SHA-256) with the reference SplitBVH's answers."""
    import hashlib
    from mcrt_gb300 import GpuScene, scenes
    fx = golden("ref_traverse_cfg1.npz")
    desc = scenes.cfg1_scene()
    verts = np.ascontiguousarray(desc.vertices, np.float32)
    assert hashlib.sha256(verts.tobytes()).hexdigest() == str(fx["verts_sha256"]), "cfg1 geometry differs"
    return fx, verts, GpuScene(desc)


CFG1_SETS = ["primary", "bounce", "incoherent", "segment"]


def test_fast_mode_nonmarginal_at_1_3m_triangles(cfg1_hits, cuda_device):
    """The hit contract at full scale: on the library's own tree of the 1,310,722-triangle
    scene, the watertight traversal returns the reference SplitBVH's prim with t within 4 ulp
    on every non-marginal ray, 65,536 rays per class.  At this scale the reference's absolute
    |det| < 1e-6 cull rejects grazing hits on the ~4.7e-3 edges, and the FAST test applies
    the same cull."""
    from mcrt_gb300 import TRAVERSE_FAST
    fx, verts, sc = cfg1_hits
    report = {}
    for k in CFG1_SETS:
        rays = fx[f"rays_{k}"]
        out = sc.trace_closest(rays, TRAVERSE_FAST)
        bad, marginal = classify(verts, rays, fx[f"t_{k}"], fx[f"prim_{k}"], out[:, 0], out[:, 3].view(np.int32))
        assert not bad.any(), f"cfg1/{k}: {bad.sum()} non-marginal mismatches, e.g. ray {np.argmax(bad)}"
        report[k] = int(marginal.sum())
        assert marginal.sum() <= rays.shape[0] // 200, f"cfg1/{k}: {marginal.sum()} marginal disagreements"
    print("marginal disagreements per 65,536 rays:", report)


def test_fast_any_hit_matches_occluded_at_1_3m_triangles(cfg1_hits, cuda_device):
    """SceneBVH::occluded(ray, tfar) on the full-scale scene: the any-hit traversal over
    [1e-4, tfar - 1e-4] agrees with the reference except on rays whose reference closest hit
    is marginal or lies within 4 ulp of the bound."""
    from mcrt_gb300 import TRAVERSE_FAST
    from parity import ulp_diff
    fx, verts, sc = cfg1_hits
    for k in CFG1_SETS:
        rays = fx[f"rays_{k}"].copy()
        rays[:, 3] = np.float32(1e-4)
        rays[:, 7] = (rays[:, 7] - np.float32(1e-4)).astype(np.float32)
        occ = sc.trace_any(rays, TRAVERSE_FAST)
        diff = occ != fx[f"occ_{k}"].astype(np.int32)
        if diff.any():
            got = sc.trace_closest(fx[f"rays_{k}"], TRAVERSE_FAST)
            _, marginal = classify(verts, fx[f"rays_{k}"], fx[f"t_{k}"], fx[f"prim_{k}"], got[:, 0],
                                   got[:, 3].view(np.int32))
            near_bound = (fx[f"prim_{k}"] >= 0) & (ulp_diff(fx[f"t_{k}"], rays[:, 7]) <= 4)
            unexplained = diff & ~marginal & ~near_bound
            assert unexplained.sum() <= max(2, rays.shape[0] // 5000), f"cfg1/{k}: {unexplained.sum()} of {diff.sum()}"


def test_concurrent_host_buffer_calls_on_the_default_stream(cuda_device):
    """Several host threads tracing with host buffers on the default stream at once (what
    the SceneBVH backend does under the reference's OpenMP loops): every call gets its own
    hits, equal to one batched call's."""
    from concurrent.futures import ThreadPoolExecutor
    from mcrt_gb300 import TRAVERSE_FAST
    fx = golden("ref_traverse_cfg0.npz")
    sc = _scene(fx, "sah")
    rays = fx["rays_incoherent"][:2048]
    want = sc.trace_closest(rays, TRAVERSE_FAST)
    want_occ = sc.trace_any(rays, TRAVERSE_FAST)
    chunks = [(i, min(i + s, rays.shape[0])) for i, s in zip(range(0, rays.shape[0], 7), [1, 3, 7] * 1000)]

    def one(c):
        a, b = c
        return a, b, sc.trace_closest(rays[a:b], TRAVERSE_FAST), sc.trace_any(rays[a:b], TRAVERSE_FAST)

    with ThreadPoolExecutor(max_workers=8) as ex:
        for a, b, got, occ in ex.map(one, chunks):
            assert np.array_equal(got.view(np.int32), want[a:b].view(np.int32)), (a, b)
            assert np.array_equal(occ, want_occ[a:b]), (a, b)


def test_ref_mode_bit_exact_at_1_3m_triangles(cfg1_hits, cuda_device):
    """REF mode at full scale: the reference's own SplitBVH of the 1,310,722 triangles,
    built here by the reference's code (oracle/_ref, about a minute), traversed on the GPU in
    the reference's order and arithmetic: prim, t, u and v identical to the reference's
    SplitBVH::intersect on every ray of the four classes, and prim and t identical to the
    fixture's (made on another machine from the same sources)."""
    import ctypes
    from mcrt_gb300 import GpuScene, TRAVERSE_REF
    from mcrt_gb300.scene import DIFF, Material, SceneDesc
    from oracle.oracle import load_reference, ptr
    ref = load_reference()
    if ref is None:
        pytest.skip("the reference build (oracle/_ref) is not present")
    fx, verts, _ = cfg1_hits
    h = ref.ref_bvh_create(ptr(verts), verts.shape[0], 0)
    try:
        nn, nr = ctypes.c_int(), ctypes.c_int()
        ref.ref_bvh_dump_sizes(h, ctypes.byref(nn), ctypes.byref(nr))
        tree = dict(node_box=np.zeros((nn.value, 6), np.float32), node_info=np.zeros((nn.value, 6), np.int32),
                    ref_prim=np.zeros(nr.value, np.int32), ref_box=np.zeros((nr.value, 6), np.float32))
        ref.ref_bvh_dump(h, ptr(tree["node_box"]), ptr(tree["node_info"]), ptr(tree["ref_prim"]), ptr(tree["ref_box"]))
        sc = GpuScene(SceneDesc(verts, np.zeros(verts.shape[0], np.int32), [Material(DIFF)]), builder="external",
                      external_tree=tree)
        for k in CFG1_SETS:
            rays = np.ascontiguousarray(fx[f"rays_{k}"])
            n = rays.shape[0]
            t, p, u, v = (np.zeros(n, np.float32), np.zeros(n, np.int32), np.zeros(n, np.float32),
                          np.zeros(n, np.float32))
            ref.ref_bvh_intersect(h, ptr(rays), n, ptr(t), ptr(p), ptr(u), ptr(v), os.cpu_count() or 1)
            out = sc.trace_closest(rays, TRAVERSE_REF)
            prim = out[:, 3].view(np.int32)
            assert np.array_equal(prim, p), f"cfg1/{k}: {np.sum(prim != p)} prim mismatches"
            hit = p >= 0
            for c, want in ((0, t), (1, u), (2, v)):
                assert np.array_equal(out[hit, c].view(np.int32), want[hit].view(np.int32)), f"cfg1/{k}: column {c}"
            assert np.array_equal(p, fx[f"prim_{k}"]), f"cfg1/{k}: the reference's hits differ from the fixture's"
            assert np.array_equal(t[hit].view(np.int32), fx[f"t_{k}"][hit].view(np.int32))
        sc.close()
    finally:
        ref.ref_bvh_destroy(h)


@pytest.mark.parametrize("traverse", [0, 1])
def test_linear_scan_known_answer_1m_rays(traverse, cuda_device):
    """The reference's own known-answer check at its full size (demo_splitbvh.cpp:194-238):
    1,000,000 rays from U[-1,1]^3 in directions normalize(U[-0.5,0.5]^3) against 1000
    random triangles, closest-hit t compared with a linear scan of every triangle
    (DebugMesh::intersect, debug_mesh.cpp:780-809) by the reference's own rule |dt| < 1e-6
    (checkEqual, demo_splitbvh.cpp:62-65; both missing counts as agreement).  On the
    library's own tree, in REF and FAST traversal: the reference's rule met on all but 1 in
    10,000 rays, and the same triangle on every non-marginal ray unless the two triangles'
    hits (in double) lie within that same 1e-6.  Random triangles cross one another: a ray
    near a crossing meets two of them at nearly the same t, and float Moller-Trumbore, whose
    t is accurate to a few ulp of the coordinates (not of a small t), may order them either
    way (1 ray in 10^6 here, 88 float ulp of t apart)."""
    from mcrt_gb300 import GpuScene
    from mcrt_gb300.scene import DIFF, Material, SceneDesc
    from oracle.oracle import OracleScene
    rng = np.random.default_rng(194238)
    verts = rng.uniform(-1, 1, (1000, 9)).astype(np.float32)
    desc = SceneDesc(verts, np.zeros(1000, np.int32), [Material(DIFF, (0.5, 0.5, 0.5))])
    n = 1_000_000
    d = rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    rays[:, 3] = 1e-4  # Ray::s_ray_epsilon = NUM_EPS_RAY (ray.cpp:8)
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    t_lin, p_lin = OracleScene(desc, 32).linear_trace(rays)
    out = GpuScene(desc).trace_closest(rays, traverse)
    t_gpu, p_gpu = out[:, 0], out[:, 3].view(np.int32)
    agree = ((p_lin < 0) & (p_gpu < 0)) | ((p_lin >= 0) & (p_gpu >= 0) & (np.abs(t_gpu - t_lin) < 1e-6))
    assert (p_lin >= 0).mean() > 0.5
    bad, marginal = classify(verts, rays, t_lin, p_lin, t_gpu, p_gpu)
    _, _, t_a = mt_terms(verts, p_lin, rays)
    _, _, t_b = mt_terms(verts, p_gpu, rays)
    tie = (p_lin >= 0) & (p_gpu >= 0) & (np.abs(t_a - t_b) < 1e-6)
    bad &= ~tie
    assert not bad.any(), f"{bad.sum()} non-marginal mismatches, e.g. ray {np.argmax(bad)}"
    assert (~agree).sum() <= n // 10000, f"{(~agree).sum()} of {n} rays outside |dt| < 1e-6"
