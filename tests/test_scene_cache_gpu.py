"""Scene cache files: save, load (bit-identical renders), and rejection of files written
for another description, of damaged and of truncated files."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(sc, cam):
    img, st = sc.render(cam, spp=4, max_depth=6, seed=3)
    return img, st


def test_saved_scene_loads_and_renders_identically(cuda_device, tmp_path):
    from mcrt_gb300 import GpuScene, scenes
    desc = scenes.cfg1_scene(level=5, env_size=(256, 128), patch_tris=64)
    cam = scenes.cfg1_camera(48, 40)
    a = GpuScene(desc)
    path = tmp_path / "scene.mcrt"
    a.save(str(path))
    b = GpuScene.load(str(path), desc)
    assert a.info() == b.info()
    ia, sa = _render(a, cam)
    ib, sb = _render(b, cam)
    np.testing.assert_array_equal(ia, ib)
    assert sa["rays"] == sb["rays"]
    # REF traversal (reference-layout tree) survives the round trip too
    t1, _ = a.render(cam, spp=2, max_depth=4, seed=9, traverse=1)
    t2, _ = b.render(cam, spp=2, max_depth=4, seed=9, traverse=1)
    np.testing.assert_array_equal(t1, t2)


def test_cache_for_another_description_is_rejected(cuda_device, tmp_path):
    from mcrt_gb300 import GpuScene, McrtError, scenes
    path = tmp_path / "scene.mcrt"
    GpuScene(scenes.cfg0_scene()).save(str(path))
    with pytest.raises(McrtError, match="hash"):
        GpuScene.load(str(path), scenes.cfg0_scene(sphere_level=3))
    GpuScene.load(str(path))  # no expected description: accepted


def test_damaged_and_truncated_files_are_rejected(cuda_device, tmp_path):
    from mcrt_gb300 import GpuScene, McrtError, scenes
    path = tmp_path / "scene.mcrt"
    GpuScene(scenes.cfg0_scene()).save(str(path))
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.mcrt"
    raw2 = bytearray(raw)
    raw2[len(raw2) // 2] ^= 0x40
    bad.write_bytes(bytes(raw2))
    with pytest.raises(McrtError, match="corrupt"):
        GpuScene.load(str(bad))
    bad.write_bytes(bytes(raw[: len(raw) - 100]))
    with pytest.raises(McrtError):
        GpuScene.load(str(bad))
    bad.write_bytes(b"not a scene")
    with pytest.raises(McrtError, match="not a scene cache"):
        GpuScene.load(str(bad))


def test_cached_builds_once_then_loads(cuda_device, tmp_path):
    from mcrt_gb300 import GpuScene, scenes
    desc = scenes.cfg0_scene()
    path = tmp_path / "c.mcrt"
    a = GpuScene.cached(desc, str(path))
    assert path.exists()
    b = GpuScene.cached(desc, str(path))
    cam = scenes.cfg0_camera(32, 32)
    np.testing.assert_array_equal(_render(a, cam)[0], _render(b, cam)[0])
