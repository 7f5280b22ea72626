"""MCRT's scene-building calls (mcrt_gb300.mcrt_scene) describe the same scene as the
library's own description: the reference's Cornell box built triangle by triangle, and an
OBJ added with Scene::loadModel, on the CPU (no GPU: the description, not the upload)."""
import numpy as np
import pytest

from conftest import golden


def test_triangles_materials_camera_as_the_reference_api_builds_them(tmp_path):
    from mcrt_gb300 import McrtError, scenes
    from mcrt_gb300.mcrt_scene import Material, Scene, TriangleObject, todo_addMaterial
    fx = golden("ref_image_cornell.npz")
    sc = Scene()
    with pytest.raises(McrtError):
        sc.desc()
    ids = [todo_addMaterial(Material(tuple(float(x) for x in c), 0.0, int(t)))
           for t, c in zip(fx["mat_types"], fx["mat_colors"])]
    for v, m in zip(fx["verts"], ids):
        sc.add(TriangleObject(tuple(v[0:3]), tuple(v[3:6]), tuple(v[6:9])), m)
    c = fx["camera"]
    sc.setCamera(c[0:3], c[3:6], 32, 32, c[6])
    env = scenes.sky_envmap(16, 8, sun_diameter_deg=6.0, sun_radiance=5.0)
    scenes.write_envmap_bin(str(tmp_path / "env.bin"), env)
    sc.setEnvmap(str(tmp_path / "env.bin"))
    d = sc.desc()
    assert sc.numTrangles() == fx["verts"].shape[0]
    np.testing.assert_array_equal(d.vertices, fx["verts"].astype(np.float32))
    assert d.normals is None  # face normals left to the library, as the reference computes them
    types = np.array([d.materials[k].type for k in d.material_ids])
    np.testing.assert_array_equal(types, fx["mat_types"])
    np.testing.assert_array_equal(d.envmap, env.astype(np.float32))
    assert sc.camera().width == 32 and sc.camera().fov_y == pytest.approx(float(c[6]))


def test_load_model_adds_the_obj_with_a_new_material(tmp_path):
    from mcrt_gb300.mcrt_scene import SPEC, Material, Scene, todo_getMaterial
    g = golden("ref_obj.npz")
    p = tmp_path / "mesh.obj"
    p.write_bytes(g["obj"].tobytes())
    sc = Scene()
    sc.loadModel(str(p), g["transform"], Material((0.9, 0.9, 0.9), 0.0, SPEC))
    d = sc.desc()
    np.testing.assert_array_equal(d.vertices, g["verts"])
    np.testing.assert_array_equal(d.normals, g["normals"])
    assert len(d.materials) == 1 and d.materials[0].type == SPEC
    from mcrt_gb300 import mcrt_scene
    assert todo_getMaterial(len(mcrt_scene._mat_lib) - 1).type == SPEC
