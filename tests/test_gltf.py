"""glTF input (inmyroom_vulkan_gb300.gltf): the draw-mode expansion of
CreateIndicesTriplets (src/Geometry/Triangle.cpp:10-58), a save/load round
trip, and, where the reference checkout is present, its sample scenes
(testGames/SnakeGame Apple and Table_room) loaded and built into trees by the
oracle. No device involved."""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import gltf, scenes
from oracle import REF_ROOT_DEFAULT

SNAKE = os.path.join(REF_ROOT_DEFAULT, "inMyRoom_vulkan", "testGames", "SnakeGame")


def test_triplets_by_mode():
    idx = np.array([10, 11, 12, 13, 14])
    assert gltf.triplets(idx[:3], 4).tolist() == [[10, 11, 12]]
    # strip: (i, i + 1 + i % 2, i + 2 - i % 2)
    assert gltf.triplets(idx, 5).tolist() == [[10, 11, 12], [11, 13, 12], [12, 13, 14]]
    # fan: (i + 1, i + 2, 0)
    assert gltf.triplets(idx, 6).tolist() == [[11, 12, 10], [12, 13, 10], [13, 14, 10]]
    assert gltf.triplets(idx[:4], 1).tolist() == [[10, 10, 11], [12, 12, 13]]
    assert gltf.triplets(idx[:3], 3).tolist() == [[10, 10, 11], [11, 11, 12]]
    assert gltf.triplets(idx[:2], 0).tolist() == [[10, 10, 10], [11, 11, 11]]
    assert gltf.triplets(idx, 2).shape == (0, 3)


def test_round_trip(tmp_path):
    sc = scenes.scene(n_entities=6)
    meshes = [gltf.Mesh(f"m{k}", m.points, m.normals if k % 2 == 0 else None, m.indices)
              for k, m in enumerate(sc.meshes)]
    inst = [gltf.Instance(k, sc.mats[k], f"e{k}") for k in range(6)]
    path = str(tmp_path / "scene.gltf")
    gltf.save(path, gltf.Scene(meshes, inst))
    back = gltf.load(path)
    assert len(back.meshes) == 6 and len(back.instances) == 6
    for a, b in zip(meshes, back.meshes):
        assert np.array_equal(a.points, b.points)
        assert np.array_equal(np.asarray(a.indices).reshape(-1, 3), b.indices)
        assert (a.normals is None) == (b.normals is None)
        if a.normals is not None:
            assert np.array_equal(a.normals, b.normals)
    for a, b in zip(inst, back.instances):
        assert a.mesh == b.mesh and np.array_equal(a.matrix, b.matrix)


@pytest.mark.skipif(not os.path.isdir(SNAKE), reason="the reference's sample assets are not here")
def test_sample_scenes(port):
    for name, min_tris in (("Apple", 500), ("Table_room", 5000)):
        sc = gltf.load(os.path.join(SNAKE, name, "scene.gltf"))
        assert sc.instances
        total = 0
        for m in sc.meshes:
            if not m.n_tris:
                continue  # skinned meshes: no tree, as in the engine
            assert m.indices.max() < len(m.points)
            assert np.isfinite(m.points).all()
            t = port.tree_build(m.points, m.indices, m.normals)
            n, tris = t.sizes()
            assert tris == m.n_tris
            total += m.n_tris
        assert total >= min_tris, (name, total)
        for inst in sc.instances:
            assert np.isfinite(inst.matrix).all()
