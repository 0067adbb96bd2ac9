"""The .mscene reader (host C++ in libmpcore.so) and writer on the CPU:
round trips, the transform conventions of Scene.cpp, rejection of malformed
files, and the reference's own packed test scenes when its tree is present."""
import os

import numpy as np
import pytest

from micropolis_gb300 import _lib, mscene, scenes


def _ref_scenes():
    """The reference's packed scenes, where its tree is present (the one
    oracle/build_ref.sh compiled the pin from)."""
    from oracle import oracle
    d = oracle.reference_dir()
    return os.path.join(d, "testscene") if d else ""


REF_SCENES = _ref_scenes()


def _records():
    sc = scenes.mixed4096_1920x1080(n=64, width=256, height=256)
    meshes, objects, cams = mscene.records_from_scene(sc, mscene.camera_from_view(sc.draws[0].mv))
    objects[1].transform = mscene.Transform((0.5, -1.0, 2.0), (np.cos(0.3), 0.0, np.sin(0.3), 0.0))
    objects[1].color = (0.25, 0.5, 0.75)
    lights = [mscene.LightRecord("sun", color=(1, 0.9, 0.8), intensity=2.0)]
    return meshes, objects, cams, lights


def test_round_trip(built):
    meshes, objects, cams, lights = _records()
    s = mscene.SceneFile.parse(mscene.encode_mscene(meshes, objects, cams, lights))
    assert s.counts() == (2, 2, 1, 1)
    for a, b in zip(s.meshes(), meshes):
        assert a.name == b.name and a.type == b.type
        assert np.array_equal(a.positions.view(np.uint32), np.asarray(b.positions, np.float32).view(np.uint32))
    objs = s.objects()
    assert [o[0] for o in objs] == ["object0", "object1"] and [o[1] for o in objs] == [0, 1]
    assert np.array_equal(objs[0][2], np.eye(4, dtype=np.float32).reshape(-1))
    assert np.allclose(objs[1][3], [0.25, 0.5, 0.75, 1.0])
    name, cm, near, far, fovy = s.cameras()[0]
    assert name == "camera" and near == np.float32(cams[0].near) and fovy == np.float32(cams[0].fovy)
    assert far == np.float32(1000.0)


def test_transform_conventions(built):
    """translate(t) * mat4_cast(q) column major; modelview = inverse(camera) * object."""
    meshes, objects, cams, _ = _records()
    s = mscene.SceneFile.parse(mscene.encode_mscene(meshes, objects, cams))
    _, _, m, _ = s.objects()[1]
    a = 0.6   # q = (cos 0.3, 0, sin 0.3, 0): rotation by 0.6 rad about y
    want = np.array([[np.cos(a), 0, np.sin(a), 0.5], [0, 1, 0, -1.0], [-np.sin(a), 0, np.cos(a), 2.0], [0, 0, 0, 1]])
    assert np.allclose(m.reshape(4, 4).T, want, atol=1e-6)
    cam = s.cameras()[0][1].reshape(4, 4).T.astype(np.float64)
    mv = s.modelview(0, 1).reshape(4, 4).T
    assert np.allclose(mv, np.linalg.inv(cam) @ m.reshape(4, 4).T.astype(np.float64), atol=1e-5)
    sc = scenes.mixed4096_1920x1080(n=64, width=256, height=256)
    assert np.abs(s.modelview(0, 0) - sc.draws[0].mv).max() < 1e-5


def test_malformed_inputs_are_rejected(built):
    meshes, objects, cams, lights = _records()
    data = mscene.encode_mscene(meshes, objects, cams, lights)
    for bad in (b"", b"\x00", data[:len(data) // 2], b"\xff" * 9, bytes(64)):
        with pytest.raises(_lib.MpError) as e:
            mscene.SceneFile.parse(bad)
        assert e.value.status == _lib.MP_ERR_INVALID_ARG
    rng = np.random.default_rng(7)
    arr = np.frombuffer(data, np.uint8)
    for _ in range(300):   # corrupted bytes: decoded or rejected, never a crash
        c = arr.copy()
        idx = rng.integers(0, len(c), size=4)
        c[idx] = rng.integers(0, 256, size=4)
        try:
            s = mscene.SceneFile.parse(c.tobytes())
            s.meshes(), s.objects(), s.cameras()
        except _lib.MpError as e:
            assert e.status == _lib.MP_ERR_INVALID_ARG
    with pytest.raises(_lib.MpError):
        mscene.SceneFile.load("/nonexistent/scene.mscene")


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference test scenes not present")
def test_reference_scenes_decode(built):
    """The reference's packed scenes (written by the Cap'n Proto library)."""
    want = {"teapot.mscene": (1, 0, 32), "teapot_greg.mscene": (1, 1, 32), "killeroo.mscene": (1, 0, 11532),
            "eye_split.mscene": (1, 1, 1)}
    for f, (n_mesh, typ, patches) in want.items():
        s = mscene.SceneFile.load(os.path.join(REF_SCENES, f))
        ms = s.meshes()
        assert len(ms) == n_mesh and ms[0].type == typ
        assert len(ms[0].positions) == patches * (48 if typ == 0 else 60)
        assert np.all(np.isfinite(ms[0].positions))
        assert len(s.cameras()) >= 1 and all(o[1] >= 0 for o in s.objects())
    s = mscene.SceneFile.load(os.path.join(REF_SCENES, "killeroos.mscene"))
    assert s.counts()[1] == 20
    for f in sorted(os.listdir(REF_SCENES)):
        if f.endswith(".mscene"):
            s = mscene.SceneFile.load(os.path.join(REF_SCENES, f))
            for m in s.meshes():
                assert len(m.positions) % (48 if m.type == 0 else 60) == 0
            sc = s.to_scene(640, 480)
            assert sc.n_patches > 0
