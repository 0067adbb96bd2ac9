"""The reference's .mscene scene files (src/micropolis/mscene.capnp).

`SceneFile` reads one through libmpcore.so (the decoder is host C++,
micropolis_gb300/csrc/mp_scene.cu) and either draws it the way
Reyes::Scene::draw does (src/micropolis/Scene.cpp:179-197) or converts it to
a `scenes.Scene` for the oracle and the tests.  `write_mscene` writes the
same format (Cap'n Proto packed, one segment), the counterpart of
Scene::save (Scene.cpp:200-294).
"""
from __future__ import annotations

import ctypes
import dataclasses
import struct
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import MpError, lib


@dataclasses.dataclass
class MeshRecord:
    name: str
    type: int                 # 0 Bezier, 1 Gregory
    positions: np.ndarray     # float32, 3 per point


@dataclasses.dataclass
class Transform:
    translation: Sequence[float] = (0.0, 0.0, 0.0)
    rotation: Sequence[float] = (1.0, 0.0, 0.0, 0.0)   # quaternion (r, i, j, k)


@dataclasses.dataclass
class ObjectRecord:
    name: str
    meshname: str
    transform: Transform = dataclasses.field(default_factory=Transform)
    color: Sequence[float] = (1.0, 1.0, 1.0)


@dataclasses.dataclass
class CameraRecord:
    name: str
    transform: Transform = dataclasses.field(default_factory=Transform)
    near: float = 0.01
    far: float = 1000.0
    fovy: float = 60.0


@dataclasses.dataclass
class LightRecord:
    name: str
    transform: Transform = dataclasses.field(default_factory=Transform)
    color: Sequence[float] = (1.0, 1.0, 1.0)
    intensity: float = 1.0
    type: int = 1             # point, directional, hemi


def _ck(st: int, what: str) -> None:
    if st != _lib.MP_OK:
        raise MpError(st, what)


class SceneFile:
    """A decoded .mscene scene (host memory, owned by libmpcore.so)."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @classmethod
    def load(cls, path: str) -> "SceneFile":
        h = ctypes.c_void_p()
        _ck(lib().mp_scene_load(path.encode(), ctypes.byref(h)), f"cannot read scene {path}")
        return cls(h)

    @classmethod
    def parse(cls, data: bytes) -> "SceneFile":
        h = ctypes.c_void_p()
        _ck(lib().mp_scene_parse(data, len(data), ctypes.byref(h)), "not a packed .mscene message")
        return cls(h)

    def close(self) -> None:
        if self._h:
            lib().mp_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def counts(self):
        c = [ctypes.c_int32() for _ in range(4)]
        _ck(lib().mp_scene_counts(self._h, *[ctypes.byref(x) for x in c]), "scene")
        return tuple(x.value for x in c)   # meshes, objects, cameras, lights

    def meshes(self) -> List[MeshRecord]:
        out = []
        for i in range(self.counts()[0]):
            name, typ = ctypes.c_char_p(), ctypes.c_int32()
            xyz, n = ctypes.POINTER(ctypes.c_float)(), ctypes.c_int64()
            _ck(lib().mp_scene_mesh(self._h, i, ctypes.byref(name), ctypes.byref(typ), ctypes.byref(xyz),
                                    ctypes.byref(n)), "mesh")
            pos = np.ctypeslib.as_array(xyz, shape=(n.value,)).copy() if n.value else np.zeros(0, np.float32)
            out.append(MeshRecord(name.value.decode(errors="replace"), typ.value, pos))
        return out

    def objects(self):
        """(name, mesh index, 4x4 column-major matrix as float32[16], colour rgba)."""
        out = []
        for i in range(self.counts()[1]):
            name, mesh = ctypes.c_char_p(), ctypes.c_int32()
            m = np.zeros(16, np.float32)
            c = np.zeros(4, np.float32)
            _ck(lib().mp_scene_object(self._h, i, ctypes.byref(name), ctypes.byref(mesh),
                                      m.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                      c.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "object")
            out.append((name.value.decode(errors="replace"), mesh.value, m, c))
        return out

    def cameras(self):
        """(name, matrix float32[16], near, far, fovy in degrees)."""
        out = []
        for i in range(self.counts()[2]):
            name = ctypes.c_char_p()
            m = np.zeros(16, np.float32)
            nf = [ctypes.c_float() for _ in range(3)]
            _ck(lib().mp_scene_camera(self._h, i, ctypes.byref(name), m.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                      *[ctypes.byref(x) for x in nf]), "camera")
            out.append((name.value.decode(errors="replace"), m, nf[0].value, nf[1].value, nf[2].value))
        return out

    def modelview(self, camera: int, obj: int) -> np.ndarray:
        mv = np.zeros(16, np.float32)
        _ck(lib().mp_scene_modelview(self._h, camera, obj, mv.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
            "modelview")
        return mv

    def draw(self, renderer, camera: int = 0) -> None:
        """Reyes::Scene::draw through the C ABI (one prepare ... finish)."""
        renderer._ck(lib().mp_scene_draw(renderer._ctx, self._h, camera))

    def to_scene(self, width: int, height: int, camera: int = 0, name: str = "mscene"):
        """A scenes.Scene with the same draws (one per object with a mesh)."""
        from . import scenes
        meshes = self.meshes()
        cams = self.cameras()
        mesh_objs = {}
        draws = []
        for k, (oname, mi, _, color) in enumerate(self.objects()):
            if mi < 0:
                continue
            if mi not in mesh_objs:
                m = meshes[mi]
                per = 16 if m.type == 0 else 20
                mesh_objs[mi] = scenes.Mesh(m.type, m.positions.reshape(-1, per, 3).copy())
            draws.append(scenes.Draw(mesh_objs[mi], self.modelview(camera, k), tuple(float(x) for x in color)))
        _, _, near, _, fovy = cams[camera]
        return scenes.Scene(name, width, height, draws, fovy=fovy, near=near)


# ----------------------------------------------------------------------------
# writer: Cap'n Proto message (one segment), packed

class _Builder:
    """Words of one segment; structs, lists and text laid out in order."""

    def __init__(self):
        self.words: List[int] = [0]          # word 0: the root pointer

    def alloc(self, n: int) -> int:
        at = len(self.words)
        self.words.extend([0] * n)
        return at

    def struct_ptr(self, at_ptr: int, target: int, dwords: int, pwords: int) -> None:
        off = target - at_ptr - 1
        self.words[at_ptr] = ((off << 2) & 0xffffffff) | (dwords << 32) | (pwords << 48)

    def list_ptr(self, at_ptr: int, target: int, size_code: int, count: int) -> None:
        off = target - at_ptr - 1
        self.words[at_ptr] = ((off << 2) & 0xffffffff) | 1 | (size_code << 32) | (count << 35)

    def set_bytes(self, word_at: int, byte_off: int, data: bytes) -> None:
        raw = bytearray(b"".join(w.to_bytes(8, "little") for w in self.words[word_at:word_at + (byte_off + len(data) + 7) // 8]))
        raw[byte_off:byte_off + len(data)] = data
        for k in range(len(raw) // 8):
            self.words[word_at + k] = int.from_bytes(raw[8 * k:8 * k + 8], "little")

    def struct(self, at_ptr: int, dwords: int, pwords: int) -> int:
        s = self.alloc(dwords + pwords)
        self.struct_ptr(at_ptr, s, dwords, pwords)
        return s

    def struct_list(self, at_ptr: int, n: int, dwords: int, pwords: int) -> List[int]:
        tag = self.alloc(1 + n * (dwords + pwords))
        self.list_ptr(at_ptr, tag, 7, n * (dwords + pwords))
        self.words[tag] = ((n << 2) & 0xffffffff) | (dwords << 32) | (pwords << 48)
        return [tag + 1 + k * (dwords + pwords) for k in range(n)]

    def text(self, at_ptr: int, s: str) -> None:
        data = s.encode() + b"\0"
        t = self.alloc((len(data) + 7) // 8)
        self.list_ptr(at_ptr, t, 2, len(data))
        self.set_bytes(t, 0, data)

    def floats(self, at_ptr: int, values: np.ndarray) -> None:
        data = np.ascontiguousarray(values, "<f4").tobytes()
        t = self.alloc((len(data) + 7) // 8)
        self.list_ptr(at_ptr, t, 4, len(data) // 4)
        if data:
            padded = data + b"\0" * (-len(data) % 8)
            for k in range(len(padded) // 8):
                self.words[t + k] = int.from_bytes(padded[8 * k:8 * k + 8], "little")

    def f32s(self, s: int, values: Sequence[float]) -> None:
        self.set_bytes(s, 0, struct.pack("<%df" % len(values), *values))

    def transform(self, at_ptr: int, t: Transform) -> None:
        tr = self.struct(at_ptr, 0, 2)
        v = self.struct(tr, 2, 0)
        self.f32s(v, list(t.translation))
        q = self.struct(tr + 1, 2, 0)
        self.f32s(q, list(t.rotation))

    def vec3(self, at_ptr: int, c: Sequence[float]) -> None:
        v = self.struct(at_ptr, 2, 0)
        self.f32s(v, list(c))


def _pack(words: List[int]) -> bytes:
    out = bytearray()
    i, n = 0, len(words)
    while i < n:
        w = words[i].to_bytes(8, "little")
        tag = 0
        for b in range(8):
            if w[b]:
                tag |= 1 << b
        out.append(tag)
        out.extend(x for x in w if x)
        i += 1
        if tag == 0:
            run = 0
            while i < n and words[i] == 0 and run < 255:
                run += 1
                i += 1
            out.append(run)
        elif tag == 0xFF:
            out.append(0)   # no raw run: every following word is tagged on its own
    return bytes(out)


def encode_mscene(meshes: Sequence[MeshRecord], objects: Sequence[ObjectRecord], cameras: Sequence[CameraRecord],
                  lights: Sequence[LightRecord] = ()) -> bytes:
    """The packed message Scene::save writes for these records (field layout
    of src/micropolis/mscene.capnp)."""
    b = _Builder()
    root = b.struct(0, 0, 4)
    ms = b.struct_list(root + 0, len(meshes), 1, 2)
    for s, m in zip(ms, meshes):
        b.text(s + 1, m.name)
        b.set_bytes(s, 0, struct.pack("<H", int(m.type)))
        b.floats(s + 2, np.asarray(m.positions, np.float32).reshape(-1))
    ls = b.struct_list(root + 1, len(lights), 1, 3)
    for s, l in zip(ls, lights):
        b.text(s + 1, l.name)
        b.transform(s + 2, l.transform)
        b.vec3(s + 3, l.color)
        b.set_bytes(s, 0, struct.pack("<fH", float(l.intensity), int(l.type)))
    os_ = b.struct_list(root + 2, len(objects), 0, 4)
    for s, o in zip(os_, objects):
        b.text(s + 0, o.name)
        b.transform(s + 1, o.transform)
        b.text(s + 2, o.meshname)
        b.vec3(s + 3, o.color)
    cs = b.struct_list(root + 3, len(cameras), 2, 2)
    for s, c in zip(cs, cameras):
        b.text(s + 2, c.name)
        b.transform(s + 3, c.transform)
        b.f32s(s, [c.near, c.far, c.fovy])
    seg = b.words
    frame = [len(seg) << 32]              # segment count - 1 = 0, then the segment's size
    return _pack(frame + seg)


def write_mscene(path: str, meshes, objects, cameras, lights=()) -> None:
    with open(path, "wb") as f:
        f.write(encode_mscene(meshes, objects, cameras, lights))


def records_from_scene(scene, camera_transform: Optional[Transform] = None):
    """Mesh and object records for a scenes.Scene whose draws each use their
    own mesh with an identity object transform; the modelview of draw 0 is
    carried by the camera, which must be a rigid motion."""
    meshes, objects = [], []
    seen = {}
    for k, d in enumerate(scene.draws):
        key = id(d.mesh)
        if key not in seen:
            seen[key] = "mesh%d" % len(meshes)
            meshes.append(MeshRecord(seen[key], int(d.mesh.type), d.mesh.cp.reshape(-1)))
        objects.append(ObjectRecord("object%d" % k, seen[key], Transform(), tuple(d.color[:3])))
    cam = CameraRecord("camera", camera_transform or Transform(), near=scene.near, fovy=scene.fovy)
    return meshes, objects, [cam]


def camera_from_view(mv) -> Transform:
    """The camera transform (translation + unit quaternion) whose inverse is
    the rigid view matrix mv (column-major float[16])."""
    m = np.asarray(mv, np.float64).reshape(4, 4).T          # row-major view matrix
    cam = np.linalg.inv(m)
    r = cam[:3, :3]
    t = cam[:3, 3]
    # rotation matrix -> quaternion (Shepperd's method)
    tr = np.trace(r)
    if tr > 0:
        s = np.sqrt(tr + 1.0) * 2
        w, x, y, z = 0.25 * s, (r[2, 1] - r[1, 2]) / s, (r[0, 2] - r[2, 0]) / s, (r[1, 0] - r[0, 1]) / s
    elif r[0, 0] > r[1, 1] and r[0, 0] > r[2, 2]:
        s = np.sqrt(1.0 + r[0, 0] - r[1, 1] - r[2, 2]) * 2
        w, x, y, z = (r[2, 1] - r[1, 2]) / s, 0.25 * s, (r[0, 1] + r[1, 0]) / s, (r[0, 2] + r[2, 0]) / s
    elif r[1, 1] > r[2, 2]:
        s = np.sqrt(1.0 + r[1, 1] - r[0, 0] - r[2, 2]) * 2
        w, x, y, z = (r[0, 2] - r[2, 0]) / s, (r[0, 1] + r[1, 0]) / s, 0.25 * s, (r[1, 2] + r[2, 1]) / s
    else:
        s = np.sqrt(1.0 + r[2, 2] - r[0, 0] - r[1, 1]) * 2
        w, x, y, z = (r[1, 0] - r[0, 1]) / s, (r[0, 2] + r[2, 0]) / s, (r[1, 2] + r[2, 1]) / s, 0.25 * s
    return Transform(tuple(float(v) for v in t), (float(w), float(x), float(y), float(z)))
