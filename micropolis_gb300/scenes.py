"""Seeded synthetic scenes standing in for the reference's .mscene inputs.

Each scene is a list of draws (mesh, modelview, colour) plus a camera, in the
layout the reference's renderer consumes: Bezier meshes hold 16 xyz control
points per patch (P[i][j] = point 4*i + j, src/base/Patch.h:24-27), Gregory
meshes 20 (p[0..3], ep[0..3], em[0..3], fp[0..3], fm[0..3],
tools/mscene_export.py:245).  A Gregory patch is made from a Bezier one with
the index map of tools/bez2mscene_greg.py:111.

Workloads (named by what they are):
  heightfield_1024x768    8x8 Bezier heightfield, 1024x768, split limit 8
  mixed4096_1920x1080     4096 patches, half Bezier half Gregory, 1920x1080
  views64_512x512         64 independent scenes of 100..10000 patches
  heightfield16_512x512   16x16 heightfield with displacement (gradients)
  heightfield512_3840x2160  512x512 fractal heightfield at 4K, split limit 4
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

BEZIER = 0
GREGORY = 1

# tools/bez2mscene_greg.py:111 -- 16-point Bezier patch -> 20-point Gregory patch
BEZIER_TO_GREGORY = np.array([0, 3, 15, 12, 1, 7, 14, 8, 4, 2, 11, 13, 5, 6, 10, 9, 5, 6, 10, 9])


@dataclasses.dataclass
class Mesh:
    type: int                 # BEZIER or GREGORY
    cp: np.ndarray            # float32 [n_patches, 16 | 20, 3]

    @property
    def n_patches(self) -> int:
        return int(self.cp.shape[0])


@dataclasses.dataclass
class Draw:
    mesh: Mesh
    mv: np.ndarray            # float32 [16], column-major modelview (glm layout)
    color: tuple = (1.0, 1.0, 1.0, 1.0)
    view: int = 0             # framebuffer layer (batched views)


@dataclasses.dataclass
class Scene:
    name: str
    width: int
    height: int
    draws: list
    fovy: float = 60.0
    near: float = 0.01
    options: dict = dataclasses.field(default_factory=dict)
    seed: int = 0

    @property
    def n_patches(self) -> int:
        return sum(d.mesh.n_patches for d in self.draws)


def look_at(eye, center, up) -> np.ndarray:
    """Right-handed view matrix (the camera inverse of src/micropolis/Scene.cpp:190),
    returned column-major as float32[16]."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(center, np.float64) - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -s @ eye
    m[1, 3] = -u @ eye
    m[2, 3] = f @ eye
    return m.T.reshape(-1).astype(np.float32)


def heightfield_mesh(n: int, z: np.ndarray, extent: float = 1.0) -> Mesh:
    """n x n Bezier patches over [-extent, extent]^2 sharing border control
    points (C0): one (3n+1)^2 control grid with heights z."""
    g = 3 * n + 1
    xs = np.linspace(-extent, extent, g)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    grid = np.stack([X, Y, z.reshape(g, g)], axis=-1)
    cp = np.empty((n * n, 16, 3), np.float64)
    for a in range(n):
        for b in range(n):
            # P[i][j] with i along y and j along x keeps the +z side front-facing
            blk = grid[3 * b:3 * b + 4, 3 * a:3 * a + 4]          # [x, y]
            cp[a * n + b] = blk.transpose(1, 0, 2).reshape(16, 3)  # i = y, j = x
    return Mesh(BEZIER, cp.astype(np.float32))


def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z)
    r[:, 0, 1] = 2 * (x * y - z * w)
    r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w)
    r[:, 1, 1] = 1 - 2 * (x * x + z * z)
    r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w)
    r[:, 2, 1] = 2 * (y * z + x * w)
    r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def scattered_patches(rng, n: int, gregory: bool) -> Mesh:
    """Planar 4x4 patches, centres U[-10,10]^3, side lognormal(-1, 1), random
    orientation, every control point jittered N(0, 0.1*side)."""
    centre = rng.uniform(-10, 10, size=(n, 3))
    scale = rng.lognormal(mean=-1.0, sigma=1.0, size=n)
    rot = _random_rotations(rng, n)
    t = np.arange(4) / 3.0 - 0.5
    I, J = np.meshgrid(t, t, indexing="ij")
    planar = np.stack([J.reshape(-1), I.reshape(-1), np.zeros(16)], axis=-1)  # [16, 3]
    pts = np.einsum("nij,kj->nki", rot, planar) * scale[:, None, None] + centre[:, None, :]
    if gregory:
        pts = pts[:, BEZIER_TO_GREGORY, :]
    pts = pts + rng.normal(size=pts.shape) * (0.1 * scale)[:, None, None]
    return Mesh(GREGORY if gregory else BEZIER, pts.astype(np.float32))


def heightfield_1024x768(seed: int = 1234) -> Scene:
    rng = np.random.default_rng(seed)
    n = 8
    z = rng.uniform(-0.2, 0.2, size=(3 * n + 1) ** 2)
    mesh = heightfield_mesh(n, z)
    mv = look_at((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1))
    return Scene("heightfield_1024x768", 1024, 768, [Draw(mesh, mv, (0.9, 0.7, 0.3, 1.0))],
                 options=dict(bound_n_split_limit=8.0, reyes_patch_size=8, reyes_patches_per_pass=1024),
                 seed=seed)


# Camera distance for the mixed scene, chosen so that the mean depth
# complexity (covered fragments / frame pixels) is about 6.
MIXED_CAMERA_DISTANCE = 13.0


def mixed4096_1920x1080(seed: int = 1235, n: int = 4096, width: int = 1920, height: int = 1080,
                        distance: float = MIXED_CAMERA_DISTANCE) -> Scene:
    rng = np.random.default_rng(seed)
    bez = scattered_patches(rng, n // 2, gregory=False)
    greg = scattered_patches(rng, n - n // 2, gregory=True)
    eye = np.array([0.6, -0.8, 0.35])
    eye = eye / np.linalg.norm(eye) * distance
    mv = look_at(eye, (0, 0, 0), (0, 0, 1))
    return Scene("mixed4096_1920x1080", width, height,
                 [Draw(bez, mv, (0.9, 0.6, 0.3, 1.0)), Draw(greg, mv, (0.3, 0.7, 0.9, 1.0))],
                 options=dict(bound_n_split_limit=8.0, reyes_patch_size=8), seed=seed)


def fibonacci_sphere(n: int, radius: float) -> np.ndarray:
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    theta = math.pi * (1 + 5 ** 0.5) * i
    return radius * np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], -1)


def views64_512x512(seed: int = 1236, n_views: int = 64, size: int = 512) -> Scene:
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(100), np.log(10000), size=n_views)).astype(int)
    eyes = fibonacci_sphere(n_views, 15.0)
    draws = []
    for v in range(n_views):
        mesh = scattered_patches(rng, int(counts[v]), gregory=False)
        up = (0, 0, 1) if abs(eyes[v][2]) < 14.5 else (0, 1, 0)
        draws.append(Draw(mesh, look_at(eyes[v], (0, 0, 0), up), (0.8, 0.8, 0.8, 1.0), view=v))
    return Scene("views64_512x512", size, size, draws,
                 options=dict(bound_n_split_limit=8.0, batch_views=n_views), seed=seed)


def heightfield16_512x512(seed: int = 1237) -> Scene:
    rng = np.random.default_rng(seed)
    n = 16
    z = rng.uniform(-0.2, 0.2, size=(3 * n + 1) ** 2)
    mesh = heightfield_mesh(n, z)
    mv = look_at((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1))
    return Scene("heightfield16_512x512", 512, 512, [Draw(mesh, mv, (0.9, 0.7, 0.3, 1.0))],
                 options=dict(bound_n_split_limit=8.0, reyes_patch_size=8, displacement=1,
                              displacement_amplitude=1.0), seed=seed)


def value_noise_fbm(rng, g: int, octaves: int = 4, amplitude: float = 0.3, lacunarity: float = 2.0,
                    base_cells: int = 8) -> np.ndarray:
    """Fractal value noise on a g x g grid: bilinear lattice noise, octaves
    summed with frequency x lacunarity and amplitude x 0.5 per octave."""
    out = np.zeros((g, g))
    x = np.linspace(0, 1, g)
    amp = amplitude
    cells = base_cells
    for _ in range(octaves):
        lat = rng.uniform(-1, 1, size=(int(cells) + 2, int(cells) + 2))
        u = x * cells
        i0 = np.floor(u).astype(int)
        f = u - i0
        a = lat[i0][:, i0]
        b = lat[i0 + 1][:, i0]
        c = lat[i0][:, i0 + 1]
        d = lat[i0 + 1][:, i0 + 1]
        fx = f[:, None]
        fy = f[None, :]
        out += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        amp *= 0.5
        cells *= lacunarity
    return out


def heightfield512_3840x2160(seed: int = 1238, n: int = 512, width: int = 3840, height: int = 2160) -> Scene:
    rng = np.random.default_rng(seed)
    g = 3 * n + 1
    z = value_noise_fbm(rng, g)
    mesh = heightfield_mesh(n, z)
    mv = look_at((0.0, -1.9, 0.9), (0, 0, 0), (0, 0, 1))
    return Scene("heightfield512_3840x2160", width, height, [Draw(mesh, mv, (0.9, 0.7, 0.3, 1.0))],
                 options=dict(bound_n_split_limit=4.0, reyes_patch_size=8, displacement=1,
                              displacement_amplitude=1.0), seed=seed)


WORKLOADS = {
    "heightfield_1024x768": heightfield_1024x768,
    "mixed4096_1920x1080": mixed4096_1920x1080,
    "views64_512x512": views64_512x512,
    "heightfield16_512x512": heightfield16_512x512,
    "heightfield512_3840x2160": heightfield512_3840x2160,
}
