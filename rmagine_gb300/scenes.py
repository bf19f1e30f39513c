"""Procedural meshes and pose sets (seeded, float32), the inputs of the workloads.

* gen_cube: the 12-triangle unit cube of rmagine's genCube
  (src/rmagine_core/src/util/synthetic.cpp:183-221): the same 8 vertices and
  12 faces in the same order, so face ids agree with the reference's.
* box_room: a closed axis-aligned room plus random boxes (a plain LiDAR scene).
* terrain: a heightfield of fractional-Brownian-motion value noise plus boxes
  standing on it (the large-mesh scene).
* euler_to_quat: EulerAngles -> Quaternion (math/types/EulerAngles.tcc:40-61).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .sensors import cosf, sinf

F32 = np.float32

# genCube: 8 corners of the +-0.5 cube, then 12 triangles.
_CUBE_V = np.array([
    [-0.5, -0.5, -0.5], [-0.5, -0.5, 0.5], [-0.5, 0.5, 0.5], [-0.5, 0.5, -0.5],
    [0.5, 0.5, -0.5], [0.5, 0.5, 0.5], [0.5, -0.5, 0.5], [0.5, -0.5, -0.5],
], np.float32)
_CUBE_F = np.array([
    [0, 1, 2], [2, 3, 0],
    [4, 5, 6], [6, 7, 4],
    [0, 7, 1], [1, 7, 6], [1, 6, 5], [5, 2, 1], [2, 5, 4], [3, 2, 4], [3, 4, 7], [3, 7, 0],
], np.uint32)


def gen_cube():
    """Unit cube centred at the origin: (vertices [8,3] float32, faces [12,3] uint32)."""
    return _CUBE_V.copy(), _CUBE_F.copy()


def box_mesh(lo, hi):
    """Axis-aligned box [lo, hi] with the cube's topology."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    v = lo + (_CUBE_V + F32(0.5)) * (hi - lo)
    return v.astype(np.float32), _CUBE_F.copy()


def merge(meshes):
    vs, fs, off = [], [], 0
    for v, f in meshes:
        vs.append(np.asarray(v, np.float32))
        fs.append(np.asarray(f, np.uint32) + np.uint32(off))
        off += len(v)
    return np.concatenate(vs).astype(np.float32), np.concatenate(fs).astype(np.uint32)


def boxes_mesh(centers_xy, base_z, edges):
    """Many boxes at once: centre (x, y), bottom z, edge lengths (ex, ey, ez)."""
    n = len(centers_xy)
    lo = np.empty((n, 3), np.float32)
    hi = np.empty((n, 3), np.float32)
    lo[:, 0] = centers_xy[:, 0] - edges[:, 0] / 2
    hi[:, 0] = centers_xy[:, 0] + edges[:, 0] / 2
    lo[:, 1] = centers_xy[:, 1] - edges[:, 1] / 2
    hi[:, 1] = centers_xy[:, 1] + edges[:, 1] / 2
    lo[:, 2] = base_z
    hi[:, 2] = base_z + edges[:, 2]
    unit = _CUBE_V + F32(0.5)
    v = lo[:, None, :] + unit[None, :, :] * (hi - lo)[:, None, :]
    f = _CUBE_F[None, :, :] + (np.arange(n, dtype=np.uint32) * 8)[:, None, None]
    return v.reshape(-1, 3).astype(np.float32), f.reshape(-1, 3).astype(np.uint32)


# ---- rotations -----------------------------------------------------------------
def euler_to_quat(roll, pitch, yaw) -> np.ndarray:
    """EulerAngles.tcc:40-61 in binary32 with the C library's cosf/sinf: returns [N, 4] (x, y, z, w)."""
    roll = np.asarray(roll, np.float32)
    pitch = np.asarray(pitch, np.float32)
    yaw = np.asarray(yaw, np.float32)
    half = F32(2.0)
    cr, sr = cosf(roll / half), sinf(roll / half)
    cp, sp = cosf(pitch / half), sinf(pitch / half)
    cy, sy = cosf(yaw / half), sinf(yaw / half)
    q = np.stack([
        sr * cp * cy - cr * sp * sy,
        cr * sp * cy + sr * cp * sy,
        cr * cp * sy - sr * sp * cy,
        cr * cp * cy + sr * sp * sy,
    ], axis=-1)
    return q.astype(np.float32).reshape(-1, 4)


def random_quats(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniformly distributed unit quaternions (normalised Gaussian 4-vectors)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


# ---- scene: room with boxes --------------------------------------------------------
@dataclass
class Scene:
    vertices: np.ndarray
    faces: np.ndarray
    height_at: object = None  # callable (x, y) -> ground height, when the scene has a ground

    @property
    def n_faces(self) -> int:
        return int(self.faces.shape[0])


def box_room(seed: int = 0, n_boxes: int = 200, half: float = 10.0, height: float = 4.0) -> Scene:
    """Closed room [-half, half]^2 x [0, height] plus n_boxes boxes on the floor
    (centres uniform in the room, edges U[0.2, 2] per axis)."""
    rng = np.random.default_rng(seed)
    room = box_mesh([-half, -half, 0.0], [half, half, height])
    c = rng.uniform(-half, half, (n_boxes, 2)).astype(np.float32)
    e = rng.uniform(0.2, 2.0, (n_boxes, 3)).astype(np.float32)
    boxes = boxes_mesh(c, np.zeros(n_boxes, np.float32), e)
    v, f = merge([room, boxes])
    return Scene(v, f, lambda x, y: np.zeros_like(np.asarray(x, np.float32)))


def room_poses(n: int, seed: int = 1, half: float = 10.0, z: float = 1.0) -> np.ndarray:
    """Poses in the room: xy uniform, z fixed, yaw U(-pi, pi).  [n, 8] Transform records."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-half, half, (n, 2)).astype(np.float32)
    yaw = rng.uniform(-math.pi, math.pi, n).astype(np.float32)
    q = euler_to_quat(np.zeros(n), np.zeros(n), yaw)
    out = np.zeros((n, 8), np.float32)
    out[:, :4] = q
    out[:, 4:6] = xy
    out[:, 6] = z
    return out


# ---- scene: terrain ---------------------------------------------------------------------
def _value_noise(x, y, freq, rng):
    """Bilinear value noise on a lattice of period 1/freq with smoothstep blending."""
    gx, gy = x * freq, y * freq
    ix, iy = np.floor(gx).astype(np.int64), np.floor(gy).astype(np.int64)
    fx, fy = gx - ix, gy - iy
    ox, oy = ix.min(), iy.min()
    nx, ny = ix.max() - ox + 2, iy.max() - oy + 2
    lat = rng.uniform(-1.0, 1.0, (nx, ny))
    ix, iy = ix - ox, iy - oy
    sx, sy = fx * fx * (3 - 2 * fx), fy * fy * (3 - 2 * fy)
    a = lat[ix, iy] * (1 - sx) + lat[ix + 1, iy] * sx
    b = lat[ix, iy + 1] * (1 - sx) + lat[ix + 1, iy + 1] * sx
    return a * (1 - sy) + b * sy


def fbm_heights(n: int, size: float, amplitude: float, octaves: int, seed: int) -> np.ndarray:
    """n x n heights over [-size/2, size/2]^2: sum_o gain^o * noise(lacunarity^o * f0), gain 0.5,
    lacunarity 2, base period size/4, scaled so the amplitude is `amplitude` metres."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-size / 2, size / 2, n)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    h = np.zeros_like(X)
    amp, total, freq = 1.0, 0.0, 4.0 / size
    for _ in range(octaves):
        h += amp * _value_noise(X, Y, freq, rng)
        total += amp
        amp *= 0.5
        freq *= 2.0
    return (h / total * amplitude).astype(np.float32)


class _Heightfield:
    def __init__(self, heights: np.ndarray, size: float):
        self.h = heights
        self.n = heights.shape[0]
        self.size = size

    def __call__(self, x, y):
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        s = (self.n - 1) / self.size
        gx = np.clip((x + self.size / 2) * s, 0, self.n - 1 - 1e-9)
        gy = np.clip((y + self.size / 2) * s, 0, self.n - 1 - 1e-9)
        i, j = np.floor(gx).astype(np.int64), np.floor(gy).astype(np.int64)
        fx, fy = gx - i, gy - j
        h = self.h
        a = h[i, j] * (1 - fx) + h[i + 1, j] * fx
        b = h[i, j + 1] * (1 - fx) + h[i + 1, j + 1] * fx
        return (a * (1 - fy) + b * fy).astype(np.float32)


def terrain(grid: int = 1024, size: float = 500.0, amplitude: float = 20.0, octaves: int = 6,
            n_boxes: int = 2000, seed: int = 0) -> Scene:
    """grid x grid heightfield (2*(grid-1)^2 triangles) plus n_boxes boxes standing on it."""
    h = fbm_heights(grid, size, amplitude, octaves, seed)
    xs = np.linspace(-size / 2, size / 2, grid).astype(np.float32)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    v = np.stack([X, Y, h], axis=-1).reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(grid - 1), np.arange(grid - 1), indexing="ij")
    v00 = (i * grid + j).reshape(-1)
    v10 = ((i + 1) * grid + j).reshape(-1)
    v11 = ((i + 1) * grid + j + 1).reshape(-1)
    v01 = (i * grid + j + 1).reshape(-1)
    f = np.empty((2 * v00.size, 3), np.uint32)
    f[0::2] = np.stack([v00, v10, v11], axis=1)
    f[1::2] = np.stack([v00, v11, v01], axis=1)
    hf = _Heightfield(h, size)
    mesh = [(v, f)]
    if n_boxes:
        rng = np.random.default_rng(seed + 1)
        c = rng.uniform(-0.45 * size, 0.45 * size, (n_boxes, 2)).astype(np.float32)
        e = rng.uniform(0.2, 2.0, (n_boxes, 3)).astype(np.float32)
        base = hf(c[:, 0], c[:, 1]) - F32(0.1)
        mesh.append(boxes_mesh(c, base, e))
    v, f = merge(mesh)
    return Scene(v, f, hf)


def terrain_poses(scene: Scene, n: int, seed: int = 2, size: float = 500.0, above: float = 1.5) -> np.ndarray:
    """Poses over the inner 90% of the terrain, `above` metres over the ground, yaw U(-pi, pi)."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-0.45 * size, 0.45 * size, (n, 2)).astype(np.float32)
    yaw = rng.uniform(-math.pi, math.pi, n).astype(np.float32)
    q = euler_to_quat(np.zeros(n), np.zeros(n), yaw)
    out = np.zeros((n, 8), np.float32)
    out[:, :4] = q
    out[:, 4:6] = xy
    out[:, 6] = scene.height_at(xy[:, 0], xy[:, 1]) + F32(above)
    return out


def million_triangle_terrain(seed: int = 0) -> Scene:
    """The ~1M-triangle terrain: 708 x 708 grid (999,698 triangles) + 2000 boxes (24,000)."""
    return terrain(grid=708, n_boxes=2000, seed=seed)


def instanced_terrain(grid: int = 708, n_boxes: int = 2000, seed: int = 0, size: float = 500.0):
    """terrain(grid, n_boxes=n_boxes, seed) as an instanced scene: the heightfield is geometry 0
    (one identity instance, ids 0), the boxes are instances of one unit box (geometry 1,
    [-0.5, 0.5]^2 x [0, 1]) scaled by their edge lengths and moved to their centre and base, with
    geom_id 0 and object_id 1 + i -- the same boxes, to binary32 rounding, that terrain() bakes
    into the mesh.  Returns (meshes [(vertices, faces)], instances [dict]) and the baked Scene."""
    baked = terrain(grid=grid, size=size, n_boxes=n_boxes, seed=seed)
    n_terrain_v = grid * grid
    n_terrain_f = 2 * (grid - 1) ** 2
    tv = baked.vertices[:n_terrain_v]
    tf = baked.faces[:n_terrain_f]
    ub_v, ub_f = box_mesh([-0.5, -0.5, 0.0], [0.5, 0.5, 1.0])
    rng = np.random.default_rng(seed + 1)
    c = rng.uniform(-0.45 * size, 0.45 * size, (n_boxes, 2)).astype(np.float32)
    e = rng.uniform(0.2, 2.0, (n_boxes, 3)).astype(np.float32)
    base = baked.height_at(c[:, 0], c[:, 1]) - F32(0.1)
    ident = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
    insts = [dict(geometry=0, T=ident.copy(), scale=np.ones(3, np.float32), geom_id=0, object_id=0)]
    for i in range(n_boxes):
        T = ident.copy()
        T[4:7] = (c[i, 0], c[i, 1], base[i])
        insts.append(dict(geometry=1, T=T, scale=e[i].copy(), geom_id=0, object_id=1 + i))
    return [(tv, tf), (ub_v, ub_f)], insts, baked


def perturb_poses(poses: np.ndarray, seed: int, sigma_t: float = 0.1, sigma_r_deg: float = 2.0) -> np.ndarray:
    """Poses moved by R <- R exp(N(0, sigma_r)^3) and t <- t + N(0, sigma_t)^3 (seeded)."""
    from .transforms import compose

    rng = np.random.default_rng(seed)
    n = poses.shape[0]
    d = np.zeros((n, 8), np.float32)
    w = rng.normal(0, np.radians(sigma_r_deg), (n, 3))
    th = np.linalg.norm(w, axis=1, keepdims=True)
    d[:, :3] = (w / np.maximum(th, 1e-30) * np.sin(th / 2)).astype(np.float32)
    d[:, 3] = np.cos(th[:, 0] / 2).astype(np.float32)
    out = compose(poses, d)
    out[:, 4:7] += rng.normal(0, sigma_t, (n, 3)).astype(np.float32)
    return out

