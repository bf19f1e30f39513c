"""Sensor models, mirroring rmagine's (src/rmagine_core/include/rmagine/types/sensor_models.h).

Field names and meanings follow the reference: SphericalModel has `phi`
(vertical, rows) and `theta` (horizontal, columns) DiscreteIntervals and a
`range` Interval; PinholeModel has width/height/range/f/c; O1DnModel one
origin and width*height directions; OnDnModel width*height origins and
directions.  All values are binary32, as in the reference structs.

The presets restate src/rmagine_core/src/types/sensors.cpp:6-137 with the
same mixed float/double constant arithmetic, so they produce the same binary32
field values (checked against the compiled reference in the tests).
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

F32 = np.float32
DEG_TO_RAD = 0.017453292519943295
DEG_TO_RAD_F = float(F32(0.017453292519943295))  # the reference's float literal


def f32(x: float) -> float:
    return float(F32(x))


_libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _n in ("cosf", "sinf"):
    getattr(_libm, _n).restype = C.c_float
    getattr(_libm, _n).argtypes = [C.c_float]


def cosf(x) -> np.ndarray:
    """The C library's binary32 cosine (what `cos(float)` calls in the reference's C++)."""
    return np.array([_libm.cosf(float(v)) for v in np.ravel(x)], np.float32).reshape(np.shape(x))


def sinf(x) -> np.ndarray:
    return np.array([_libm.sinf(float(v)) for v in np.ravel(x)], np.float32).reshape(np.shape(x))


@dataclass
class Interval:
    min: float = 0.0
    max: float = 0.0

    def invalidValue(self) -> float:
        return f32(self.max + 1.0)

    def inside(self, v: float) -> bool:
        return self.min <= v <= self.max


@dataclass
class DiscreteInterval:
    min: float = 0.0
    inc: float = 0.0
    size: int = 0

    def getValue(self, i: int) -> float:
        return f32(F32(self.min) + F32(F32(i) * F32(self.inc)))

    def max(self) -> float:
        return self.getValue(self.size - 1)


@dataclass
class SphericalModel:
    """sensor_models.h:118-215 -- phi: vertical (rows), theta: horizontal (cols)."""
    phi: DiscreteInterval = field(default_factory=DiscreteInterval)
    theta: DiscreteInterval = field(default_factory=DiscreteInterval)
    range: Interval = field(default_factory=Interval)
    kind = L.RMG_MODEL_SPHERICAL

    def getWidth(self) -> int:
        return int(self.theta.size)

    def getHeight(self) -> int:
        return int(self.phi.size)

    def size(self) -> int:
        return self.getWidth() * self.getHeight()

    def getBufferId(self, vid: int, hid: int) -> int:
        return vid * self.getWidth() + hid

    def to_c(self) -> L.ModelC:
        m = L.ModelC()
        m.kind = self.kind
        m.width, m.height = self.getWidth(), self.getHeight()
        m.range = L.Interval(self.range.min, self.range.max)
        m.phi = L.DiscreteInterval(self.phi.min, self.phi.inc, self.phi.size)
        m.theta = L.DiscreteInterval(self.theta.min, self.theta.inc, self.theta.size)
        return m


@dataclass
class PinholeModel:
    """sensor_models.h:217-315 -- f = (fx, fy), c = (cx, cy)."""
    width: int = 0
    height: int = 0
    range: Interval = field(default_factory=Interval)
    f: tuple = (0.0, 0.0)
    c: tuple = (0.0, 0.0)
    kind = L.RMG_MODEL_PINHOLE

    def getWidth(self) -> int:
        return int(self.width)

    def getHeight(self) -> int:
        return int(self.height)

    def size(self) -> int:
        return self.getWidth() * self.getHeight()

    def getBufferId(self, vid: int, hid: int) -> int:
        return vid * self.width + hid

    def to_c(self) -> L.ModelC:
        m = L.ModelC()
        m.kind = self.kind
        m.width, m.height = self.width, self.height
        m.range = L.Interval(self.range.min, self.range.max)
        m.f[0], m.f[1] = self.f
        m.c[0], m.c[1] = self.c
        return m


@dataclass
class O1DnModel:
    """sensor_models.h:338-417 -- one origin, width*height directions."""
    width: int = 0
    height: int = 0
    range: Interval = field(default_factory=Interval)
    orig: tuple = (0.0, 0.0, 0.0)
    dirs: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    kind = L.RMG_MODEL_O1DN

    def getWidth(self) -> int:
        return int(self.width)

    def getHeight(self) -> int:
        return int(self.height)

    def size(self) -> int:
        return self.getWidth() * self.getHeight()

    def getBufferId(self, vid: int, hid: int) -> int:
        return vid * self.width + hid

    def to_c(self) -> L.ModelC:
        m = L.ModelC()
        m.kind = self.kind
        m.width, m.height = self.width, self.height
        m.range = L.Interval(self.range.min, self.range.max)
        m.orig = L.Vec3(*self.orig)
        self._dirs = np.ascontiguousarray(self.dirs, dtype=np.float32).reshape(-1, 3)
        if self._dirs.shape[0] != self.size():
            raise ValueError("O1DnModel: dirs must hold width*height directions")
        m.dirs = self._dirs.ctypes.data_as(C.c_void_p)
        return m


@dataclass
class OnDnModel:
    """sensor_models.h:422-502 -- width*height origins and directions."""
    width: int = 0
    height: int = 0
    range: Interval = field(default_factory=Interval)
    origs: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    dirs: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    kind = L.RMG_MODEL_ONDN

    def getWidth(self) -> int:
        return int(self.width)

    def getHeight(self) -> int:
        return int(self.height)

    def size(self) -> int:
        return self.getWidth() * self.getHeight()

    def getBufferId(self, vid: int, hid: int) -> int:
        return vid * self.width + hid

    def to_c(self) -> L.ModelC:
        m = L.ModelC()
        m.kind = self.kind
        m.width, m.height = self.width, self.height
        m.range = L.Interval(self.range.min, self.range.max)
        self._dirs = np.ascontiguousarray(self.dirs, dtype=np.float32).reshape(-1, 3)
        self._origs = np.ascontiguousarray(self.origs, dtype=np.float32).reshape(-1, 3)
        if self._dirs.shape[0] != self.size() or self._origs.shape[0] != self.size():
            raise ValueError("OnDnModel: origs and dirs must hold width*height entries")
        m.dirs = self._dirs.ctypes.data_as(C.c_void_p)
        m.origs = self._origs.ctypes.data_as(C.c_void_p)
        return m


LiDARModel = SphericalModel
CameraModel = PinholeModel
DepthCameraModel = PinholeModel


# ---- presets: src/rmagine_core/src/types/sensors.cpp -------------------------
def vlp16_900() -> SphericalModel:
    """sensors.cpp:6-20."""
    return SphericalModel(
        phi=DiscreteInterval(f32(-15.0 * DEG_TO_RAD_F), f32(2.0 * DEG_TO_RAD_F), 16),
        theta=DiscreteInterval(f32(-math.pi), f32((360.0 / 900.0) * DEG_TO_RAD_F), 900),
        range=Interval(0.5, 130.0))


def vlp16_360() -> SphericalModel:
    """sensors.cpp:22-36."""
    return SphericalModel(
        phi=DiscreteInterval(f32(-15.0 * DEG_TO_RAD_F), f32(2.0 * DEG_TO_RAD_F), 16),
        theta=DiscreteInterval(f32(-math.pi), f32(1.0 * DEG_TO_RAD_F), 360),
        range=Interval(0.5, 130.0))


def example_spherical() -> SphericalModel:
    """sensors.cpp:39-54."""
    return SphericalModel(
        phi=DiscreteInterval(f32(-15.0 * math.pi / 180.0), f32(2.0 * math.pi / 180.0), 16),
        theta=DiscreteInterval(f32(-math.pi), f32(0.4 * math.pi / 180.0), 900),
        range=Interval(0.0, 100.0))


def example_pinhole() -> PinholeModel:
    """sensors.cpp:56-68."""
    return PinholeModel(width=200, height=150, range=Interval(0.0, 100.0), f=(100.0, 100.0),
                        c=(100.0, 75.0))


def _normalize_f32(v: np.ndarray) -> np.ndarray:
    """Vector3::normalize (Vector3.tcc:180-211): divide by sqrtf(x*x + y*y + z*z)."""
    v = v.astype(np.float32)
    n2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    n = np.sqrt(n2, dtype=np.float32)
    return (v / n[:, None]).astype(np.float32)


def example_o1dn() -> O1DnModel:
    """sensors.cpp:70-102: 200 directions (cos(y)*2+2, y, -1) normalised, y = -(i-100)*0.05,
    with the binary32 cosine the reference's `cos(float)` resolves to."""
    i = np.arange(200)
    y = (-(i - 100).astype(np.float32) * F32(0.05)).astype(np.float32)
    x = (cosf(y).astype(np.float64) * 2.0 + 2.0).astype(np.float32)
    z = np.full(200, -1.0, np.float32)
    dirs = _normalize_f32(np.stack([x, y, z], axis=1))
    return O1DnModel(width=200, height=1, range=Interval(0.0, 100.0), orig=(0.0, 0.0, 0.0), dirs=dirs)


def example_ondn() -> OnDnModel:
    """sensors.cpp:104-137: origins on a scaled arc in the y-z plane, all directions +x."""
    i = np.arange(200)
    percent = (i.astype(np.float32) / F32(200)).astype(np.float32)
    step = (-(i - 100).astype(np.float32) * F32(0.05)).astype(np.float32)
    y = sinf(step)
    x = cosf(step)
    origs = np.stack([np.zeros(200, np.float32), (y * percent).astype(np.float32),
                      (x * percent).astype(np.float32)], axis=1)
    dirs = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (200, 1))
    return OnDnModel(width=200, height=1, range=Interval(0.0, 100.0), origs=origs, dirs=dirs)


# ---- workload models ---------------------------------------------------------
def ouster_like(rows: int = 128, cols: int = 1024, vfov_deg: float = 45.0,
                range_min: float = 0.5, range_max: float = 130.0) -> SphericalModel:
    """Spherical model with `rows` beams over +-vfov/2 and `cols` columns over 360 deg."""
    half = vfov_deg / 2.0
    return SphericalModel(
        phi=DiscreteInterval(f32(-half * math.pi / 180.0), f32(vfov_deg * math.pi / 180.0 / (rows - 1)), rows),
        theta=DiscreteInterval(f32(-math.pi), f32(2.0 * math.pi / cols), cols),
        range=Interval(range_min, range_max))


def depth_camera(width: int = 640, height: int = 480, hfov_deg: float = 90.0,
                 range_min: float = 0.3, range_max: float = 130.0) -> PinholeModel:
    """Pinhole model with focal length from the horizontal field of view."""
    fx = (width / 2.0) / math.tan(math.radians(hfov_deg) / 2.0)
    return PinholeModel(width=width, height=height, range=Interval(range_min, range_max),
                        f=(f32(fx), f32(fx)), c=(f32((width - 1) / 2.0), f32((height - 1) / 2.0)))


def sphere_directions(n: int, seed: int) -> np.ndarray:
    """n unit vectors uniform on the sphere (normalised Gaussian triplets)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, 3)).astype(np.float32)
    return _normalize_f32(g)
