"""Map and simulators with rmagine's interface, computing on the GB300 through librmg_gb300.

Mirrors, for the GPU:
  * SimulatorEmbree::setMap / setTsb            (SimulatorEmbree.hpp:58-61)
  * XSimulator::setModel                         (SphereSimulatorEmbree.hpp:115-116)
  * XSimulator::simulate(Tbm, bundle) / simulate<BundleT>(Tbm)
                                                 (SphereSimulatorEmbree.hpp:130-155,
                                                  SphereSimulatorOptix.hpp:141-160)
  * Bundle / IntAttrAll / resize_memory_bundle   (SimulationResults.hpp:56-215)

Device memory is torch CUDA tensors (torch is used for allocation and
streams only).  Bundles whose tensors live on the device are filled
asynchronously on the current stream, like the OptiX simulators; bundles in
host memory go through a device staging buffer and the call synchronises,
like the reference's RAM overloads.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable

import numpy as np
import torch

from . import _lib as L
from .sensors import O1DnModel, OnDnModel, PinholeModel, SphericalModel

ATTRIBUTES = ("hits", "ranges", "points", "normals", "face_ids", "geom_ids", "object_ids")
_DTYPES = {
    "hits": (torch.uint8, ()),
    "ranges": (torch.float32, ()),
    "points": (torch.float32, (3,)),
    "normals": (torch.float32, (3,)),
    "face_ids": (torch.int32, ()),    # uint32 bit patterns (torch has no uint32 arithmetic)
    "geom_ids": (torch.int32, ()),
    "object_ids": (torch.int32, ()),
}


def _stream_ptr(device: torch.device | None = None) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _ptr(t: torch.Tensor | None) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


# ---- transforms ----------------------------------------------------------------
def make_transforms(q_xyzw, t, device=None) -> torch.Tensor:
    """Packs rotations (x, y, z, w) and translations into rmagine Transform records.

    Returns a float32 tensor [N, 8] whose rows are byte-identical to
    rmagine::Transform (Quaternion R; Vector3 t; uint32 stamp = 0).
    """
    q = np.asarray(q_xyzw, dtype=np.float32).reshape(-1, 4)
    tt = np.asarray(t, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((q.shape[0], 8), np.float32)
    out[:, :4] = q
    out[:, 4:7] = tt
    ten = torch.from_numpy(out)
    return ten.to(device) if device is not None else ten


def identity_transforms(n: int, device=None) -> torch.Tensor:
    q = np.tile(np.array([[0.0, 0.0, 0.0, 1.0]], np.float32), (n, 1))
    return make_transforms(q, np.zeros((n, 3), np.float32), device)


def transform_c(T) -> L.TransformC:
    a = np.asarray(T, dtype=np.float32).reshape(-1)
    if a.size == 7:
        a = np.concatenate([a, np.zeros(1, np.float32)])
    tc = L.TransformC()
    tc.R = L.Quat(float(a[0]), float(a[1]), float(a[2]), float(a[3]))
    tc.t = L.Vec3(float(a[4]), float(a[5]), float(a[6]))
    tc.stamp = 0
    return tc


# ---- map ------------------------------------------------------------------------
class Map:
    """A triangle mesh with its BVH on the current CUDA device (rmg_map).  builder: "sah" (the
    default: binned surface area heuristic) or "lbvh" (Morton-code linear BVH, the fastest build);
    every query gives the same result with either."""

    BUILDERS = {"sah": L.RMG_BUILD_SAH, "lbvh": L.RMG_BUILD_LBVH}

    def __init__(self, vertices, faces, stream=None, builder: str = "sah"):
        self._h = None
        if builder not in self.BUILDERS:
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "Map", f"builder must be one of {sorted(self.BUILDERS)}")
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        self.n_vertices, self.n_faces = v.shape[0], f.shape[0]
        self.builder = builder
        h = C.c_void_p()
        L.call("rmg_map_build_ex", v.ctypes.data_as(C.c_void_p), v.shape[0], f.ctypes.data_as(C.c_void_p),
               f.shape[0], self.BUILDERS[builder], stream if stream is not None else _stream_ptr(), C.byref(h))
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "Map", "map was destroyed")
        return self._h

    def refit(self, vertices, stream=None) -> None:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        L.call("rmg_map_refit", self.handle, v.ctypes.data_as(C.c_void_p), v.shape[0],
               stream if stream is not None else _stream_ptr())

    def info(self) -> dict:
        inf = L.MapInfoC()
        L.call("rmg_map_info_get", self.handle, C.byref(inf))
        return {"n_vertices": inf.n_vertices, "n_faces": inf.n_faces, "n_nodes": inf.n_nodes,
                "depth": inf.depth, "device_bytes": inf.device_bytes,
                "bounds_lo": list(inf.bounds_lo), "bounds_hi": list(inf.bounds_hi)}

    def export(self) -> dict:
        """Downloads the tree: nodes [n_nodes, 16] (12 float + 4 int32 views), tris [n_faces, 12]."""
        inf = self.info()
        nodes = np.zeros((inf["n_nodes"], 16), np.float32)
        tris = np.zeros((inf["n_faces"], 12), np.float32)
        order = np.zeros(inf["n_faces"], np.uint32)
        L.call("rmg_map_export", self.handle, nodes.ctypes.data_as(C.c_void_p),
               tris.ctypes.data_as(C.c_void_p), order.ctypes.data_as(C.c_void_p))
        return {"boxes": nodes[:, :12].copy(), "links": nodes.view(np.int32)[:, 12:].copy(),
                "tris": tris, "leaf_order": order}

    def build_wide8(self) -> "Map":
        """Adds the 8-wide tree with quantized boxes (rmg_map_build_wide8) for launch_config(bvh_width=8)."""
        L.call("rmg_map_build_wide8", self.handle, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self

    def status(self, clear: bool = True) -> int:
        return int(L.load().rmg_map_status(self.handle, 1 if clear else 0))

    def save(self, path) -> None:
        """The built map (mesh + tree) to a file (rmg_map_save)."""
        from .meshio import save_map

        save_map(self, path)

    @classmethod
    def load(cls, path) -> "Map":
        """A map saved by save(), without a rebuild (rmg_map_load)."""
        from .meshio import load_map

        return load_map(path)

    def destroy(self) -> None:
        if self._h is not None:
            L.load().rmg_map_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Instance:
    """One placement of a geometry in a Scene: x_map = T * (scale (.) x_mesh)
    (EmbreeInstance::setTransform / setScale / apply, EmbreeInstance.cpp:46-60), reporting
    geom_id / object_id for its hits."""

    def __init__(self, geometry: int, T=None, scale=(1.0, 1.0, 1.0), geom_id: int = 0, object_id: int = 0):
        self.geometry = int(geometry)
        self.T = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32) if T is None else \
            np.asarray(T, np.float32).reshape(-1)[:8].copy()
        if self.T.size == 7:
            self.T = np.concatenate([self.T, np.zeros(1, np.float32)])
        self.scale = np.asarray(scale, np.float32).reshape(3).copy()
        self.geom_id = int(geom_id)
        self.object_id = int(object_id)

    def to_c(self) -> L.InstanceDescC:
        d = L.InstanceDescC()
        d.geometry, d.geom_id, d.object_id = self.geometry, self.geom_id, self.object_id
        d.T = transform_c(self.T)
        d.scale[:] = [float(x) for x in self.scale]
        return d


def _instances_c(instances):
    arr = (L.InstanceDescC * max(1, len(instances)))()
    for i, inst in enumerate(instances):
        arr[i] = inst.to_c()
    return arr


class Scene:
    """Several meshes and instances of them under a top-level tree (rmg_scene): EmbreeScene /
    OptixScene with instance children.  Usable wherever a Map is (setMap)."""

    def __init__(self, geometries, instances, stream=None):
        self._h = None
        self.geometries = list(geometries)  # keeps the meshes alive as long as the scene
        self.instances = list(instances)
        handles = (C.c_void_p * max(1, len(self.geometries)))(*[g.handle.value for g in self.geometries])
        h = C.c_void_p()
        L.call("rmg_scene_create", handles, len(self.geometries), _instances_c(self.instances), len(self.instances),
               stream if stream is not None else _stream_ptr(), C.byref(h))
        self._h = h

    @classmethod
    def from_meshes(cls, meshes, instances=None):
        """meshes: list of (vertices, faces).  instances: list of Instance; default one identity
        instance per mesh with geom_id = object_id = the mesh index (meshes added without instancing)."""
        geoms = [Map(v, f) for v, f in meshes]
        if instances is None:
            instances = [Instance(i, geom_id=i, object_id=i) for i in range(len(geoms))]
        return cls(geoms, instances)

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "Scene", "scene was destroyed")
        return self._h

    def update(self, instances, rebuild: bool = False, stream=None) -> None:
        """New instance poses / scales / ids (same count): refits the top-level tree, or rebuilds it."""
        instances = list(instances)
        L.call("rmg_scene_update", self.handle, _instances_c(instances), len(instances), 1 if rebuild else 0,
               stream if stream is not None else _stream_ptr())
        self.instances = instances

    def status(self, clear: bool = True) -> int:
        return int(L.load().rmg_scene_status(self.handle, 1 if clear else 0))

    def destroy(self) -> None:
        if self._h is not None:
            L.load().rmg_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Sensor:
    """A sensor model with its device direction table (rmg_sensor)."""

    def __init__(self, model, stream=None):
        self._h = None
        self.model = model
        mc = model.to_c()
        h = C.c_void_p()
        L.call("rmg_sensor_create", C.byref(mc), stream if stream is not None else _stream_ptr(), C.byref(h))
        self._h = h
        w, hh = C.c_uint32(), C.c_uint32()
        L.call("rmg_sensor_size", h, C.byref(w), C.byref(hh))
        self.width, self.height = w.value, hh.value

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def directions(self) -> np.ndarray:
        out = np.zeros((self.width * self.height, 3), np.float32)
        L.call("rmg_sensor_directions", self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def visit_order(self):
        """The sorted order in which the kernels visit this sensor's rays (table indices), or None when
        they visit them in the table's own order (O1Dn/OnDn tables of scattered directions get one)."""
        sorted_ = C.c_int()
        L.call("rmg_sensor_visit_order", self._h, None, C.byref(sorted_))
        if not sorted_.value:
            return None
        out = np.zeros(self.width * self.height, np.uint32)
        L.call("rmg_sensor_visit_order", self._h, out.ctypes.data_as(C.c_void_p), C.byref(sorted_))
        return out

    def destroy(self) -> None:
        if self._h is not None:
            L.load().rmg_sensor_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


# ---- result bundles ----------------------------------------------------------------
class Bundle:
    """A set of result attributes (rmagine Bundle<Hits, Ranges, ...>).

    Attributes not in the bundle stay None and are not computed, like a
    Bundle type without that attribute in the reference."""

    def __init__(self, *attrs: str):
        for a in attrs:
            if a not in ATTRIBUTES:
                raise ValueError(f"unknown attribute {a!r}")
        self.attrs = tuple(a for a in ATTRIBUTES if a in attrs)
        for a in ATTRIBUTES:
            setattr(self, a, None)

    def has(self, attr: str) -> bool:
        return attr in self.attrs

    def tensors(self) -> dict:
        return {a: getattr(self, a) for a in self.attrs if getattr(self, a) is not None}


def IntAttrAll() -> Bundle:
    """SimulationResults.hpp:152-159."""
    return Bundle(*ATTRIBUTES)


def resize_memory_bundle(bundle: Bundle, W: int, H: int, N: int = 1, device="cuda",
                         pin_memory: bool = False) -> Bundle:
    """SimulationResults.hpp:176-215: sizes every attribute buffer to W*H*N."""
    n = int(W) * int(H) * int(N)
    for a in bundle.attrs:
        dt, tail = _DTYPES[a]
        if str(device) == "cpu":
            t = torch.empty((n, *tail), dtype=dt, pin_memory=pin_memory)
        else:
            t = torch.empty((n, *tail), dtype=dt, device=device)
        setattr(bundle, a, t)
    return bundle


def outputs_c(bundle: Bundle) -> L.OutputsC:
    o = L.OutputsC()
    for a in ATTRIBUTES:
        t = getattr(bundle, a, None)
        setattr(o, a, None if t is None or t.numel() == 0 else t.data_ptr())
    return o


def launch_config(stack_depth=16, block_warps=4, tile_w=8, tile_h=4, refill=0, chunk=4, bvh_width=0,
                  packet=2) -> L.LaunchConfigC:
    return L.LaunchConfigC(stack_depth, block_warps, tile_w, tile_h, refill, chunk, bvh_width, packet)


# ---- simulators -------------------------------------------------------------------
class _Simulator:
    model_type: type = object

    def __init__(self, map: Map | None = None):
        self._map = map
        self._sensor: Sensor | None = None
        self._model = None
        self._Tsb = transform_c([0, 0, 0, 1, 0, 0, 0])
        self.launch_config: L.LaunchConfigC | None = None
        self._copy_stream = None
        self._side_streams: list | None = None

    # SimulatorEmbree::setMap (a Map or a Scene)
    def setMap(self, map: "Map | Scene") -> None:
        self._map = map

    def map(self) -> Map | None:
        return self._map

    # SimulatorEmbree::setTsb
    def setTsb(self, T) -> None:
        if isinstance(T, torch.Tensor):
            T = T.detach().cpu().numpy()
        self._Tsb = transform_c(np.asarray(T).reshape(-1)[:8])

    def setModel(self, model) -> None:
        if not isinstance(model, self.model_type):
            raise TypeError(f"{type(self).__name__}.setModel expects {self.model_type.__name__}")
        self._model = model
        if self._sensor is not None:
            self._sensor.destroy()
        self._sensor = Sensor(model)

    def model(self):
        return self._model

    @property
    def sensor(self) -> Sensor:
        if self._sensor is None:
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate", "no model set")
        return self._sensor

    def _compute_streams(self, k: int = 2) -> list:
        """The current stream and k-1 cached side streams (each made to wait for the current one)
        that the chunked host paths alternate their launches over: a launch of a few poses lasts
        as long as its slowest warps, and the next chunk's launch on another stream fills the SMs
        those stragglers leave idle.  The caller joins them with _join_streams."""
        cur = torch.cuda.current_stream()
        if self._side_streams is None or len(self._side_streams) != k - 1:
            self._side_streams = [torch.cuda.Stream() for _ in range(k - 1)]
        for s in self._side_streams:
            s.wait_stream(cur)
        return [cur] + self._side_streams

    @staticmethod
    def _join_streams(streams: list) -> None:
        for s in streams[1:]:
            streams[0].wait_stream(s)

    def _check_ready(self) -> None:
        if self._map is None:
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate", "no map set")
        self.sensor  # noqa: B018

    def simulate(self, Tbm, bundle: Bundle | None = None, attrs: Iterable[str] | None = None) -> Bundle:
        """simulate(Tbm, bundle) fills `bundle`; simulate(Tbm) allocates an IntAttrAll-like
        bundle (or `attrs`) on the device, like simulate<BundleT>(Tbm)."""
        self._check_ready()
        if not isinstance(Tbm, torch.Tensor):
            Tbm = torch.as_tensor(np.asarray(Tbm, np.float32).reshape(-1, 8))
        Tbm = Tbm.reshape(-1, 8)
        n = Tbm.shape[0]
        W, H = self.sensor.width, self.sensor.height
        if bundle is None:
            bundle = Bundle(*(attrs if attrs is not None else ATTRIBUTES))
            resize_memory_bundle(bundle, W, H, n, device="cuda")
        for a, t in bundle.tensors().items():
            if t.shape[0] != W * H * n:
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate",
                                 f"{a} holds {t.shape[0]} elements, expected {W * H * n}")
        on_host = any(not t.is_cuda for t in bundle.tensors().values())
        if on_host:
            return self._simulate_host(Tbm, bundle, n)
        Tbm_d = Tbm if Tbm.is_cuda else Tbm.to("cuda", non_blocking=True)
        Tbm_d = Tbm_d.contiguous()
        self._launch(Tbm_d, n, bundle, _stream_ptr())
        return bundle

    def _launch(self, Tbm_d: torch.Tensor, n: int, bundle: Bundle, stream) -> None:
        out = outputs_c(bundle)
        lib = L.load()
        if isinstance(self._map, Scene):
            st = lib.rmg_simulate_scene(self._map.handle, self.sensor.handle, C.byref(self._Tsb),
                                        C.c_void_p(Tbm_d.data_ptr()), n, C.byref(out), stream)
            L.check(st, "rmg_simulate_scene")
            return
        if self.launch_config is None:
            st = lib.rmg_simulate(self._map.handle, self.sensor.handle, C.byref(self._Tsb),
                                  C.c_void_p(Tbm_d.data_ptr()), n, C.byref(out), stream)
        else:
            st = lib.rmg_simulate_ex(self._map.handle, self.sensor.handle, C.byref(self._Tsb),
                                     C.c_void_p(Tbm_d.data_ptr()), n, C.byref(out),
                                     C.byref(self.launch_config), stream)
        L.check(st, "rmg_simulate")

    def autotune(self, Tbm, bundle: Bundle | None = None, attrs: Iterable[str] | None = None, reps: int = 3):
        """Times the launch configurations of rmg_autotune_launch_config on these poses (and this
        bundle, or one with `attrs`) and keeps the fastest in self.launch_config.  Single-mesh maps
        only; results do not depend on the choice."""
        if isinstance(self._map, Scene):
            raise L.RmgError(L.RMG_ERR_UNSUPPORTED, "autotune", "needs a single-mesh Map")
        self._check_ready()
        if not isinstance(Tbm, torch.Tensor):
            Tbm = torch.as_tensor(np.asarray(Tbm, np.float32).reshape(-1, 8))
        Tbm_d = Tbm.reshape(-1, 8).to("cuda").contiguous()
        n = Tbm_d.shape[0]
        if bundle is None:
            bundle = Bundle(*(attrs if attrs is not None else ATTRIBUTES))
            resize_memory_bundle(bundle, self.sensor.width, self.sensor.height, n, device="cuda")
        out = outputs_c(bundle)
        best = L.LaunchConfigC()
        L.call("rmg_autotune_launch_config", self._map.handle, self.sensor.handle, C.byref(self._Tsb),
               C.c_void_p(Tbm_d.data_ptr()), n, C.byref(out), int(reps), C.byref(best), _stream_ptr())
        self.launch_config = best
        return best

    def simulate_statistics(self, Tbm, dataset_points, dataset_mask=None, dataset_ids=None, pre=None,
                            params=None, point_to_plane: bool = True, want_stats: bool = True,
                            want_transforms: bool = True):
        """Fused simulate -> statistics_p2l (or _p2p) -> umeyama_transform for every pose in Tbm:
        the model scan is cast at Tbm[p] and paired ray by ray with the dataset scan, without
        writing Points/Normals (rmg_simulate_statistics).  dataset_points is [W*H, 3] (one scan
        for every pose) or [n, W*H, 3] (one per pose), in the sensor frame and ray order of
        simulate(); dataset_mask (e.g. the scan's hits) and dataset_ids follow its shape.  pre is
        one transform or one per pose.  Returns (stats [n,16] or None, transforms [n,8] or None)
        on the device, asynchronously on the current stream.  A dataset in host memory goes
        through rmg_simulate_statistics_host instead: per-pose scans are uploaded in pose chunks
        while earlier chunks are reduced, and the results come back in host memory when the call
        returns (the same values as one call on device data: every pose is reduced on its own)."""
        from . import statistics as S

        self._check_ready()
        if isinstance(self._map, Scene):
            raise L.RmgError(L.RMG_ERR_UNSUPPORTED, "simulate_statistics", "needs a single-mesh Map")
        if not (isinstance(dataset_points, torch.Tensor) and dataset_points.is_cuda):
            return self._simulate_statistics_host(Tbm, dataset_points, dataset_mask, dataset_ids, pre, params,
                                                  point_to_plane, want_stats, want_transforms)
        Tbm = S._dev(Tbm, torch.float32).reshape(-1, 8)
        n = Tbm.shape[0]
        W, H = self.sensor.width, self.sensor.height
        dp = S._dev(dataset_points, torch.float32)
        per_pose = dp.dim() == 3
        if dp.shape[-2:] != (W * H, 3) or (per_pose and dp.shape[0] != n):
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate_statistics",
                             f"dataset points {tuple(dp.shape)} do not match {n} poses x {W * H} rays")
        dm, di = S._u8(dataset_mask), S._i32(dataset_ids)
        for name, t in (("mask", dm), ("ids", di)):
            if t is not None and t.numel() != dp.numel() // 3:
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate_statistics", f"dataset {name} size mismatch")
        pre_t, stride = S._pre(pre, n)
        params = params or S.UmeyamaReductionConstraints()
        stats = torch.empty((n, 16), dtype=torch.float32, device="cuda") if want_stats else None
        T = torch.empty((n, 8), dtype=torch.float32, device="cuda") if want_transforms else None
        scan = L.ScanC(dp.data_ptr(), None if dm is None else dm.data_ptr(), None if di is None else di.data_ptr(),
                       1 if per_pose else 0)
        pc = params.to_c()
        L.call("rmg_simulate_statistics", self._map.handle, self.sensor.handle, C.byref(self._Tsb),
               C.c_void_p(Tbm.data_ptr()), n, C.byref(scan), _ptr(pre_t), stride, C.byref(pc),
               1 if point_to_plane else 0, _ptr(stats), _ptr(T), _stream_ptr())
        return stats, T

    def _simulate_statistics_host(self, Tbm, dp_h, dm_h, di_h, pre, params, point_to_plane, want_stats,
                                  want_transforms):
        from . import statistics as S

        T_in = (Tbm if isinstance(Tbm, torch.Tensor) else torch.as_tensor(np.asarray(Tbm, np.float32)))
        T_in = T_in.reshape(-1, 8).to(torch.float32).contiguous()
        n = T_in.shape[0]
        W, H = self.sensor.width, self.sensor.height
        per = W * H
        dp = torch.as_tensor(dp_h).to(torch.float32).contiguous()
        per_pose = dp.dim() == 3
        if dp.shape[-2:] != (per, 3) or (per_pose and dp.shape[0] != n):
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate_statistics",
                             f"dataset points {tuple(dp.shape)} do not match {n} poses x {per} rays")
        dm = None if dm_h is None else torch.as_tensor(dm_h).to(torch.uint8).contiguous()
        di = None
        if di_h is not None:
            di = (di_h if isinstance(di_h, torch.Tensor) else
                  torch.as_tensor(np.asarray(di_h).astype(np.uint32).view(np.int32))).to(torch.int32).contiguous()
        for name, t in (("mask", dm), ("ids", di)):
            if t is not None and t.numel() != dp.numel() // 3:
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate_statistics", f"dataset {name} size mismatch")
        pre_t, stride = None, 0
        if pre is not None:
            pre_t = (pre if isinstance(pre, torch.Tensor) else torch.as_tensor(np.asarray(pre, np.float32)))
            pre_t = pre_t.reshape(-1, 8).to(torch.float32).contiguous()
            stride = 1 if pre_t.shape[0] > 1 else 0
            if stride and pre_t.shape[0] != n:
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate_statistics", "pre: one transform or one per pose")
        params = params or S.UmeyamaReductionConstraints()
        stats = torch.empty((n, 16), dtype=torch.float32) if want_stats else None
        T = torch.empty((n, 8), dtype=torch.float32) if want_transforms else None
        scan = L.ScanC(dp.data_ptr(), None if dm is None else dm.data_ptr(), None if di is None else di.data_ptr(),
                       1 if per_pose else 0)
        pc = params.to_c()
        L.call("rmg_simulate_statistics_host", self._map.handle, self.sensor.handle, C.byref(self._Tsb),
               C.c_void_p(T_in.data_ptr()), n, C.byref(scan), _ptr(pre_t), stride, C.byref(pc),
               1 if point_to_plane else 0, _ptr(stats), _ptr(T), _stream_ptr())
        return stats, T

    def _simulate_host(self, Tbm: torch.Tensor, bundle: Bundle, n: int) -> Bundle:
        """Host bundle (the Embree simulators' RAM form): rmg_simulate_host / rmg_simulate_scene_host
        cast the poses in chunks into device staging memory and copy each chunk back on a second
        stream while the next ones are cast.  Synchronises."""
        for a, t in bundle.tensors().items():
            if not t.is_contiguous():
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "simulate", f"{a} is not contiguous")
        T = Tbm.to(torch.float32).contiguous()
        out = outputs_c(bundle)
        if isinstance(self._map, Scene):
            L.call("rmg_simulate_scene_host", self._map.handle, self.sensor.handle, C.byref(self._Tsb),
                   C.c_void_p(T.data_ptr()), n, C.byref(out), _stream_ptr())
        else:
            L.call("rmg_simulate_host", self._map.handle, self.sensor.handle, C.byref(self._Tsb),
                   C.c_void_p(T.data_ptr()), n, C.byref(out),
                   None if self.launch_config is None else C.byref(self.launch_config), _stream_ptr())
        return bundle


class SphereSimulator(_Simulator):
    """SphereSimulatorEmbree / SphereSimulatorOptix on the GB300."""
    model_type = SphericalModel


class PinholeSimulator(_Simulator):
    model_type = PinholeModel


class O1DnSimulator(_Simulator):
    model_type = O1DnModel


class OnDnSimulator(_Simulator):
    model_type = OnDnModel


def pose_shard(n_poses: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous pose range [lo, hi) of `rank` among `world` replicas: poses are independent and
    the map is replicated, so N GPUs split the poses with no collective on the data path."""
    base, extra = divmod(n_poses, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def make_simulator(model, map: Map | None = None) -> _Simulator:
    """Simulator.hpp:52-78 (SimulatorType<ModelT, CompT>) for this backend."""
    for cls in (SphereSimulator, PinholeSimulator, O1DnSimulator, OnDnSimulator):
        if isinstance(model, cls.model_type):
            sim = cls(map)
            sim.setModel(model)
            return sim
    raise TypeError(f"no simulator for model {type(model).__name__}")
