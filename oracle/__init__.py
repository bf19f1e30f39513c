"""ORACLE -- test infrastructure only.

CPU restatement of rmagine's Embree simulation path (oracle.cpp, via ctypes)
plus binary64 numpy restatements of its statistics / Umeyama math
(stats.py) and of the pose gradient (grad.py).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this package,
and only as the checker: the GPU library never calls it.

Models are read duck-typed (the attributes of rmagine's model structs), so
this package imports nothing from the GPU library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_P = C.c_void_p
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        sig = {
            "orc_max_threads": (C.c_int, []),
            "orc_dirs_spherical": (None, [C.c_float, C.c_float, C.c_uint32, C.c_float, C.c_float, C.c_uint32, _P]),
            "orc_dirs_pinhole": (None, [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, _P]),
            "orc_bvh_build": (_P, [_P, C.c_uint32, _P, C.c_uint32]),
            "orc_bvh_build_ex": (_P, [_P, C.c_uint32, _P, C.c_uint32, C.c_int]),
            "orc_bvh_count": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_float, _P, _P, _P, _P, C.c_int]),
            "orc_bvh_save_map": (C.c_int, [_P, C.c_char_p]),
            "orc_tree_count": (C.c_int, [_P, _P, C.c_uint32, _P, _P, C.c_uint64, C.c_float, _P, _P, _P, _P,
                                         C.c_int]),
            "orc_bvh_free": (None, [_P]),
            "orc_bvh_num_nodes": (C.c_uint32, [_P]),
            "orc_simulate": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_uint32, C.c_float, C.c_float, _P, _P, _P,
                                       _P, _P, C.c_uint32, _P, _P, _P, _P, _P, _P, _P, C.c_int, _P]),
            "orc_bvh4_build": (_P, [_P]),
            "orc_bvh4_free": (None, [_P]),
            "orc_simulate4": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_uint32, C.c_float, C.c_float, _P, _P, _P,
                                        _P, _P, C.c_uint32, _P, _P, _P, _P, _P, _P, _P, C.c_int]),
            "orc_stats_batched": (C.c_int, [_P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_float, C.c_int, _P]),
            "orc_pose_grad": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_uint32, C.c_float, C.c_float, _P, _P, _P, _P,
                                        _P, C.c_uint32, _P, _P, _P, C.c_double, C.c_int, _P, _P]),
            "orc_noise_apply": (C.c_int, [C.c_int, _P, _P, C.c_uint64, C.c_uint64, C.c_uint64, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
            "orc_rays": (C.c_int, [C.c_int, C.c_uint32, C.c_uint32, _P, _P, _P, _P, _P, _P, C.c_uint64, _P, _P]),
            "orc_intersect_f64": (C.c_int, [_P, _P, _P, C.c_uint32, _P, _P]),
            "orc_trace_rays": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_float, _P, _P, C.c_int]),
            "orc_lbvh_build": (_P, [_P, C.c_uint32, _P, C.c_uint32]),
            "orc_lbvh_free": (None, [_P]),
            "orc_lbvh_num_nodes": (C.c_uint32, [_P]),
            "orc_lbvh_export": (None, [_P, _P, _P, _P]),
            "orc_lbvh_count": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_float, _P, _P, _P, _P, C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


KIND = {"spherical": 0, "pinhole": 1, "o1dn": 2, "ondn": 3}


def model_kind(model) -> int:
    if hasattr(model, "phi") and hasattr(model, "theta"):
        return 0
    if hasattr(model, "f") and hasattr(model, "c"):
        return 1
    if hasattr(model, "origs"):
        return 3
    if hasattr(model, "orig"):
        return 2
    raise TypeError(f"not a sensor model: {type(model).__name__}")


def model_size(model) -> tuple[int, int]:
    if model_kind(model) == 0:
        return int(model.theta.size), int(model.phi.size)
    return int(model.width), int(model.height)


def directions(model) -> np.ndarray:
    """Sensor-frame ray directions [H*W, 3] (row-major: vid*W + hid)."""
    k = model_kind(model)
    W, H = model_size(model)
    out = np.zeros((W * H, 3), np.float32)
    if k == 0:
        lib().orc_dirs_spherical(model.phi.min, model.phi.inc, model.phi.size, model.theta.min,
                                 model.theta.inc, model.theta.size, _p(out))
    elif k == 1:
        lib().orc_dirs_pinhole(W, H, model.f[0], model.f[1], model.c[0], model.c[1], _p(out))
    else:
        out[:] = np.asarray(model.dirs, np.float32).reshape(-1, 3)
    return out


class Scene:
    """A mesh with the oracle's binned-SAH BVH."""

    def __init__(self, vertices, faces, max_leaf: int = 4):
        self.v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        self.h = lib().orc_bvh_build_ex(_p(self.v), self.v.shape[0], _p(self.f), self.f.shape[0], int(max_leaf))

    def __del__(self):
        if getattr(self, "h4", None):
            lib().orc_bvh4_free(self.h4)
            self.h4 = None
        if getattr(self, "h", None):
            lib().orc_bvh_free(self.h)
            self.h = None

    def num_nodes(self) -> int:
        return int(lib().orc_bvh_num_nodes(self.h))

    def _bvh4(self):
        if getattr(self, "h4", None) is None:
            self.h4 = lib().orc_bvh4_build(self.h)
            if not self.h4:
                raise ValueError("the SAH tree is too deep for the 4-wide walk's stack")
        return self.h4

    def save_map(self, path) -> int:
        """Writes this tree (built with max_leaf=1) as a GPU map file (rmg_map_load reads it);
        returns its depth."""
        d = int(lib().orc_bvh_save_map(self.h, str(path).encode()))
        if d < 0:
            raise ValueError("save_map needs a one-triangle-per-leaf tree and a writable path")
        return d

    def count(self, o, d, tfar: float, nthreads: int = 0):
        """Per-ray internal-node visits and triangle tests through this SAH tree (nearest child
        first, t-culling), with the hit t and face: the tree-quality yardstick for the LBVH counts."""
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = o.shape[0]
        visits = np.zeros(n, np.uint32)
        tests = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        f = np.zeros(n, np.uint32)
        lib().orc_bvh_count(self.h, _p(o), _p(d), n, float(tfar), _p(visits), _p(tests), _p(t), _p(f), int(nthreads))
        return visits, tests, t, f

    def _model_args(self, model):
        k = model_kind(model)
        W, H = model_size(model)
        dirs = directions(model)
        origs = np.ascontiguousarray(model.origs, np.float32).reshape(-1, 3) if k == 3 else None
        orig = np.asarray(model.orig, np.float32).reshape(3) if k == 2 else None
        return k, W, H, dirs, origs, orig

    def simulate(self, model, Tsb, Tbm, attrs=("hits", "ranges", "points", "normals", "face_ids", "geom_ids",
                                                "object_ids"), nthreads: int = 0, count_tests: bool = False,
                 fast: bool = False):
        """Embree-path simulation of all (pose, row, col) rays; returns numpy arrays.  fast: through
        the Embree-class 4-wide SIMD walk (orc_simulate4; the same outputs, the timed CPU baseline)."""
        k, W, H, dirs, origs, orig = self._model_args(model)
        Tsb = np.ascontiguousarray(Tsb, np.float32).reshape(8)
        Tbm = np.ascontiguousarray(Tbm, np.float32).reshape(-1, 8)
        n = Tbm.shape[0] * W * H
        out = {}
        shapes = {"hits": ((n,), np.uint8), "ranges": ((n,), np.float32), "points": ((n, 3), np.float32),
                  "normals": ((n, 3), np.float32), "face_ids": ((n,), np.uint32),
                  "geom_ids": ((n,), np.uint32), "object_ids": ((n,), np.uint32)}
        for a in attrs:
            shp, dt = shapes[a]
            out[a] = np.empty(shp, dt)
        if fast:
            if count_tests:
                raise ValueError("the 4-wide walk does not count triangle tests")
            lib().orc_simulate4(self._bvh4(), k, W, H, float(model.range.min), float(model.range.max), _p(dirs),
                                _p(origs), _p(orig), _p(Tsb), _p(Tbm), Tbm.shape[0], _p(out.get("hits")),
                                _p(out.get("ranges")), _p(out.get("points")), _p(out.get("normals")),
                                _p(out.get("face_ids")), _p(out.get("geom_ids")), _p(out.get("object_ids")),
                                int(nthreads))
            return out
        tests = np.zeros(1, np.uint64)
        lib().orc_simulate(self.h, k, W, H, float(model.range.min), float(model.range.max), _p(dirs), _p(origs),
                           _p(orig), _p(Tsb), _p(Tbm), Tbm.shape[0], _p(out.get("hits")), _p(out.get("ranges")),
                           _p(out.get("points")), _p(out.get("normals")), _p(out.get("face_ids")),
                           _p(out.get("geom_ids")), _p(out.get("object_ids")), int(nthreads),
                           _p(tests) if count_tests else None)
        if count_tests:
            out["tri_tests"] = int(tests[0])
        return out

    def rays(self, model, Tsb, Tbm, gids):
        """Map-frame origins and directions of the given global ray ids."""
        k, W, H, dirs, origs, orig = self._model_args(model)
        Tsb = np.ascontiguousarray(Tsb, np.float32).reshape(8)
        Tbm = np.ascontiguousarray(Tbm, np.float32).reshape(-1, 8)
        gids = np.ascontiguousarray(gids, np.uint64)
        o = np.zeros((gids.size, 3), np.float32)
        d = np.zeros((gids.size, 3), np.float32)
        lib().orc_rays(k, W, H, _p(dirs), _p(origs), _p(orig), _p(Tsb), _p(Tbm), _p(gids), gids.size, _p(o), _p(d))
        return o, d

    def intersect_f64(self, o, d, face: int):
        t = np.zeros(1, np.float64)
        b = np.zeros(1, np.float64)
        if not 0 <= int(face) < self.f.shape[0]:
            raise ValueError(f"intersect_f64: face {int(face)} is not a face of this mesh")
        hit = lib().orc_intersect_f64(self.h, _p(np.ascontiguousarray(o, np.float32)),
                                      _p(np.ascontiguousarray(d, np.float32)), int(face), _p(t), _p(b))
        return bool(hit), float(t[0]), float(b[0])

    def trace_rays(self, o, d, tfar: float, nthreads: int = 0):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        t = np.zeros(o.shape[0], np.float32)
        f = np.zeros(o.shape[0], np.uint32)
        lib().orc_trace_rays(self.h, _p(o), _p(d), o.shape[0], float(tfar), _p(t), _p(f), int(nthreads))
        return t, f


def stats_batched(dataset, model, normals=None, dmask=None, mmask=None, max_dist=np.inf, nthreads: int = 0):
    """stats.stats(*stats.correspondences(dataset, model, dmask=dmask, mmask=mmask, max_dist=max_dist,
    normals=normals)) on all host threads in C++ (orc_stats_batched: the same binary32 filters, binary64
    two-pass means and covariance).  dataset / model / normals: [B, N, 3]; masks [B, N]."""
    D = np.ascontiguousarray(dataset, np.float32)
    B, N = D.shape[0], D.shape[1]
    M = np.ascontiguousarray(model, np.float32).reshape(B, N, 3)
    Nn = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(B, N, 3)
    dm = None if dmask is None else np.ascontiguousarray(np.asarray(dmask).reshape(B, N) > 0, np.uint8)
    mm = None if mmask is None else np.ascontiguousarray(np.asarray(mmask).reshape(B, N) > 0, np.uint8)
    out = np.zeros((B, 16), np.float64)
    lib().orc_stats_batched(_p(D), _p(M), _p(Nn), _p(dm), _p(mm), B, N, float(max_dist), int(nthreads), _p(out))
    return {"dataset_mean": out[:, 0:3].copy(), "model_mean": out[:, 3:6].copy(),
            "covariance": out[:, 6:15].reshape(B, 3, 3).copy(), "n": out[:, 15].astype(np.int64)}


def pose_grad(scene, model, Tsb, Tbm, face_ids, ranges, r_obs, delta: float, nthreads: int = 0):
    """grad.RayFaceSet(...).analytic(P, delta) over every valid ray of the simulated scans (face set,
    range >= range.min, range.min <= r_obs <= range.max) on all host threads in C++ (orc_pose_grad).
    Returns (grad [P, 6], loss [P])."""
    k, W, H, dirs, origs, orig = scene._model_args(model)
    Tsb = np.ascontiguousarray(Tsb, np.float32).reshape(8)
    Tbm = np.ascontiguousarray(Tbm, np.float32).reshape(-1, 8)
    P = Tbm.shape[0]
    f = np.ascontiguousarray(face_ids, np.uint32).reshape(-1)
    r = np.ascontiguousarray(ranges, np.float32).reshape(-1)
    o = np.ascontiguousarray(r_obs, np.float32).reshape(-1)
    assert f.size == r.size == o.size == P * W * H
    g = np.zeros((P, 6), np.float64)
    L = np.zeros(P, np.float64)
    lib().orc_pose_grad(scene.h, k, W, H, float(model.range.min), float(model.range.max), _p(dirs), _p(origs),
                        _p(orig), _p(Tsb), _p(Tbm), P, _p(f), _p(r), _p(o), float(delta), int(nthreads), _p(g),
                        _p(L))
    return g, L


def noise_apply(kind, ranges, seed, call, mean=0.0, stddev=0.0, range_exp=1.0, hit_p=0.0, ret_p=0.0,
                max_range=10000.0, nthreads: int = 0):
    """noise.apply(...)'s new ranges (binary64) on all host threads in C++ (orc_noise_apply)."""
    r = np.ascontiguousarray(ranges, np.float32).reshape(-1)
    out = np.empty(r.size, np.float64)
    if lib().orc_noise_apply(int(kind), _p(r), _p(out), r.size, int(seed), int(call), float(mean), float(stddev),
                             float(range_exp), float(hit_p), float(ret_p), float(max_range), int(nthreads)) != 0:
        raise ValueError(f"noise kind {kind}")
    return out


class CanonicalLbvh:
    """The oracle's restatement of the GPU LBVH construction (for tree equality and work counts)."""

    def __init__(self, vertices, faces):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        self.n_faces = f.shape[0]
        self.h = lib().orc_lbvh_build(_p(v), v.shape[0], _p(f), f.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_lbvh_free(self.h)
            self.h = None

    def export(self) -> dict:
        n = int(lib().orc_lbvh_num_nodes(self.h))
        nodes = np.zeros((n, 16), np.float32)
        tris = np.zeros((self.n_faces, 12), np.float32)
        order = np.zeros(self.n_faces, np.uint32)
        lib().orc_lbvh_export(self.h, _p(nodes), _p(tris), _p(order))
        return {"boxes": nodes[:, :12].copy(), "links": nodes.view(np.int32)[:, 12:].copy(), "tris": tris,
                "leaf_order": order}

    def count(self, o, d, tfar: float, nthreads: int = 0):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = o.shape[0]
        visits = np.zeros(n, np.uint32)
        tests = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        f = np.zeros(n, np.uint32)
        lib().orc_lbvh_count(self.h, _p(o), _p(d), n, float(tfar), _p(visits), _p(tests), _p(t), _p(f), int(nthreads))
        return visits, tests, t, f


def tree_count(export: dict, o, d, tfar: float, nthreads: int = 0):
    """Per-ray node visits, triangle tests, hit t and face through a GPU map's exported tree
    (rmg_map_export / Map.export()), in the kernel's visiting order."""
    nodes = np.ascontiguousarray(np.concatenate([export["boxes"], export["links"].view(np.float32)], axis=1),
                                 np.float32)
    tris = np.ascontiguousarray(export["tris"], np.float32)
    o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
    n = o.shape[0]
    visits = np.zeros(n, np.uint32)
    tests = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    f = np.zeros(n, np.uint32)
    lib().orc_tree_count(_p(nodes), _p(tris), tris.shape[0], _p(o), _p(d), n, float(tfar), _p(visits), _p(tests),
                         _p(t), _p(f), int(nthreads))
    return visits, tests, t, f


def certify(scene: Scene, model, Tsb, Tbm, got: dict, want: dict, band: float = 1e-6, tol: float = 1e-4,
            gids=None):
    """Compares two simulation results ray by ray (hits, face ids, ranges).

    `gids`, when given, holds the global ray id of every entry of the arrays (a
    sample of a larger simulation); otherwise entry i is ray i.

    A ray is disputed when the hit flag or face id differ, or |dr| > tol.
    It is excused when binary64 re-intersection puts the relevant hit within
    `band` barycentric of a triangle edge, when the two faces' binary64 t agree
    within `band` relative (a tie), or when t lies within 1e-5 relative of
    range.min / range.max (the flag threshold).  Returns a report dict; the
    caller asserts report["unexcused"] == 0.
    """
    rmin, rmax = float(model.range.min), float(model.range.max)
    # face ids as unsigned 32-bit (a result held in int32 reads a miss as -1)
    f_got = np.asarray(got["face_ids"]).astype(np.int64) & 0xFFFFFFFF
    f_want = np.asarray(want["face_ids"]).astype(np.int64) & 0xFFFFFFFF
    r_got, r_want = got["ranges"], want["ranges"]
    h_got = got.get("hits")
    h_want = want.get("hits")
    bad = (f_got != f_want) | (np.abs(r_got.astype(np.float64) - r_want.astype(np.float64)) > tol)
    if h_got is not None and h_want is not None:
        bad |= h_got != h_want
    idx = np.nonzero(bad)[0]
    rep = {"rays": int(f_got.size), "disputed": int(idx.size), "excused": 0, "unexcused": 0, "examples": []}
    if idx.size == 0:
        return rep
    ray_ids = idx if gids is None else np.asarray(gids, np.uint64)[idx]
    o, d = scene.rays(model, Tsb, Tbm, np.ascontiguousarray(ray_ids, np.uint64))
    for j, gid in enumerate(idx):
        reasons = []
        faces = {int(x) for x in (f_got[gid], f_want[gid]) if int(x) != 0xFFFFFFFF}
        res = {fc: scene.intersect_f64(o[j], d[j], fc) for fc in faces}
        for fc, (hit, t, b) in res.items():
            if abs(b) <= band:
                reasons.append(f"edge(face {fc}, bary {b:.2e})")
            if hit and (abs(t - rmin) <= 1e-5 * max(1.0, rmin) or abs(t - rmax) <= 1e-5 * max(1.0, rmax)):
                reasons.append(f"range bound (t {t:.7g})")
        if len(res) == 2:
            (ha, ta, _), (hb, tb, _) = res.values()
            if ha and hb and abs(ta - tb) <= band * max(1.0, abs(ta)):
                reasons.append("tie")
        if reasons:
            rep["excused"] += 1
        else:
            rep["unexcused"] += 1
            if len(rep["examples"]) < 10:
                rep["examples"].append({"gid": int(ray_ids[j]), "face_got": int(f_got[gid]), "face_want": int(f_want[gid]),
                                        "r_got": float(r_got[gid]), "r_want": float(r_want[gid]),
                                        "f64": {k: v for k, v in res.items()}})
    return rep
