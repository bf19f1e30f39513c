"""ORACLE -- test infrastructure only.

Restatement of ray casting on an instanced scene (several meshes placed by instances) for
checking rmg_simulate_scene.  The reference resolves instances inside Embree / OptiX
(EmbreeScene.cpp:246-406, EmbreeInstance.cpp:33-60, SphereSimulatorEmbree.tcc:160-186,
SensorProgramHit.cu:120-136, 220-262); this oracle states the same result without a top-level
tree: every instance is tried (brute force), the ray is taken into the instance's mesh frame in
binary32 with the kernel's operation order (o_l = s^-1 (.) conj(q) (o - t) q, d_l likewise),
each mesh's closest hit comes from the oracle's own BVH (`Scene.trace_rays`), and the overall
hit is the smallest range, then the smaller instance index, then the smaller face index.
Normals go mesh -> map by R s^-1 (the OptiX path's object-to-world normal transform) and then
to the sensor frame as for a single mesh.
"""
from __future__ import annotations

import numpy as np

from . import Scene, directions, model_kind, model_size
from .stats import _qmul

F32 = np.float32
MISS = 0xFFFFFFFF


def _qrot(q, v):
    """q (v, 0) conj(q) in binary32, Quaternion.tcc:68-75 term order."""
    q = np.asarray(q, F32)
    v = np.asarray(v, F32)
    lead = np.broadcast_shapes(q.shape[:-1], v.shape[:-1])
    q = np.broadcast_to(q, lead + (4,)).astype(F32)
    v = np.broadcast_to(v, lead + (3,)).astype(F32)
    P = np.concatenate([v, np.zeros(v.shape[:-1] + (1,), F32)], axis=-1)
    return _qmul(_qmul(q, P), (q * np.array([-1, -1, -1, 1], F32)).astype(F32))[..., :3]


def _compose(T1, T2):
    """Transform::mult (Transform.tcc:34-42) in binary32."""
    out = np.zeros(np.broadcast_shapes(T1.shape, T2.shape), F32)
    rt = _qrot(T1[..., :4], T2[..., 4:7])
    out[..., :4] = _qmul(T1[..., :4], T2[..., :4])
    out[..., 4:7] = rt + T1[..., 4:7]
    return out


def _unit(n):
    n = n.astype(F32)
    ln = np.sqrt((n[..., 0] * n[..., 0] + n[..., 1] * n[..., 1]) + n[..., 2] * n[..., 2]).astype(F32)
    return (n / ln[..., None]).astype(F32)


class InstancedScene:
    """meshes: list of (vertices, faces); instances: list of dicts with geometry, T [8], scale [3],
    geom_id, object_id."""

    def __init__(self, meshes, instances):
        self.meshes = [(np.asarray(v, F32).reshape(-1, 3), np.asarray(f, np.uint32).reshape(-1, 3)) for v, f in meshes]
        self.scenes = [Scene(v, f) if f.shape[0] > 0 else None for v, f in self.meshes]
        self.instances = []
        for inst in instances:
            T = np.asarray(inst["T"], F32).reshape(-1)[:8]
            if T.size == 7:
                T = np.concatenate([T, np.zeros(1, F32)])
            s = np.asarray(inst.get("scale", (1, 1, 1)), F32).reshape(3)
            self.instances.append({"geometry": int(inst["geometry"]), "T": T, "scale": s,
                                   "inv_s": (F32(1) / s).astype(F32), "geom_id": int(inst.get("geom_id", 0)),
                                   "object_id": int(inst.get("object_id", 0))})
        # any triangle scene generates rays (they do not depend on the mesh)
        self._ray_scene = Scene(np.zeros((3, 3), F32), np.array([[0, 1, 2]], np.uint32))

    def local_rays(self, i, o, d):
        I = self.instances[i]
        qinv = (I["T"][:4] * np.array([-1, -1, -1, 1], F32)).astype(F32)
        ol = (_qrot(qinv, (o - I["T"][4:7]).astype(F32)) * I["inv_s"]).astype(F32)
        dl = (_qrot(qinv, d) * I["inv_s"]).astype(F32)
        return ol, dl

    def trace(self, o, d, tfar):
        n = o.shape[0]
        best_t = np.full(n, F32(tfar), F32)
        best_i = np.full(n, -1, np.int64)
        best_f = np.full(n, MISS, np.uint32)
        for i, I in enumerate(self.instances):
            sc = self.scenes[I["geometry"]]
            if sc is None:
                continue
            ol, dl = self.local_rays(i, o, d)
            t, f = sc.trace_rays(ol, dl, tfar)
            better = np.isfinite(t) & ((best_i < 0) | (t < best_t))
            best_t[better] = t[better]
            best_i[better] = i
            best_f[better] = f[better]
        return best_t, best_i, best_f

    def simulate(self, model, Tsb, Tbm, attrs=("hits", "ranges", "points", "normals", "face_ids", "geom_ids",
                                                "object_ids")):
        W, H = model_size(model)
        Tbm = np.asarray(Tbm, F32).reshape(-1, 8)
        Tsb = np.asarray(Tsb, F32).reshape(8)
        P = Tbm.shape[0]
        n = P * W * H
        gids = np.arange(n, dtype=np.uint64)
        o, d = self._ray_scene.rays(model, Tsb, Tbm, gids)
        rmin, rmax = F32(model.range.min), F32(model.range.max)
        t, inst, face = self.trace(o, d, float(rmax))
        hit = inst >= 0
        out = {"instance": inst}
        dirs = directions(model).reshape(-1, 3).astype(F32)
        loc = (gids % (W * H)).astype(np.int64)
        dir_s = dirs[loc]
        if "hits" in attrs:
            out["hits"] = (hit & (t >= rmin)).astype(np.uint8)
        if "ranges" in attrs:
            out["ranges"] = np.where(hit, t, (rmax + F32(1)).astype(F32)).astype(F32)
        if "points" in attrs:
            p = (dir_s * t[:, None]).astype(F32)
            kind = model_kind(model)
            if kind == 2:
                p = (p + np.asarray(model.orig, F32).reshape(1, 3)).astype(F32)
            elif kind == 3:
                p = (p + np.asarray(model.origs, F32).reshape(-1, 3)[loc]).astype(F32)
            p[~hit] = np.nan
            out["points"] = p
        if "normals" in attrs:
            nrm = np.full((n, 3), np.nan, F32)
            idx = np.nonzero(hit)[0]
            if idx.size:
                Tsm = _compose(Tbm[(idx // (W * H)).astype(np.int64)], Tsb[None, :])
                for i in np.unique(inst[idx]):
                    sel = idx[inst[idx] == i]
                    I = self.instances[int(i)]
                    v, f = self.meshes[I["geometry"]]
                    tri = v[f[face[sel].astype(np.int64)]]
                    e1 = (tri[:, 1] - tri[:, 0]).astype(F32)
                    e2 = (tri[:, 2] - tri[:, 0]).astype(F32)
                    c = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                                  e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1).astype(F32)
                    nl = (_unit(c) * I["inv_s"]).astype(F32)
                    nm = _qrot(I["T"][:4], nl)
                    k = np.searchsorted(idx, sel)
                    qc = (Tsm[k, :4] * np.array([-1, -1, -1, 1], F32)).astype(F32)
                    ns = _qrot(qc, nm)
                    ds = dir_s[sel]
                    dp = (ds[:, 0] * ns[:, 0] + ds[:, 1] * ns[:, 1]) + ds[:, 2] * ns[:, 2]
                    ns[dp > 0] = -ns[dp > 0]
                    nrm[sel] = _unit(ns)
            out["normals"] = nrm
        if "face_ids" in attrs:
            out["face_ids"] = np.where(hit, face, MISS).astype(np.uint32)
        gi = np.array([I["geom_id"] for I in self.instances] + [MISS], np.uint32)
        oi = np.array([I["object_id"] for I in self.instances] + [MISS], np.uint32)
        if "geom_ids" in attrs:
            out["geom_ids"] = gi[inst]
        if "object_ids" in attrs:
            out["object_ids"] = oi[inst]
        return out

    def certify(self, model, Tsb, Tbm, got: dict, want: dict, band: float = 1e-6, tol: float = 1e-4, gids=None):
        """Rays on which two results differ (hit, face, object id or |dr| > tol) are excused when a
        binary64 re-intersection of the involved (instance, face) pairs puts a hit within `band`
        barycentric of an edge, or two candidate hits tie within `band` relative.  got / want
        must carry face_ids, ranges and object_ids (object ids unique per instance).  `gids`, when
        given, holds the global ray id of every entry (a sample of a larger simulation)."""
        f_got, f_want = got["face_ids"], want["face_ids"]
        bad = (f_got != f_want) | (got["object_ids"] != want["object_ids"]) | \
            (np.abs(got["ranges"].astype(np.float64) - want["ranges"].astype(np.float64)) > tol)
        idx = np.nonzero(bad)[0]
        rep = {"rays": int(f_got.size), "disputed": int(idx.size), "excused": 0, "unexcused": 0, "examples": []}
        if idx.size == 0:
            return rep
        by_obj = {I["object_id"]: i for i, I in enumerate(self.instances)}
        ray_ids = idx if gids is None else np.asarray(gids, np.uint64)[idx]
        o, d = self._ray_scene.rays(model, Tsb, Tbm, np.ascontiguousarray(ray_ids, np.uint64))
        for j, gid in enumerate(idx):
            cands = []
            for res in (got, want):
                f, ob = int(res["face_ids"][gid]), int(res["object_ids"][gid])
                if f != MISS and ob in by_obj:
                    cands.append((by_obj[ob], f))
            reasons, ts = [], []
            for i, f in set(cands):
                ol, dl = self.local_rays(i, o[j:j + 1], d[j:j + 1])
                h, t, b = self.scenes[self.instances[i]["geometry"]].intersect_f64(ol[0], dl[0], f)
                if abs(b) <= band:
                    reasons.append("edge")
                if h:
                    ts.append(t)
            if len(ts) == 2 and abs(ts[0] - ts[1]) <= band * max(1.0, abs(ts[0])):
                reasons.append("tie")
            if reasons:
                rep["excused"] += 1
            else:
                rep["unexcused"] += 1
                if len(rep["examples"]) < 10:
                    rep["examples"].append({"gid": int(gid), "got": (int(f_got[gid]), int(got["object_ids"][gid]),
                                                                     float(got["ranges"][gid])),
                                            "want": (int(f_want[gid]), int(want["object_ids"][gid]),
                                                     float(want["ranges"][gid]))})
        return rep
