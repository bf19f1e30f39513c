"""Many heterogeneous sensors in one persistent, graph-replayed launch (rmg_batch plans).

    plan = BatchPlan(map, [(simulator_or_sensor, Tbm_device, bundle), ...])
    plan.autotune()          # optional: picks stack depth / warps / tile / grab, cached on disk
    plan.launch()            # all sensors' rays, one kernel, one graph launch

Outputs are bit-identical to one `simulate` per entry.  The plan holds the device tensors it
was built with: to move poses, write into the same Tbm tensors and launch again.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path

import torch

from . import _lib as L
from .simulation import Bundle, Map, Sensor, _Simulator, outputs_c, transform_c


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def default_cache_path() -> Path:
    return Path(os.environ.get("RMG_AUTOTUNE_CACHE", Path.home() / ".cache" / "rmagine_gb300" / "autotune.json"))


class BatchPlan:
    def __init__(self, map: Map, jobs, config: L.BatchConfigC | None = None):
        self._h = None
        self.map = map
        self._keep = []  # tensors and sensors the device table points into
        entries = (L.BatchEntryC * max(1, len(jobs)))()
        sig = []
        for i, job in enumerate(jobs):
            who, Tbm, bundle = job[0], job[1], job[2]
            Tsb = job[3] if len(job) > 3 else None
            if isinstance(who, _Simulator):
                sensor, tsb = who.sensor, who._Tsb
            else:
                sensor, tsb = who, transform_c(Tsb if Tsb is not None else [0, 0, 0, 1, 0, 0, 0])
            Tbm = Tbm.reshape(-1, 8)
            if not Tbm.is_cuda or not Tbm.is_contiguous():
                raise L.RmgError(L.RMG_ERR_INVALID_ARG, "BatchPlan", "Tbm must be a contiguous CUDA tensor")
            n = Tbm.shape[0]
            for a, t in bundle.tensors().items():
                if not t.is_cuda or t.shape[0] != sensor.width * sensor.height * n:
                    raise L.RmgError(L.RMG_ERR_INVALID_ARG, "BatchPlan", f"{a}: wrong size or not on the device")
            entries[i].sensor = sensor.handle
            entries[i].Tsb = tsb
            entries[i].Tbm = Tbm.data_ptr()
            entries[i].n_poses = n
            entries[i].out = outputs_c(bundle)
            self._keep.extend([sensor, Tbm, bundle])
            sig.append((sensor.model.kind, sensor.width, sensor.height, n))
        h = C.c_void_p()
        L.call("rmg_batch_create", map.handle, entries, len(jobs), C.byref(h))
        self._h = h
        self.signature = sig
        if config is not None:
            self.set_config(config)

    def config(self) -> L.BatchConfigC:
        c = L.BatchConfigC()
        L.call("rmg_batch_get_config", self._h, C.byref(c))
        return c

    def set_config(self, c: L.BatchConfigC) -> None:
        L.call("rmg_batch_set_config", self._h, C.byref(c))

    def info(self) -> dict:
        r, t = C.c_uint64(), C.c_uint64()
        L.call("rmg_batch_info", self._h, C.byref(r), C.byref(t))
        return {"rays": r.value, "tiles": t.value}

    def launch(self) -> None:
        L.call("rmg_batch_launch", self._h, _stream())

    def _cache_key(self) -> str:
        name = torch.cuda.get_device_name()
        mesh = self.map.info()["n_faces"]
        bucket = 1 << max(0, int(mesh).bit_length() - 1)
        return json.dumps([name, bucket, sorted(self.signature)])

    def autotune(self, reps: int = 3, cache: Path | None = None, use_cache: bool = True) -> L.BatchConfigC:
        """Finds the fastest launch options for this plan (in the library), cached per GPU,
        mesh-size bucket and job signature in a JSON file."""
        cache = Path(cache) if cache else default_cache_path()
        key = self._cache_key()
        table = {}
        if use_cache and cache.exists():
            try:
                table = json.loads(cache.read_text())
            except ValueError:
                table = {}
        if use_cache and key in table:
            c = L.BatchConfigC(*table[key])
            self.set_config(c)
            return c
        best = L.BatchConfigC()
        L.call("rmg_batch_autotune", self._h, _stream(), reps, C.byref(best))
        if use_cache:
            table[key] = [best.stack_depth, best.block_warps, best.tile_w, best.tile_h, best.grab, best.ctas_per_sm,
                          best.use_graph]
            cache.parent.mkdir(parents=True, exist_ok=True)
            cache.write_text(json.dumps(table, indent=1))
        return best

    def destroy(self) -> None:
        if self._h is not None:
            L.load().rmg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class ChunkedBatchPlan:
    """Host-result form of a batch: every job's poses are split into n_chunks ranges and one
    BatchPlan is built per range.  run_to_host() launches the plans in order on the current stream
    and copies each plan's outputs to host memory on a second stream while the next plan runs, so
    the device->host copy of all but the last range overlaps the ray casting.  Outputs are
    bit-identical to one BatchPlan over all poses (every ray is independent).  Jobs are given as
    for BatchPlan, with device Tbm and device bundles; a job with fewer poses than n_chunks sits in
    the first ranges only."""

    def __init__(self, map: Map, jobs, n_chunks: int = 4, config: L.BatchConfigC | None = None):
        self.jobs = list(jobs)
        self.plans: list[BatchPlan] = []
        self.slices: list[list[tuple[int, int, int]]] = []  # per plan: (job, first ray, end ray)
        for k in range(max(1, int(n_chunks))):
            sub, sl = [], []
            for j, job in enumerate(self.jobs):
                who, Tbm, bundle = job[0], job[1].reshape(-1, 8), job[2]
                n = Tbm.shape[0]
                p0, p1 = n * k // n_chunks, n * (k + 1) // n_chunks
                if p1 <= p0:
                    continue
                sensor = who.sensor if isinstance(who, _Simulator) else who
                per = sensor.width * sensor.height
                b = Bundle(*bundle.attrs)
                for a, t in bundle.tensors().items():
                    setattr(b, a, t[p0 * per:p1 * per])
                sub.append((who, Tbm[p0:p1], b) + tuple(job[3:]))
                sl.append((j, p0 * per, p1 * per))
            if sub:
                self.plans.append(BatchPlan(map, sub, config))
                self.slices.append(sl)
        self._copy = None

    def launch(self) -> None:
        """All ranges on the device, asynchronously on the current stream."""
        for p in self.plans:
            p.launch()

    def run_to_host(self, host_bundles) -> None:
        """host_bundles[j]: host Bundle of job j (same attributes and sizes as its device bundle;
        pinned memory copies fastest).  Synchronous."""
        if self._copy is None:
            self._copy = torch.cuda.Stream()
        cur = torch.cuda.current_stream()
        self._copy.wait_stream(cur)
        for plan, sl in zip(self.plans, self.slices):
            plan.launch()
            ev = torch.cuda.Event()
            ev.record(cur)
            self._copy.wait_event(ev)
            with torch.cuda.stream(self._copy):
                for j, r0, r1 in sl:
                    host = host_bundles[j]
                    for a, t in self.jobs[j][2].tensors().items():
                        getattr(host, a)[r0:r1].copy_(t[r0:r1], non_blocking=True)
        cur.wait_stream(self._copy)
        cur.synchronize()


def batch_config(stack_depth=8, block_warps=4, tile_w=8, tile_h=4, grab=2, ctas_per_sm=0, use_graph=1):
    return L.BatchConfigC(stack_depth, block_warps, tile_w, tile_h, grab, ctas_per_sm, use_graph)


def mixed_sensor_set(n_sensors: int, seed: int, max_poses: int = 4096):
    """Cfg of the batched workload: sensors drawn uniformly from {VLP-16 16x900, spherical 128x2048,
    pinhole 640x480, O1Dn 10k directions uniform on the sphere with origin (0.1, 0, 0.2)}; pose
    count per sensor floor(exp(U(ln 1, ln max_poses)))."""
    import numpy as np

    from . import sensors

    rng = np.random.default_rng(seed)
    kinds = rng.integers(0, 4, n_sensors)
    counts = np.floor(np.exp(rng.uniform(0.0, np.log(max_poses), n_sensors))).astype(int)
    out = []
    o1 = sensors.O1DnModel(width=10000, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.1, 0.0, 0.2),
                           dirs=sensors.sphere_directions(10000, seed=seed + 7))
    for k, c in zip(kinds, counts):
        if k == 0:
            m = sensors.vlp16_900()
        elif k == 1:
            m = sensors.ouster_like(128, 2048, 45.0, 0.5, 130.0)
        elif k == 2:
            m = sensors.depth_camera(640, 480, 90.0, 0.3, 130.0)
        else:
            m = o1
        out.append((m, int(max(1, c))))
    return out


def small_sensor_set(n_sensors: int, seed: int, max_poses: int = 8):
    """Many small sensors, where one launch per sensor is launch-bound: O1Dn sensors of 256
    directions (each its own set, uniform on the sphere, origin (0.05, 0, 0.1)) and 32x8 pinhole
    cameras, alternating, with floor(exp(U(ln 1, ln max_poses))) poses per sensor."""
    import numpy as np

    from . import sensors

    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(0.0, np.log(max_poses), n_sensors))).astype(int)
    out = []
    for i, c in enumerate(counts):
        if i % 2 == 0:
            m = sensors.O1DnModel(width=256, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.05, 0.0, 0.1),
                                  dirs=sensors.sphere_directions(256, seed=seed + 1000 + i))
        else:
            m = sensors.depth_camera(32, 8, 60.0, 0.3, 130.0)
        out.append((m, int(max(1, c))))
    return out
