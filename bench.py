#!/usr/bin/env python
"""Throughput of the range-sensor ray-casting path on the GB300.

A step = one rmg_simulate call over all poses of the workload (one launch of
the traversal kernel), inputs (map, sensor table, poses) resident in HBM.
Default workload: the ~1M-triangle terrain (708 x 708 heightfield, 999,698
triangles, plus 2,000 boxes = 1,023,698 triangles), an Ouster-like spherical
sensor 128 x 1024 (+-22.5 deg), 1,000 poses 1.5 m above the ground, all five
attributes (Hits, Ranges, Points, Normals, FaceIds): 131,072,000 rays.

Prints one JSON line (rank 0).  `--impl reference` times the CPU path of the
reference's semantics on the host cores instead (see cpu_leg()).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
ALL = ("hits", "ranges", "points", "normals", "face_ids")
OUT_BYTES = {"hits": 1, "ranges": 4, "points": 12, "normals": 12, "face_ids": 4, "geom_ids": 4, "object_ids": 4}

# Mean internal-node visits and triangle tests per ray of the canonical LBVH
# in the kernel's traversal order, measured by the oracle's instrumented
# traversal (oracle.CanonicalLbvh.count) on a fixed 0.1% ray sample
# (rng seed 0) of each workload; tests/test_work_constants.py re-derives them.
WORK_PER_RAY = {
    "terrain1m_spherical": {"nodes": 39.94, "tris": 1.886},
}


def workload(name: str):
    from rmagine_gb300 import scenes, sensors

    if name == "terrain1m_spherical":
        sc = scenes.million_triangle_terrain(seed=0)
        model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
        poses = scenes.terrain_poses(sc, 1000, seed=2)
        desc = {"workload": "terrain 708x708 + 2000 boxes (1,023,698 tris), spherical 128x1024, 1000 poses, "
                            "Hits+Ranges+Points+Normals+FaceIds"}
        return sc, model, poses, ALL, desc
    if name == "terrain1m_pinhole":
        sc = scenes.million_triangle_terrain(seed=0)
        model = sensors.depth_camera(640, 480, 90.0, 0.3, 130.0)
        poses = scenes.terrain_poses(sc, 1000, seed=2)
        desc = {"workload": "terrain 708x708 + 2000 boxes (1,023,698 tris), pinhole 640x480, 1000 poses, "
                            "Hits+Ranges+Points+Normals+FaceIds"}
        return sc, model, poses, ALL, desc
    if name == "terrain2m_spherical":
        sc = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
        model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
        poses = scenes.terrain_poses(sc, 1000, seed=2)
        desc = {"workload": "terrain 1024x1024 + 2000 boxes (2,117,058 tris), spherical 128x1024, 1000 poses, "
                            "Hits+Ranges+Points+Normals+FaceIds"}
        return sc, model, poses, ALL, desc
    if name == "room_vlp16":
        sc = scenes.box_room(seed=0, n_boxes=200)
        model = sensors.vlp16_900()
        poses = scenes.room_poses(100, seed=1)
        desc = {"workload": "box room + 200 boxes (2,412 tris), VLP-16 16x900, 100 poses, Hits+Ranges"}
        return sc, model, poses, ("hits", "ranges"), desc
    raise SystemExit(f"unknown workload {name}")


def model_size(model):
    import oracle

    return oracle.model_size(model)


# ---- clocks --------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return None
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                rows.append((float(p[1]), float(p[2]), p[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- CPU leg (oracle port of the reference semantics) -------------------------------------------
def cpu_leg(sc, model, poses, attrs, target_s: float = 15.0, max_poses: int | None = None):
    """Times the oracle's OpenMP restatement of rmagine's Embree path on all host cores over a
    bounded pose sample (map build excluded, as in the reference's benchmark loop)."""
    import oracle

    ocs = oracle.Scene(sc.vertices, sc.faces)
    threads = oracle.lib().orc_max_threads()
    W, H = model_size(model)
    # probe with one pose to size the sample
    t0 = time.perf_counter()
    ocs.simulate(model, IDENT, poses[:1], attrs=attrs, nthreads=threads)
    per_pose = max(time.perf_counter() - t0, 1e-4)
    n = int(max(1, min(len(poses), target_s / per_pose)))
    if max_poses:
        n = min(n, max_poses)
    t0 = time.perf_counter()
    ocs.simulate(model, IDENT, poses[:n], attrs=attrs, nthreads=threads)
    dt = time.perf_counter() - t0
    rays = n * W * H
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": int(threads), "kind": "port",
            "sample": f"{n} of {len(poses)} poses ({rays} rays), all host threads, oracle SAH-BVH restatement "
                      f"of the Embree path (Embree itself is not buildable here)", "seconds": dt}


# ---- GPU leg ---------------------------------------------------------------------------------------
def gpu_leg(args, sc, model, poses, attrs, desc, rank, world):
    import torch

    import rmagine_gb300 as rm

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W, H = model_size(model)
    n = poses.shape[0]
    rays = n * W * H
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(model, m)
    Tbm = torch.from_numpy(poses).to(dev)
    bundle = rm.resize_memory_bundle(rm.Bundle(*attrs), W, H, n, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > L2
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    for _ in range(args.warmup):
        sim.simulate(Tbm, bundle)
    torch.cuda.synchronize(dev)
    if m.status() != 0:
        raise RuntimeError("device status error during warm-up")

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(dev.index) as clk:
        for i in range(args.steps):
            flush.zero_()  # evict L2 between timed steps (outside the events)
            starts[i].record(stream)
            sim.simulate(Tbm, bundle)
            ends[i].record(stream)
        torch.cuda.synchronize(dev)
    barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    if m.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * rays * args.steps / (total_ms / 1e3) / 1e6

    # e2e through the public API: host (pinned) poses in, host (pinned) bundle out, synchronous
    host_poses = torch.from_numpy(poses).pin_memory()
    hb = rm.resize_memory_bundle(rm.Bundle(*attrs), W, H, n, device="cpu", pin_memory=True)
    sim.simulate(host_poses, hb)  # warm the staging buffers
    e2e_t = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sim.simulate(host_poses, hb)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = rays / (sum(e2e_t) / len(e2e_t)) / 1e6
    d2h = rays * sum(OUT_BYTES[a] for a in attrs)

    bytes_per_ray = None
    wk = WORK_PER_RAY.get(args.workload)
    peak, peak_kind = measured_peaks()
    roofline = None
    if wk:
        bytes_per_ray = sum(OUT_BYTES[a] for a in attrs) + 64 * wk["nodes"] + 48 * wk["tris"]
        per_launch_s = total_ms / args.steps / 1e3
        achieved = bytes_per_ray * rays / per_launch_s / 1e9
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": peak_kind,
                    "algorithmic_bytes_per_ray": round(bytes_per_ray, 1),
                    "note": "algorithmic bytes = outputs + 64 B per node visit + 48 B per triangle test; "
                            "node and triangle fetches are served mostly from L2"}
        tr = TRAFFIC.get(args.workload)
        if tr:
            roofline["traffic"] = tr
    return {
        "value": value, "ms_per_step": total_ms / args.steps, "step_ms": step_ms, "rays_per_step": rays,
        "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": int(poses.nbytes),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": roofline, "clocks": clk.summary(), "map": m.info(),
    }


# Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the
# traversal kernel from one ncu capture of the workload; see profiles/.
TRAFFIC: dict = {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="terrain1m_spherical")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--poses", type=int, default=0, help="use only the first N poses (small profiling case)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    sc, model, poses, attrs, desc = workload(args.workload)
    if args.poses:
        poses = poses[:args.poses]
    W, H = model_size(model)
    config = dict(desc)
    config.update({"poses": int(poses.shape[0]), "rays_per_step": int(poses.shape[0] * W * H),
                   "triangles": int(sc.n_faces), "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas{world}" if world > 1 else "single"})
    base = {"metric": "Mrays/s", "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural terrain and poses)", "config": config}

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import build as ob

        ob.build()
        vals = []
        leg = None
        for _ in range(args.warmup + args.steps):
            leg = cpu_leg(sc, model, poses, attrs, target_s=max(2.0, 60.0 / (args.steps + args.warmup)))
            vals.append(leg["value"])
        v = statistics.mean(vals[args.warmup:]) if len(vals) > args.warmup else vals[-1]
        out = dict(base)
        out.update({"impl": "reference", "value": round(v, 3), "ms_per_step": round(1e3 * leg["seconds"], 1),
                    "gpu_launches": 0,
                    "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": leg["cores"],
                                     "kind": "port", "sample": leg["sample"]},
                    "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}})
        print(json.dumps(out))
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    res = gpu_leg(args, sc, model, poses, attrs, desc, rank, world)
    if rank != 0:
        return
    out = dict(base)
    out.update({"value": round(res["value"], 2), "ms_per_step": round(res["ms_per_step"], 3),
                "e2e": res["e2e"], "roofline": res["roofline"], "clocks": res["clocks"],
                "gpu_launches": args.steps, "step_ms": [round(x, 3) for x in res["step_ms"]],
                "map": {k: res["map"][k] for k in ("n_faces", "n_nodes", "depth", "device_bytes")}})
    if not args.no_cpu_baseline:
        from oracle import build as ob

        ob.build()
        cpu = cpu_leg(sc, model, poses, attrs)
        out["cpu_baseline"] = {k: (round(v, 3) if isinstance(v, float) else v) for k, v in cpu.items()
                               if k != "seconds"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
