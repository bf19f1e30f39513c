#!/usr/bin/env python
"""Throughput of the range-sensor ray-casting path (and its companions) on the GB300.

Default workload (`--workload terrain1m_spherical`): a step = one rmg_simulate call over all
poses (one launch of the traversal kernel), map / sensor table / poses resident in HBM.  The
~1M-triangle terrain (708 x 708 heightfield = 999,698 triangles + 2,000 boxes = 1,023,698),
an Ouster-like spherical sensor 128 x 1024 (+-22.5 deg), 1,000 poses 1.5 m above the ground,
all five attributes (Hits, Ranges, Points, Normals, FaceIds): 131,072,000 rays per step.

Other workloads: terrain1m_pinhole, terrain2m_spherical (2,117,058 triangles), room_vlp16;
icp_stats (8192 batches x 32768 correspondences: statistics_p2p + Umeyama forward and the
backward, correspondences/s); pose_grad (2.1M-triangle terrain, spherical 64 x 1024, 4096
poses: fused ray cast + range adjoint, pose-gradient evaluations/s); rcc_fused (the
correction loop's inner step fused: model ray cast at 1,000 pose estimates paired ray by ray
with per-pose scans into statistics_p2l + Umeyama, sensor rays/s, with the two-step
simulate + statistics path timed beside it); batched (64 mixed sensors in one launch).

Prints one JSON line (rank 0).  `--impl reference` times the CPU restatement of the reference's
semantics on the host cores instead (see the cpu_* functions).
"""
from __future__ import annotations

import argparse
import json
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


def host_link_bytes(attrs, rays):
    """Bytes per ray the host-buffer forms move device -> host: with Ranges requested and at least
    64 MB of Points, the points are formed on the host from the ranges (csrc/host.cu, HostDerive)
    and not copied."""
    derived = {"points"} if "ranges" in attrs and "points" in attrs and rays * 12 >= (64 << 20) else set()
    return sum(OUT_BYTES[a] for a in attrs if a not in derived)

# Mean internal-node visits and triangle tests per ray of the canonical LBVH in the kernel's
# traversal order, measured by the oracle's instrumented traversal (oracle.CanonicalLbvh.count)
# on a fixed 0.1% ray sample (rng seed 0) of each workload; tests/test_work_constants.py
# re-derives them on smaller samples.
WORK_PER_RAY = {
    "terrain1m_spherical": {"nodes": 30.521, "tris": 1.800},
    "terrain1m_pinhole": {"nodes": 27.285, "tris": 1.657},
    "terrain2m_spherical": {"nodes": 30.580, "tris": 1.764},
    "room_vlp16": {"nodes": 65.651, "tris": 3.919},
    "pose_grad": {"nodes": 30.260, "tris": 1.763},
    # averaged over all sensor rays; rays without a valid dataset point (1 - data_frac) are not cast
    "rcc_fused": {"nodes": 21.417, "tris": 1.715, "data_frac": 0.554},
}

# Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernel,
# from one ncu capture of the workload (profiles/).
TRAFFIC: dict = {
    # captured on 100 poses (13.1 M rays) and scaled by the ray count to the 1,000-pose launch
    "terrain1m_spherical": 10 * (292245504 + 441846016),
    # captured on 512 batches (16.8 M correspondences) and scaled by 16 to the 8,192-batch launch
    "icp_stats_fwd": 16 * (402915328 + 3088384),
    "icp_stats_bwd": 16 * (403369216 + 357416960),
    # captured on 64 poses (4.19 M rays) and scaled by 64 to the 4,096-pose launch
    "pose_grad": 64 * (224337920 + 14536960),
    # captured on 50 poses (15.4 M rays) / 100 poses (13.1 M rays) and scaled to the 1,000-pose launch
    "terrain1m_pinhole": 20 * (87372800 + 503376896),
    "terrain2m_spherical": 10 * (545676032 + 467888640),
    # captured on 100 poses (13.1 M rays) and scaled by the ray count to the 1,000-pose launch
    "rcc_fused": 10 * (295333888 + 25030912),
    # full-size launch (131,072,000 ranges)
    "noise": 524465664 + 463988224,
    # captured on 100 poses (13.1 M rays) and scaled by the ray count to the 1,000-pose launch
    "scene_terrain1m": 10 * (364896000 + 665387776),
    # the whole 1,024-sensor launch (780,800 rays)
    "batched_small": 207004928 + 27197184,
    # captured with every sensor cut to 16 poses (143,238,688 rays) and scaled by the ray count to the
    # full 64-sensor launch (9,025,081,856 rays)
    "batched": round(9025081856 / 143238688 * (2130438912 + 852212224)),
}

SRC_COUNTERS = "profiles/traversal_counters_by_workload.md (small cases)"

# Warp instructions per unit (ray) of the dominant kernel, `smsp__inst_executed.sum` of one ncu
# capture on the small case of the workload divided by its rays (profiles/), keyed by kernel walk.
ISSUE: dict = {
    "terrain1m_spherical/full_stack": {"warp_inst_per_unit": 1601428820 / 13107200, "source":
                                       "profiles/k_trace_terrain1m_spherical.md (100 poses, 13,107,200 rays)"},
    "pose_grad/k_range_grad": {"warp_inst_per_unit": 591709423 / 4194304, "source":
                               "profiles/k_range_grad_terrain2m_posegrad.md (64 poses, 4,194,304 rays)"},
    "terrain1m_pinhole/packet": {"warp_inst_per_unit": 1218427530 / 15360000, "source": SRC_COUNTERS},
    "terrain1m_pinhole/full_stack": {"warp_inst_per_unit": 1300374245 / 15360000, "source": SRC_COUNTERS},
    "terrain2m_spherical/full_stack": {"warp_inst_per_unit": 1716707653 / 13107200, "source": SRC_COUNTERS},
    "room_vlp16/packet": {"warp_inst_per_unit": 117898004 / 1440000, "source": SRC_COUNTERS},
    "room_vlp16/full_stack": {"warp_inst_per_unit": 129417314 / 1440000, "source": SRC_COUNTERS},
    "rcc_fused/k_trace_stats": {"warp_inst_per_unit": 1329978711 / 13107200, "source": SRC_COUNTERS},
    "scene_terrain1m/k_trace_scene": {"warp_inst_per_unit": 2033824909 / 13107200, "source": SRC_COUNTERS},
    "batched_small/k_trace_batched": {"warp_inst_per_unit": 164797836 / 780800, "source": SRC_COUNTERS},
    "batched/k_trace_batched": {"warp_inst_per_unit": 14365424579 / 143238688, "source":
                                "profiles/k_trace_batched_mixed64.md (16 poses per sensor, 143,238,688 rays, "
                                "autotuned launch options)"},
}

RAYCAST = ("terrain1m_spherical", "terrain1m_pinhole", "terrain2m_spherical", "terrain33m_spherical", "room_vlp16")


def raycast_workload(name: str):
    from rmagine_gb300 import scenes, sensors

    if name in ("terrain1m_spherical", "terrain1m_pinhole"):
        sc = scenes.million_triangle_terrain(seed=0)
        tri = "terrain 708x708 + 2000 boxes (1,023,698 tris)"
    elif name == "terrain2m_spherical":
        sc = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
        tri = "terrain 1024x1024 + 2000 boxes (2,117,058 tris)"
    elif name == "terrain33m_spherical":
        sc = scenes.terrain(grid=4096, size=2000.0, n_boxes=2000, seed=0)
        tri = "terrain 4096x4096 over 2 km + 2000 boxes (33,562,050 tris)"
    elif name == "room_vlp16":
        sc = scenes.box_room(seed=0, n_boxes=200)
        model = sensors.vlp16_900()
        poses = scenes.room_poses(100, seed=1)
        return sc, model, poses, ("hits", "ranges"), {
            "workload": "box room + 200 boxes (2,412 tris), VLP-16 16x900, 100 poses, Hits+Ranges"}
    else:
        raise SystemExit(f"unknown workload {name}")
    if name.endswith("pinhole"):
        model = sensors.depth_camera(640, 480, 90.0, 0.3, 130.0)
        mdesc = "pinhole 640x480 (90 deg hfov)"
    else:
        model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
        mdesc = "spherical 128x1024 (+-22.5 deg)"
    poses = scenes.terrain_poses(sc, 1000, seed=2, size=2000.0 if name.startswith("terrain33m") else 500.0)
    return sc, model, poses, ALL, {"workload": f"{tri}, {mdesc}, 1000 poses, Hits+Ranges+Points+Normals+FaceIds"}


def model_size(model):
    return int(model.getWidth()), int(model.getHeight())


# ---- clocks ------------------------------------------------------------------------------
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


def measured_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def sm_count():
    import ctypes as C

    from rmagine_gb300 import _lib

    n, a, b = C.c_int(0), C.c_int(0), C.c_int(0)
    _lib.check(_lib.load().rmg_device_info(C.byref(n), C.byref(a), C.byref(b)), "rmg_device_info")
    return int(n.value)


def issue_roofline(kernel, units_per_launch, launch_s, clocks, traffic, note):
    """The traversal kernels are bound by instruction issue (ALU pipe, divergence, dependent node
    fetches), not by DRAM: `achieved` = warp instructions per ray (ncu, `ISSUE` below) x rays per
    launch / the launch's CUDA-event time, `peak` = SMs x 4 schedulers x the SM clock sampled during
    the timed region (one warp instruction per scheduler per cycle).  `hbm` beside it is the measured
    DRAM traffic per launch over the same time against the measured copy peak."""
    inst = ISSUE.get(kernel)
    if inst is None:
        return None
    sms = sm_count()
    mhz = (clocks or {}).get("sm_mhz") or float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"]
                                                if (ROOT / "MEASURED_PEAKS.json").exists() else 2070.0)
    achieved = inst["warp_inst_per_unit"] * units_per_launch / launch_s / 1e9
    peak = sms * 4 * mhz * 1e6 / 1e9
    hbm_peak, kind = measured_hbm()
    out = {"bound": "issue", "achieved": round(achieved, 1), "peak": round(peak, 1), "unit": "Gwarp-inst/s",
           "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": "SMs x 4 x sampled SM clock",
           "sm_count": sms, "sm_mhz": mhz, "warp_inst_per_unit": inst["warp_inst_per_unit"],
           "inst_source": inst["source"], "units_per_launch": int(units_per_launch), "note": note}
    if traffic:
        hb = traffic / launch_s / 1e9
        out["hbm"] = {"achieved": round(hb, 1), "peak": hbm_peak, "unit": "GB/s", "frac": round(hb / hbm_peak, 4),
                      "peak_kind": kind}
    return out


def traffic_roofline(traffic, launch_s, note):
    """Measured DRAM bytes per launch (ncu) over the launch's CUDA-event time against the measured HBM
    copy peak, where no instruction count is recorded; None without a capture."""
    if not traffic:
        return None
    peak, kind = measured_hbm()
    achieved = traffic / launch_s / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": kind,
            "note": note + "; bytes = the measured DRAM traffic of the dominant kernel"}


def roofline(bytes_per_unit, units_per_launch, launch_s, note, traffic=None):
    peak, kind = measured_hbm()
    achieved = bytes_per_unit * units_per_launch / launch_s / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": kind,
            "algorithmic_bytes_per_unit": round(bytes_per_unit, 2), "units_per_launch": int(units_per_launch),
            "note": note}


def nvtx_range(name):
    """Pushes an NVTX range; returns the function that pops it (a no-op where NVTX is missing)."""
    try:
        import torch

        torch.cuda.nvtx.range_push(name)
        return torch.cuda.nvtx.range_pop
    except Exception:
        return lambda: None


class Timer:
    """Per-step CUDA events on the launching stream with an L2 flush between steps."""

    def __init__(self, dev, steps):
        import torch

        self.torch = torch
        self.dev = dev
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
        self.ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]

    def run(self, fn, world):
        torch = self.torch
        stream = torch.cuda.current_stream(self.dev)
        barrier(world)
        torch.cuda.synchronize(self.dev)
        with ClockSampler(self.dev.index) as clk:
            # one more untimed step after the sampler's start-up pause: the GPU idles during the pause,
            # and the first step after it would otherwise run while the clocks ramp back up
            fn()
            torch.cuda.synchronize(self.dev)
            barrier(world)
            nvtx = nvtx_range("timed")  # lets a profiler select the timed launches (ncu --nvtx-include timed/)
            for s, e in self.ev:
                self.flush.zero_()  # evict L2 between timed steps (outside the events)
                s.record(stream)
                fn()
                e.record(stream)
            nvtx()
            torch.cuda.synchronize(self.dev)
        barrier(world)
        ms = [s.elapsed_time(e) for s, e in self.ev]
        total = sum(ms)
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([total], device=self.dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            total = float(t.item())
        return total, ms, clk.summary()


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---- ray casting -------------------------------------------------------------------------
def raycast_config(desc, n_poses, rays, n_faces, world):
    """The `config` of a ray-cast line; both arms print this same dict for the same workload."""
    config = dict(desc)
    config.update({"poses": int(n_poses), "rays_per_step": int(rays), "triangles": int(n_faces),
                   "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas{world}" if world > 1 else "single"})
    return config


# --walk: a fixed traversal instead of the autotuned one (profiling cases)
WALKS = {"full_stack": dict(packet=0, bvh_width=2), "packet": dict(packet=1), "wide4": dict(bvh_width=4, packet=0)}


def walk_name(cfg, depth):
    """Which traversal the launch configuration selects on a tree of `depth` levels (the rules of
    make_trace_params in csrc/simulate.cu)."""
    if cfg.refill:
        return "refill"
    if cfg.bvh_width == 4:
        return "wide4"
    if cfg.packet == 1 and depth <= 32:
        return "packet"
    if cfg.stack_depth > 0 and depth <= 32:
        return "full_stack"
    return "trail"


def cpu_raycast(sc, model, poses, attrs, target_s=15.0):
    """rmagine's Embree path restated on all host cores (the oracle's simulation with its Embree-style
    4-wide SIMD walk, outputs equal to the restatement's) over a bounded pose sample (map build
    excluded, as in the reference's benchmark loop)."""
    import oracle

    ocs = oracle.Scene(sc.vertices, sc.faces)
    threads = oracle.lib().orc_max_threads()
    W, H = model_size(model)
    t0 = time.perf_counter()
    ocs.simulate(model, IDENT, poses[:1], attrs=attrs, nthreads=threads, fast=True)
    per_pose = max(time.perf_counter() - t0, 1e-4)
    n = int(max(1, min(len(poses), target_s / per_pose)))
    t0 = time.perf_counter()
    ocs.simulate(model, IDENT, poses[:n], attrs=attrs, nthreads=threads, fast=True)
    dt = time.perf_counter() - t0
    rays = n * W * H
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": int(threads), "kind": "port",
            "sample": f"{n} of {len(poses)} poses ({rays} rays), all host threads, Embree-style 4-wide SIMD single-ray walk over the oracle's binned-SAH tree "
                      f"(Embree itself is not buildable here)", "seconds": dt}


def cpu_batched(sc, spec, pose_seed=100, target_s=10.0):
    """The oracle's OpenMP ray cast (4-wide walk) over every sensor of a batched set, each with its first k poses
    (k the same for all sensors, sized to about target_s): rays per second over the whole sample."""
    import oracle
    from rmagine_gb300 import scenes

    ocs = oracle.Scene(sc.vertices, sc.faces)
    threads = oracle.lib().orc_max_threads()
    poses = [scenes.terrain_poses(sc, c, seed=pose_seed + i) for i, (_, c) in enumerate(spec)]

    def run(k):
        rays = 0
        t0 = time.perf_counter()
        for (mod, c), p in zip(spec, poses):
            kk = min(k, c)
            ocs.simulate(mod, IDENT, p[:kk], attrs=("hits", "ranges"), nthreads=threads, fast=True)
            W, H = model_size(mod)
            rays += kk * W * H
        return rays, time.perf_counter() - t0

    r1, t1 = run(1)
    k = int(max(1, min(64, target_s / max(t1, 1e-3))))
    rays, dt = run(k)
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": int(threads), "kind": "port",
            "sample": f"the first {k} poses of each of the {len(spec)} sensors ({rays} rays), all host threads, "
                      f"Embree-style 4-wide SIMD single-ray walk over the oracle's binned-SAH tree", "seconds": dt}


def gpu_raycast(args, world):
    import torch

    import rmagine_gb300 as rm

    sc, model, poses, attrs, desc = raycast_workload(args.workload)
    if args.poses:
        poses = poses[:args.poses]
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W, H = model_size(model)
    n = poses.shape[0]
    rays = n * W * H
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    m = rm.Map(sc.vertices, sc.faces)  # binned-SAH tree (the default builder); includes the host->device copy
    build_ms = 1e3 * (time.perf_counter() - t0)
    sim = rm.make_simulator(model, m)
    Tbm = torch.from_numpy(poses).to(dev)
    bundle = rm.resize_memory_bundle(rm.Bundle(*attrs), W, H, n, device=dev)
    if args.walk:
        tuned = rm.launch_config(**WALKS[args.walk])
        sim.launch_config = tuned
    elif args.no_autotune:
        tuned = rm.launch_config()
        sim.launch_config = tuned
    else:
        tuned = sim.autotune(Tbm, bundle, reps=3)  # fastest launch configuration for this map, sensor and poses
    for _ in range(args.warmup):
        sim.simulate(Tbm, bundle)
    torch.cuda.synchronize(dev)
    if m.status() != 0:
        raise RuntimeError("device status error during warm-up")
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(lambda: sim.simulate(Tbm, bundle), world)
    if m.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * rays * args.steps / (total_ms / 1e3) / 1e6

    # e2e through the host-buffer C entry point (rmg_simulate_host, behind the simulator's RAM-bundle
    # overload): pinned host poses in, pinned host bundle out, synchronous
    host_poses = torch.from_numpy(poses).pin_memory()
    hb = rm.resize_memory_bundle(rm.Bundle(*attrs), W, H, n, device="cpu", pin_memory=True)
    sim.simulate(host_poses, hb)
    e2e_t = []
    for _ in range(max(3, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sim.simulate(host_poses, hb)
        e2e_t.append(time.perf_counter() - t0)
    e2e = rays / float(np.median(e2e_t)) / 1e6
    out_b = sum(OUT_BYTES[a] for a in attrs)
    attrs_e2e = attrs
    wk = WORK_PER_RAY.get(args.workload)
    walk = walk_name(tuned, int(m.info()["depth"]))
    launch_s = total_ms / args.steps / 1e3
    rl = issue_roofline(f"{args.workload}/{walk}", rays, launch_s, clocks, TRAFFIC.get(args.workload),
                        f"{walk} walk of k_trace: issue-bound (ALU pipe, SIMD divergence, dependent node fetches); "
                        f"DRAM carries the outputs and tree re-reads")
    if rl is None:
        rl = traffic_roofline(TRAFFIC.get(args.workload), launch_s,
                              f"no instruction count is recorded for the {walk} walk on this workload")
    if rl is not None and wk:
        rl["algorithmic_bytes_per_unit"] = round(out_b + 64 * wk["nodes"] + 48 * wk["tris"], 2)
    config = raycast_config(desc, n, rays, sc.n_faces, world)
    line = {"metric": "Mrays/s", "unit": "Mrays/s", "value": round(value, 2), "ms_per_step": round(total_ms / args.steps, 3),
            "dtype": "f32", "config": config, "gpu_launches": args.steps,
            "run": {"launch": {k: int(getattr(tuned, k)) for k, _ in tuned._fields_}, "walk": walk,
                    "tree": {"builder": m.builder, "depth": int(m.info()["depth"]), "build_ms": round(build_ms, 1)}},
            "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": int(poses.nbytes),
                    "d2h_bytes_per_step": int(rays * host_link_bytes(attrs_e2e, rays)),
                    "step_ms": [round(1e3 * x, 3) for x in e2e_t]},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms],
            "map": {k: m.info()[k] for k in ("n_faces", "n_nodes", "depth", "device_bytes")}}
    return line, lambda: cpu_raycast(sc, model, poses, attrs, target_s=getattr(args, "cpu_target_s", 15.0)), config


# ---- instanced scene (two-level BVH) ----------------------------------------------------------
SCENE_ATTRS = ALL + ("geom_ids", "object_ids")


def gpu_scene(args, world):
    """The 1M-triangle terrain with its 2,000 boxes placed by instances of one unit box (a two-level
    tree: 2,001 instances over 2 meshes), all seven attributes; the same geometry baked into one
    mesh is timed beside it."""
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import scenes, sensors

    meshes, insts, baked = scenes.instanced_terrain(grid=708, n_boxes=2000, seed=0)
    model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
    poses = scenes.terrain_poses(baked, 1000, seed=2)
    if args.poses:
        poses = poses[:args.poses]
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W, H = model_size(model)
    n = poses.shape[0]
    rays = n * W * H
    geoms = [rm.Map(v, f) for v, f in meshes]
    scene = rm.Scene(geoms, [rm.Instance(i["geometry"], i["T"], i["scale"], i["geom_id"], i["object_id"])
                             for i in insts])
    sim = rm.make_simulator(model, scene)
    Tbm = torch.from_numpy(poses).to(dev)
    bundle = rm.resize_memory_bundle(rm.Bundle(*SCENE_ATTRS), W, H, n, device=dev)
    for _ in range(args.warmup):
        sim.simulate(Tbm, bundle)
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(lambda: sim.simulate(Tbm, bundle), world)
    if scene.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * rays * args.steps / (total_ms / 1e3) / 1e6
    # the same geometry as one mesh
    m = rm.Map(baked.vertices, baked.faces)
    bsim = rm.make_simulator(model, m)
    for _ in range(2):
        bsim.simulate(Tbm, bundle)
    reps = max(3, min(args.steps, 5))
    baked_ms, _, _ = Timer(dev, reps).run(lambda: bsim.simulate(Tbm, bundle), world)
    baked_ms /= reps
    del bsim, m
    # e2e through rmg_simulate_scene_host: pinned host poses in, pinned host bundle out, synchronous
    host_poses = torch.from_numpy(poses).pin_memory()
    hb = rm.resize_memory_bundle(rm.Bundle(*SCENE_ATTRS), W, H, n, device="cpu", pin_memory=True)
    sim.simulate(host_poses, hb)
    e2e_t = []
    for _ in range(max(3, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sim.simulate(host_poses, hb)
        e2e_t.append(time.perf_counter() - t0)
    e2e = rays / float(np.median(e2e_t)) / 1e6
    out_b = sum(OUT_BYTES[a] for a in SCENE_ATTRS)
    attrs_e2e = SCENE_ATTRS
    rl = issue_roofline("scene_terrain1m/k_trace_scene", rays, total_ms / args.steps / 1e3, clocks,
                        TRAFFIC.get("scene_terrain1m"),
                        "k_trace_scene (identity geometry walked directly, then the top-level walk with nested instance walks): issue-bound")
    rl = rl or traffic_roofline(TRAFFIC.get("scene_terrain1m"), total_ms / args.steps / 1e3,
                                "no instruction count is recorded for k_trace_scene")
    config = {"workload": "instanced scene: terrain 708x708 (999,698 tris) + 2,000 instances of one 12-triangle "
                          "unit box (scaled, placed), spherical 128x1024, 1000 poses, all seven attributes",
              "poses": int(n), "rays_per_step": int(rays), "instances": len(insts), "geometries": len(meshes),
              "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas{world}" if world > 1 else "single"}
    line = {"metric": "Mrays/s", "unit": "Mrays/s", "value": round(value, 2),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32", "config": config,
            "gpu_launches": args.steps,
            "baked_single_mesh": {"value": round(rays / (baked_ms / 1e3) / 1e6, 2), "unit": "Mrays/s",
                                  "ms_per_step": round(baked_ms, 3)},
            "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": int(poses.nbytes),
                    "d2h_bytes_per_step": int(rays * host_link_bytes(attrs_e2e, rays)),
                    "step_ms": [round(1e3 * x, 3) for x in e2e_t]},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms]}
    return line, lambda: cpu_raycast(baked, model, poses, SCENE_ATTRS, target_s=getattr(args, "cpu_target_s", 15.0)), config


# ---- range noise ---------------------------------------------------------------------------------
def gpu_noise(args, world):
    """Gaussian range noise over the Ranges of one 1M-terrain step (131,072,000 floats), in place:
    an HBM stream of 8 bytes per range."""
    import torch

    from rmagine_gb300 import noise

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = 131_072_000
    r = torch.rand(n, device=dev) * 100.0
    nz = noise.GaussianNoise(0.0, 0.02, noise.NoiseOptions(seed=42, max_range=130.0))
    for _ in range(args.warmup):
        nz.apply(r)
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(lambda: nz.apply(r), world)
    value = world * n * args.steps / (total_ms / 1e3) / 1e9
    rl = roofline(8.0, n, total_ms / args.steps / 1e3, "read + write of one float per range", TRAFFIC.get("noise"))
    # e2e: an eighth of the ranges from pinned host memory, noised on the device, back to pinned
    # host memory (buffers allocated once, like a caller's)
    host = r[: n // 8].cpu().pin_memory()
    host_out = torch.empty_like(host).pin_memory()
    d = torch.empty_like(host, device=dev)
    e2e_t = []
    for _ in range(5):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        d.copy_(host, non_blocking=True)
        nz.apply(d)
        host_out.copy_(d, non_blocking=True)
        torch.cuda.synchronize(dev)
        e2e_t.append(time.perf_counter() - t0)
    line = {"metric": "Granges/s", "unit": "Granges/s", "value": round(value, 2),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32",
            "config": {"workload": "GaussianNoise(0, 0.02) on 131,072,000 ranges in HBM", "l2": "inputs > L2"},
            "gpu_launches": args.steps,
            "e2e": {"value": round(n // 8 / float(np.median(e2e_t)) / 1e9, 3), "unit": "Granges/s",
                    "h2d_bytes_per_step": 4 * (n // 8), "d2h_bytes_per_step": 4 * (n // 8)},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms]}

    return line, cpu_noise, line["config"]


def cpu_noise(n=64_000_000):
    """GaussianNoise(0, 0.02) on n ranges: the oracle's C++ OpenMP restatement (Philox4x32-10,
    binary64 Box-Muller; equal to the numpy restatement) on all host threads."""
    import oracle

    threads = oracle.lib().orc_max_threads()
    rr = np.random.default_rng(0).uniform(0, 100, n).astype(np.float32)
    oracle.noise_apply(0, rr[:1_000_000], 42, 0, stddev=0.02, max_range=130.0, nthreads=threads)
    t0 = time.perf_counter()
    oracle.noise_apply(0, rr, 42, 0, stddev=0.02, max_range=130.0, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": rr.size / dt / 1e9, "unit": "Granges/s", "cores": int(threads), "kind": "port",
            "sample": f"{n:,} ranges, C++ OpenMP restatement (Philox4x32-10, binary64 Box-Muller), all host threads",
            "seconds": dt}


# ---- ICP statistics + Umeyama (forward and backward) -----------------------------------------
def icp_data(B, N, dev, seed=0):
    """Source points U([-25,25]^3); targets = R src + t + N(0, 0.01) with 5% outliers + U(-5,5)^3;
    per-batch uniform random R and t ~ U(-5,5)^3.  Generated on the device (seeded)."""
    import torch

    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    src = torch.rand((B, N, 3), generator=g, device=dev) * 50 - 25
    q = torch.randn((B, 4), generator=g, device=dev)
    q = q / q.norm(dim=1, keepdim=True)
    x, y, z, w = q.unbind(1)
    R = torch.stack([torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
                     torch.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
                     torch.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)], 1)
    t = torch.rand((B, 3), generator=g, device=dev) * 10 - 5
    tgt = torch.empty_like(src)
    for b0 in range(0, B, 512):
        b1 = min(B, b0 + 512)
        tgt[b0:b1] = torch.bmm(src[b0:b1], R[b0:b1].transpose(1, 2)) + t[b0:b1, None, :]
    tgt += torch.randn(tgt.shape, generator=g, device=dev) * 0.01
    out = torch.rand((B, N), generator=g, device=dev) < 0.05
    tgt += out[..., None] * (torch.rand(tgt.shape, generator=g, device=dev) * 10 - 5)
    return src.contiguous(), tgt.contiguous()


def cpu_icp(src_h, tgt_h, target_s=10.0):
    """statistics_p2p + Umeyama of a bounded batch sample on all host threads: the oracle's C++
    OpenMP statistics (binary32 filter, binary64 two-pass means and covariance; equal to the numpy
    restatement) and numpy's batched binary64 SVD for Umeyama."""
    import oracle
    from oracle import stats as ost

    B = src_h.shape[0]
    threads = oracle.lib().orc_max_threads()

    def run(n):
        return ost.umeyama(oracle.stats_batched(src_h[:n], tgt_h[:n], nthreads=threads))

    t0 = time.perf_counter()
    run(min(B, 4))
    per = max((time.perf_counter() - t0) / min(B, 4), 1e-5)
    n = int(max(1, min(B, target_s / per)))
    reps = int(max(1, min(50, target_s / (per * n))))  # a small batch set is timed over repeated passes
    t0 = time.perf_counter()
    for _ in range(reps):
        run(n)
    dt = time.perf_counter() - t0
    corr = reps * n * src_h.shape[1]
    return {"value": corr / dt / 1e9, "unit": "Gcorr/s", "cores": int(threads), "kind": "port",
            "sample": f"{n} of {B} batches x {reps} passes ({corr} correspondences), forward statistics + Umeyama "
                      f"only: C++ OpenMP statistics_p2p in binary64 on all host threads + numpy binary64 Umeyama",
            "seconds": dt}


def gpu_icp(args, world):
    import ctypes as C

    import torch

    from rmagine_gb300 import _lib
    from rmagine_gb300 import statistics as rs

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    B, N = (args.poses or 8192), 32768
    src, tgt = icp_data(B, N, dev)
    corr = B * N
    stats = torch.empty((B, 16), dtype=torch.float32, device=dev)
    T = torch.empty((B, 8), dtype=torch.float32, device=dev)
    gR = torch.randn((B, 9), device=dev)
    gt = torch.randn((B, 3), device=dev)
    gd = torch.empty_like(src)
    gm = torch.empty_like(tgt)
    pc = rs.UmeyamaReductionConstraints().to_c()
    lib = _lib.load()
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def fwd():
        st = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(lib.rmg_statistics_p2p(None, 0, p(src), None, None, p(tgt), None, None, C.byref(pc), B, N,
                                          p(stats), p(T), C.c_void_p(st)), "rmg_statistics_p2p")

    def bwd():
        st = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(lib.rmg_umeyama_backward(None, 0, p(src), None, None, p(tgt), None, None, C.byref(pc), B, N,
                                            p(stats), p(gR), p(gt), p(gd), p(gm), C.c_void_p(st)),
                   "rmg_umeyama_backward")

    def step():
        fwd()
        bwd()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(step, world)
    f_ms, _, _ = Timer(dev, args.steps).run(fwd, world)
    b_ms, _, _ = Timer(dev, args.steps).run(bwd, world)
    value = world * corr * args.steps / (total_ms / 1e3) / 1e9
    # e2e: host (pinned) clouds in, transforms + gradients back, through the public API; batches in
    # chunks whose uploads, statistics + backward and downloads overlap on three streams (the copies
    # in the two directions share the host link: 340 GB/s together against 193-211 GB/s alone)
    hs, ht = src.cpu().pin_memory(), tgt.cpu().pin_memory()
    hgd = torch.empty(hs.shape, dtype=torch.float32, pin_memory=True)
    hgm = torch.empty(hs.shape, dtype=torch.float32, pin_memory=True)
    hT = torch.empty((B, 8), dtype=torch.float32, pin_memory=True)
    ds, dt_ = torch.empty_like(src), torch.empty_like(tgt)
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    compute = torch.cuda.current_stream(dev)
    cstep = max(1, B // 32)  # 32 chunks: 6.74 Gcorr/s; 8 / 16 / 64: 6.44 / 6.69 / 6.68

    def e2e_step():
        up.wait_stream(compute)
        down.wait_stream(compute)
        for c0 in range(0, B, cstep):
            c1 = min(B, c0 + cstep)
            with torch.cuda.stream(up):
                ds[c0:c1].copy_(hs[c0:c1], non_blocking=True)
                dt_[c0:c1].copy_(ht[c0:c1], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(up)
            compute.wait_event(ev)
            s_, T_ = rs.statistics(ds[c0:c1], dt_[c0:c1])
            a, b = rs.umeyama_backward(ds[c0:c1], dt_[c0:c1], s_, grad_R=gR[c0:c1], grad_t=gt[c0:c1])
            done = torch.cuda.Event()
            done.record(compute)
            down.wait_event(done)
            with torch.cuda.stream(down):
                hgd[c0:c1].copy_(a, non_blocking=True)
                hgm[c0:c1].copy_(b, non_blocking=True)
                hT[c0:c1].copy_(T_, non_blocking=True)
            for t in (a, b, T_, s_):
                t.record_stream(down)
        compute.wait_stream(down)

    e2e_step()
    e2e_t = []
    for _ in range(max(3, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize(dev)
        e2e_t.append(time.perf_counter() - t0)
    e2e = corr / float(np.median(e2e_t)) / 1e9
    fwd_s, bwd_s = f_ms / args.steps / 1e3, b_ms / args.steps / 1e3
    rl_f = roofline(24, corr, fwd_s, "k_stats: 24 B per correspondence read (dataset + model points)",
                    TRAFFIC.get("icp_stats_fwd"))
    rl_b = roofline(48, corr, bwd_s, "k_umeyama_bwd_stream: 24 B read + 24 B gradients written per correspondence",
                    TRAFFIC.get("icp_stats_bwd"))
    dominant, other = (rl_b, rl_f) if bwd_s >= fwd_s else (rl_f, rl_b)
    config = {"workload": f"ICP statistics_p2p + Umeyama forward and backward, {B} batches x {N} correspondences "
                          f"(src U[-25,25]^3, tgt = R src + t + N(0,0.01), 5% outliers)",
              "batches": B, "correspondences_per_step": corr, "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas{world}" if world > 1 else "single"}
    line = {"metric": "Gcorr/s", "unit": "Gcorr/s", "value": round(value, 3),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32 (f64 accumulation)", "config": config,
            "gpu_launches": 4 * args.steps,
            "forward_ms": round(f_ms / args.steps, 3), "backward_ms": round(b_ms / args.steps, 3),
            "e2e": {"value": round(e2e, 3), "unit": "Gcorr/s", "h2d_bytes_per_step": int(2 * 12 * corr),
                    "d2h_bytes_per_step": int(2 * 12 * corr + 32 * B)},
            "roofline": dominant, "roofline_other_kernel": other, "clocks": clocks,
            "step_ms": [round(x, 3) for x in step_ms]}
    src_h = src[:min(B, 64)].cpu().numpy()
    tgt_h = tgt[:min(B, 64)].cpu().numpy()
    return line, lambda: cpu_icp(src_h, tgt_h, target_s=getattr(args, "cpu_target_s", 10.0)), config


# ---- pose gradient -----------------------------------------------------------------------------
def posegrad_workload(n_poses):
    from rmagine_gb300 import scenes, sensors

    sc = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
    model = sensors.ouster_like(64, 1024, 45.0, 0.5, 130.0)
    true = scenes.terrain_poses(sc, n_poses, seed=3)
    est = scenes.perturb_poses(true, 4, 0.1, 2.0)
    return sc, model, true, est


def cpu_posegrad(sc, model, true, est, obs_h, target_s=10.0):
    """Ray cast of the estimates (the oracle's 4-wide walk) + the analytic range adjoint (the oracle's
    C++ OpenMP restatement in binary64, equal to oracle/grad.py's) on all host threads."""
    import oracle

    ocs = oracle.Scene(sc.vertices, sc.faces)
    threads = oracle.lib().orc_max_threads()
    W, H = model_size(model)

    def run(n):
        sim = ocs.simulate(model, IDENT, est[:n], attrs=("ranges", "face_ids"), nthreads=threads, fast=True)
        return oracle.pose_grad(ocs, model, IDENT, est[:n], sim["face_ids"], sim["ranges"], obs_h[:n * W * H], 0.2,
                                nthreads=threads)

    run(1)  # builds the 4-wide tree
    t0 = time.perf_counter()
    run(1)
    per = max(time.perf_counter() - t0, 1e-4)
    n = int(max(1, min(len(est), obs_h.size // (W * H), target_s / per)))
    t0 = time.perf_counter()
    run(n)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "poses/s", "cores": int(threads), "kind": "port",
            "sample": f"{n} of {len(est)} poses: oracle ray cast (4-wide SIMD walk) + C++ OpenMP binary64 adjoint, "
                      f"all host threads", "seconds": dt}


def gpu_posegrad(args, world):
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import grad as rg

    n_poses = args.poses or 4096
    sc, model, true, est = posegrad_workload(n_poses)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W, H = model_size(model)
    rays = n_poses * W * H
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    obs = sim.simulate(torch.from_numpy(true).to(dev), attrs=("ranges",)).ranges
    Test = torch.from_numpy(est).to(dev)
    for _ in range(args.warmup):
        rg.range_pose_grad(sim, Test, obs, 0.2)
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(lambda: rg.range_pose_grad(sim, Test, obs, 0.2), world)
    if m.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * n_poses * args.steps / (total_ms / 1e3)
    host_est = torch.from_numpy(est).pin_memory()
    host_obs = obs.cpu().pin_memory()
    e2e_t = []
    for _ in range(max(3, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        g, l_ = rg.range_pose_grad(sim, host_est, host_obs, 0.2)  # rmg_range_pose_grad_host: results in host memory
        g.cpu()
        l_.cpu()
        e2e_t.append(time.perf_counter() - t0)
    e2e = n_poses / float(np.median(e2e_t))
    rl = issue_roofline("pose_grad/k_range_grad", rays, total_ms / args.steps / 1e3, clocks, TRAFFIC.get("pose_grad"),
                        "k_range_grad (ray cast fused with the range adjoint and the per-pose reduction): "
                        "issue-bound like k_trace")
    rl = rl or traffic_roofline(TRAFFIC.get("pose_grad"), total_ms / args.steps / 1e3,
                                "no instruction count is recorded for k_range_grad")
    config = {"workload": f"pose gradient: terrain 1024x1024 + 2000 boxes (2,117,058 tris), spherical 64x1024, "
                          f"{n_poses} poses perturbed N(0,0.1 m) / N(0,2 deg), Huber 0.2 m",
              "poses": n_poses, "rays_per_step": rays, "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas{world}" if world > 1 else "single"}
    line = {"metric": "pose-grad evals/s", "unit": "poses/s", "value": round(value, 1),
            "mrays_per_s": round(world * rays * args.steps / (total_ms / 1e3) / 1e6, 1),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32", "config": config,
            "gpu_launches": 2 * args.steps,
            "e2e": {"value": round(e2e, 1), "unit": "poses/s", "h2d_bytes_per_step": int(est.nbytes + 4 * rays),
                    "d2h_bytes_per_step": int(28 * n_poses)},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms]}
    obs_h = obs[:128 * W * H].cpu().numpy()  # the CPU leg times up to 128 poses
    return line, lambda: cpu_posegrad(sc, model, true, est, obs_h, target_s=getattr(args, "cpu_target_s", 10.0)), config


# ---- fused simulate -> statistics (RCC / MICP-L inner step) ---------------------------------
def rcc_workload(n_poses=1000):
    """1M-triangle terrain, spherical 128x1024, n pose estimates (the ray-cast workload's poses
    perturbed by N(0, 0.1 m) / N(0, 2 deg)), each against the scan taken at its true pose."""
    from rmagine_gb300 import scenes, sensors

    sc = scenes.million_triangle_terrain(seed=0)
    model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
    true = scenes.terrain_poses(sc, 1000, seed=2)[:n_poses]
    est = scenes.perturb_poses(true, 4, 0.1, 2.0)
    return sc, model, true, est


def cpu_rcc(sc, model, true, est, data_h, target_s=10.0):
    """The step on the host: ray cast of the model scan (the oracle's 4-wide walk), statistics_p2l in
    binary64 (the oracle's C++ OpenMP statistics) and numpy binary64 Umeyama, all host threads; the
    same results as oracle/stats.py's simulate_statistics."""
    import oracle
    from oracle import stats as ost

    ocs = oracle.Scene(sc.vertices, sc.faces)
    threads = oracle.lib().orc_max_threads()
    W, H = model_size(model)

    def run(n):
        sim = ocs.simulate(model, IDENT, est[:n], attrs=("hits", "points", "normals"), nthreads=threads, fast=True)
        st = oracle.stats_batched(data_h["points"][:n * W * H].reshape(n, W * H, 3),
                                  sim["points"].reshape(n, W * H, 3), normals=sim["normals"].reshape(n, W * H, 3),
                                  dmask=data_h["hits"][:n * W * H], mmask=sim["hits"], max_dist=0.5, nthreads=threads)
        return ost.umeyama(st)

    run(1)  # builds the 4-wide tree
    t0 = time.perf_counter()
    run(1)
    per = max(time.perf_counter() - t0, 1e-4)
    n = int(max(1, min(len(est), data_h["hits"].size // (W * H), target_s / per)))
    t0 = time.perf_counter()
    run(n)
    dt = time.perf_counter() - t0
    return {"value": n * W * H / dt / 1e6, "unit": "Mrays/s", "cores": int(threads), "kind": "port",
            "sample": f"{n} of {len(est)} poses ({n * W * H} rays): oracle ray cast (4-wide SIMD walk) + C++ OpenMP "
                      f"binary64 statistics_p2l + numpy Umeyama, all host threads", "seconds": dt}


def gpu_rcc(args, world):
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import statistics as rs

    n_poses = args.poses or 1000
    sc, model, true, est = rcc_workload(n_poses)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W, H = model_size(model)
    rays = n_poses * W * H
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    data = sim.simulate(torch.from_numpy(true).to(dev), attrs=("hits", "points"))
    dp, dm = data.points.reshape(n_poses, W * H, 3), data.hits.reshape(n_poses, W * H)
    Est = torch.from_numpy(est).to(dev)
    P = rs.UmeyamaReductionConstraints(max_dist=0.5)

    def fused():
        return sim.simulate_statistics(Est, dp, dataset_mask=dm, params=P)

    mod = rm.Bundle("hits", "points", "normals")
    rm.resize_memory_bundle(mod, W, H, n_poses, device=dev)

    def two_step():
        sim.simulate(Est, mod)
        return rs.statistics_p2l(dp, mod.points.reshape(n_poses, W * H, 3), mod.normals.reshape(n_poses, W * H, 3),
                                 params=P, dataset_mask=dm, model_mask=mod.hits.reshape(n_poses, W * H))

    for _ in range(args.warmup):
        fused()
        two_step()
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(fused, world)
    two_ms, _, _ = Timer(dev, max(3, min(args.steps, 5))).run(two_step, world)
    two_ms /= max(3, min(args.steps, 5))
    if m.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * rays * args.steps / (total_ms / 1e3) / 1e6
    # end to end through rmg_simulate_statistics_host: estimates and scans from pinned host memory,
    # statistics + transforms back in host memory
    host_est = torch.from_numpy(est).pin_memory()
    host_dp, host_dm = dp.cpu().pin_memory(), dm.cpu().pin_memory()
    e2e_t = []
    for _ in range(max(3, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        st, T = sim.simulate_statistics(host_est, host_dp, dataset_mask=host_dm, params=P)
        st.cpu()
        T.cpu()
        e2e_t.append(time.perf_counter() - t0)
    e2e = rays / float(np.median(e2e_t)) / 1e6
    rl = issue_roofline("rcc_fused/k_trace_stats", rays, total_ms / args.steps / 1e3, clocks, TRAFFIC.get("rcc_fused"),
                        "k_trace_stats (ray cast fused with statistics_p2l and the per-pose reduction): issue-bound")
    rl = rl or traffic_roofline(TRAFFIC.get("rcc_fused"), total_ms / args.steps / 1e3,
                                "no instruction count is recorded for k_trace_stats")
    config = {"workload": f"fused simulate -> statistics_p2l -> Umeyama: terrain 708x708 + 2000 boxes (1,023,698 "
                          f"tris), spherical 128x1024, {n_poses} pose estimates (perturbed N(0,0.1 m) / N(0,2 deg)) "
                          f"each against the scan at its true pose, max_dist 0.5 m",
              "poses": n_poses, "rays_per_step": rays, "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas{world}" if world > 1 else "single"}
    line = {"metric": "Mrays/s", "unit": "Mrays/s", "value": round(value, 1),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32", "config": config,
            "gpu_launches": 2 * args.steps,
            "two_step": {"value": round(rays / (two_ms / 1e3) / 1e6, 1), "unit": "Mrays/s",
                         "ms_per_step": round(two_ms, 3),
                         "what": "rmg_simulate (Hits, Points, Normals) + rmg_statistics_p2l with Umeyama"},
            "e2e": {"value": round(e2e, 1), "unit": "Mrays/s", "h2d_bytes_per_step": int(est.nbytes + 13 * rays),
                    "d2h_bytes_per_step": int(96 * n_poses)},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms]}
    data_h = {"points": dp[:64].reshape(-1, 3).cpu().numpy(), "hits": dm[:64].reshape(-1).cpu().numpy()}  # CPU leg: up to 64 poses
    return line, lambda: cpu_rcc(sc, model, true, est, data_h, target_s=getattr(args, "cpu_target_s", 10.0)), config


# ---- batched heterogeneous sensors ------------------------------------------------------------
def gpu_batched(args, world):
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import batched, scenes

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    sc = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
    m = rm.Map(sc.vertices, sc.faces)
    small = args.workload == "batched_small"
    spec = batched.small_sensor_set(1024, seed=0) if small else batched.mixed_sensor_set(64, seed=0)
    if args.poses:
        spec = [(mod, min(c, args.poses)) for mod, c in spec]
    attrs = ("hits", "ranges")
    # every job's poses and outputs are views into one contiguous buffer each, so the host side of a
    # step is one upload and one download per attribute
    sims = [rm.make_simulator(mod, m) for mod, _ in spec]
    counts = [c for _, c in spec]
    n_rays = [s_.sensor.width * s_.sensor.height * c for s_, c in zip(sims, counts)]
    all_poses = torch.from_numpy(np.concatenate([scenes.terrain_poses(sc, c, seed=100 + i)
                                                 for i, c in enumerate(counts)])).to(dev)
    all_out = {"hits": torch.empty(sum(n_rays), dtype=torch.uint8, device=dev),
               "ranges": torch.empty(sum(n_rays), dtype=torch.float32, device=dev)}
    jobs = []
    p0 = r0 = 0
    for sim, c, nr in zip(sims, counts, n_rays):
        b = rm.Bundle(*attrs)
        for a in attrs:
            setattr(b, a, all_out[a][r0:r0 + nr])
        jobs.append((sim, all_poses[p0:p0 + c], b))
        p0 += c
        r0 += nr
    rays = sum(s.sensor.width * s.sensor.height * p.shape[0] for s, p, _ in jobs)
    # autotune on a sample of the plan (each job cut to its first 8 poses), apply to the full plan
    sample = []
    for sim, poses, b in jobs:
        k = min(8, poses.shape[0])
        n = sim.sensor.width * sim.sensor.height * k
        sb = rm.Bundle(*attrs)
        for a in attrs:
            setattr(sb, a, getattr(b, a)[:n])
        sample.append((sim, poses[:k], sb))
    t0 = time.perf_counter()
    if args.no_autotune:  # the plan's default launch options
        best = batched.BatchPlan(m, sample).config()
    else:
        best = batched.BatchPlan(m, sample).autotune(reps=3, use_cache=False)
    tune_s = time.perf_counter() - t0
    plan = batched.BatchPlan(m, jobs, best)
    for _ in range(args.warmup):
        plan.launch()
    torch.cuda.synchronize(dev)
    total_ms, step_ms, clocks = Timer(dev, args.steps).run(plan.launch, world)

    def plain():
        for sim, poses, b in jobs:
            sim.simulate(poses, b)

    plain()
    torch.cuda.synchronize(dev)
    plain_ms, _, _ = Timer(dev, max(2, args.steps // 2)).run(plain, world)
    plain_ms = plain_ms / max(2, args.steps // 2)

    # the same launches through the C ABI with every argument built beforehand: launch cost only
    import ctypes as C

    from rmagine_gb300 import _lib
    from rmagine_gb300.simulation import _stream_ptr, outputs_c

    lib = _lib.load()
    prebuilt = [(sim.sensor.handle, C.byref(sim._Tsb), C.c_void_p(p.data_ptr()), p.shape[0], outputs_c(b))
                for sim, p, b in jobs]
    stream = _stream_ptr()

    def plain_abi():
        for sh, tsb, tp, n, out in prebuilt:
            lib.rmg_simulate(m.handle, sh, tsb, tp, n, C.byref(out), stream)

    plain_abi()
    torch.cuda.synchronize(dev)
    abi_ms, _, _ = Timer(dev, max(2, args.steps // 2)).run(plain_abi, world)
    abi_ms = abi_ms / max(2, args.steps // 2)
    if m.status() != 0:
        raise RuntimeError("device status error in the timed region")
    value = world * rays * args.steps / (total_ms / 1e3) / 1e6
    # e2e: host poses in, host hits+ranges out, through the chunked plan (16 pose ranges of every
    # job; each range's outputs copy to the host while the next range is cast)
    host_poses = all_poses.cpu().pin_memory()
    host_out = {a: torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for a, t in all_out.items()}
    host_jobs = []
    r0 = 0
    for nr in n_rays:
        hb = rm.Bundle(*attrs)
        for a in attrs:
            setattr(hb, a, host_out[a][r0:r0 + nr])
        host_jobs.append(hb)
        r0 += nr
    # 16 ranges when the outputs are large (their copies then hide behind the casting); one plan and
    # one copy per attribute of the whole contiguous output when they are small (the 1,024-sensor set:
    # 3.9 MB, where per-job copies would cost more than they hide)
    e2e_chunks = 16 if rays * 5 > (256 << 20) else 1
    cplan = batched.ChunkedBatchPlan(m, jobs, e2e_chunks, best) if e2e_chunks > 1 else None

    def e2e_step():
        all_poses.copy_(host_poses, non_blocking=True)
        if cplan is not None:
            cplan.run_to_host(host_jobs)
        else:
            plan.launch()
            for a in attrs:
                host_out[a].copy_(all_out[a], non_blocking=True)
            torch.cuda.synchronize(dev)

    e2e_step()
    e2e_t = []
    for _ in range(3):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    e2e = rays / float(np.median(e2e_t)) / 1e6
    key = "batched_small" if small else "batched"
    rl = issue_roofline(f"{key}/k_trace_batched", rays, total_ms / args.steps / 1e3, clocks, TRAFFIC.get(key),
                        "k_trace_batched (persistent warps over all sensors' tiles, per-ray walk of k_trace): "
                        "issue-bound")
    rl = rl or traffic_roofline(TRAFFIC.get(key), total_ms / args.steps / 1e3,
                                "no instruction count is recorded for this batch")
    config = {"workload": ("batched small sensors: terrain 1024x1024 + 2000 boxes (2,117,058 tris), 1024 sensors "
                           "(O1Dn 256 dirs / pinhole 32x8, alternating), poses log-uniform [1,8], Hits+Ranges") if small
              else ("batched: terrain 1024x1024 + 2000 boxes (2,117,058 tris), 64 sensors from {VLP-16 16x900, "
                    "spherical 128x2048, pinhole 640x480, O1Dn 10k dirs}, poses log-uniform [1,4096], Hits+Ranges"),
              "sensors": len(jobs), "poses": int(sum(p.shape[0] for _, p, _ in jobs)), "rays_per_step": int(rays),
              "autotuned": {"stack_depth": best.stack_depth, "block_warps": best.block_warps,
                            "tile": f"{best.tile_w}x{best.tile_h}", "grab": best.grab, "tuning_s": round(tune_s, 2)},
              "l2": "flushed between timed steps (256 MB write)",
              "parallelism": f"replicas{world}" if world > 1 else "single"}
    line = {"metric": "Mrays/s", "unit": "Mrays/s", "value": round(value, 2),
            "ms_per_step": round(total_ms / args.steps, 3), "dtype": "f32", "config": config,
            "gpu_launches": args.steps,
            "plain_one_launch_per_sensor": {"value": round(rays / (plain_ms / 1e3) / 1e6, 2), "unit": "Mrays/s",
                                            "ms_per_step": round(plain_ms, 3), "launches_per_step": len(jobs)},
            "speedup_vs_plain": round(plain_ms / (total_ms / args.steps), 3),
            "plain_c_abi_loop": {"value": round(rays / (abi_ms / 1e3) / 1e6, 2), "unit": "Mrays/s",
                                 "ms_per_step": round(abi_ms, 3),
                                 "what": "one rmg_simulate per sensor, arguments built before the timed region"},
            "speedup_vs_c_abi_loop": round(abi_ms / (total_ms / args.steps), 3),
            "e2e": {"value": round(e2e, 2), "unit": "Mrays/s",
                    "h2d_bytes_per_step": int(sum(p.numel() * 4 for _, p, _ in jobs)),
                    "d2h_bytes_per_step": int(5 * rays)},
            "roofline": rl, "clocks": clocks, "step_ms": [round(x, 3) for x in step_ms]}

    def cpu():
        return cpu_batched(sc, spec, target_s=getattr(args, "cpu_target_s", 10.0))

    return line, cpu, config


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="terrain1m_spherical")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="ray-cast workloads: the default launch configuration")
    ap.add_argument("--poses", type=int, default=0, help="use only the first N poses / batches (profiling case)")
    ap.add_argument("--walk", choices=sorted(WALKS), default=None,
                    help="ray-cast workloads: this traversal instead of the autotuned one (profiling cases)")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: skip the batched and pose-gradient parts of the line")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    base = {"n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic (seeded procedural inputs)"}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(args, base)))
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if args.workload in RAYCAST:
        line, cpu, _ = gpu_raycast(args, world)
    elif args.workload == "icp_stats":
        line, cpu, _ = gpu_icp(args, world)
    elif args.workload == "pose_grad":
        line, cpu, _ = gpu_posegrad(args, world)
    elif args.workload in ("batched", "batched_small"):
        line, cpu, _ = gpu_batched(args, world)
    elif args.workload == "rcc_fused":
        line, cpu, _ = gpu_rcc(args, world)
    elif args.workload == "scene_terrain1m":
        line, cpu, _ = gpu_scene(args, world)
    elif args.workload == "noise":
        line, cpu, _ = gpu_noise(args, world)
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    subs = {}
    if args.workload == "terrain1m_spherical" and not args.headline_only and not args.poses and world == 1:
        # (at N = 1 only: the scaling run measures the headline; a sub-line failing on one rank would
        # leave the others waiting at its barriers)
        # the other two parts of the headline metric ("plain vs batched", "pose-grad evals/s"), each
        # timed on its own workload with its own clocks, e2e, roofline and CPU baseline
        import torch

        for key, fn, steps in (("batched", gpu_batched, min(args.steps, 5)), ("pose_grad", gpu_posegrad, args.steps)):
            torch.cuda.empty_cache()
            sub_args = argparse.Namespace(**vars(args))
            sub_args.workload, sub_args.steps, sub_args.warmup = key, steps, max(3, min(args.warmup, 3))
            sline, scpu, _ = fn(sub_args, world)
            sline.update({"steps": steps, "warmup": sub_args.warmup})
            subs[key] = (sline, scpu)
        # the other measured workloads, so that every figure of the measurement table has a record
        # of this run; a failure there is reported in its own key and leaves the line intact
        for key, fn in OTHER_SUBS:
            torch.cuda.empty_cache()
            sub_args = argparse.Namespace(**vars(args))
            sub_args.workload, sub_args.steps, sub_args.warmup = key, min(args.steps, 5), 3
            sub_args.cpu_target_s = 4.0
            try:
                sline, scpu, _ = fn(sub_args, world)
                sline.update({"steps": sub_args.steps, "warmup": sub_args.warmup})
                subs[key] = (sline, scpu)
            except Exception as e:  # noqa: BLE001
                subs[key] = ({"error": f"{type(e).__name__}: {e}"[:300]}, None)
            torch.cuda.synchronize()
    if rank != 0:
        return
    out = dict(base)
    out.update(line)
    if not args.no_cpu_baseline:
        from oracle import build as ob

        ob.build()
    for key, (sline, scpu) in subs.items():
        if not args.no_cpu_baseline and scpu is not None:
            try:
                sline["cpu_baseline"] = rounded(scpu())
            except Exception as e:  # noqa: BLE001
                sline["cpu_baseline"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        out[key] = sline
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = rounded(cpu())
    print(json.dumps(out))


# Sub-lines of the default line beside batched and pose_grad: (key = workload name, GPU arm).
OTHER_SUBS = (("terrain1m_pinhole", lambda a, w: gpu_raycast(a, w)),
              ("terrain2m_spherical", lambda a, w: gpu_raycast(a, w)),
              ("room_vlp16", lambda a, w: gpu_raycast(a, w)),
              ("scene_terrain1m", lambda a, w: gpu_scene(a, w)),
              ("rcc_fused", lambda a, w: gpu_rcc(a, w)),
              ("icp_stats", lambda a, w: gpu_icp(a, w)),
              ("noise", lambda a, w: gpu_noise(a, w)))


def rounded(c):
    return {k: (round(v, 4) if isinstance(v, float) else v) for k, v in c.items() if k != "seconds"}


def cpu_leg(workload, args, target_s):
    """The CPU leg of one workload on the host cores: (run, metric, unit, config), run() timing a
    bounded sample of about target_s seconds (the reference's Embree path is not buildable; the
    oracle's port of it stands in)."""
    if workload in RAYCAST:
        sc, model, poses, attrs, desc = raycast_workload(workload)
        if args.poses and workload == args.workload:
            poses = poses[:args.poses]
        run = lambda: cpu_raycast(sc, model, poses, attrs, target_s=target_s)  # noqa
        W, H = model_size(model)
        config = raycast_config(desc, poses.shape[0], poses.shape[0] * W * H, sc.n_faces,
                                int(os.environ.get("WORLD_SIZE", "1")))
        return run, "Mrays/s", "Mrays/s", config
    if workload == "icp_stats":
        rng = np.random.default_rng(0)
        src = rng.uniform(-25, 25, (64, 32768, 3)).astype(np.float32)
        tgt = (src + rng.normal(0, 0.01, src.shape)).astype(np.float32)
        return (lambda: cpu_icp(src, tgt, target_s=target_s), "Gcorr/s", "Gcorr/s",
                {"workload": "ICP statistics_p2p + Umeyama (CPU sample)"})
    if workload == "pose_grad":
        sc, model, true, est = posegrad_workload(64)
        import oracle

        obs = oracle.Scene(sc.vertices, sc.faces).simulate(model, IDENT, true, attrs=("ranges",), fast=True)["ranges"]
        return (lambda: cpu_posegrad(sc, model, true, est, obs, target_s=target_s), "pose-grad evals/s", "poses/s",
                {"workload": "pose gradient (CPU sample)"})
    if workload == "scene_terrain1m":
        from rmagine_gb300 import scenes, sensors

        _, _, baked = scenes.instanced_terrain(grid=708, n_boxes=2000, seed=0)
        model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
        poses = scenes.terrain_poses(baked, 1000, seed=2)
        return (lambda: cpu_raycast(baked, model, poses, SCENE_ATTRS, target_s=target_s), "Mrays/s", "Mrays/s",
                {"workload": "terrain 1M + 2000 boxes (CPU: the geometry as one mesh)"})
    if workload == "noise":
        return cpu_noise, "Granges/s", "Granges/s", {"workload": "GaussianNoise(0, 0.02) (CPU sample)"}
    if workload == "rcc_fused":
        import oracle

        sc, model, true, est = rcc_workload(64)
        data_h = oracle.Scene(sc.vertices, sc.faces).simulate(model, IDENT, true, attrs=("hits", "points"), fast=True)
        return (lambda: cpu_rcc(sc, model, true, est, data_h, target_s=target_s), "Mrays/s", "Mrays/s",
                {"workload": "fused simulate -> statistics_p2l (CPU sample)"})
    raise SystemExit(f"unknown workload {workload}")


def reference_arm(args, base):
    """CPU leg on the host cores for the same workload and metric (the reference's Embree path is not
    buildable; the oracle's port of it stands in)."""
    from oracle import build as ob

    ob.build()
    run, metric, unit, config = cpu_leg(args.workload, args, max(2.0, 60.0 / (args.steps + args.warmup)))
    single = int(os.environ.get("WORLD_SIZE", "1")) == 1  # sub-line legs at N = 1 only, as in the GPU arm
    extras = {}
    if args.workload == "terrain1m_spherical" and not args.headline_only and not args.poses and single:
        # the CPU legs of the line's batched and pose-gradient parts, one bounded sample each
        import oracle
        from rmagine_gb300 import batched, scenes

        sc2 = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
        extras["batched"] = cpu_batched(sc2, batched.mixed_sensor_set(64, seed=0), target_s=8.0)
        psc, pmodel, ptrue, pest = posegrad_workload(64)
        pobs = oracle.Scene(psc.vertices, psc.faces).simulate(pmodel, IDENT, ptrue, attrs=("ranges",),
                                                              fast=True)["ranges"]
        extras["pose_grad"] = cpu_posegrad(psc, pmodel, ptrue, pest, pobs, target_s=8.0)
    vals, leg = [], None
    for _ in range(args.warmup + args.steps):
        leg = run()
        vals.append(leg["value"])
    v = statistics.mean(vals[args.warmup:]) if len(vals) > args.warmup else vals[-1]
    out = dict(base)
    out.update({"impl": "reference", "metric": metric, "unit": unit, "value": round(v, 4), "dtype": "f32",
                "ms_per_step": round(1e3 * leg["seconds"], 1), "config": config, "gpu_launches": 0,
                "cpu_baseline": {"value": round(v, 4), "unit": unit, "cores": leg["cores"], "kind": leg["kind"],
                                 "sample": leg["sample"]},
                "e2e": {"value": round(v, 4), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    for key, leg2 in extras.items():
        out[key] = {"metric": "Mrays/s" if key == "batched" else "pose-grad evals/s", "unit": leg2["unit"],
                    "value": round(leg2["value"], 4), "cpu_baseline": rounded(leg2)}
    if args.workload == "terrain1m_spherical" and not args.headline_only and not args.poses and single:
        for key, _ in OTHER_SUBS:  # the CPU legs of the default line's other sub-lines
            try:
                run2, metric2, unit2, _ = cpu_leg(key, args, 4.0)
                leg2 = run2()
                out[key] = {"metric": metric2, "unit": unit2, "value": round(leg2["value"], 4),
                            "cpu_baseline": rounded(leg2)}
            except Exception as e:  # noqa: BLE001
                out[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out


if __name__ == "__main__":
    main()
