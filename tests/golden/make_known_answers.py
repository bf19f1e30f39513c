"""Extracts the known-answer constants of rmagine's own tests into known_answers.json.

Run in a checkout that has the reference at RMAGINE_REF (default
/root/reference); it reads the test sources as text, takes the numeric
literals at the cited lines, and records each with its path:line inside the
rmagine project.  The committed JSON is what the tests read; the reference
tree is not needed at test time.

    python tests/golden/make_known_answers.py
"""
from __future__ import annotations

import json
import os
import re
from pathlib import Path

REF = Path(os.environ.get("RMAGINE_REF", "/root/reference"))
OUT = Path(__file__).resolve().parent / "known_answers.json"
NUM = r"(-?[0-9]+(?:\.[0-9]*)?(?:[eE][-+]?[0-9]+)?)"


def grab(rel: str, line: int, pattern: str, n: int = 1):
    text = (REF / rel).read_text().splitlines()[line - 1]
    m = re.search(pattern, text)
    if not m:
        raise SystemExit(f"pattern {pattern!r} not found at {rel}:{line}: {text!r}")
    vals = [float(g) for g in m.groups()[:n]]
    return (vals[0] if n == 1 else vals), f"{rel}:{line}"


def vec3(rel, line, prefix):
    return grab(rel, line, re.escape(prefix) + r"\s*\{\s*" + NUM + r"\s*,\s*" + NUM + r"\s*,\s*" + NUM, 3)


def main() -> None:
    answers = {}

    v, src = grab("tests/embree/simulation_spherical.cpp", 60, r"range - " + NUM)
    tol, tsrc = grab("tests/embree/simulation_spherical.cpp", 61, r"error > " + NUM)
    answers["spherical_cube_range"] = {
        "model": "example_spherical", "map": "genCube", "poses": 100, "pose": "identity",
        "vid": "phi.size/2", "hid": 0, "expect": v, "tol": tol, "source": src, "tol_source": tsrc}

    p, src = vec3("tests/embree/simulation_pinhole.cpp", 64, "Vector3")
    tol, tsrc = grab("tests/embree/simulation_pinhole.cpp", 68, r"error > " + NUM)
    answers["pinhole_cube_point"] = {
        "model": "example_pinhole", "map": "genCube", "poses": 100, "pose": "identity",
        "vid": 0, "hid": 0, "expect": p, "metric": "L1(dir*range - expect)", "tol": tol,
        "source": src, "tol_source": tsrc}

    p, src = vec3("tests/embree/simulation_o1dn.cpp", 64, "Vector3")
    tol, tsrc = grab("tests/embree/simulation_o1dn.cpp", 67, r"error > " + NUM)
    answers["o1dn_cube_point"] = {
        "model": "example_o1dn", "map": "genCube", "poses": 100, "pose": "identity", "ray": 0,
        "expect": p, "metric": "L1(orig + dir*range - expect)", "tol": tol, "source": src, "tol_source": tsrc}

    n, src = vec3("tests/optix/simulation_o1dn.cpp", 84, "Vector")
    tol, tsrc = grab("tests/optix/simulation_o1dn.cpp", 85, r"normal_error > " + NUM)
    answers["o1dn_cube_normal"] = {
        "model": "example_o1dn", "map": "genCube", "poses": 100, "pose": "identity", "ray": 0,
        "expect": n, "metric": "L2(normal - expect)", "tol": tol, "source": src, "tol_source": tsrc}

    v, src = grab("tests/optix/simulation_o1dn.cpp", 109, r"last_scan\[0\] - " + NUM)
    answers["o1dn_cube_range"] = {
        "model": "example_o1dn", "map": "genCube", "poses": 100, "pose": "identity", "ray": 0,
        "expect": v, "tol": 1e-4, "source": src}

    v, src = grab("tests/embree/simulation_single_ray.cpp", 59, r"range - " + NUM)
    answers["ondn_single_ray_range"] = {
        "model": "OnDn 1x1, orig (0,0,0), dir (1,0,0), range [0,100]", "map": "genCube", "poses": 100,
        "pose": "identity", "ray": 0, "expect": v, "tol": 1e-4, "source": src}

    v, src = grab("tests/embree/simulation_ondn.cpp", 63, r"last_scan\[0\] - " + NUM)
    answers["ondn_cube_range"] = {
        "model": "example_ondn", "map": "genCube", "poses": 100, "pose": "identity", "ray": 0,
        "expect": v, "tol": 1e-4, "source": src}

    rel = "tests/core/math_statistics.cpp"
    parts = []
    for dl, ml in ((329, 330), (334, 335), (339, 340), (344, 345)):
        d, _ = vec3(rel, dl, "dataset_mean =")
        m, _ = vec3(rel, ml, "model_mean   =")
        parts.append({"dataset_mean": d, "model_mean": m})
    gd, s1 = vec3(rel, 363, "gt.dataset_mean =")
    gm, _ = vec3(rel, 364, "gt.model_mean =")
    gc, _ = grab(rel, 366, r"gt\.covariance\(0,0\) = " + NUM)
    gn, _ = grab(rel, 367, r"gt\.n_meas = " + NUM)
    answers["cross_stats_paper"] = {
        "inputs": parts, "merge": "((c11+c12)+(c13+c14))",
        "expect": {"dataset_mean": gd, "model_mean": gm, "cov00": gc, "n_meas": int(gn)},
        "tol": 1e-4, "source": f"{rel}:329-367"}

    npts, src = grab(rel, 28, r"n_points = " + NUM)
    answers["p2p_filter_counts"] = {
        "n_points": int(npts), "n_points_source": src,
        "fill": "p = i/n; d = (-p, 10p, p); m = (p, p, -p); dataset_mask = i%2; dataset_ids = i%4",
        "fill_source": f"{rel}:495-509", "max_dist": 20000.0,
        "cases": [{"use": "none", "expect": int(npts)},
                  {"use": "dataset_mask", "expect": int(npts) // 2},
                  {"use": "dataset_mask+dataset_ids==2", "expect": 0}],
        "source": f"{rel}:542,554,566"}

    OUT.write_text(json.dumps(answers, indent=1) + "\n")
    print(f"wrote {OUT} ({len(answers)} entries)")


if __name__ == "__main__":
    main()
