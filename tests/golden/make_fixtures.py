"""Generates the committed fixtures in tests/golden/ from the oracle.

algorithmic_bytes.json: per-ray algorithmic bytes of each benchmark workload,
counted by the oracle under the reference's GLSL traversal order
(src/shaders/scene.glsl:218-267: near-first, both child boxes read per inner
node): 64 B per inner node visited + 48 B per triangle tested + 24 B ray in +
16 B hit out. bench.py divides these by the measured kernel time for its
roofline; tests/test_fixtures.py re-derives the cheap ones so they cannot go
stale.

Run: python tests/golden/make_fixtures.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from lucent_gb300 import workloads  # noqa: E402


def closest_bytes(n_rays=200_000):
    """Random soup workload; the mean over the first n_rays of its 10^6 rays."""
    pos, rays = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=1_000_000)
    ob = oracle.build_bvh(pos)
    geo = oracle.leaf_order_geometry(ob, pos)
    inner, tris, _ = oracle.glsl_traversal_counts(ob.nodes, ob.node_count, geo, rays[:n_rays], 1e-5)
    popped, tests = oracle.ts_traversal_counts(ob, pos, rays[:n_rays])
    per_ray = 64.0 * inner.mean() + 48.0 * tris.mean() + 24 + 16
    return {"bytes_per_ray": round(float(per_ray), 2), "inner_nodes_per_ray": round(float(inner.mean()), 3),
            "triangles_per_ray": round(float(tris.mean()), 3), "rays_sampled": n_rays,
            "reference_order_nodes_per_ray": round(float(popped.mean()), 3),
            "reference_order_triangles_per_ray": round(float(tests.mean()), 3)}


def box_scene_bytes(samples=1):
    """Path-tracing workload (box scene, seed 0, 81,956 triangles, 512 x 512,
    depth 8): the oracle renders `samples` spp of the full frame and tallies,
    for every closest-hit ray, the reference GLSL traversal's inner nodes and
    triangles (64 B / 48 B each) and, for every shadow ray, the occluded()
    traversal's visited nodes and triangles (32 B / 48 B); + 24 B ray in and
    16 B result out per ray."""
    from oracle import render as R
    prep = R.prepare(workloads.box_scene(0, 6))
    w = R.render_work(prep, 512, 512, 0, samples, max_bounces=8)
    c, s = w["closest_rays"], w["shadow_rays"]
    return {"bytes_per_closest_ray": round((64.0 * w["closest_inner"] + 48.0 * w["closest_tris"]) / c + 40, 2),
            "bytes_per_shadow_ray": round((32.0 * w["shadow_nodes"] + 48.0 * w["shadow_tris"]) / s + 40, 2),
            "closest_rays_per_path": round(c / (512 * 512 * samples), 4),
            "shadow_rays_per_path": round(s / (512 * 512 * samples), 4),
            "inner_nodes_per_closest_ray": round(w["closest_inner"] / c, 3),
            "triangles_per_closest_ray": round(w["closest_tris"] / c, 3), "samples": samples}


def knot_bytes(samples=1, crop=(720, 405, 480, 270)):
    """Large-mesh workload (2,000,000-triangle displaced torus knot, 1920 x
    1080, depth 12): the oracle renders `samples` spp of a centred 480 x 270
    crop (a sixteenth of the frame) and tallies the reference GLSL traversal
    work as box_scene_bytes does."""
    from oracle import render as R
    prep = R.prepare(workloads.knot_scene(0))
    w = R.render_work(prep, 1920, 1080, 0, samples, max_bounces=12, crop=crop)
    c, s = w["closest_rays"], w["shadow_rays"]
    px = crop[2] * crop[3] * samples
    return {"bytes_per_closest_ray": round((64.0 * w["closest_inner"] + 48.0 * w["closest_tris"]) / c + 40, 2),
            "bytes_per_shadow_ray": round((32.0 * w["shadow_nodes"] + 48.0 * w["shadow_tris"]) / s + 40, 2),
            "closest_rays_per_path": round(c / px, 4), "shadow_rays_per_path": round(s / px, 4),
            "inner_nodes_per_closest_ray": round(w["closest_inner"] / c, 3),
            "triangles_per_closest_ray": round(w["closest_tris"] / c, 3), "samples": samples,
            "crop": list(crop)}


def main():
    path = os.path.join(HERE, "algorithmic_bytes.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    out["closest"] = closest_bytes()
    out["pt_box"] = box_scene_bytes()
    out["pt_knot"] = knot_bytes()
    json.dump(out, open(path, "w"), indent=1, sort_keys=True)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
