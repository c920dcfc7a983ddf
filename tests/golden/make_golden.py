"""Generates the traversal golden vectors in tests/golden/*.npz by running the
reference libYafaRay kd-tree itself (oracle/_ref/kdtree_dump, built from the
reference sources by oracle/ref/Makefile) ray by ray.

    make -C oracle/ref -j8 && python tests/golden/make_golden.py

Each file holds the scene (vertices, faces), the rays, and what the reference
returned: closest hit (Accelerator::intersect) prim/t/u/v and shadow
occlusion (Accelerator::isShadowed) as a hit flag, plus the tree bound.

    python tests/golden/make_golden.py normals   # smooth_normals.npz only
    python tests/golden/make_golden.py binding   # binding_translation.npz only
    python tests/golden/make_golden.py procedural   # procedural.npz only

smooth_normals.npz holds the reference's yafaray_smoothObjectMesh results;
binding_translation.npz the scenes the reference-side binding
(oracle/ref/gb300_binding.cc) translates for the GPU library;
procedural.npz the reference's noise tables and procedural textures
evaluated at seeded points (oracle/_ref/noise_dump).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import orc  # noqa: E402
from libyafaray_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def edge_rays(verts, faces, n, seed):
    """Rays aimed at face vertices and edge midpoints (shared-edge cases) and
    axis-aligned rays (zero direction components)."""
    rng = np.random.default_rng(seed)
    lo, hi = verts.min(0), verts.max(0)
    ext = hi - lo
    rays = np.zeros((n, 8), np.float32)
    for i in range(n):
        f = faces[rng.integers(len(faces))]
        nv = 3 if f[3] == scenes.TRI else 4
        a, b = rng.choice(nv, 2, replace=False)
        target = 0.5 * (verts[f[a]].astype(np.float64) + verts[f[b]]) if i % 2 else verts[f[a]].astype(np.float64)
        o = lo - 0.3 * ext + rng.random(3) * 1.6 * ext
        if i % 7 == 0:  # axis-aligned
            ax = rng.integers(3)
            o = target.copy(); o[ax] = lo[ax] - 0.5 * ext[ax] if rng.random() < 0.5 else hi[ax] + 0.5 * ext[ax]
        d = target - o
        d /= np.linalg.norm(d)
        rays[i, :3] = o; rays[i, 3] = 0.0; rays[i, 4:7] = d; rays[i, 7] = -1.0
    return rays


def bounded_rays(rays, seed):
    """Copies with tmin > 0 and finite tmax (shadow-ray style segments)."""
    rng = np.random.default_rng(seed)
    r = rays.copy()
    r[:, 3] = rng.choice([0.0, 1e-4, 5e-4, 0.01], len(r)).astype(np.float32)
    r[:, 7] = np.where(rng.random(len(r)) < 0.3, -1.0, rng.uniform(0.05, 2.0, len(r))).astype(np.float32)
    return r


def run_case(name, verts, faces, rays):
    b0, bs, ts, p0, t0, u0, v0 = orc.run_reference_kdtree(verts, faces, rays, 0)
    b1, _, _, p1, _, _, _ = orc.run_reference_kdtree(verts, faces, rays, 1)
    assert np.array_equal(b0, b1)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), vertices=verts, faces=faces, rays=rays, bound=b0,
                        closest_prim=p0, closest_t=t0, closest_u=u0, closest_v=v0,
                        shadow_hit=(p1 >= 0).astype(np.uint8))
    print(f"{name}: {len(faces)} faces, {len(rays)} rays, {int((p0 >= 0).sum())} closest hits, "
          f"{int((p1 >= 0).sum())} occluded, kd build {bs:.3f}s trace {ts:.3f}s")


def main():
    only = sys.argv[1:]
    if not orc.reference_available():
        sys.exit("oracle/_ref/kdtree_dump missing: run make -C oracle/ref first")
    # 1. triangle soup, the traversal micro-benchmark's distribution, small
    v, f = scenes.random_triangles(4096, seed=1)
    r = scenes.random_rays(4096, seed=2)
    run_case("tri_soup_4k", v, f, r)
    # 1b. denser soup (larger triangles, many overlaps), incl. bounded segments
    v, f = scenes.random_triangles(4096, seed=12, spread=0.06)
    r = scenes.random_rays(6144, seed=13)
    r = np.concatenate([r, bounded_rays(scenes.random_rays(2048, seed=14), seed=15)])
    run_case("tri_soup_dense", v, f, r)
    # 2. Cornell box, quads (one primitive per quad, shared edges)
    v, f, _ = scenes.cornell_mesh(as_quads=True)
    cam = scenes.camera_rays(48, 48, (0.0, 1.0, 3.7), (0.0, 1.0, 0.0), seed=5)
    inside = scenes.random_rays(2048, seed=6, lo=-0.95, hi=0.95)
    inside[:, 1] += 1.0
    er = edge_rays(v, f, 1024, seed=7)
    r = np.concatenate([cam, inside, er, bounded_rays(inside, seed=8)])
    run_case("cornell_quads", v, f, r)
    # 3. Cornell box as triangles
    v, f, _ = scenes.cornell_mesh(as_quads=False)
    er = edge_rays(v, f, 1024, seed=9)
    r = np.concatenate([cam, inside, er, bounded_rays(inside, seed=10)])
    run_case("cornell_tris", v, f, r)
    # 4. one triangle, incl. degenerate neighbours (zero area)
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0], [0.5, 0.5, 0], [0.2, 0.2, 0]], np.float32)
    f = np.array([[0, 1, 2, scenes.TRI], [3, 4, 5, scenes.TRI]], np.uint32)
    rng = np.random.default_rng(11)
    r = np.zeros((512, 8), np.float32)
    r[:, 0:2] = rng.uniform(-0.2, 1.2, (512, 2)); r[:, 2] = 1.0
    r[:, 6] = -1.0; r[:, 7] = -1.0
    r[::3, 6] = 1.0   # pointing away
    r[::5, 2] = 0.0; r[::5, 4] = 1.0; r[::5, 6] = 0.0  # in-plane rays
    run_case("single_tri", v, f, r)
    # 5. displaced sphere (Perlin amplitude 0.05), the micro-benchmark's second
    # mesh at 16k triangles: camera-coherent primary rays + random rays
    v, f = scenes.perlin_sphere(128, 64)
    cam = scenes.camera_rays(96, 54, (0.0, 0.6, 3.2), (0.0, 0.0, 0.0), seed=16)
    r = np.concatenate([cam, scenes.random_rays(2048, seed=17, lo=-1.5, hi=1.5), edge_rays(v, f, 512, seed=18)])
    run_case("perlin_sphere_16k", v, f, r)
    normals_golden()


def normals_golden():
    """smooth_normals.npz: per face corner the normal index and normal the
    reference's yafaray_smoothObjectMesh gives: a coarse icosphere at 181 /
    100 / 30 / 0.05 degrees, a torus of quads at 40 and 181, the Cornell
    short box at 30, and a noisy height field at 50 (many merges)."""
    cases = {}
    v, f = scenes.icosphere((0.1, 0.2, 0.3), 0.7, 1)
    for a in (181.0, 100.0, 30.0, 0.05):
        cases[f"ico_{a:g}"] = (v, f, a)
    v, f = scenes.torus_quads((0.0, 0.1, 0.0), 0.5, 0.2, 12, 8)
    for a in (40.0, 181.0):
        cases[f"torus_{a:g}"] = (v, f, a)
    sc = scenes.smooth_cornell_scene(res=8, glass=False)
    box = [o for o in sc["objects"] if o["name"] == "group3"][0]
    cases["box_30"] = (box["vertices"], box["faces"], 30.0)
    rng = np.random.default_rng(21)
    n = 9
    gx, gz = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    hv = np.stack([gx, 0.15 * rng.random((n, n)), gz], -1).reshape(-1, 3).astype(np.float32)
    quads = [[i * n + j, i * n + j + 1, (i + 1) * n + j + 1, (i + 1) * n + j] for i in range(n - 1) for j in range(n - 1)]
    hf = np.array([[a, b, c, scenes.TRI] if k % 3 else [a, b, c, d] for k, (a, b, c, d) in enumerate(quads)], np.uint32)
    cases["height_50"] = (hv, hf, 50.0)
    out = {}
    for name, (v, f, a) in cases.items():
        idx, nrm = orc.run_reference_normals(v, f, a)
        out[f"{name}_vertices"] = np.asarray(v, np.float32)
        out[f"{name}_faces"] = np.asarray(f, np.uint32)
        out[f"{name}_angle"] = np.float32(a)
        out[f"{name}_index"] = idx
        out[f"{name}_normal"] = nrm
    out["cases"] = np.array(sorted(cases))
    np.savez_compressed(os.path.join(OUT, "smooth_normals.npz"), **out)
    print(f"smooth_normals.npz: {len(cases)} meshes")


BINDING_CASES = {
    # the glass Cornell box with smoothed meshes (shading normals per corner)
    "smooth": lambda: scenes.smooth_cornell_scene(res=48),
    # pathtracing with a caustic photon map and the film's AA_clamp_indirect
    "pt_photon": lambda: scenes.cornell_pt_variant_scene(res=48, caustic_type="both", clamp_indirect=2.0),
}


def binding_golden():
    """binding_translation.npz: the scenes of BINDING_CASES as the
    reference-side binding (oracle/ref/gb300_binding.cc, run by
    oracle/_ref/binding_dump) hands them to the GPU library: arrays, and the
    descriptor structures as raw bytes (gbrt.h layouts)."""
    out = {}
    for name, make in BINDING_CASES.items():
        tr = orc.run_reference_translation(make(), spp=8)
        assert tr["ok"], tr["error"]
        for k in ("vertices", "faces", "face_material", "normals", "face_normals"):
            if k in tr:
                out[f"{name}_{k}"] = tr[k]
        for k in ("materials", "lights"):
            out[f"{name}_{k}"] = np.frombuffer(b"".join(bytes(x) for x in tr[k]), np.uint8)
        for k in ("camera", "params", "aa", "caustic"):
            out[f"{name}_{k}"] = np.frombuffer(bytes(tr[k]), np.uint8)
    out["cases"] = np.array(sorted(BINDING_CASES))
    np.savez_compressed(os.path.join(OUT, "binding_translation.npz"), **out)
    print(f"binding_translation.npz: {len(BINDING_CASES)} scenes")


def procedural_cases():
    """The procedural textures the golden covers: every texture type, every
    noise generator, every voronoi metric and colour mode, every Musgrave
    type, every blend progression, colour ramps in each mode and hue
    interpolation, and the colour adjustments."""
    ramp3 = {"ramp_num_items": 3, "ramp_item_0_color": (1.0, 0.1, 0.0, 1.0), "ramp_item_0_position": 0.15,
             "ramp_item_1_color": (0.1, 0.9, 0.2, 0.5), "ramp_item_1_position": 0.55,
             "ramp_item_2_color": (0.2, 0.1, 1.0, 0.8), "ramp_item_2_position": 0.85}
    cases = []
    noises = ["blender", "stdperlin", "newperlin", "cellnoise", "voronoi_f1", "voronoi_f2", "voronoi_f3", "voronoi_f4",
              "voronoi_f2f1", "voronoi_crackle"]
    for i, n in enumerate(noises):
        cases.append({"type": "clouds", "noise_type": n, "depth": i % 4, "size": 0.6 + 0.1 * i, "hard": i % 2 == 1,
                      "color1": (0.1, 0.2, 0.3), "color2": (0.9, 0.7, 0.4)})
    cases += [{"type": "clouds", "noise_type": "blender", "bias": "positive", "depth": 3},
              {"type": "clouds", "noise_type": "stdperlin", "bias": "negative", "depth": 2, "hard": True}]
    for i, (shape, n) in enumerate([("sin", "newperlin"), ("saw", "blender"), ("tri", "voronoi_f1")]):
        cases.append({"type": "marble", "shape": shape, "noise_type": n, "sharpness": 1.0 + 1.5 * i, "turbulence": 2.0 + i,
                      "depth": 1 + i, "hard": i == 1})
        cases.append({"type": "wood", "shape": shape, "noise_type": n, "wood_type": "rings" if i % 2 else "bands",
                      "turbulence": 0.0 if i == 2 else 0.7, "depth": i, "size": 0.8})
    metrics = ["real", "squared", "manhattan", "chebychev", "minkovsky_half", "minkovsky_four", "minkovsky"]
    modes = ["intensity-without-color", "position", "position-outline", "position-outline-intensity"]
    for i, m in enumerate(metrics):
        cases.append({"type": "voronoi", "distance_metric": m, "color_mode": modes[i % 4], "mk_exponent": 1.7, "size": 1.3,
                      "weight1": 1.0, "weight2": -0.5 if i % 2 else 0.3, "weight3": 0.2 * (i % 3), "weight4": 0.1,
                      "intensity": 0.9})
    for i, (mt, n) in enumerate([("fBm", "newperlin"), ("multifractal", "blender"), ("heteroterrain", "stdperlin"),
                                 ("hybridmf", "voronoi_crackle"), ("ridgedmf", "newperlin")]):
        cases.append({"type": "musgrave", "musgrave_type": mt, "noise_type": n, "octaves": 2.0 + 0.75 * i, "H": 0.6 + 0.1 * i,
                      "lacunarity": 2.2, "offset": 0.9 + 0.1 * i, "gain": 1.3, "intensity": 0.8, "size": 0.7})
    cases += [{"type": "distorted_noise", "noise_type1": "blender", "noise_type2": "voronoi_f2f1", "distort": 1.5, "size": 0.8},
              {"type": "distorted_noise", "noise_type1": "stdperlin", "noise_type2": "cellnoise", "distort": 0.4}]
    for bt in ["linear", "quadratic", "easing", "diagonal", "sphere", "quad_sphere", "radial"]:
        cases.append({"type": "blend", "blend_type": bt, "use_flip_axis": bt in ("easing", "diagonal")})
    cases.append({"type": "rgb_cube"})
    cases.append({"type": "rgb_cube", "adj_contrast": 1.4, "adj_clamp": True})
    for mode, interp, hue in [("RGB", "LINEAR", "NEAR"), ("RGB", "CONSTANT", "NEAR"), ("HSV", "LINEAR", "NEAR"),
                              ("HSV", "LINEAR", "FAR"), ("HSV", "LINEAR", "CW"), ("HSL", "LINEAR", "CCW")]:
        cases.append({"type": "clouds", "noise_type": "newperlin", "depth": 2, **ramp3, "ramp_color_mode": mode,
                      "ramp_interpolation": interp, "ramp_hue_interpolation": hue})
    cases.append({"type": "voronoi", "color_mode": "position", **ramp3})
    cases.append({"type": "blend", "blend_type": "sphere", **ramp3, "ramp_color_mode": "HSV"})
    cases += [{"type": "clouds", "adj_intensity": 1.2, "adj_contrast": 0.8, "adj_saturation": 0.5, "adj_hue": 30.0,
               "adj_mult_factor_red": 1.3, "color1": (0.2, 0.4, 0.1), "color2": (0.9, 0.3, 0.6)},
              {"type": "marble", "adj_mult_factor_green": 0.5, "adj_hue": -50.0, "adj_clamp": True, "color1": (0.9, 0.2, 0.1)},
              {"type": "voronoi", "color_mode": "position-outline-intensity", "adj_intensity": 0.7, "adj_saturation": 1.6}]
    return cases


def procedural_golden():
    """procedural.npz: the reference's noise tables and, at 768 seeded
    texture-space points, each case of procedural_cases: getColor RGBA and
    getFloat (oracle/_ref/noise_dump)."""
    import json
    rng = np.random.default_rng(31)
    pts = np.concatenate([rng.uniform(-3.0, 3.0, (512, 3)), rng.uniform(-0.5, 0.5, (192, 3)),
                          np.round(rng.uniform(-4, 4, (64, 3))) + rng.choice([0.0, 1e-4, -1e-4, 0.5], (64, 3))]).astype(np.float32)
    cases = procedural_cases()
    tables, tex, _, _ = orc.run_reference_textures(cases, pts)
    out = {f"table_{k}": v for k, v in tables.items()}
    out["points"] = pts
    out["cases"] = np.array(json.dumps(cases))
    for i, (status, rgba, val) in enumerate(tex):
        assert status == 0, cases[i]
        out[f"rgba_{i}"] = rgba
        out[f"value_{i}"] = val
    np.savez_compressed(os.path.join(OUT, "procedural.npz"), **out)
    print(f"procedural.npz: {len(cases)} textures at {len(pts)} points")


if __name__ == "__main__":
    if sys.argv[1:] == ["normals"]:
        normals_golden()
    elif sys.argv[1:] == ["binding"]:
        binding_golden()
    elif sys.argv[1:] == ["procedural"]:
        procedural_golden()
    else:
        main()
