"""Generates the traversal golden vectors in tests/golden/*.npz by running the
reference libYafaRay kd-tree itself (oracle/_ref/kdtree_dump, built from the
reference sources by oracle/ref/Makefile) ray by ray.

    make -C oracle/ref -j8 && python tests/golden/make_golden.py

Each file holds the scene (vertices, faces), the rays, and what the reference
returned: closest hit (Accelerator::intersect) prim/t/u/v and shadow
occlusion (Accelerator::isShadowed) as a hit flag, plus the tree bound.

    python tests/golden/make_golden.py normals   # smooth_normals.npz only
    python tests/golden/make_golden.py binding   # binding_translation.npz only

smooth_normals.npz holds the reference's yafaray_smoothObjectMesh results;
binding_translation.npz the scenes the reference-side binding
(oracle/ref/gb300_binding.cc) translates for the GPU library.
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


if __name__ == "__main__":
    if sys.argv[1:] == ["normals"]:
        normals_golden()
    elif sys.argv[1:] == ["binding"]:
        binding_golden()
    else:
        main()
