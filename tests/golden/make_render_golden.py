"""Generates render and sampler golden fixtures from the compiled reference
(oracle/_ref/render_dump and oracle/_ref/sampler_dump, built from the
reference sources by oracle/ref/Makefile).

    make -C oracle/ref -j8 && python tests/golden/make_render_golden.py

cornell_64_render.npz: the Cornell-box configuration at 64x64, `pathtracing`
(path_samples 1, bounces 5, russian_roulette_min_bounces 3), 16 spp per
batch, 32 batches with distinct adv_base_sampling_offset; per-pixel mean and
standard error of the batch means.
sampler.npz: the reference's lowDiscrepancySampling / riVdC / riLp / riS /
fnv32ABuf / Halton(2,3) / FAST_TRIG sin and cos on a fixed input grid.

Other groups, by command-line name (python make_render_golden.py NAME ...):
cornell_glossy, cornell_glass, cornell_point, cornell_shiny, indoor, pm,
cornell_pm, dl, batch, hashgrid, film (gauss film), aa (adaptive-AA film
states + flags and an adaptive render), aa_pm (adaptive passes of
photonmapping / directlighting), cornell_tshadow (transparent shadows,
shadowDepth 4 and 1), cornell_textured (image textures, mapper and layer
nodes), cornell_bicubic (the same textures with bicubic interpolation),
cornell_sppm (SPPM with and without pmIRE), cornell_smooth (smoothed
vertex normals), cornell_pt_caustics (pathtracing caustic_type / no_recursive),
pm_full (config-5 photon maps at full size, as bucketed digests),
cornell_512 (the Cornell configuration at 512x512), cornell_procedural
(procedural textures; needs procedural.npz from make_golden.py procedural),
cornell_nodes (shader node trees on every colour slot; the same tables),
cornell_bump (bump mapping; the same tables).
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import orc  # noqa: E402
from libyafaray_gb300 import scenes  # noqa: E402
from tests.parity import photon_buckets  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SAMPLER = os.path.join(ROOT, "oracle", "_ref", "sampler_dump")


def sampler_golden():
    with tempfile.TemporaryDirectory() as d:
        fo = os.path.join(d, "s.bin")
        subprocess.run([SAMPLER, fo], check=True)
        raw = open(fo, "rb").read()
    nd, ni = struct.unpack("<ii", raw[:8])
    o = 8
    lds = np.frombuffer(raw, np.float64, nd * ni, o).reshape(nd, ni); o += 8 * nd * ni
    vdc = np.frombuffer(raw, np.float32, ni, o); o += 4 * ni
    lp = np.frombuffer(raw, np.float32, ni, o); o += 4 * ni
    ss = np.frombuffer(raw, np.float32, ni, o); o += 4 * ni
    fnv = np.frombuffer(raw, np.uint32, ni, o); o += 4 * ni
    h2 = np.frombuffer(raw, np.float32, ni, o); o += 4 * ni
    h3 = np.frombuffer(raw, np.float32, ni, o); o += 4 * ni
    na = struct.unpack("<i", raw[o:o + 4])[0]; o += 4
    ang = np.frombuffer(raw, np.float32, na, o); o += 4 * na
    sn = np.frombuffer(raw, np.float32, na, o); o += 4 * na
    cs = np.frombuffer(raw, np.float32, na, o); o += 4 * na
    npow = struct.unpack("<i", raw[o:o + 4])[0]; o += 4
    pb = np.frombuffer(raw, np.float32, npow, o); o += 4 * npow
    pe = np.frombuffer(raw, np.float32, npow, o); o += 4 * npow
    pv = np.frombuffer(raw, np.float32, npow, o)
    k = 512
    np.savez_compressed(os.path.join(OUT, "sampler.npz"),
                        lds=lds[:, :k].copy(), lds_index_mult=np.uint32(7919),
                        vdc=vdc[:1024].copy(), lp=lp[:1024].copy(), s=ss[:1024].copy(), fnv=fnv[:1024].copy(),
                        seq_index_mult=np.uint32(2654435761), h2=h2[:1024].copy(), h3=h3[:1024].copy(),
                        halton_start=np.uint32(1000), angle=ang[::4].copy(), sin=sn[::4].copy(), cos=cs[::4].copy(),
                        pow_base=pb.copy(), pow_exp=pe.copy(), pow=pv.copy())
    print("sampler.npz written")


def render_golden(res=64, spp=16, batches=32, glossy=False):
    sc = scenes.cornell_scene(res=res, glossy=glossy)
    rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    name = f"cornell_{'glossy_' if glossy else ''}{res}_render.npz"
    np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32),
                        se=se.astype(np.float32), batches=np.int32(batches), spp=np.int32(spp),
                        seconds=secs)
    print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


HASHGRID = os.path.join(ROOT, "oracle", "_ref", "hashgrid_dump")


def hashgrid_golden():
    """hashgrid.npz: the reference HashGrid's bucket (updateGrid) of every
    photon of photons_small.npz, for two cell sizes and grid sizes, box a =
    the photons' own minimum corner."""
    g = np.load(os.path.join(OUT, "photons_small.npz"))
    pos = np.concatenate([g["diffuse"][:, 3:6], g["caustic"][:, 3:6]]).astype(np.float32)
    lo = pos.min(0) - np.float32(0.001)
    hi = pos.max(0) + np.float32(0.001)
    cases = [(0.02 * (1.0 + 1.0 / 1024.0), 1700), (0.05, 1024), (0.3, 97)]
    out = {"pos": pos, "lo": lo}
    for i, (cell, size) in enumerate(cases):
        with tempfile.TemporaryDirectory() as d:
            fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
            with open(fi, "wb") as f:
                f.write(struct.pack("<dI", cell, size) + np.concatenate([lo, hi]).astype(np.float32).tobytes()
                        + struct.pack("<I", len(pos)) + pos.tobytes())
            subprocess.run([HASHGRID, fi, fo], check=True)
            out[f"bucket{i}"] = np.frombuffer(open(fo, "rb").read(), np.uint32).copy()
        out[f"cell{i}"] = np.float64(cell)
        out[f"size{i}"] = np.uint32(size)
    np.savez_compressed(os.path.join(OUT, "hashgrid.npz"), **out)
    print(f"hashgrid.npz: {len(pos)} points, {len(cases)} cases")


def film_golden(spp=16, batches=32):
    """Cornell at 48x36 through the reference's default film filter (gauss,
    AA_pixelwidth 1.5): each sample splats over neighbouring pixels."""
    sc = scenes.cornell_scene(res=48)
    sc["camera"]["resy"] = 36
    sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5}
    rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    name = "cornell_gauss_48x36_render.npz"
    np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32), se=se.astype(np.float32),
                        batches=np.int32(batches), spp=np.int32(spp), seconds=secs)
    print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


# Adaptive-AA cases: (resx, resy, focal scale, AA_minsamples, film AA_* entries)
AA_CASES = [
    (40, 30, 1.0, 16, dict(AA_threshold=0.15)),
    (40, 30, 1.0, 16, dict(AA_threshold=0.2, AA_variance_pixels=4, AA_variance_edge_size=6, AA_detect_color_noise=True)),
    (40, 30, 1.0, 16, dict(AA_threshold=0.12, AA_dark_detection_type="linear", AA_dark_threshold_factor=0.6,
                           AA_resampled_floor=60.0)),
    (40, 30, 1.0, 16, dict(AA_threshold=0.2, AA_resampled_floor=50.0, AA_sample_multiplier_factor=1.5,
                           AA_light_sample_multiplier_factor=2.0)),
    (24, 18, 6.0, 1024, dict(AA_threshold=0.05, AA_dark_detection_type="curve", AA_inc_samples=64)),
]
AA_RENDER = dict(AA_passes=4, AA_inc_samples=4, AA_threshold=0.2, AA_resampled_floor=50.0,
                 AA_sample_multiplier_factor=1.5, AA_light_sample_multiplier_factor=2.0)


def aa_scene(resx, resy, focal_scale, aa):
    sc = scenes.cornell_scene(res=resx)
    sc["camera"]["resy"] = resy
    sc["camera"]["focal"] = sc["camera"]["focal"] * focal_scale
    sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5, "AA_passes": 3, "AA_inc_samples": 4, **aa}
    return sc


def aa_golden(batches=24, stride=4096):
    """aa_flags.npz: the film state (combined sums, weights, threshold) of the
    reference's adaptive passes and the pixels ImageFilm::nextPass flagged on
    it, for every AA_CASES entry (first two detections each).
    cornell_aa_48x36_render.npz: Cornell 48x36, gauss film, AA_RENDER passes
    from 16 samples, `batches` renders at adv_base_sampling_offset k x stride:
    mean, standard error and the pixels flagged per detection of batch 0."""
    import json
    out = {}
    for i, (rx, ry, fs, spp, aa) in enumerate(AA_CASES):
        sc = aa_scene(rx, ry, fs, aa)
        _, _, passes = orc.run_reference_aa(sc, spp, 1, stride, threads=os.cpu_count() or 1)
        out[f"c{i}_film"] = np.array(json.dumps(sc["film"]))
        for j, p in enumerate(passes[:2]):
            # opaque samples: the alpha sum is the weight sum
            assert np.array_equal(p["sums"][..., 3], p["weights"])
            mask = np.zeros(rx * ry, bool)
            mask[p["flagged"]] = True
            out[f"c{i}_p{j}_sums"] = p["sums"][..., :3].copy()
            out[f"c{i}_p{j}_weights"] = p["weights"]
            out[f"c{i}_p{j}_threshold"] = np.float32(p["threshold"])
            out[f"c{i}_p{j}_flags"] = np.packbits(mask)
        print(f"aa case {i}: flagged {[len(p['flagged']) for p in passes]}")
    np.savez_compressed(os.path.join(OUT, "aa_flags.npz"), n_cases=np.int32(len(AA_CASES)), **out)
    sc = aa_scene(48, 36, 1.0, AA_RENDER)
    rgb, secs, passes = orc.run_reference_aa(sc, 16, batches, stride, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    np.savez_compressed(os.path.join(OUT, "cornell_aa_48x36_render.npz"), mean=mean.astype(np.float32),
                        se=se.astype(np.float32), batches=np.int32(batches), spp=np.int32(16), stride=np.int32(stride),
                        film=np.array(json.dumps(sc["film"])), seconds=secs,
                        flagged=np.array([len(p["flagged"]) for p in passes], np.int32))
    print(f"cornell_aa_48x36_render.npz: mean {mean.mean(axis=(0, 1))}, flagged {[len(p['flagged']) for p in passes]}, "
          f"{secs.sum():.1f} s of reference rendering")


def variant_golden(name, res=64, spp=16, batches=32, **kw):
    """Cornell variants: glass (glass + rough-glass spheres, the recursive
    split) and point (a pointlight instead of the area light)."""
    sc = scenes.cornell_scene(res=res, **kw)
    rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32), se=se.astype(np.float32),
                        batches=np.int32(batches), spp=np.int32(spp), seconds=secs)
    print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


def pm_full_golden():
    """pm_full_maps.npz: the photon maps of the photon-mapping configuration
    at full size (200,000-triangle geodesic glass sphere, 10M diffuse + 10M
    caustic photon paths, threads_photons 1) as bucketed digests (4096
    buckets of count and hash sum per map) with the photon and path counts."""
    sc = scenes.caustic_scene(res=32, geodesic=100, diffuse_photons=10_000_000, caustic_photons=10_000_000,
                              final_gather=False, radius=0.02, search=50)
    (d, dp), (c, cp) = orc.run_reference_photons(sc)
    out = {}
    for name, ph, paths in (("diffuse", d, dp), ("caustic", c, cp)):
        counts, sums = photon_buckets(ph)
        out.update({f"{name}_n": np.int64(len(ph)), f"{name}_paths": np.int64(paths), f"{name}_counts": counts,
                    f"{name}_sums": sums})
    np.savez_compressed(os.path.join(OUT, "pm_full_maps.npz"), **out)
    print(f"pm_full_maps.npz: {len(d)} diffuse / {len(c)} caustic photons of {dp} / {cp} paths")


def pm_golden(spp=8, batches=16):
    """photons_small.npz: diffuse and caustic photon maps of the reference
    (threads_photons 1, so photon path i uses Halton index i) for a 20k-path
    version of the scene; pm_*_render.npz: photonmapping renders."""
    sc = scenes.caustic_scene(res=32, subdiv=3, diffuse_photons=20000, caustic_photons=20000, final_gather=False)
    (d, dp), (c, cp) = orc.run_reference_photons(sc)
    np.savez_compressed(os.path.join(OUT, "photons_small.npz"), diffuse=d, diffuse_paths=np.int32(dp), caustic=c,
                        caustic_paths=np.int32(cp))
    print(f"photons_small.npz: {len(d)} diffuse / {len(c)} caustic photons of {dp} / {cp} paths")
    # area light (Cornell box): 5k diffuse photon paths
    (d, dp), _ = orc.run_reference_photons(scenes.cornell_pm_scene(16, False, diffuse_photons=5000))
    np.savez_compressed(os.path.join(OUT, "photons_cornell.npz"), diffuse=d, diffuse_paths=np.int32(dp))
    print(f"photons_cornell.npz: {len(d)} diffuse photons of {dp} paths")
    for fg in (False, True):
        sc = scenes.caustic_scene_small(fg)
        rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
        mean = rgb.mean(0)
        se = rgb.std(0, ddof=1) / np.sqrt(batches)
        name = f"pm_{'fg' if fg else 'direct'}_48_render.npz"
        # the reference's photonmapping renders of these scenes are
        # deterministic (Halton photon indices, batch-invariant sample
        # positions): its first two batches are kept for a batch-by-batch check
        np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32), se=se.astype(np.float32),
                            batches=np.int32(batches), spp=np.int32(spp), seconds=secs, batch01=rgb[:2].astype(np.float32))
        print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


def cornell_pm_golden(spp=8, batches=24):
    """cornell_pm_{direct,fg}_48_render.npz: the Cornell box (area light) with
    photonmapping: 100k diffuse photon paths, diffuse_search 50; direct
    estimate with diffuse_radius 0.005 (taken as r^2), or final gather with
    diffuse_radius 0.1, fg_samples 8, fg_bounces 2."""
    for fg in (False, True):
        sc = scenes.cornell_pm_scene(48, fg)
        rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
        mean = rgb.mean(0)
        se = rgb.std(0, ddof=1) / np.sqrt(batches)
        name = f"cornell_pm_{'fg' if fg else 'direct'}_48_render.npz"
        np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32), se=se.astype(np.float32),
                            batches=np.int32(batches), spp=np.int32(spp), seconds=secs, batch01=rgb[:2].astype(np.float32))
        print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


BATCH_CASES = (5, 26, 10, 18)        # 18: every object rough glass


def batch_golden(spp=8, batches=24):
    """batch_scene_{i}_48_render.npz: scenes of the 64-scene batch (seed
    1000 + i; spheres / tori, shinydiffuse + glossy + rough glass, 2-4 area
    lights, bounces 8) at 48x48."""
    for i in BATCH_CASES:
        name = f"batch_scene_{i}_48_render.npz"
        if os.path.exists(os.path.join(OUT, name)) and "--force" not in sys.argv:
            continue
        sc = scenes.batch_scene(i, res=48)
        rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
        mean = rgb.mean(0)
        se = rgb.std(0, ddof=1) / np.sqrt(batches)
        name = f"batch_scene_{i}_48_render.npz"
        np.savez_compressed(os.path.join(OUT, name), mean=mean.astype(np.float32), se=se.astype(np.float32),
                            batches=np.int32(batches), spp=np.int32(spp), seconds=secs)
        print(f"{name}: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


def dl_golden(spp=8, batches=24):
    """cornell_dl_48_render.npz: the glass Cornell box with directlighting
    and a 200k-path caustic photon map."""
    sc = scenes.cornell_dl_scene(48)
    rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    np.savez_compressed(os.path.join(OUT, "cornell_dl_48_render.npz"), mean=mean.astype(np.float32), se=se.astype(np.float32),
                        batches=np.int32(batches), spp=np.int32(spp), seconds=secs)
    print(f"cornell_dl_48_render.npz: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


def indoor_golden(spp=16, batches=24):
    sc = scenes.indoor_scene(n_boxes=120, subdiv=1, res=(96, 54))
    rgb, secs = orc.run_reference_render(sc, spp, batches, threads=os.cpu_count() or 1)
    mean = rgb.mean(0)
    se = rgb.std(0, ddof=1) / np.sqrt(batches)
    np.savez_compressed(os.path.join(OUT, "indoor_small_render.npz"), mean=mean.astype(np.float32),
                        se=se.astype(np.float32), batches=np.int32(batches), spp=np.int32(spp), seconds=secs)
    print(f"indoor_small_render.npz: mean {mean.mean(axis=(0, 1))}, {secs.sum():.1f} s of reference rendering")


if __name__ == "__main__":
    if not os.path.exists(SAMPLER) or not os.path.exists(orc.REF_RENDER):
        sys.exit("reference harnesses missing: run make -C oracle/ref first")
    what = sys.argv[1:] or ["sampler", "cornell"]
    if "sampler" in what:
        sampler_golden()
    if "cornell" in what:
        render_golden()
    if "cornell_glossy" in what or "cornell" in what:
        render_golden(glossy=True)
    if "indoor" in what:
        indoor_golden()
    if "cornell_glass" in what:
        variant_golden("cornell_glass_64_render.npz", glass=True)
    if "pm" in what:
        pm_golden()
    if "pm_full" in what:
        pm_full_golden()
    if "hashgrid" in what:
        hashgrid_golden()
    if "dl" in what:
        dl_golden()
    if "batch" in what:
        batch_golden()
    if "cornell_pm" in what:
        cornell_pm_golden()
    if "film" in what:
        film_golden()
    if "cornell_shiny" in what:
        variant_golden("cornell_shiny_64_render.npz", shiny=True)
    if "aa" in what:
        aa_golden()
    if "cornell_tshadow" in what:
        # transparent shadows: a transparent shinydiffuse box and fake_shadows
        # glass balls, shadowDepth 4 (both balls pass) and 1 (a ball's second
        # surface blocks)
        variant_golden("cornell_tshadow_64_render.npz", shiny=("transparent",), glass=True, transparent_shadows=4)
        variant_golden("cornell_tshadow1_48_render.npz", res=48, batches=24, shiny=("transparent",), glass=True,
                       transparent_shadows=1)
    if "cornell_textured" in what:
        # image textures: a UV-mapped bilinear checker on the back wall and a
        # cube-mapped global-coordinate texture on the tall box
        sc = scenes.textured_cornell_scene(res=64)
        rgb, secs = orc.run_reference_render(sc, 16, 32, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_textured_64_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(32)).astype(np.float32), batches=np.int32(32),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_textured_64_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_bicubic" in what:
        # the same textures with bicubic interpolation (repeat + mirror, extend
        # and checker-clipped lookups)
        sc = scenes.textured_cornell_scene(res=48, interpolate="bicubic")
        rgb, secs = orc.run_reference_render(sc, 16, 24, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_bicubic_48_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_bicubic_48_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_procedural" in what:
        # procedural textures (marble, clouds with an HSV ramp, voronoi cells,
        # wood rings under a layer node, a tube-mapped ridged Musgrave fractal);
        # the noise tables are those of procedural.npz (the reference's own)
        g = np.load(os.path.join(OUT, "procedural.npz"))
        tables = {k[len("table_"):]: g[k] for k in g.files if k.startswith("table_")}
        sc = scenes.procedural_cornell_scene(tables, res=64)
        rgb, secs = orc.run_reference_render(sc, 16, 32, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_procedural_64_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(32)).astype(np.float32), batches=np.int32(32),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_procedural_64_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_nodes" in what:
        # shader node trees on every colour slot (mix nodes in each mode, value
        # and layer nodes, mappers over procedural and image textures)
        g = np.load(os.path.join(OUT, "procedural.npz"))
        tables = {k[len("table_"):]: g[k] for k in g.files if k.startswith("table_")}
        sc = scenes.node_cornell_scene(tables, res=64)
        rgb, secs = orc.run_reference_render(sc, 16, 32, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_nodes_64_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(32)).astype(np.float32), batches=np.int32(32),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_nodes_64_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_bump" in what:
        # bump mapping: an image through uvs, marble in global coordinates, a
        # layer chain over clouds and voronoi, blender noise on glass
        g = np.load(os.path.join(OUT, "procedural.npz"))
        tables = {k[len("table_"):]: g[k] for k in g.files if k.startswith("table_")}
        sc = scenes.bump_cornell_scene(tables, res=64)
        rgb, secs = orc.run_reference_render(sc, 16, 32, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_bump_64_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(32)).astype(np.float32), batches=np.int32(32),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_bump_64_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_sppm_dense" in what:
        # SPPM with 1,000,000 photon paths x 2 passes: in the glass ball's
        # caustic thousands of photons lie within the initial radius, so the
        # reference's 1,000-photon gather cap decides those pixels
        sc = scenes.cornell_sppm_scene(res=48, photons=1000000, passes=2)
        rgb, secs = orc.run_reference_render(sc, 1, 24, threads=os.cpu_count() or 1, offset_stride=2)
        np.savez_compressed(os.path.join(OUT, "cornell_sppm_dense_48_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24), passes=np.int32(2),
                            photons=np.int32(1000000), seconds=secs)
        print(f"cornell_sppm_dense_48_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_sppm" in what:
        # SPPM: the glass Cornell box, 100,000 photon paths x 8 passes; batch k
        # at sample offsets 8k .. 8k + 7 (a fresh integrator per batch)
        sc = scenes.cornell_sppm_scene(res=48, photons=100000, passes=8)
        rgb, secs = orc.run_reference_render(sc, 1, 24, threads=os.cpu_count() or 1, offset_stride=8)
        np.savez_compressed(os.path.join(OUT, "cornell_sppm_48_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24), passes=np.int32(8),
                            photons=np.int32(100000), seconds=secs)
        print(f"cornell_sppm_48_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
        # the same with the initial radius estimate (pmIRE, photonRadius 0.1, searchNum 10)
        sc = scenes.cornell_sppm_scene(res=48, photons=100000, passes=8, pm_ire=True)
        rgb, secs = orc.run_reference_render(sc, 1, 24, threads=os.cpu_count() or 1, offset_stride=8)
        np.savez_compressed(os.path.join(OUT, "cornell_sppm_ire_48_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24), passes=np.int32(8),
                            photons=np.int32(100000), seconds=secs)
        print(f"cornell_sppm_ire_48_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "aa_pm" in what:
        # adaptive AA passes of the photonmapping (direct estimate) and
        # directlighting integrators
        for name, sc in (("cornell_pm_aa_48_render.npz", scenes.cornell_pm_scene(48, False)),
                         ("cornell_dl_aa_48_render.npz", scenes.cornell_dl_scene(48))):
            sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5, "AA_passes": 3, "AA_inc_samples": 2,
                          "AA_threshold": 0.08}
            rgb, secs, passes = orc.run_reference_aa(sc, 8, 24, 4096, threads=os.cpu_count() or 1)
            np.savez_compressed(os.path.join(OUT, name), mean=rgb.mean(0).astype(np.float32),
                                se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24), spp=np.int32(8),
                                stride=np.int32(4096), film=np.array(__import__("json").dumps(sc["film"])), seconds=secs,
                                flagged=np.array([len(p["flagged"]) for p in passes], np.int32))
            print(f"{name}: mean {rgb.mean(axis=(0, 1, 2))}, flagged {[len(p['flagged']) for p in passes]}, {secs.sum():.1f} s")
    if "cornell_point" in what:
        variant_golden("cornell_point_64_render.npz", point_light=True)
    if "cornell_512" in what:
        # the Cornell-box configuration at its benchmark size: 512x512, 16 spp
        # per batch, 16 batches; mean and standard error kept as float16
        sc = scenes.cornell_scene(res=512)
        rgb, secs = orc.run_reference_render(sc, 16, 16, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_512_render.npz"), mean=rgb.mean(0).astype(np.float16),
                            se=(rgb.std(0, ddof=1) / np.sqrt(16)).astype(np.float16), batches=np.int32(16),
                            spp=np.int32(16), seconds=secs)
        print(f"cornell_512_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_pt_caustics" in what:
        # pathtracing's caustic options on the glass Cornell box: photon
        # caustics, both (path + photon) with AA_clamp_indirect, no_recursive
        for name, kw in (("cornell_pt_photon_48_render.npz", dict(caustic_type="photon")),
                         ("cornell_pt_both_clamp_48_render.npz", dict(caustic_type="both", clamp_indirect=0.3)),
                         ("cornell_pt_norec_48_render.npz", dict(no_recursive=True))):
            sc = scenes.cornell_pt_variant_scene(res=48, **kw)
            rgb, secs = orc.run_reference_render(sc, 8, 24, threads=os.cpu_count() or 1)
            np.savez_compressed(os.path.join(OUT, name), mean=rgb.mean(0).astype(np.float32),
                                se=(rgb.std(0, ddof=1) / np.sqrt(24)).astype(np.float32), batches=np.int32(24),
                                spp=np.int32(8), seconds=secs)
            print(f"{name}: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
    if "cornell_smooth" in what:
        # shading normals: yafaray_smoothObjectMesh at 181 (a coarse ball, a
        # glass ball), 40 (a torus of quads) and 30 degrees (the short box)
        sc = scenes.smooth_cornell_scene(res=64)
        rgb, secs = orc.run_reference_render(sc, 16, 32, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_smooth_64_render.npz"), mean=rgb.mean(0).astype(np.float32),
                            se=(rgb.std(0, ddof=1) / np.sqrt(32)).astype(np.float32), batches=np.int32(32),
                            spp=np.int32(16), seconds=secs)
        # the normals the reference's MeshObject::smoothVerticesNormals makes
        # for the same objects are pinned by the render; the flat render of the
        # same scene shows that the smoothing is visible
        flat = scenes.smooth_cornell_scene(res=64)
        for o in flat["objects"]:
            o.pop("smooth", None)
        rgb_f, _ = orc.run_reference_render(flat, 16, 8, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(OUT, "cornell_smooth_flat_64_render.npz"), mean=rgb_f.mean(0).astype(np.float32),
                            batches=np.int32(8), spp=np.int32(16))
        print(f"cornell_smooth_64_render.npz: mean {rgb.mean(axis=(0, 1, 2))}, {secs.sum():.1f} s")
