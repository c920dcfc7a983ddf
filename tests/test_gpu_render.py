"""GPU path tracer parity with the reference renderer.

Statistical rule: at equal spp, for each pixel and channel the difference of
the per-pixel means must lie within 3 combined standard errors
(sqrt(se_gpu^2 + se_ref^2), from independent batches with distinct sampling
offsets) on at least 99.5 % of pixel channels; pixels whose standard errors
are both zero (constant radiance, e.g. the visible emitter) must agree to
1e-4 relative.  relMSE = mean (x - r)^2 / (r^2 + 1e-2) against the reference
mean is reported."""
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes
from tests.sampler_check import check_sampler

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def batches(renderer, spp, k):
    return np.stack([renderer.render(spp, base_offset=b * spp, seed=1000 + b)[0] for b in range(k)])


def parity(gpu_batches, ref_mean, ref_se):
    k = len(gpu_batches)
    m = gpu_batches.mean(0)
    se = gpu_batches.std(0, ddof=1) / np.sqrt(k)
    comb = np.sqrt(se ** 2 + ref_se ** 2)
    zero = comb == 0
    z = np.where(zero, 0.0, np.abs(m - ref_mean) / np.where(zero, 1.0, comb))
    ok_zero = np.abs(m - ref_mean) <= 1e-4 * np.maximum(1.0, np.abs(ref_mean))
    frac = float(np.mean(np.where(zero, ok_zero, z <= 3.0)))
    relmse = float(np.mean((m - ref_mean) ** 2 / (ref_mean ** 2 + 1e-2)))
    return frac, relmse, m


def test_gpu_sampler_bitexact(cuda_device):
    assert check_sampler(on_device=True) == {}


def test_gpu_cornell_matches_reference(cuda_device):
    g = np.load(os.path.join(GOLD, "cornell_64_render.npz"))
    sc = scenes.cornell_scene(res=64)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_cornell_512_benchmark_size_matches_reference(cuda_device):
    """The Cornell-box configuration at the size the benchmark renders it
    (512x512, 16 spp per batch): per-pixel means of 16 batches within 3
    combined standard errors of the reference's on >= 99.5 % of pixel
    channels."""
    g = np.load(os.path.join(GOLD, "cornell_512_render.npz"))
    r = gbrt.Renderer(scenes.cornell_scene(res=512))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"].astype(np.float32), g["se"].astype(np.float32))
    print(f"cornell 512x512: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].astype(np.float32).mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_render_accumulates_and_counts_rays(cuda_device):
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_scene(res=32)
    r = gbrt.Renderer(sc)
    film = torch.zeros(32 * 32 * 3, dtype=torch.float32, device="cuda")
    st = r.render_device(4, film.data_ptr(), stats=True)
    assert st["camera_samples"] == 32 * 32 * 4
    assert st["extension_rays"] >= st["camera_samples"] and st["shadow_rays"] > 0
    s1 = film.sum().item()
    r.render_device(4, film.data_ptr(), base_offset=4)
    torch.cuda.synchronize()
    assert film.sum().item() > 1.5 * s1
    img64, _ = r.render(8, fp64=True)
    img32, _ = r.render(8)
    assert np.allclose(img64, img32, rtol=1e-4, atol=1e-5)


def test_gpu_cornell_glossy_matches_reference(cuda_device):
    g = np.load(os.path.join(GOLD, "cornell_glossy_64_render.npz"))
    sc = scenes.cornell_scene(res=64, glossy=True)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell glossy 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_indoor_small_matches_reference(cuda_device):
    """Indoor scene (door ajar, outdoor light, glossy and diffuse boxes), 120
    untessellated boxes at 96x54, depth 12 with Russian roulette."""
    g = np.load(os.path.join(GOLD, "indoor_small_render.npz"))
    sc = scenes.indoor_scene(n_boxes=120, subdiv=1, res=(96, 54))
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"indoor small: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_cornell_glass_matches_reference(cuda_device):
    """Glass (specular reflect + refract children, the reflection inside the
    ball limited to ray levels < 3) and rough glass (8-way glossy split with
    both GGX directions, division-scaled light samples and decorrelated
    first bounces in the children) through the recursive split, raydepth 5."""
    g = np.load(os.path.join(GOLD, "cornell_glass_64_render.npz"))
    sc = scenes.cornell_scene(res=64, glass=True)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell glass 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


@pytest.mark.parametrize("name,res,depth", [("cornell_tshadow_64_render.npz", 64, 4), ("cornell_tshadow1_48_render.npz", 48, 1)])
def test_gpu_cornell_transparent_shadows_match_reference(cuda_device, name, res, depth):
    """Transparent shadows (transpShad, shadowDepth): the transparent
    shinydiffuse box and the fake_shadows glass balls let shadow rays pass
    times their filter colour; with shadowDepth 1 a ball's second surface
    blocks."""
    g = np.load(os.path.join(GOLD, name))
    sc = scenes.cornell_scene(res=res, shiny=("transparent",), glass=True, transparent_shadows=depth)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell transparent shadows (depth {depth}) {res}x{res}: {100 * frac:.2f}% of pixel channels within 3 SE, "
          f"relMSE {relmse:.3g}, means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995
    # the same scene with opaque shadows differs from the reference's
    sc0 = scenes.cornell_scene(res=res, shiny=("transparent",), glass=True, transparent_shadows=depth)
    sc0["integrator"]["transpShad"] = False
    r0 = gbrt.Renderer(sc0)
    f0, _, _ = parity(batches(r0, int(g["spp"]), int(g["batches"])), g["mean"], g["se"])
    assert f0 < frac - 0.01


def test_gpu_cornell_textured_matches_reference(cuda_device):
    """Image textures through texture-mapper nodes on shinydiffuse diffuse
    colour: UV coordinates (bilinear, repeat x 2) on the back wall, global
    coordinates with cube mapping, scale / offset, no interpolation, clip
    extend and intensity / contrast adjustments on the tall box."""
    g = np.load(os.path.join(GOLD, "cornell_textured_64_render.npz"))
    r = gbrt.Renderer(scenes.textured_cornell_scene(res=64))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell textured 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_cornell_bicubic_matches_reference(cuda_device):
    """The textured Cornell box with bicubic image interpolation on all three
    textures (ImageTexture::bicubicInterpolation: the repeat + mirror lookup
    of the back wall, the extend and checker-clipped lookups of the boxes).
    The same scene with bilinear lookups is scored against the bicubic
    golden for comparison (printed)."""
    g = np.load(os.path.join(GOLD, "cornell_bicubic_48_render.npz"))
    r = gbrt.Renderer(scenes.textured_cornell_scene(res=48, interpolate="bicubic"))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    rl = gbrt.Renderer(scenes.textured_cornell_scene(res=48, interpolate="bilinear"))
    fl, rel_l, _ = parity(batches(rl, int(g["spp"]), int(g["batches"])), g["mean"], g["se"])
    print(f"cornell bicubic 48x48: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g} "
          f"(bilinear lookups against the same golden: {100 * fl:.2f}%, relMSE {rel_l:.3g})")
    assert frac >= 0.995


@pytest.mark.parametrize("name,ire", [("cornell_sppm_48_render.npz", False), ("cornell_sppm_ire_48_render.npz", True),
                                      ("cornell_sppm_dense_48_render.npz", False)])
def test_gpu_cornell_sppm_matches_reference(cuda_device, name, ire):
    """SPPM (SppmIntegrator): per pass a caustic photon map, one eye sample per
    pixel with direct light and the specular / glossy split, the caustic
    gather within each pixel's shrinking radius and the progressive update;
    with pmIRE the first pass's radius estimate from the diffuse and caustic
    maps; with 1,000,000 photon paths per pass the gather keeps the 1,000
    nearest photons where more lie within the radius."""
    g = np.load(os.path.join(GOLD, name))
    passes = int(g["passes"])
    r = gbrt.Renderer(scenes.cornell_sppm_scene(res=48, photons=int(g["photons"]), passes=passes, pm_ire=ire))
    gb = np.stack([r.render(1, base_offset=b * passes, seed=1000 + b)[0] for b in range(int(g["batches"]))])
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"{name}: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_cornell_smooth_normals_match_reference(cuda_device):
    """Shading normals (PrimitivePolygon::getSurfacePolygon's smooth branch)
    from the reference's yafaray_smoothObjectMesh: a coarse ball averaged at
    every vertex (181 degrees), a glossy torus of quads smoothed within 40
    degrees (bilinear interpolation over each quad), the short box at 30
    degrees (sharp edges kept) and a smoothed glass ball through the
    recursive split.  The flat-shaded render of the same scene does not
    agree with the reference's smooth one."""
    g = np.load(os.path.join(GOLD, "cornell_smooth_64_render.npz"))
    r = gbrt.Renderer(scenes.smooth_cornell_scene(res=64))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell smooth normals 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995
    flat = scenes.smooth_cornell_scene(res=64)
    for o in flat["objects"]:
        o.pop("smooth", None)
    f0, _, _ = parity(batches(gbrt.Renderer(flat), int(g["spp"]), int(g["batches"])), g["mean"], g["se"])
    print(f"flat-shaded render against the smooth reference: {100 * f0:.2f}%")
    assert f0 < frac - 0.02


@pytest.mark.parametrize("name,kw", [("cornell_pt_photon_48_render.npz", dict(caustic_type="photon")),
                                     ("cornell_pt_both_clamp_48_render.npz", dict(caustic_type="both", clamp_indirect=0.3)),
                                     ("cornell_pt_norec_48_render.npz", dict(no_recursive=True))])
def test_gpu_pathtracing_caustic_options_match_reference(cuda_device, name, kw):
    """PathIntegrator's caustic_type photon (a caustic photon map estimated at
    diffuse camera hits, no path caustics after the first bounce), both (path
    + photon, the photon estimate clamped by AA_clamp_indirect 0.3) and
    no_recursive (the path loop at every first hit, all BSDF components) on
    the glass Cornell box."""
    g = np.load(os.path.join(GOLD, name))
    r = gbrt.Renderer(scenes.cornell_pt_variant_scene(res=48, **kw))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"{name}: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_explicit_normals_equal_smoothing(cuda_device):
    """Vertex normals given per vertex (yafaray_addNormal: one normal per
    vertex, every face corner using its vertex's) render like the same
    normals made by smoothing at 181 degrees."""
    sc = scenes.smooth_cornell_scene(res=32, glass=False)
    a = gbrt.Renderer(sc).render(4, base_offset=0, seed=5)[0]
    sc2 = scenes.smooth_cornell_scene(res=32, glass=False)
    for o in sc2["objects"]:
        if o.get("smooth") == 181.0:
            o["normals"], _ = gbrt.smooth_normals(o["vertices"], o["faces"], 181.0)
            del o["smooth"]
    b = gbrt.Renderer(sc2).render(4, base_offset=0, seed=5)[0]
    # equal up to the film's float atomics (their order varies from run to run)
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)


def test_gpu_cornell_shiny_layers_match_reference(cuda_device):
    """ShinyDiffuseMaterial's layers: a Fresnel mirror (specular_reflect 0.8,
    IOR 1.5), transparency 0.5 with transmit_filter 0.7 and translucency 0.3,
    a plain 0.4 mirror over a diffuse layer and an emissive wall, through the
    recursive split (getSpecular) and the path loop (component sampling)."""
    g = np.load(os.path.join(GOLD, "cornell_shiny_64_render.npz"))
    sc = scenes.cornell_scene(res=64, shiny=True)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell shiny 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_cornell_pointlight_matches_reference(cuda_device):
    """A pointlight (MonteCarloIntegrator::diracLight: one shadow ray, colour x
    power / d^2, no MIS) instead of the area light."""
    g = np.load(os.path.join(GOLD, "cornell_point_64_render.npz"))
    sc = scenes.cornell_scene(res=64, point_light=True)
    r = gbrt.Renderer(sc)
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell pointlight 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_recursive_split_small_waves_agree(cuda_device):
    """The depth-first processing of spawned integrate() calls gives the same
    image whether a render runs as one wave or as many small ones (chunked
    spawn levels): means agree within float summation order."""
    sc = scenes.cornell_scene(res=32, glass=True)
    r = gbrt.Renderer(sc)
    torch = pytest.importorskip("torch")
    a = torch.zeros(32 * 32 * 3, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    st_a = r.render_device(8, 0, film64_ptr=a.data_ptr(), stats=True)
    st_b = r.render_device(8, 0, film64_ptr=b.data_ptr(), stats=True, wave_paths=1000)
    torch.cuda.synchronize()
    assert st_a["extension_rays"] == st_b["extension_rays"] and st_a["shadow_rays"] == st_b["shadow_rays"]
    assert torch.allclose(a, b, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("i", [5, 26])
def test_gpu_batch_scene_matches_reference(cuda_device, i):
    """Scenes of the 64-scene batch (tessellated spheres / tori, shinydiffuse +
    glossy + rough glass, several area lights, bounces 8) at 48x48."""
    g = np.load(os.path.join(GOLD, f"batch_scene_{i}_48_render.npz"))
    r = gbrt.Renderer(scenes.batch_scene(i, res=48))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"batch scene {i} 48x48: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_gpu_batch_wavefront_matches_reference(cuda_device):
    """Four scenes of the 64-scene batch rendered together in one wavefront
    (gbrt_pt_render_multi) - scene 18 all rough glass, scene 10 two rough
    glass objects - each against the reference's render of that scene
    alone: per-pixel means of the batches within 3 SE on >= 99.5 %."""
    torch = pytest.importorskip("torch")
    cases = (5, 26, 10, 18)
    gs = [np.load(os.path.join(GOLD, f"batch_scene_{i}_48_render.npz")) for i in cases]
    rs = [gbrt.Renderer(scenes.batch_scene(i, res=48)) for i in cases]
    spp, k = int(gs[0]["spp"]), int(gs[0]["batches"])
    imgs = [[] for _ in cases]
    tuning = None
    for b in range(k):
        films = [torch.zeros(48 * 48 * 3, dtype=torch.float32, device="cuda") for _ in rs]
        _, tuning = gbrt.render_multi(rs, spp, [f.data_ptr() for f in films], tuning=tuning, base_offset=b * spp, seed=1000 + b)
        for j, f in enumerate(films):
            imgs[j].append(f.cpu().numpy().reshape(48, 48, 3) / spp)
    print(f"autotuned: {tuning}")
    for i, g, im in zip(cases, gs, imgs):
        frac, relmse, m = parity(np.stack(im), g["mean"], g["se"])
        print(f"batch wavefront, scene {i}: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}")
        assert frac >= 0.995


def test_gpu_render_batch_equals_single_renders(cuda_device):
    """One wavefront over scenes of different sizes and materials (rough
    glass splits included) gives each scene the image its own render gives
    (up to the order of the film's float atomics) and the same ray counts;
    also with small waves that cut across scene boundaries, 64-thread
    shading blocks and one traversal block per SM."""
    torch = pytest.importorskip("torch")
    rs = [gbrt.Renderer(scenes.batch_scene(i, res=32)) for i in (5, 26, 30)]
    sc = scenes.cornell_scene(res=40, glass=True)
    sc["camera"]["resy"] = 24
    rs.append(gbrt.Renderer(sc))
    singles, rays = [], [0, 0]
    for r in rs:
        n = r.scene["camera"]["resx"] * r.scene["camera"]["resy"] * 3
        f = torch.zeros(n, dtype=torch.float32, device="cuda")
        s1 = r.render_device(4, f.data_ptr(), stats=True)
        torch.cuda.synchronize()
        singles.append(f)
        rays[0] += s1["extension_rays"]
        rays[1] += s1["shadow_rays"]
    for tuning in (None, {"wave_paths": 3000, "shade_block": 64, "trace_blocks_per_sm": 1, "streams": 3}):
        films = [torch.zeros_like(f) for f in singles]
        st, used = gbrt.render_multi(rs, 4, [f.data_ptr() for f in films], tuning=tuning)
        torch.cuda.synchronize()
        print(f"tuning {used}: {st}")
        assert st["extension_rays"] == rays[0] and st["shadow_rays"] == rays[1]
        for f, single in zip(films, singles):
            assert torch.allclose(f, single, rtol=1e-4, atol=1e-6)
        if tuning is None:
            assert used["wave_paths"] in (1 << 19, 1 << 20, 1 << 21, 1 << 22) and used["shade_block"] in (64, 128)
