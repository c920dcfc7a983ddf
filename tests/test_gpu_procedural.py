"""Procedural textures on the GPU: the device evaluation
(gbrt_texture_eval on_device) against the compiled reference's values
(tests/golden/procedural.npz), and a Cornell box textured procedurally
everywhere against the reference's render (cornell_procedural_64_render.npz)."""
import json
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes
from tests.test_gpu_render import batches, parity

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden():
    g = np.load(os.path.join(GOLD, "procedural.npz"))
    tables = {k[len("table_"):]: g[k] for k in g.files if k.startswith("table_")}
    return g, tables, json.loads(str(g["cases"]))


@pytest.mark.gpu
def test_gpu_procedural_textures_match_reference(cuda_device):
    """Every case bit for bit, except the radial blend progression, whose
    atan2f is the device's (within 2 ulp of the host's)."""
    g, tables, cases = golden()
    pts = g["points"]
    for i, t in enumerate(cases):
        rgba, val = gbrt.texture_eval(t, tables, pts, on_device=True)
        if t.get("blend_type") == "radial":
            np.testing.assert_allclose(rgba, g[f"rgba_{i}"], rtol=3e-7, atol=3e-7, err_msg=str(t))
            np.testing.assert_allclose(val, g[f"value_{i}"], rtol=3e-7, atol=3e-7, err_msg=str(t))
            continue
        assert np.array_equal(rgba.view(np.uint32), g[f"rgba_{i}"].view(np.uint32)), (i, t)
        assert np.array_equal(val.view(np.uint32), g[f"value_{i}"].view(np.uint32)), (i, t)


@pytest.mark.gpu
def test_gpu_cornell_procedural_matches_reference(cuda_device):
    """Marble, clouds through an HSV ramp, voronoi cells, wood rings under a
    multiply layer node, and a tube-mapped ridged Musgrave fractal with
    adjustments, all as shinydiffuse diffuse shaders."""
    _, tables, _ = golden()
    g = np.load(os.path.join(GOLD, "cornell_procedural_64_render.npz"))
    r = gbrt.Renderer(scenes.procedural_cornell_scene(tables, res=64))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell procedural 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


@pytest.mark.gpu
def test_gpu_procedural_texture_needs_noise_tables(cuda_device):
    """gbrt_scene_set_textures refuses a procedural texture until the
    scene has the host's noise tables."""
    import ctypes
    r = gbrt.Renderer(scenes.cornell_scene(res=8))
    d, _ = gbrt.texture_desc({"type": "clouds"})
    descs = (gbrt.TextureDesc * 1)(d)
    mt = np.full(len(r.mat_names), -1, np.int32)
    mt[0] = 0
    with pytest.raises(gbrt.GbrtError):
        gbrt.check(gbrt.load().gbrt_scene_set_textures(r._h, None, 0, None, descs, 1, gbrt._ptr(mt), len(mt)))
    _, tables, _ = golden()
    nt, keep = gbrt.noise_tables(tables)
    gbrt.check(gbrt.load().gbrt_scene_set_noise_tables(r._h, ctypes.byref(nt)))
    gbrt.check(gbrt.load().gbrt_scene_set_textures(r._h, None, 0, None, descs, 1, gbrt._ptr(mt), len(mt)))
    img, _ = r.render(2)
    assert np.isfinite(img).all()


@pytest.mark.gpu
def test_gpu_cornell_shader_nodes_match_reference(cuda_device):
    """Shader node trees on every colour slot: mix nodes in the multiply
    (with a texture's scalar as factor), overlay, darken, lighten, screen,
    subtract, difference and add modes, a value node, two chained layer
    nodes (stencil, upper_layer), texture mappers over procedural and image
    textures; on shinydiffuse and glossy diffuse, glossy colour, glass and
    rough-glass filter and mirror colours."""
    _, tables, _ = golden()
    g = np.load(os.path.join(GOLD, "cornell_nodes_64_render.npz"))
    r = gbrt.Renderer(scenes.node_cornell_scene(tables, res=64))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell shader nodes 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


@pytest.mark.gpu
def test_gpu_shader_nodes_reject_bad_trees(cuda_device):
    """Inputs must lie below a node, slots must exist on the material type."""
    _, tables, _ = golden()
    sc = scenes.node_cornell_scene(tables, res=8)
    sc["material_shaders"]["grey"] = {"glossy_shader": "m_clouds"}     # shinydiffuse has no glossy slot
    with pytest.raises(gbrt.GbrtError):
        gbrt.Renderer(sc)


@pytest.mark.gpu
def test_gpu_cornell_bump_matches_reference(cuda_device):
    """Bump mapping on four materials: an image bump map through uv
    coordinates (the texture-space slope branch), marble in global
    coordinates (shinydiffuse), a negated, stencilled layer over clouds with
    a voronoi upper layer (glossy), blender-noise clouds (glass)."""
    _, tables, _ = golden()
    g = np.load(os.path.join(GOLD, "cornell_bump_64_render.npz"))
    r = gbrt.Renderer(scenes.bump_cornell_scene(tables, res=64))
    gb = batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m = parity(gb, g["mean"], g["se"])
    print(f"cornell bump 64x64: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995
