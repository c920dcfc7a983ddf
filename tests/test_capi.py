"""CPU-side checks of the C ABI library: it builds, loads, and exports every
function include/gbrt.h declares; error paths work without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from libyafaray_gb300 import gbrt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name):
    src = open(os.path.join(ROOT, "include", name)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbrt_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected_entry_points():
    fns = header_functions("gbrt.h")
    for f in ["gbrt_bvh_build", "gbrt_bvh_build_host", "gbrt_bvh_destroy", "gbrt_trace_closest",
              "gbrt_trace_shadow", "gbrt_trace_closest_host", "gbrt_trace_shadow_host", "gbrt_bvh_get_bound"]:
        assert f in fns


def test_library_exports_every_declared_symbol(gbrt_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", gbrt.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gbrt_[a-z0-9_]+)", out))
    missing = [f for f in header_functions("gbrt.h") if f not in exported]
    assert not missing, missing
    # and the ctypes binding covers the same set
    assert set(gbrt.SIGNATURES) == set(header_functions("gbrt.h"))


def test_null_arguments_are_errors_not_crashes(gbrt_lib):
    L = gbrt_lib
    assert L.gbrt_bvh_build_host(None, 0, None, 1, None, None) == -1
    assert b"NULL" in L.gbrt_last_error()
    assert L.gbrt_trace_closest(None, None, 10, None, None) == -1
    assert L.gbrt_bvh_destroy(None) == 0
    assert L.gbrt_version() >= 1


def test_guide_and_tensor_core_argument_checks(gbrt_lib):
    """Argument errors are reported before any CUDA call."""
    import numpy as np
    from libyafaray_gb300 import gbrt
    L = gbrt_lib
    assert L.gbrt_guide_set_eval_mode(None, 0) == -1
    assert L.gbrt_guide_status(None, None) == -1
    a = np.zeros((128, 16), np.float32)
    with pytest.raises(gbrt.GbrtError, match="multiple of 16"):
        gbrt.tc_selftest(np.zeros((128, 8), np.float32), np.zeros((8, 8), np.float32))
    with pytest.raises(gbrt.GbrtError, match="multiple of 16"):
        gbrt.tc_selftest(a, np.zeros((80, 16), np.float32))


def test_photon_mapping_argument_checks(gbrt_lib):
    """Photon-mapping defaults are the reference's; argument errors are
    reported before any CUDA call."""
    from libyafaray_gb300 import gbrt
    p = gbrt.PmParams()
    assert gbrt_lib.gbrt_pm_default_params(ctypes.byref(p)) == 0
    assert (p.diffuse_photons, p.caustic_photons, p.diffuse_search, p.caustic_mix, p.caustic_depth, p.bounces) == (100000, 500000, 50, 50, 10, 3)
    assert abs(p.diffuse_radius - 0.1) < 1e-7 and abs(p.caustic_radius - 0.25) < 1e-7
    assert (p.caustics, p.diffuse, p.final_gather, p.fg_samples, p.fg_bounces) == (0, 1, 1, 32, 2)
    assert gbrt_lib.gbrt_pm_render(None, None, None, None, None, None, None, None) == -1
    with pytest.raises(gbrt.GbrtError, match="k in"):
        gbrt.knn_gather([[0, 0, 0]], [[0, 0, 0]], cell=0.1, k=65, r2=0.01)
    with pytest.raises(gbrt.GbrtError, match="below the search radius"):
        gbrt.knn_gather([[0, 0, 0]], [[0, 0, 0]], cell=0.05, k=8, r2=0.01)


def test_new_entry_points_reject_bad_arguments_before_cuda(gbrt_lib):
    """Adaptive AA, SPPM and texture entry points check their arguments on
    the host (NULL scene / parameters) and report them as errors."""
    L = gbrt_lib
    assert L.gbrt_pt_render_aa(None, None, None, None, None, None, None, None) == -1
    assert b"NULL" in L.gbrt_last_error()
    assert L.gbrt_pt_render_aa_host(None, None, None, None, None, None, None) == -1
    assert L.gbrt_aa_flags(None, None, 4, 4, None, 0.05, None, None) == -1
    assert L.gbrt_sppm_render(None, None, None, None, None, None, None) == -1
    assert L.gbrt_sppm_render_host(None, None, None, None, None, None) == -1
    assert L.gbrt_scene_set_textures(None, None, 0, None, None, 0, None, 0) == -1


def test_parameter_structs_follow_reference_names_and_defaults():
    """AA, SPPM and texture parameters parsed from scene dicts with the
    reference's parameter names and defaults."""
    a = gbrt.aa_params({})
    assert (a.passes, a.inc_samples, a.detect_color_noise, a.dark_detection_type, a.variance_edge_size,
            a.variance_pixels) == (1, 1, 0, 0, 10, 0)
    assert abs(a.threshold - 0.05) < 1e-7 and a.sample_multiplier_factor == 1.0
    a = gbrt.aa_params({"AA_passes": 3, "AA_dark_detection_type": "curve", "AA_detect_color_noise": True})
    assert (a.passes, a.dark_detection_type, a.detect_color_noise) == (3, 2, 1)
    sp = gbrt.sppm_params({"type": "SPPM"})
    assert (sp.photons, sp.passes, sp.bounces) == (500000, 1000, 5)
    import numpy as np
    d, img = gbrt.texture_desc({"image": np.zeros((4, 6, 4), np.float32)})
    assert (d.width, d.height, d.interpolate, d.clipping, d.texco, d.mapping) == (6, 4, 1, 3, 0, 0)
    assert list(d.proj) == [1, 2, 3] and list(d.scale) == [1.0, 1.0, 1.0] and list(d.crop) == [0.0, 0.0, 1.0, 1.0]


def test_uv_flattening_offsets_per_object_uvs():
    """flatten_uvs: object uvs are appended after a shared (0, 0) entry and
    each face's uv indices shifted by the object's offset; objects without
    uvs point at the shared entry."""
    import numpy as np
    from libyafaray_gb300 import scenes
    sc = scenes.textured_cornell_scene(res=16)
    uv, fuv = scenes.flatten_uvs(sc)
    verts, faces, _, _ = scenes.flatten(sc)
    assert len(fuv) == len(faces) and uv.shape[1] == 2
    back = [i for i, o in enumerate(sc["objects"]) if "uvs" in o]
    assert len(back) == 1
    start = sum(len(o["faces"]) for o in sc["objects"][:back[0]])
    n = len(sc["objects"][back[0]]["faces"])
    assert (fuv[start:start + n, :3] >= 1).all() and (fuv[:start] == 0).all()
    # the back wall's uvs span [0, 1] across it
    assert uv[1:].min() >= 0.0 and uv[1:].max() <= 1.0 + 1e-6


def test_reference_scene_text_carries_textures_nodes_and_aa():
    """The reference harness input holds images, textures, mapper nodes,
    uv meshes and AA film parameters in the harness's own syntax."""
    from libyafaray_gb300 import scenes
    from oracle import orc
    sc = scenes.textured_cornell_scene(res=16)
    sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5, "AA_passes": 3, "AA_detect_color_noise": True}
    text = orc.reference_scene_text(sc, 4, 2, 1, offset_stride=100)
    lines = text.splitlines()
    assert any(l.startswith("image checker_img 16 16") for l in lines)
    assert any(l.startswith("texture checker type=image image_name=checker_img") for l in lines)
    node = [l for l in lines if l.startswith("node name=back_tex_dtex")]
    assert node and "texco=uv" in node[0] and "proj_x=1" in node[0]
    assert any(l.startswith("material back_tex shinydiffusemat") and "diffuse_shader=back_tex_dtex" in l for l in lines)
    assert any(l.startswith("object back_wall back_tex 4 2 4") for l in lines)
    aa = [l for l in lines if l.startswith("aa ")]
    assert aa and "AA_passes=3" in aa[0] and "AA_detect_color_noise=true" in aa[0]
    assert lines[-1] == "render 4 2 1 100"
