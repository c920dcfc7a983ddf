"""The reference-side binding (oracle/ref/gb300_binding.cc): the scene, the
integrator parameters and the film parameters a libYafaRay build hands to the
GPU library through gb300::translate / pt_params / film_params must be what
this package's host API (scenes.flatten, gbrt._material_desc,
Renderer.params) hands it for the same scene, so the parity the GPU tests
prove through the host API holds for the reference's own C API too.

The binding is compiled against the reference's sources (oracle/_ref/
binding_dump); these tests run where that harness was built and skip
elsewhere.  They need no GPU: the reference builds the scene, the binding
translates it, and the translation is compared field by field."""
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes
from oracle import orc

pytestmark = pytest.mark.skipif(not orc.binding_available(), reason="reference binding harness not built here")

TRI = 0xFFFFFFFF


def _corners(vertices, faces):
    """Per face its 4 corner positions (the 4th NaN for a triangle)."""
    v = np.asarray(vertices, np.float32)
    f = np.asarray(faces, np.uint32)
    out = np.full((len(f), 4, 3), np.nan, np.float32)
    out[:, :3] = v[f[:, :3]]
    quad = f[:, 3] != TRI
    out[quad, 3] = v[f[quad, 3]]
    return out


def _fields(s):
    vals = []
    for name, _ in s._fields_:
        x = getattr(s, name)
        vals.extend(list(x) if hasattr(x, "__len__") else [x])
    return np.array(vals, np.float64)


def _geometric_normals(corners):
    e1 = corners[:, 1] - corners[:, 0]
    e2 = corners[:, 2] - corners[:, 0]
    n = np.cross(e1, e2).astype(np.float32)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def _check_translation(sc, spp=2):
    tr = orc.run_reference_translation(sc, spp)
    assert tr["ok"], tr["error"]
    v, f, fm, names = scenes.flatten(sc)
    # faces in the reference's primitive order with the same corners
    assert len(tr["faces"]) == len(f)
    assert np.array_equal(tr["faces"][:, 3] == TRI, f[:, 3] == TRI)
    np.testing.assert_array_equal(_corners(tr["vertices"], tr["faces"]), _corners(v, f))
    # every face's material description, field by field
    host = [_fields(gbrt._material_desc(sc["materials"][n])) for n in names]
    ref = [_fields(m) for m in tr["materials"]]
    for i in range(len(f)):
        np.testing.assert_array_equal(ref[tr["face_material"][i]], host[fm[i]], err_msg=f"face {i}")
    # lights in the same order (the light selection index)
    r = gbrt.Renderer.__new__(gbrt.Renderer)
    r.scene = sc
    assert len(tr["lights"]) == len(sc["lights"])
    for i, L in enumerate(sc["lights"]):
        got = tr["lights"][i]
        if L["type"] == "arealight":
            exp = [0, *L["corner"], *L["point1"], *L["point2"], *L["color"], L["power"], L["samples"]]
        else:
            exp = [1, *L["from"], 0, 0, 0, 0, 0, 0, *L["color"], L["power"], 1]
        np.testing.assert_array_equal(_fields(got), np.array(exp, np.float32).astype(np.float64), err_msg=f"light {i}")
    # camera
    np.testing.assert_array_equal(_fields(tr["camera"]), _fields(r.camera_desc()))
    # integrator parameters
    r._caustic = None
    p = r.params(spp)
    got = tr["params"]
    for name in ("spp", "path_samples", "bounces", "russian_roulette_min_bounces", "base_sampling_offset", "raydepth",
                 "transparent_shadows", "shadow_depth", "caustic_type", "no_recursive", "clamp_indirect"):
        assert getattr(got, name) == getattr(p, name), name
    film = sc.get("film", {})
    if film.get("filter_type", "pixel") == "pixel":
        # the single-pixel splat reaches the reference as its box filter of width 1
        assert (got.filter_type, got.aa_pixel_width) == (gbrt.FILTERS["box"], 1.0)
    else:
        assert got.filter_type == p.filter_type and got.aa_pixel_width == np.float32(film.get("AA_pixelwidth", 1.5))
    np.testing.assert_array_equal(_fields(tr["aa"]), _fields(gbrt.aa_params(film)))
    if p.caustic_type in (2, 3):
        c, exp = tr["caustic"], gbrt.pm_params(sc["integrator"])
        for name in ("caustic_photons", "caustic_radius", "caustic_mix", "caustic_depth"):
            assert getattr(c, name) == getattr(exp, name), name
    return tr, (v, f)


@pytest.mark.parametrize("kw", [{}, {"glossy": True}, {"glass": True}, {"point_light": True}, {"shiny": True},
                                {"transparent_shadows": 4}],
                         ids=["cornell", "glossy", "glass", "pointlight", "shiny", "tshadow"])
def test_cornell_translation_matches_host_api(kw):
    _check_translation(scenes.cornell_scene(res=16, **kw))


@pytest.mark.parametrize("kw", [{"caustic_type": "photon"}, {"caustic_type": "both", "clamp_indirect": 2.0},
                                {"no_recursive": True}, {"caustic_type": "none"}],
                         ids=["photon", "both_clamp", "norec", "none"])
def test_pathtracing_options_translate(kw):
    _check_translation(scenes.cornell_pt_variant_scene(res=16, caustic_photons=1000, **kw))


@pytest.mark.parametrize("i", [5, 26])
def test_batch_scene_translation(i):
    _check_translation(scenes.batch_scene(i, res=16))


def test_film_parameters_translate():
    sc = scenes.cornell_scene(res=16)
    sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5, "AA_passes": 3, "AA_inc_samples": 2,
                  "AA_threshold": 0.03, "AA_resampled_floor": 5.0, "AA_dark_detection_type": "linear",
                  "AA_dark_threshold_factor": 0.2, "AA_variance_edge_size": 8, "AA_variance_pixels": 2,
                  "AA_detect_color_noise": True}
    _check_translation(sc)


def test_smooth_normals_translate():
    """Smoothed meshes: every face corner of a smoothed object carries the
    reference's vertex normal where smoothing gave one (equal to the host
    API's gbrt_mesh_smooth_normals result) and the face's geometric normal
    elsewhere; flat objects stay flat."""
    sc = scenes.smooth_cornell_scene(res=16)
    tr, (v, f) = _check_translation(sc)
    hn, hfn, base = [], [], 0
    smooth_face = []
    for o in sc["objects"]:
        ov = np.asarray(o["vertices"], np.float32)
        of = np.asarray(o["faces"], np.uint32)
        if "smooth" in o:
            n, fn = gbrt.smooth_normals(ov, of, float(o["smooth"]))
            fn = fn.copy()
            live = fn != gbrt.NO_NORMAL
            fn[live] += base
            hn.append(n)
            base += len(n)
            smooth_face.append(np.ones(len(of), bool))
        else:
            fn = np.full((len(of), 4), gbrt.FLAT_FACE, np.uint32)
            smooth_face.append(np.zeros(len(of), bool))
        hfn.append(fn)
    hn = np.concatenate(hn)
    hfn = np.concatenate(hfn)
    smooth_face = np.concatenate(smooth_face)
    rfn, rn = tr["face_normals"], tr["normals"]
    assert np.array_equal(rfn[~smooth_face] == gbrt.FLAT_FACE, np.ones_like(rfn[~smooth_face], bool))
    corners = _corners(v, f)
    ng = _geometric_normals(corners)
    tri = f[:, 3] == TRI
    checked = 0
    for i in np.nonzero(smooth_face)[0]:
        for k in range(3 if tri[i] else 4):
            got = rn[rfn[i, k]]
            if hfn[i, k] != gbrt.NO_NORMAL:
                np.testing.assert_array_equal(got, hn[hfn[i, k]], err_msg=f"face {i} corner {k}")
            else:
                np.testing.assert_allclose(got, ng[i], atol=2e-6, err_msg=f"face {i} corner {k}")
            checked += 1
        if tri[i]:
            assert rfn[i, 3] == gbrt.NO_NORMAL
    assert checked > 1000


def test_binding_refuses_what_the_gpu_does_not_build():
    """A textured material (a shader node) is refused with a message, not
    rendered without its texture."""
    tr = orc.run_reference_translation(scenes.textured_cornell_scene(res=16))
    assert not tr["ok"] and "shader node" in tr["error"]


def test_gpu_integrator_fails_cleanly_without_a_device():
    """PathIntegratorGb300 in the reference's render loop on a host without a
    GPU: the library's error reaches the integrator, which reports the
    render as failed; the process ends normally with an empty film."""
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    text = orc.reference_scene_text(scenes.cornell_scene(res=8), 1, 1)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "scene.txt"), os.path.join(d, "out.bin")
        open(fin, "w").write(text)
        env = dict(os.environ, GB300_INTEGRATOR="1")
        r = subprocess.run([orc.REF_BINDING, fin, fout], env=env, stdout=subprocess.DEVNULL, timeout=120)
        assert r.returncode == 0
        raw = open(fout, "rb").read()
    K, H, W = struct.unpack("<iii", raw[:12])
    img = np.frombuffer(raw[12 + 8 * K:], np.float32)
    assert (K, H, W) == (1, 8, 8) and not img.any()
