"""The GPU render of scenes as the reference-side binding translates them
(tests/golden/binding_translation.npz, made by tests/golden/make_golden.py
binding from oracle/ref/gb300_binding.cc): built and rendered through the
same C-ABI calls PathIntegratorGb300::render makes (gbrt_bvh_build_host,
gbrt_scene_create, gbrt_scene_set_normals, gbrt_pt_render_aa_host), the image
must be the one this package's host API renders for the same scene, whose
parity with the reference the render tests establish.  The binding gives
every face its own vertices and puts the reference's default material first;
neither may change a pixel beyond float-summation order."""
import ctypes
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "binding_translation.npz")

# the scenes of tests/golden/make_golden.py BINDING_CASES, for the host API
CASES = {
    "smooth": lambda: scenes.smooth_cornell_scene(res=48),
    "pt_photon": lambda: scenes.cornell_pt_variant_scene(res=48, caustic_type="both", clamp_indirect=2.0),
}


def _struct(cls, raw):
    return cls.from_buffer_copy(np.asarray(raw, np.uint8).tobytes())


def _structs(cls, raw):
    b = np.asarray(raw, np.uint8).tobytes()
    n = len(b) // ctypes.sizeof(cls)
    arr = (cls * max(1, n))()
    ctypes.memmove(arr, b, len(b))
    return arr, n


def _render_translated(g, name):
    L = gbrt.load()
    v = np.ascontiguousarray(g[f"{name}_vertices"], np.float32)
    f = np.ascontiguousarray(g[f"{name}_faces"], np.uint32)
    fm = np.ascontiguousarray(g[f"{name}_face_material"], np.int32)
    mats, nm = _structs(gbrt.MaterialDesc, g[f"{name}_materials"])
    lights, nl = _structs(gbrt.LightDesc, g[f"{name}_lights"])
    bvh = gbrt.Bvh.build_host(v, f)
    h = ctypes.c_void_p()
    gbrt.check(L.gbrt_scene_create(bvh.handle, gbrt._ptr(v), len(v), gbrt._ptr(f), len(f), gbrt._ptr(fm), mats, nm, lights,
                                   nl, ctypes.byref(h)))
    try:
        if f"{name}_normals" in g:
            n = np.ascontiguousarray(g[f"{name}_normals"], np.float32)
            fn = np.ascontiguousarray(g[f"{name}_face_normals"], np.uint32)
            gbrt.check(L.gbrt_scene_set_normals(h, gbrt._ptr(n), len(n), gbrt._ptr(fn)))
        cam = _struct(gbrt.CameraDesc, g[f"{name}_camera"])
        p = _struct(gbrt.PtParams, g[f"{name}_params"])
        caustic = _struct(gbrt.PmParams, g[f"{name}_caustic"])
        p.guide = None
        p.film_weight_dev = None
        p.caustic = ctypes.addressof(caustic) if p.caustic_type in (2, 3) else None
        aa = _struct(gbrt.AaParams, g[f"{name}_aa"])
        img = np.empty((cam.resy, cam.resx, 3), np.float32)
        st = gbrt.PtStats()
        gbrt.check(L.gbrt_pt_render_aa_host(h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(aa), gbrt._ptr(img),
                                            ctypes.byref(st), None))
        return img, p
    finally:
        L.gbrt_scene_destroy(h)
        bvh.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_binding_translation_renders_like_host_api(name):
    g = dict(np.load(GOLD))
    img, p = _render_translated(g, name)
    sc = CASES[name]()
    film = dict(sc.get("film", {}))
    # the film the reference hands over: its box filter of width 1
    film.update({"filter_type": "box", "AA_pixelwidth": 1.0})
    sc["film"] = film
    ref, _, _ = gbrt.Renderer(sc).render_aa(spp=p.spp)
    assert np.isfinite(img).all() and img.mean() > 0.01
    np.testing.assert_allclose(img, ref, rtol=2e-5, atol=1e-6)
