"""Procedural textures on the host (gbrt_texture_eval, on_device 0) against
the compiled reference (tests/golden/procedural.npz, made by
tests/golden/make_golden.py procedural from oracle/_ref/noise_dump): every
texture type, noise generator, voronoi metric and colour mode, Musgrave
type, blend progression, colour-ramp mode and the colour adjustments, at
768 seeded points — getColor and getFloat bit for bit."""
import ctypes
import json
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "procedural.npz")


def golden():
    g = np.load(GOLD)
    tables = {k[len("table_"):]: g[k] for k in g.files if k.startswith("table_")}
    return g, tables, json.loads(str(g["cases"]))


def test_every_procedural_texture_matches_reference_bit_for_bit():
    gbrt.load()
    g, tables, cases = golden()
    pts = g["points"]
    for i, t in enumerate(cases):
        rgba, val = gbrt.texture_eval(t, tables, pts)
        assert np.array_equal(rgba.view(np.uint32), g[f"rgba_{i}"].view(np.uint32)), (i, t)
        assert np.array_equal(val.view(np.uint32), g[f"value_{i}"].view(np.uint32)), (i, t)
    assert len(cases) >= 50


def test_texture_eval_rejects_image_kind_and_long_ramps():
    gbrt.load()
    _, tables, _ = golden()
    nt, keep = gbrt.noise_tables(tables)
    pts = np.zeros((1, 3), np.float32)
    out, val = np.zeros((1, 4), np.float32), np.zeros(1, np.float32)
    d, img = gbrt.texture_desc({"type": "image", "image": np.zeros((2, 2, 4), np.float32)})
    with pytest.raises(gbrt.GbrtError):
        gbrt.check(gbrt.load().gbrt_texture_eval(ctypes.byref(d), ctypes.byref(nt), gbrt._ptr(pts), 1, gbrt._ptr(out), gbrt._ptr(val), 0))
    d, _ = gbrt.texture_desc({"type": "clouds"})
    d.proc.ramp_n = gbrt.RAMP_MAX + 1
    with pytest.raises(gbrt.GbrtError):
        gbrt.check(gbrt.load().gbrt_texture_eval(ctypes.byref(d), ctypes.byref(nt), gbrt._ptr(pts), 1, gbrt._ptr(out), gbrt._ptr(val), 0))
