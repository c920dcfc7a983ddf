"""The oracle (CPU restatement, oracle/traverse_oracle.c) against golden
vectors produced by the reference kd-tree itself (tests/golden/)."""
import glob
import os

import numpy as np
import pytest

from oracle import orc
from tests import parity

TRAVERSAL_CASES = ["cornell_quads", "cornell_tris", "single_tri", "tri_soup_4k", "tri_soup_dense", "perlin_sphere_16k"]
GOLDEN = [os.path.join(os.path.dirname(__file__), "golden", n + ".npz") for n in TRAVERSAL_CASES]


def test_golden_present():
    names = {os.path.basename(g) for g in GOLDEN}
    assert {"tri_soup_4k.npz", "tri_soup_dense.npz", "cornell_quads.npz", "cornell_tris.npz", "single_tri.npz"} <= names


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_closest_matches_reference(path):
    g = np.load(path)
    s = orc.OracleScene(g["vertices"], g["faces"])
    assert np.array_equal(s.bound(), g["bound"]), "tree bound differs from Accelerator::getBound"
    got = s.trace(g["rays"], 0)
    ref = (g["closest_prim"], g["closest_t"], g["closest_u"], g["closest_v"])
    r = parity.compare_closest(g["vertices"], g["faces"], g["rays"], got, ref)
    print(os.path.basename(path), r["mismatch"], "mismatches:", r["edge"], "on edges,", r["tie"], "exact ties")
    assert not r["bad"], f"unexplained ID mismatches at rays {r['bad'][:10]}"
    assert r["t_exact"] and r["uv_ok"]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_shadow_matches_reference(path):
    g = np.load(path)
    s = orc.OracleScene(g["vertices"], g["faces"])
    occ, _, _, _ = s.trace(g["rays"], 1)
    r = parity.compare_shadow(g["vertices"], g["faces"], g["rays"], occ, g["shadow_hit"])
    assert not r["bad"], f"unexplained shadow mismatches at rays {r['bad'][:10]}"


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_bvh_equals_bruteforce(path):
    g = np.load(path)
    s = orc.OracleScene(g["vertices"], g["faces"])
    a = s.trace(g["rays"], 0, bruteforce=False)
    b = s.trace(g["rays"], 0, bruteforce=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_mt_quad_uv_remap():
    # shape_polygon.h:148-149,169: quads report (u+v, v) / (u, u+v)
    q = np.array([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0], np.float32)
    import ctypes
    L = orc.lib()
    fp = ctypes.POINTER(ctypes.c_float)
    u, v = ctypes.c_float(), ctypes.c_float()
    for (x, y) in [(0.7, 0.2), (0.2, 0.7)]:
        o = np.array([x, y, 1.0], np.float32)
        d = np.array([0, 0, -1.0], np.float32)
        t = L.orc_mt_intersect(q.ctypes.data_as(fp), 4, o.ctypes.data_as(fp), d.ctypes.data_as(fp), ctypes.byref(u), ctypes.byref(v))
        assert t == 1.0
        assert abs(u.value - x) < 1e-6 and abs(v.value - y) < 1e-6


@pytest.mark.skipif(not orc.reference_available(), reason="reference kd-tree harness not built here")
def test_oracle_against_live_reference_random():
    from libyafaray_gb300 import scenes
    v, f = scenes.random_triangles(20000, seed=21, spread=0.03)
    r = scenes.random_rays(20000, seed=22)
    b, _, _, p, t, u, vv = orc.run_reference_kdtree(v, f, r, 0)
    s = orc.OracleScene(v, f)
    res = parity.compare_closest(v, f, r, s.trace(r, 0), (p, t, u, vv))
    assert not res["bad"] and res["t_exact"]
