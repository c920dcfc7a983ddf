"""The film oracle (oracle/film_oracle.py) pinned against the reference's own
sampler values, and properties of its splat."""
import os

import numpy as np

from oracle import film_oracle as fo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampler.npz")


def test_film_oracle_sampler_functions_match_reference():
    g = np.load(GOLD)
    idx = (np.arange(1024, dtype=np.uint64) * int(g["seq_index_mult"]) % (1 << 32)).astype(np.uint32)
    assert np.array_equal(fo.ri_lp(idx), g["lp"])
    assert np.array_equal(fo.fnv32a(idx), g["fnv"])
    got = fo._exp2(fo._log2(g["pow_base"]) * g["pow_exp"])
    assert np.array_equal(got.view(np.uint32), g["pow"].view(np.uint32))


def test_film_oracle_splat_properties():
    # box, width 1: a sample lands in its own pixel unless it lies within
    # 0.001 of the right / lower pixel edge
    w = fo.splat_weights(20, 15, 16, "box", 1.0)
    assert np.median(w) == 16.0 and w.min() >= 16.0 - 1e-9
    # one sample per pixel sits at the pixel centre: every filter gives the
    # same weight per interior pixel
    for kind in ("gauss", "mitchell", "box"):
        w1 = fo.splat_weights(12, 9, 1, kind, 1.5)
        inner = w1[1:-1, 1:-1]
        assert np.allclose(inner, inner[0, 0])
    # gauss 1.5: the reference's footprint is the sample's pixel and its right
    # and lower neighbours (asymmetric rounding), so column 0 only gets its
    # own samples' weights
    t, width, scale = fo.filter_table("gauss", 1.5)
    assert width == 1.5 and t[0, 0] > t[15, 15] >= 0.0
    w4 = fo.splat_weights(16, 12, 4, "gauss", 1.5)
    assert w4[:, 0].mean() < w4[:, 5].mean()
