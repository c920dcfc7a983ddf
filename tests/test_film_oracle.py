"""The film oracle (oracle/film_oracle.py) pinned against the reference's own
sampler values and adaptive-AA flags, and properties of its splat."""
import json
import os

import numpy as np

from oracle import film_oracle as fo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampler.npz")
AA_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "aa_flags.npz")


def aa_snapshots():
    """(film params, sums [H,W,4] with alpha = weight, weights, threshold,
    reference flags [H,W]) of every adaptive pass in aa_flags.npz."""
    g = np.load(AA_GOLD)
    for i in range(int(g["n_cases"])):
        film = json.loads(str(g[f"c{i}_film"]))
        j = 0
        while f"c{i}_p{j}_sums" in g:
            rgb, w = g[f"c{i}_p{j}_sums"], g[f"c{i}_p{j}_weights"]
            sums = np.concatenate([rgb, w[..., None]], axis=-1)
            flags = np.unpackbits(g[f"c{i}_p{j}_flags"])[:w.size].reshape(w.shape).astype(bool)
            yield film, sums, w, float(g[f"c{i}_p{j}_threshold"]), flags
            j += 1


def oracle_flags(film, sums, w, thr):
    return fo.aa_flags(sums, w, thr, film.get("AA_detect_color_noise", False), film.get("AA_dark_detection_type", "none"),
                       film.get("AA_dark_threshold_factor", 0.0), film.get("AA_variance_edge_size", 10),
                       film.get("AA_variance_pixels", 0))


def test_aa_flags_oracle_matches_reference():
    n = 0
    kinds = set()
    for film, sums, w, thr, ref in aa_snapshots():
        got = oracle_flags(film, sums, w, thr)
        assert np.array_equal(got, ref), (film, int((got != ref).sum()))
        assert 0 < ref.sum() < ref.size      # every snapshot discriminates
        kinds.add(film.get("AA_dark_detection_type", "none"))
        n += 1
    assert n >= 10 and kinds == {"none", "linear", "curve"}


def test_aa_flags_oracle_edge_cases():
    # no samples -> flagged; a flat film -> nothing flagged; a single row or
    # column has no neighbour pairs
    w = np.ones((6, 8), np.float32)
    sums = np.concatenate([np.full((6, 8, 3), 0.5, np.float32), w[..., None]], -1)
    assert not fo.aa_flags(sums, w, 0.05).any()
    w2 = w.copy()
    w2[2, 3] = 0
    f = fo.aa_flags(sums * w2[..., None], w2, 0.05)
    # the empty pixel itself and the neighbours whose difference to it (0 vs 0.5) counts
    assert f[2, 3] and f.sum() > 1
    assert fo.aa_flags(sums[:1], w[:1], 0.05).sum() == 0
    # a step edge flags both sides; the variance window widens it
    s2 = sums.copy()
    s2[:, 4:, :3] = 2.0
    f = fo.aa_flags(s2, w, 0.05)
    assert f[:, 3].all() and f[:, 4].all() and not f[:, 0].any()
    fv = fo.aa_flags(s2, w, 0.05, variance_edge_size=4, variance_pixels=1)
    assert fv.sum() > f.sum()
    # dark curve knots
    assert fo.dark_curve(np.float32(0.05)) == np.float32(0.0001)
    assert fo.dark_curve(np.float32(5.0)) == np.float32(0.1)


def test_film_oracle_sampler_functions_match_reference():
    g = np.load(GOLD)
    idx = (np.arange(1024, dtype=np.uint64) * int(g["seq_index_mult"]) % (1 << 32)).astype(np.uint32)
    assert np.array_equal(fo.ri_lp(idx), g["lp"])
    assert np.array_equal(fo.ri_vdc(idx), g["vdc"])
    assert np.array_equal(fo.ri_s(idx), g["s"])
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
