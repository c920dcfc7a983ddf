"""Photon mapping on the GPU against the reference.

- k-nearest gather (PhotonMap::gather semantics: at most k photons with
  d^2 < r^2, the radius shrinking to the k-th distance) through the device
  grid equals a brute-force float32 search: same counts, same final r^2
  (bit for bit) and the same photon sets.
- Photon maps: the diffuse and caustic maps the GPU shoots for Halton
  indices 0 .. n-1 against the reference's maps (threads_photons 1), compared
  as multisets of (dir, pos, colour): the same number of photons, every one
  bit-identical; at full size (10M + 10M paths, 200,000-triangle sphere) as
  bucketed digests of the multisets.
- photonmapping renders, without and with final gather, against the
  reference renderer: per-pixel means within 3 combined standard errors."""
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def brute_knn(P, q, k, r2):
    v = (P - q).astype(np.float32)
    d = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    cand = np.nonzero(d < np.float32(r2))[0]
    if len(cand) < k:
        return len(cand), np.float32(r2), set(cand.tolist())
    order = cand[np.argsort(d[cand], kind="stable")]
    sel = order[:k]
    return k, d[sel].max(), set(sel.tolist())


@pytest.mark.parametrize("k,r2", [(50, 0.0025), (8, 0.01), (64, 0.0004)])
def test_knn_gather_matches_brute_force(cuda_device, k, r2):
    rng = np.random.default_rng(k)
    P = np.concatenate([rng.uniform(0, 1, (15000, 3)), rng.normal(0.5, 0.02, (5000, 3))]).astype(np.float32)
    P[:2000, 1] = 0.25                                    # a plane of coplanar photons
    Q = np.concatenate([rng.uniform(0, 1, (300, 3)), rng.normal(0.5, 0.02, (100, 3)), P[:100]]).astype(np.float32)
    cnt, rr, idx = gbrt.knn_gather(P, Q, cell=float(np.sqrt(r2)), k=k, r2=r2)
    bad = 0
    for i in range(len(Q)):
        c, r, s = brute_knn(P, Q[i], k, r2)
        got = set(idx[i, :cnt[i]].tolist())
        ties = False
        if c == k and got != s:
            # exactly equal distances at the k-th place may swap members
            v = (P - Q[i]).astype(np.float32)
            d = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
            ties = np.count_nonzero(d == r) > 1
        if cnt[i] != c or rr[i] != r or (got != s and not ties):
            bad += 1
    assert bad == 0, f"{bad} of {len(Q)} queries differ"


def match_photons(a, b):
    """Fraction of rows of a with a bit-identical row in b (multiset)."""
    ka = [r.tobytes() for r in np.ascontiguousarray(a)]
    kb = {}
    for r in np.ascontiguousarray(b):
        kb[r.tobytes()] = kb.get(r.tobytes(), 0) + 1
    hit = 0
    for x in ka:
        if kb.get(x, 0):
            kb[x] -= 1
            hit += 1
    return hit / max(1, len(ka))


def test_photon_maps_match_reference(cuda_device):
    g = np.load(os.path.join(GOLD, "photons_small.npz"))
    sc = scenes.caustic_scene(res=32, subdiv=3, diffuse_photons=20000, caustic_photons=20000, final_gather=False)
    r = gbrt.Renderer(sc)
    for which in ("diffuse", "caustic"):
        ph, paths = r.photons(which)
        ref = g[which]
        assert paths == int(g[f"{which}_paths"])
        exact = match_photons(ref, ph)
        print(f"{which}: gpu {len(ph)} photons, reference {len(ref)}; {100 * exact:.2f}% bit-identical")
        assert len(ph) == len(ref)
        assert exact == 1.0


def test_full_size_photon_maps_match_reference(cuda_device):
    """The photon-mapping configuration at full size: 200,000-triangle
    geodesic glass sphere, 10M diffuse + 10M caustic photon paths.  The
    photon and path counts equal the reference's, and the maps agree as
    multisets: a 4096-bucket digest (count and hash sum per bucket) of each
    map equals the reference's bucket for bucket.  A bucket that differs
    holds at least one photon that differs; those are counted and printed."""
    from tests.parity import photon_buckets
    g = np.load(os.path.join(GOLD, "pm_full_maps.npz"))
    sc = scenes.caustic_scene(res=32, geodesic=100, diffuse_photons=10_000_000, caustic_photons=10_000_000,
                              final_gather=False, radius=0.02, search=50)
    r = gbrt.Renderer(sc)
    for which in ("diffuse", "caustic"):
        ph, paths = r.photons(which)
        counts, sums = photon_buckets(ph)
        differ = int(np.count_nonzero((counts != g[f"{which}_counts"]) | (sums != g[f"{which}_sums"])))
        print(f"full-size {which} map: gpu {len(ph)} photons / {paths} paths, reference {int(g[f'{which}_n'])} / "
              f"{int(g[f'{which}_paths'])}; {differ} of 4096 digest buckets differ")
        assert paths == int(g[f"{which}_paths"])
        assert len(ph) == int(g[f"{which}_n"])
        assert differ == 0


# the reference renders these goldens through its box filter of width 1
# (render_dump's film): a sample within 0.001 of a pixel edge also lands in
# the neighbouring pixel, which the single-pixel GPU film does not do
BOX_FILM = {"filter_type": "box", "AA_pixelwidth": 1.0}


def pm_parity(gpu_batches, ref_mean, ref_se, rel_float=1e-5):
    """Per-pixel means within 3 combined standard errors.  The photon maps
    and the sample positions are the same in every batch, so where the
    estimate is smooth a pixel's batch spread falls to float rounding; the
    combined SE therefore carries a float term, rel_float x |mean| (the
    photon terms of a gather, up to 64, and the 8 samples of a pixel are
    summed in another order than the reference's).  Returns (fraction
    agreeing, relMSE, mean, channels that agree only through the float
    term)."""
    k = len(gpu_batches)
    m = gpu_batches.mean(0)
    se = gpu_batches.std(0, ddof=1) / np.sqrt(k)
    d = np.abs(m - ref_mean)
    stat = np.sqrt(se ** 2 + ref_se ** 2)
    comb = np.sqrt(stat ** 2 + (rel_float * np.abs(ref_mean)) ** 2)
    ok = d <= 3.0 * comb
    relmse = float(np.mean((m - ref_mean) ** 2 / (ref_mean ** 2 + 1e-2)))
    return float(np.mean(ok)), relmse, m, int(np.count_nonzero(ok & (d > 3.0 * stat)))


def batch_agreement(gpu_batch, ref_batch, rel=1e-4):
    """Fraction of pixel channels of one batch equal to the reference's same
    batch within rel (relative, floor 1e-3), and the positions of the rest."""
    d = np.abs(gpu_batch - ref_batch)
    ok = d <= rel * np.maximum(np.abs(ref_batch), 1e-3)
    return float(np.mean(ok)), np.argwhere(~ok)


def render_batches(r, spp, k):
    return np.stack([r.render(spp, base_offset=b * spp, seed=300 + b)[0] for b in range(k)])


def test_area_light_photon_map_matches_reference(cuda_device):
    """Diffuse photons of the Cornell box's area light (AreaLight::emitPhoton
    with its unnormalised emission frame, light_area.cc:126-133)."""
    g = np.load(os.path.join(GOLD, "photons_cornell.npz"))
    r = gbrt.Renderer(scenes.cornell_pm_scene(16, False, diffuse_photons=5000))
    ph, paths = r.photons("diffuse")
    exact = match_photons(g["diffuse"], ph)
    print(f"cornell diffuse photons: gpu {len(ph)}, reference {len(g['diffuse'])}; {100 * exact:.2f}% bit-identical")
    assert paths == int(g["diffuse_paths"])
    assert len(ph) == len(g["diffuse"])
    assert exact == 1.0


def _pm_check(name, sc, fg):
    g = np.load(os.path.join(GOLD, name))
    sc["film"] = dict(BOX_FILM)
    r = gbrt.Renderer(sc)
    gb = render_batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m, n_float = pm_parity(gb, g["mean"], g["se"])
    print(f"{name}: {100 * frac:.2f}% of pixel channels within 3 SE ({n_float} through the float term), relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995
    if not fg:
        # batch by batch: the same photon maps and sample positions give the
        # reference's pixel values to float rounding
        for b in range(2):
            agree, rest = batch_agreement(gb[b], g["batch01"][b])
            print(f"  batch {b}: {100 * agree:.3f}% of pixel channels equal the reference's within 1e-4; "
                  f"others at {rest[:8].tolist()}")
            assert agree >= 0.999


@pytest.mark.parametrize("fg", [False, True])
def test_photonmapping_caustic_scene_matches_reference(cuda_device, fg):
    """Glass ball on a plane under a pointlight: caustic map (kernel
    estimate), diffuse map (direct estimate or pre-gathered radiance map),
    specular split through the ball.  Without final gather each batch also
    equals the reference's same batch pixel by pixel."""
    _pm_check(f"pm_{'fg' if fg else 'direct'}_48_render.npz", scenes.caustic_scene_small(fg), fg)


@pytest.mark.parametrize("fg", [False, True])
def test_photonmapping_cornell_matches_reference(cuda_device, fg):
    """The Cornell box with photonmapping: area-light photons (unnormalised
    emission frame), emission counted twice, direct photon estimate or final
    gathering over the radiance map (thinned radiance points, pre-gather)."""
    _pm_check(f"cornell_pm_{'fg' if fg else 'direct'}_48_render.npz", scenes.cornell_pm_scene(48, fg), fg)


def test_directlighting_caustics_matches_reference(cuda_device):
    """directlighting on the glass Cornell box: emission, all-light
    estimation, the recursive split through the glass and rough-glass balls,
    and the caustic photon map (glossy and specular photon paths)."""
    g = np.load(os.path.join(GOLD, "cornell_dl_48_render.npz"))
    sc = scenes.cornell_dl_scene(48)
    sc["film"] = dict(BOX_FILM)
    r = gbrt.Renderer(sc)
    gb = render_batches(r, int(g["spp"]), int(g["batches"]))
    frac, relmse, m, n_float = pm_parity(gb, g["mean"], g["se"])
    print(f"directlighting glass cornell 48x48: {100 * frac:.2f}% agree ({n_float} through the float term), relMSE {relmse:.3g}, "
          f"means gpu {m.mean(axis=(0, 1))} ref {g['mean'].mean(axis=(0, 1))}")
    assert frac >= 0.995


def test_grid_cell_assignment_matches_reference_hashgrid(cuda_device):
    """The photon grid puts every photon in the bucket the reference's
    HashGrid::updateGrid puts it (cell coordinates and hash, bit for bit)."""
    g = np.load(os.path.join(GOLD, "hashgrid.npz"))
    for i in range(3):
        got = gbrt.grid_buckets(g["pos"], float(g[f"cell{i}"]), int(g[f"size{i}"]), g["lo"])
        assert np.array_equal(got, g[f"bucket{i}"]), f"case {i}: {np.count_nonzero(got != g[f'bucket{i}'])} photons differ"
