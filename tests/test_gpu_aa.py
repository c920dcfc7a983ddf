"""Adaptive anti-aliasing on the GPU (TiledIntegrator::render's passes,
integrator_tiled.cc:160-214, and ImageFilm::nextPass, imagefilm.cc:365-547):
the resample flags of the detection kernels equal the reference's on the
reference's own film states, a pass schedule that resamples every pixel
splats exactly the oracle's multipass weights, and an adaptive render agrees
with the compiled reference's."""
import json
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes
from oracle import film_oracle as fo
from tests.test_film_oracle import aa_snapshots
from tests.test_gpu_render import parity

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_gpu_aa_flags_match_reference(cuda_device):
    import torch
    n = 0
    for film, sums, w, thr, ref in aa_snapshots():
        H, W = w.shape
        f = torch.from_numpy(np.ascontiguousarray(sums[..., :3])).reshape(-1).cuda()
        wt = torch.from_numpy(np.ascontiguousarray(w)).reshape(-1).cuda()
        flags = torch.zeros(H * W, dtype=torch.uint8, device="cuda")
        cnt = gbrt.aa_flags(f.data_ptr(), wt.data_ptr(), W, H, gbrt.aa_params(film), thr, flags.data_ptr())
        got = flags.cpu().numpy().reshape(H, W).astype(bool)
        assert np.array_equal(got, ref), (film, int((got != ref).sum()))
        assert cnt == int(ref.sum())
        n += 1
    assert n >= 10


def test_gpu_aa_flags_edge_cases(cuda_device):
    import torch
    aa = gbrt.aa_params({})
    for H, W in ((1, 7), (5, 1), (1, 1), (3, 2)):
        w = np.ones((H, W), np.float32)
        w[0, 0] = 0.0
        f = torch.zeros(H * W * 3, dtype=torch.float32, device="cuda")
        wt = torch.from_numpy(w.reshape(-1)).cuda()
        flags = torch.full((H * W,), 7, dtype=torch.uint8, device="cuda")
        cnt = gbrt.aa_flags(f.data_ptr(), wt.data_ptr(), W, H, aa, 0.05, flags.data_ptr())
        sums = np.zeros((H, W, 4), np.float32)
        sums[..., 3] = w
        exp = fo.aa_flags(sums, w, 0.05)
        assert np.array_equal(flags.cpu().numpy().reshape(H, W).astype(bool), exp) and cnt == int(exp.sum())


def _cornell(resx, resy, film):
    sc = scenes.cornell_scene(res=resx)
    sc["camera"]["resy"] = resy
    sc["film"] = film
    return gbrt.Renderer(sc)


@pytest.mark.parametrize("kind,passes,inc,smult", [("gauss", 3, 2, 1.5), ("box", 4, 1, 1.0)])
def test_gpu_aa_every_pixel_passes_match_oracle_weights(cuda_device, kind, passes, inc, smult):
    # AA_threshold 0: every pass resamples every pixel, at sample offsets
    # base + samples so far, with riVdC / riS positions
    import torch
    resx, resy, spp, base = 24, 18, 3, 40
    film = {"filter_type": kind, "AA_pixelwidth": 1.5, "AA_passes": passes, "AA_inc_samples": inc,
            "AA_threshold": 0.0, "AA_sample_multiplier_factor": smult}
    r = _cornell(resx, resy, film)
    f = torch.zeros(resx * resy * 3, dtype=torch.float32, device="cuda")
    w = torch.zeros(resx * resy, dtype=torch.float32, device="cuda")
    res = r.render_aa_device(f.data_ptr(), w.data_ptr(), spp=spp, base_offset=base)
    torch.cuda.synchronize()
    assert res == [resx * resy] * passes
    exp = fo.splat_weights(resx, resy, spp, kind, 1.5, multipass=True, pass_offset=base)
    acum, mult_f = spp, 1.0
    for _ in range(1, passes):
        mult_f = np.float32(mult_f) * np.float32(smult)
        m = int(np.ceil(np.float32(inc) * mult_f))
        exp += fo.splat_weights(resx, resy, m, kind, 1.5, multipass=True, pass_offset=base + acum)
        acum += m
    got = w.cpu().numpy().reshape(resy, resx).astype(np.float64)
    assert np.allclose(got, exp, rtol=1e-5, atol=1e-5), float(np.abs(got - exp).max())


def test_gpu_aa_render_vs_reference(cuda_device):
    g = np.load(os.path.join(GOLD, "cornell_aa_48x36_render.npz"))
    film = json.loads(str(g["film"]))
    r = _cornell(48, 36, film)
    k, spp, stride = int(g["batches"]), int(g["spp"]), int(g["stride"])
    imgs, flagged = [], []
    for b in range(k):
        img, _, res = r.render_aa(spp=spp, base_offset=b * stride, seed=1000 + b)
        imgs.append(img)
        flagged.append(res[1:])
    frac, relmse, _ = parity(np.stack(imgs), g["mean"], g["se"])
    print(f"cornell adaptive AA 48x36: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}; "
          f"flagged per pass {np.mean(flagged, 0).round(1).tolist()} (reference batch 0: {g['flagged'].tolist()})")
    assert frac >= 0.995
    # the flagged counts of the reference's batch 0 against the mean of ours
    assert np.allclose(np.mean(flagged, 0), g["flagged"], rtol=0.15)


def test_gpu_aa_needs_a_filtered_film(cuda_device):
    r = _cornell(16, 12, {"filter_type": "pixel", "AA_passes": 2})
    with pytest.raises(gbrt.GbrtError):
        r.render_aa(spp=2)
    r2 = _cornell(16, 12, {"filter_type": "gauss", "AA_passes": 0})
    with pytest.raises(gbrt.GbrtError):
        r2.render_aa(spp=2)


@pytest.mark.parametrize("name,kind", [("cornell_pm_aa_48_render.npz", "pm"), ("cornell_dl_aa_48_render.npz", "dl")])
def test_gpu_aa_photon_integrators_vs_reference(cuda_device, name, kind):
    """The adaptive passes over the photonmapping (direct estimate) and
    directlighting integrators, photon maps built once per render."""
    g = np.load(os.path.join(GOLD, name))
    sc = scenes.cornell_pm_scene(48, False) if kind == "pm" else scenes.cornell_dl_scene(48)
    sc["film"] = json.loads(str(g["film"]))
    r = gbrt.Renderer(sc)
    k, spp, stride = int(g["batches"]), int(g["spp"]), int(g["stride"])
    imgs, flagged = [], []
    for b in range(k):
        img, _, res = r.render_aa(spp=spp, base_offset=b * stride, seed=1000 + b)
        imgs.append(img)
        flagged.append(res[1:])
    frac, relmse, _ = parity(np.stack(imgs), g["mean"], g["se"])
    print(f"{name}: {100 * frac:.2f}% within 3 SE, relMSE {relmse:.3g}; flagged {np.mean(flagged, 0).round(1).tolist()} "
          f"(reference batch 0: {g['flagged'].tolist()})")
    assert frac >= 0.995
