"""The reference's image-film filter on the GPU (ImageFilm::addSample and
flush, imagefilm.cc:231-264, 771-822): the weight image of a render equals
the film oracle's (every camera sample splatted with the reference's
footprint and filter table), and a Gaussian-film render agrees with the
compiled reference's."""
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes
from oracle import film_oracle as fo
from tests.test_gpu_render import parity

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cornell(resx, resy, kind, width):
    sc = scenes.cornell_scene(res=resx)
    sc["camera"]["resy"] = resy
    sc["film"] = {"filter_type": kind, "AA_pixelwidth": width}
    return gbrt.Renderer(sc)


@pytest.mark.parametrize("kind,width,spp", [("gauss", 1.5, 4), ("box", 1.0, 16), ("mitchell", 1.5, 1), ("gauss", 2.5, 3)])
def test_gpu_film_weights_match_oracle(cuda_device, kind, width, spp):
    import torch
    resx, resy = 40, 30
    r = _cornell(resx, resy, kind, width)
    film = torch.zeros(resx * resy * 3, dtype=torch.float32, device="cuda")
    w = torch.zeros(resx * resy, dtype=torch.float32, device="cuda")
    r.render_device(spp, film.data_ptr(), weight_ptr=w.data_ptr())
    torch.cuda.synchronize()
    got = w.cpu().numpy().reshape(resy, resx).astype(np.float64)
    exp = fo.splat_weights(resx, resy, spp, kind, width)
    assert np.allclose(got, exp, rtol=1e-5, atol=1e-5), float(np.abs(got - exp).max())


def test_gpu_film_needs_a_weight_buffer(cuda_device):
    import torch
    r = _cornell(16, 12, "gauss", 1.5)
    film = torch.zeros(16 * 12 * 3, dtype=torch.float32, device="cuda")
    with pytest.raises(gbrt.GbrtError):
        r.render_device(4, film.data_ptr())


def test_gpu_gauss_film_render_vs_reference(cuda_device):
    g = np.load(os.path.join(GOLD, "cornell_gauss_48x36_render.npz"))
    r = _cornell(48, 36, "gauss", 1.5)
    k, spp = int(g["batches"]), int(g["spp"])
    gpu = np.stack([r.render(spp, base_offset=b * spp, seed=1000 + b)[0] for b in range(k)])
    frac, relmse, _ = parity(gpu, g["mean"], g["se"])
    print(f"cornell gauss film 48x36: {100 * frac:.2f}% of pixel channels within 3 SE, relMSE {relmse:.3g}")
    assert frac >= 0.995
