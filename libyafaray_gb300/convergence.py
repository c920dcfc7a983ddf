"""Time-to-error measurement of the GPU path tracer, plain and guided.

relMSE(x, r) = mean over pixels and RGB of (x - r)^2 / (r^2 + 1e-2), r an
FP64-accumulated plain render.  Renders run in passes of `spp_pass` samples
into one film; after each pass the film is compared with the reference on
the device (the comparison is not counted as render time).  Guided runs
train the network online during the first `train_fraction` of the elapsed
time (the first pass is plain, later passes sample the guide with
probability alpha); every pass's samples count, so the estimate stays
unbiased.  torch is used only for device buffers and the error reduction.
"""
import time

import numpy as np


def reference_image(renderer, spp=16384, chunk=256, base_offset=1 << 24, seed=77):
    """FP64-accumulated plain render (device tensor of per-pixel means)."""
    import torch
    c = renderer.scene["camera"]
    n = int(c["resx"]) * int(c["resy"]) * 3
    acc = torch.zeros(n, dtype=torch.float64, device="cuda")
    done = 0
    while done < spp:
        k = min(chunk, spp - done)
        renderer.render_device(k, 0, film64_ptr=acc.data_ptr(), base_offset=base_offset + done, seed=seed + done)
        done += k
    torch.cuda.synchronize()
    return (acc / done).float()


def relmse_device(film_sum, spp, ref):
    import torch
    x = film_sum / spp
    return float(torch.mean((x - ref) ** 2 / (ref * ref + 1e-2)).item())


def time_to_relmse(renderer, ref, target=0.01, spp_pass=4, max_time=60.0, guide=None, alpha=0.6,
                   train_fraction=0.25, train_steps=16, batch=65536, max_vertex=2, expected_time=None, seed=1000,
                   spp_pass_after=None):
    """Returns dict(time_s, spp, relmse, reached, curve).  expected_time sets
    the training window for guided runs (train while elapsed < train_fraction
    x expected_time); defaults to max_time.  spp_pass_after: samples per pass
    once training has stopped (default spp_pass)."""
    import torch
    c = renderer.scene["camera"]
    n = int(c["resx"]) * int(c["resy"]) * 3
    film = torch.zeros(n, dtype=torch.float32, device="cuda")
    spp, t_acc, curve = 0, 0.0, []
    window = train_fraction * (expected_time if expected_time else max_time)
    err = float("inf")
    step = 0
    while t_acc < max_time:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if guide is None:
            renderer.render_device(spp_pass, film.data_ptr(), base_offset=spp, seed=seed + step)
        else:
            training = t_acc < window
            n = spp_pass if training or not spp_pass_after else spp_pass_after
            renderer.render_device(n, film.data_ptr(), base_offset=spp, seed=seed + step, guide=guide,
                                   alpha=0.0 if step == 0 else alpha, train_steps=train_steps if training else 0,
                                   batch=batch, max_vertex=max_vertex)
        torch.cuda.synchronize()
        t_acc += time.perf_counter() - t0
        spp += spp_pass if guide is None or training or not spp_pass_after else spp_pass_after
        step += 1
        err = relmse_device(film, spp, ref)
        curve.append((round(t_acc, 4), spp, err))
        if err <= target:
            return {"time_s": t_acc, "spp": spp, "relmse": err, "reached": True, "curve": curve[::max(1, len(curve) // 24)]}
    return {"time_s": t_acc, "spp": spp, "relmse": err, "reached": False, "curve": curve[::max(1, len(curve) // 24)]}
