"""Shared checks of the path tracer's sampling primitives against the
reference's own values (tests/golden/sampler.npz)."""
import os

import numpy as np

from libyafaray_gb300 import gbrt

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampler.npz")


def check_sampler(on_device):
    g = np.load(GOLD)
    mismatches = {}
    lds = g["lds"]
    n = lds.shape[1]
    for d in range(1, lds.shape[0] + 1):
        idx = (np.arange(n, dtype=np.uint64) * int(g["lds_index_mult"]) + d).astype(np.uint32)
        got = gbrt.sampler_eval(0, d, idx, on_device)
        bad = int((got.view(np.uint64) != lds[d - 1].view(np.uint64)).sum())
        if bad:
            mismatches[f"lds{d}"] = bad
    idx = (np.arange(1024, dtype=np.uint64) * int(g["seq_index_mult"]) % (1 << 32)).astype(np.uint32)
    for kind, key in [(1, "vdc"), (2, "lp"), (3, "s")]:
        got = gbrt.sampler_eval(kind, 0, idx, on_device).astype(np.float32)
        bad = int((got != g[key]).sum())
        if bad:
            mismatches[key] = bad
    got = gbrt.sampler_eval(4, 0, idx, on_device).astype(np.uint64)
    if (got != g["fnv"].astype(np.uint64)).any():
        mismatches["fnv"] = int((got != g["fnv"]).sum())
    seq = np.arange(1024, dtype=np.uint32) + np.uint32(g["halton_start"]) + 1
    for kind, key in [(5, "h2"), (6, "h3")]:
        got = gbrt.sampler_eval(kind, 0, seq, on_device).astype(np.float32)
        if (got != g[key]).any():
            mismatches[key] = int((got != g[key]).sum())
    bits = g["angle"].view(np.uint32)
    for dim, key in [(0, "sin"), (1, "cos")]:
        got = gbrt.sampler_eval(7, dim, bits, on_device).astype(np.float32)
        if (got != g[key]).any():
            mismatches[key] = int((got != g[key]).sum())
    pb = g["pow_base"].view(np.uint32)
    for e in np.unique(g["pow_exp"]):
        sel = g["pow_exp"] == e
        got = gbrt.sampler_eval(8, int(np.float32(e).view(np.int32)), pb[sel], on_device).astype(np.float32)
        bad = int((got.view(np.uint32) != g["pow"][sel].view(np.uint32)).sum())
        if bad:
            mismatches[f"pow{e}"] = bad
    mismatches.update(check_float_forms(on_device))
    return mismatches


def check_float_forms(on_device, per_dim=20000, seed=11):
    """The FP64-free float forms (kinds 9 and 10, what the kernels use) equal
    the double loops rounded to float (kinds 0 and 6, pinned to the
    reference above) on the reference's own indices, on random indices and
    on the smallest and largest ones, for every dimension."""
    g = np.load(GOLD)
    rng = np.random.default_rng(seed)
    bad = {}
    n = g["lds"].shape[1]
    for d in range(1, g["lds"].shape[0] + 1):
        idx = (np.arange(n, dtype=np.uint64) * int(g["lds_index_mult"]) + d).astype(np.uint32)
        idx = np.concatenate([idx, rng.integers(0, 2 ** 32, per_dim, dtype=np.uint64).astype(np.uint32),
                              np.arange(2000, dtype=np.uint32), (2 ** 32 - 1 - np.arange(2000)).astype(np.uint32)])
        ref = gbrt.sampler_eval(0, d, idx, on_device).astype(np.float32)
        got = gbrt.sampler_eval(9, d, idx, on_device).astype(np.float32)
        k = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
        if k:
            bad[f"lds_f{d}"] = k
    seq = np.concatenate([np.arange(1024, dtype=np.uint32) + np.uint32(g["halton_start"]) + 1,
                          rng.integers(0, 2 ** 32, 20 * per_dim, dtype=np.uint64).astype(np.uint32)])
    ref = gbrt.sampler_eval(6, 0, seq, on_device).astype(np.float32)
    got = gbrt.sampler_eval(10, 0, seq, on_device).astype(np.float32)
    k = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    if k:
        bad["h3_f"] = k
    if (gbrt.sampler_eval(10, 0, seq[:1024], on_device).astype(np.float32) != g["h3"]).any():
        bad["h3_f_golden"] = 1
    return bad
