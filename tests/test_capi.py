"""CPU-side checks of the C ABI library: it builds, loads, and exports every
function include/gbrt.h declares; error paths work without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from libyafaray_gb300 import gbrt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name):
    src = open(os.path.join(ROOT, "include", name)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbrt_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected_entry_points():
    fns = header_functions("gbrt.h")
    for f in ["gbrt_bvh_build", "gbrt_bvh_build_host", "gbrt_bvh_destroy", "gbrt_trace_closest",
              "gbrt_trace_shadow", "gbrt_trace_closest_host", "gbrt_trace_shadow_host", "gbrt_bvh_get_bound"]:
        assert f in fns


def test_library_exports_every_declared_symbol(gbrt_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", gbrt.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gbrt_[a-z0-9_]+)", out))
    missing = [f for f in header_functions("gbrt.h") if f not in exported]
    assert not missing, missing
    # and the ctypes binding covers the same set
    assert set(gbrt.SIGNATURES) == set(header_functions("gbrt.h"))


def test_null_arguments_are_errors_not_crashes(gbrt_lib):
    L = gbrt_lib
    assert L.gbrt_bvh_build_host(None, 0, None, 1, None, None) == -1
    assert b"NULL" in L.gbrt_last_error()
    assert L.gbrt_trace_closest(None, None, 10, None, None) == -1
    assert L.gbrt_bvh_destroy(None) == 0
    assert L.gbrt_version() >= 1


def test_guide_and_tensor_core_argument_checks(gbrt_lib):
    """Argument errors are reported before any CUDA call."""
    import numpy as np
    from libyafaray_gb300 import gbrt
    L = gbrt_lib
    assert L.gbrt_guide_set_eval_mode(None, 0) == -1
    assert L.gbrt_guide_status(None, None) == -1
    a = np.zeros((128, 16), np.float32)
    with pytest.raises(gbrt.GbrtError, match="multiple of 16"):
        gbrt.tc_selftest(np.zeros((128, 8), np.float32), np.zeros((8, 8), np.float32))
    with pytest.raises(gbrt.GbrtError, match="multiple of 16"):
        gbrt.tc_selftest(a, np.zeros((80, 16), np.float32))


def test_photon_mapping_argument_checks(gbrt_lib):
    """Photon-mapping defaults are the reference's; argument errors are
    reported before any CUDA call."""
    from libyafaray_gb300 import gbrt
    p = gbrt.PmParams()
    assert gbrt_lib.gbrt_pm_default_params(ctypes.byref(p)) == 0
    assert (p.diffuse_photons, p.caustic_photons, p.diffuse_search, p.caustic_mix, p.caustic_depth, p.bounces) == (100000, 500000, 50, 50, 10, 3)
    assert abs(p.diffuse_radius - 0.1) < 1e-7 and abs(p.caustic_radius - 0.25) < 1e-7
    assert (p.caustics, p.diffuse, p.final_gather, p.fg_samples, p.fg_bounces) == (0, 1, 1, 32, 2)
    assert gbrt_lib.gbrt_pm_render(None, None, None, None, None, None, None, None) == -1
    with pytest.raises(gbrt.GbrtError, match="k in"):
        gbrt.knn_gather([[0, 0, 0]], [[0, 0, 0]], cell=0.1, k=65, r2=0.01)
    with pytest.raises(gbrt.GbrtError, match="below the search radius"):
        gbrt.knn_gather([[0, 0, 0]], [[0, 0, 0]], cell=0.05, k=8, r2=0.01)
