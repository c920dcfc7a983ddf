"""Host-side mesh preparation of libgbrt against the compiled reference.

gbrt_mesh_smooth_normals restates MeshObject::smoothVerticesNormals
(src/geometry/object/object_mesh.cc:150-262), the work behind
yafaray_smoothObjectMesh.  tests/golden/smooth_normals.npz holds, per face
corner, the normal index and the normal the reference gave the same meshes
(oracle/ref/normals_dump.cc): every index and every normal must be equal,
bit for bit.  No GPU is needed (the entry point runs on the host)."""
import os

import numpy as np
import pytest

from libyafaray_gb300 import gbrt

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "smooth_normals.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLD)


def _cases():
    return [str(c) for c in np.load(GOLD)["cases"]]


@pytest.mark.parametrize("case", _cases())
def test_smooth_normals_match_reference(gbrt_lib, golden, case):
    v, f = golden[f"{case}_vertices"], golden[f"{case}_faces"]
    normals, fn = gbrt.smooth_normals(v, f, float(golden[f"{case}_angle"]))
    idx = np.where(fn == gbrt.NO_NORMAL, -1, fn.astype(np.int64))
    ref_idx = golden[f"{case}_index"]
    assert np.array_equal(idx, ref_idx), f"{np.count_nonzero(idx != ref_idx)} corner indices differ"
    got = np.zeros((len(f), 4, 3), np.float32)
    live = idx >= 0
    got[live] = normals[idx[live]]
    assert np.array_equal(got.view(np.uint32), golden[f"{case}_normal"].view(np.uint32))


def test_smooth_normals_size_query_and_capacity(gbrt_lib, golden):
    import ctypes
    v, f = golden["ico_100_vertices"], golden["ico_100_faces"]
    n = ctypes.c_uint32()
    fn = np.empty((len(f), 4), np.uint32)
    L = gbrt.load()
    assert L.gbrt_mesh_smooth_normals(gbrt._ptr(v), len(v), gbrt._ptr(f), len(f), 100.0, None, 0, ctypes.byref(n),
                                      gbrt._ptr(fn)) == 0
    assert n.value > len(v)
    small = np.empty((len(v), 3), np.float32)
    rc = L.gbrt_mesh_smooth_normals(gbrt._ptr(v), len(v), gbrt._ptr(f), len(f), 100.0, gbrt._ptr(small), len(v),
                                    ctypes.byref(n), gbrt._ptr(fn))
    assert rc == -5   # GBRT_ERR_CAPACITY
    bad = f.copy()
    bad[0, 0] = len(v)
    rc = L.gbrt_mesh_smooth_normals(gbrt._ptr(v), len(v), gbrt._ptr(bad), len(bad), 100.0, None, 0, ctypes.byref(n),
                                    gbrt._ptr(fn))
    assert rc == -1   # GBRT_ERR_INVALID
