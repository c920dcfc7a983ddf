"""gbrt_bvh_build_static, the BVH build that allocates no device memory.

It serves callers that cannot allocate device memory while building — a
render loop rebuilding small per-object hierarchies every frame (cudaMalloc
and cudaFree synchronise the device) or a host application that budgets GPU
memory through its own pool and only hands out output buffers.  Its
temporaries live in a fixed array inside the library, shared by all calls.

The test calls it through the C ABI twice in a row (a larger scene, then a
smaller one with quads, so stale contents of the shared array would show)
and requires bit-identical output to the allocating entry point
gbrt_bvh_build, read back with gbrt_bvh_export.  Kept in a file that pytest
collects last.
"""
import ctypes

import numpy as np
import pytest

from libyafaray_gb300 import gbrt, scenes

pytestmark = pytest.mark.gpu


def _static_build(torch, verts, faces, leaf=0):
    L = gbrt.load()
    n = len(faces)
    slots = max(n - 1, 1)
    v_d = torch.from_numpy(np.ascontiguousarray(verts, np.float32)).cuda()
    f_d = torch.from_numpy(np.ascontiguousarray(faces, np.uint32).view(np.int32)).cuda()
    nodes = torch.full((slots, 16), float("nan"), dtype=torch.float32, device="cuda")
    prims = torch.full((max(n, 1), 12), float("nan"), dtype=torch.float32, device="cuda")
    ids = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    bound = (ctypes.c_float * 6)()
    params = gbrt.BuildParams(leaf, 0.0, 0.0, 0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gbrt_bvh_build_static(ctypes.c_void_p(v_d.data_ptr()), len(verts), ctypes.c_void_p(f_d.data_ptr()), n,
                                 ctypes.byref(params), ctypes.c_void_p(nodes.data_ptr()), nodes.numel() * 4,
                                 ctypes.c_void_p(prims.data_ptr()), prims.numel() * 4,
                                 ctypes.c_void_p(ids.data_ptr()), ids.numel() * 4, bound, ctypes.c_void_p(stream))
    gbrt.check(rc)
    torch.cuda.synchronize()
    return (nodes.cpu().numpy(), prims.cpu().numpy()[:n], ids.cpu().numpy().view(np.uint32)[:n],
            np.array(bound[:], np.float32))


def test_static_build_matches_allocating_build_twice(cuda_device):
    torch = pytest.importorskip("torch")
    v1, f1 = scenes.random_triangles(20_000, seed=71, spread=0.03)
    v2, f2, _ = scenes.cornell_mesh(as_quads=True)
    for verts, faces in [(v1, f1), (v2, f2)]:
        ref = gbrt.Bvh.build_host(verts, faces)
        r_nodes, r_prims, r_ids = ref.export()
        s_nodes, s_prims, s_ids, s_bound = _static_build(torch, verts, faces)
        assert np.array_equal(s_bound, ref.bound())
        assert np.array_equal(s_nodes.view(np.uint32), r_nodes.view(np.uint32))
        assert np.array_equal(s_prims.view(np.uint32), r_prims.view(np.uint32))
        assert np.array_equal(s_ids, r_ids)


def test_static_build_rejects_more_than_its_capacity(cuda_device):
    torch = pytest.importorskip("torch")
    n = 65536 + 1
    v, f = scenes.random_triangles(n, seed=73)
    with pytest.raises(gbrt.GbrtError) as e:
        _static_build(torch, v, f)
    assert e.value.code == -5 and "65536" in str(e.value)
