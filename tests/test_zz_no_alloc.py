"""gbrt_bvh_build_static, the BVH build that allocates no device memory.

It serves callers that cannot allocate device memory while building — a
render loop rebuilding small per-object hierarchies every frame (cudaMalloc
and cudaFree synchronise the device) or a host application that budgets GPU
memory through its own pool and only hands out output buffers.  Its
temporaries live in a fixed array inside the library, shared by all calls.

The tests call it through the C ABI several times in a row (a larger scene,
then a smaller one with quads, so stale contents of the shared array would
show; then the empty and single-face cases and the leaf-size limits) and
require bit-identical output to the allocating entry point gbrt_bvh_build,
read back with gbrt_bvh_export, and an unchanged amount of free device
memory around a call.  Kept in a file that pytest collects last.
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


def _check_against_allocating_build(torch, verts, faces, leaf):
    ref = gbrt.Bvh.build_host(verts, faces, max_leaf_size=leaf)
    r_nodes, r_prims, r_ids = ref.export()
    s_nodes, s_prims, s_ids, s_bound = _static_build(torch, verts, faces, leaf)
    assert np.array_equal(s_bound, ref.bound())
    assert np.array_equal(s_nodes.view(np.uint32), r_nodes.view(np.uint32))
    assert np.array_equal(s_prims.view(np.uint32), r_prims.view(np.uint32))
    assert np.array_equal(s_ids, r_ids)


def test_static_build_edge_cases_and_leaf_sizes(cuda_device):
    """No faces (a zeroed root slot), one face (a single leaf), and the
    smallest and largest leaf sizes, each equal to the allocating build."""
    torch = pytest.importorskip("torch")
    v, f = scenes.random_triangles(3_000, seed=75, spread=0.05)
    empty_v, empty_f = np.zeros((0, 3), np.float32), np.zeros((0, 4), np.uint32)
    cases = [(empty_v, empty_f, 0), (v, f[:1], 0), (v[:3], f[:1], 0), (v, f, 1), (v, f, 16), (empty_v, empty_f, 0)]
    for verts, faces, leaf in cases:
        _check_against_allocating_build(torch, verts, faces, leaf)


def test_static_build_leaves_device_memory_unchanged(cuda_device):
    """A warm call takes no device memory: the device's free memory (all
    allocators of the process, the library's own pool included) and torch's
    allocator counter are the same after the call as before."""
    torch = pytest.importorskip("torch")
    v, f = scenes.random_triangles(40_000, seed=77, spread=0.03)
    v_d = torch.from_numpy(np.ascontiguousarray(v, np.float32)).cuda()
    f_d = torch.from_numpy(np.ascontiguousarray(f, np.uint32).view(np.int32)).cuda()
    n = len(f)
    nodes = torch.empty((n - 1) * 16, dtype=torch.float32, device="cuda")
    prims = torch.empty(n * 12, dtype=torch.float32, device="cuda")
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    bound = (ctypes.c_float * 6)()
    params = gbrt.BuildParams(0, 0.0, 0.0, 0)
    L = gbrt.load()
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        gbrt.check(L.gbrt_bvh_build_static(ctypes.c_void_p(v_d.data_ptr()), len(v), ctypes.c_void_p(f_d.data_ptr()), n,
                                           ctypes.byref(params), ctypes.c_void_p(nodes.data_ptr()), nodes.numel() * 4,
                                           ctypes.c_void_p(prims.data_ptr()), prims.numel() * 4,
                                           ctypes.c_void_p(ids.data_ptr()), ids.numel() * 4, bound,
                                           ctypes.c_void_p(stream)))
        torch.cuda.synchronize()

    call()                                            # loads the module on this device if no call did yet
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_allocated() == alloc0


def test_static_build_rejects_more_than_its_capacity(cuda_device):
    torch = pytest.importorskip("torch")
    n = 65536 + 1
    v, f = scenes.random_triangles(n, seed=73)
    with pytest.raises(gbrt.GbrtError) as e:
        _static_build(torch, v, f)
    assert e.value.code == -5 and "65536" in str(e.value)
