"""ctypes binding of libgbrt.so (the C ABI declared in include/gbrt.h).

There is no fallback: if the shared library is missing or no CUDA device is
visible, loading raises.  Buffers are numpy arrays (host) or raw device
pointers (ints), so torch is never needed here; callers that keep data in
torch tensors pass ``tensor.data_ptr()`` and the stream's ``cuda_stream``.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbrt.so")

GBRT_OK = 0
TRIANGLE = 0xFFFFFFFF
ERRORS = {-1: "GBRT_ERR_INVALID", -2: "GBRT_ERR_CUDA", -3: "GBRT_ERR_OOM", -4: "GBRT_ERR_TIMEOUT",
          -5: "GBRT_ERR_CAPACITY", -6: "GBRT_ERR_NO_DEVICE"}


class GbrtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class BuildParams(ctypes.Structure):
    _fields_ = [("max_leaf_size", ctypes.c_uint32), ("traversal_cost", ctypes.c_float),
                ("intersect_cost", ctypes.c_float), ("flags", ctypes.c_uint32)]


class BvhInfo(ctypes.Structure):
    _fields_ = [("n_prims", ctypes.c_uint32), ("n_nodes", ctypes.c_uint32), ("n_leaves", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32), ("sah_cost", ctypes.c_float), ("bound", ctypes.c_float * 6),
                ("device_bytes", ctypes.c_uint64)]


# Every symbol include/gbrt.h declares, with its ctypes signature.
_VP, _U32, _I, _F = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_float
SIGNATURES = {
    "gbrt_last_error": (ctypes.c_char_p, []),
    "gbrt_version": (_I, []),
    "gbrt_device_count": (_I, [ctypes.POINTER(ctypes.c_int)]),
    "gbrt_bvh_build": (_I, [_VP, _U32, _VP, _U32, ctypes.POINTER(BuildParams), _VP, ctypes.POINTER(_VP)]),
    "gbrt_bvh_build_host": (_I, [_VP, _U32, _VP, _U32, ctypes.POINTER(BuildParams), ctypes.POINTER(_VP)]),
    "gbrt_bvh_destroy": (_I, [_VP]),
    "gbrt_bvh_get_bound": (_I, [_VP, ctypes.POINTER(ctypes.c_float)]),
    "gbrt_bvh_get_info": (_I, [_VP, ctypes.POINTER(BvhInfo)]),
    "gbrt_bvh_export": (_I, [_VP, _VP, ctypes.c_size_t, _VP, ctypes.c_size_t, _VP, ctypes.c_size_t]),
    "gbrt_bvh_build_static": (_I, [_VP, _U32, _VP, _U32, ctypes.POINTER(BuildParams), _VP, ctypes.c_size_t, _VP,
                                   ctypes.c_size_t, _VP, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float), _VP]),
    "gbrt_trace_closest": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "gbrt_trace_shadow": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "gbrt_trace_closest_host": (_I, [_VP, _VP, _U32, _VP]),
    "gbrt_trace_shadow_host": (_I, [_VP, _VP, _U32, _VP]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libgbrt.so and bind every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with libyafaray_gb300.build.build()")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != GBRT_OK:
        raise GbrtError(rc, load().gbrt_last_error().decode(errors="replace"))
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Bvh:
    """Owning handle of a device BVH (gbrt_bvh)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def build_host(cls, vertices, faces, max_leaf_size=0, traversal_cost=0.0, intersect_cost=0.0):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 4)
        p = BuildParams(max_leaf_size, traversal_cost, intersect_cost, 0)
        h = ctypes.c_void_p()
        check(load().gbrt_bvh_build_host(_ptr(v), len(v), _ptr(f), len(f), ctypes.byref(p), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def build_device(cls, vertices_ptr, n_vertices, faces_ptr, n_faces, stream=0, max_leaf_size=0,
                     traversal_cost=0.0, intersect_cost=0.0):
        p = BuildParams(max_leaf_size, traversal_cost, intersect_cost, 0)
        h = ctypes.c_void_p()
        check(load().gbrt_bvh_build(ctypes.c_void_p(vertices_ptr), n_vertices, ctypes.c_void_p(faces_ptr), n_faces,
                                    ctypes.byref(p), ctypes.c_void_p(stream), ctypes.byref(h)))
        return cls(h)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            load().gbrt_bvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bound(self):
        out = (ctypes.c_float * 6)()
        check(load().gbrt_bvh_get_bound(self._h, out))
        return np.array(out[:], np.float32)

    def info(self):
        inf = BvhInfo()
        check(load().gbrt_bvh_get_info(self._h, ctypes.byref(inf)))
        return {"n_prims": inf.n_prims, "n_nodes": inf.n_nodes, "n_leaves": inf.n_leaves,
                "max_depth": inf.max_depth, "sah_cost": inf.sah_cost, "bound": list(inf.bound),
                "device_bytes": inf.device_bytes}

    def export(self):
        """(nodes float32 [slots,16], prims float32 [n,12], ids uint32 [n])."""
        inf = self.info()
        n = inf["n_prims"]
        slots = max(n - 1, 1)
        nodes = np.empty((slots, 16), np.float32)
        prims = np.empty((max(n, 1), 12), np.float32)
        ids = np.empty(max(n, 1), np.uint32)
        check(load().gbrt_bvh_export(self._h, _ptr(nodes), nodes.nbytes, _ptr(prims), prims.nbytes, _ptr(ids), ids.nbytes))
        return nodes, prims[:n], ids[:n]

    def trace_closest_host(self, rays):
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((len(r), 4), np.float32)
        check(load().gbrt_trace_closest_host(self._h, _ptr(r), len(r), _ptr(hits)))
        prim = hits[:, 0].copy().view(np.int32)
        return prim, hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].copy()

    def trace_shadow_host(self, rays):
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.empty(len(r), np.int32)
        check(load().gbrt_trace_shadow_host(self._h, _ptr(r), len(r), _ptr(occ)))
        return occ

    def trace_closest_device(self, rays_ptr, n, hits_ptr, stream=0):
        check(load().gbrt_trace_closest(self._h, ctypes.c_void_p(rays_ptr), n, ctypes.c_void_p(hits_ptr),
                                        ctypes.c_void_p(stream)))

    def trace_shadow_device(self, rays_ptr, n, occ_ptr, stream=0):
        check(load().gbrt_trace_shadow(self._h, ctypes.c_void_p(rays_ptr), n, ctypes.c_void_p(occ_ptr),
                                       ctypes.c_void_p(stream)))
