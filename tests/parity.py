"""Parity bookkeeping shared by the traversal tests.

Acceptance rule for traversal: primitive IDs must match the reference
bit-exactly, except for
  - rays that pass within EDGE_EPS (relative, plus the float32 uncertainty of
    the hit point, 8 ulps of t) of a primitive edge or vertex, where the
    reference kd-tree's answer depends on its split planes (a primitive lying
    in a split plane is only found from one side);
  - exact ties: two primitives hit at the same t (shared edges, coplanar
    overlapping faces), which the reference resolves by traversal order and
    this build by the lower primitive ID.
Those rays are counted and reported, not failed.  For
matching IDs, t must agree within T_RTOL relative (the GPU path is in fact
bit-exact) and (u, v) likewise.
"""
import numpy as np

EDGE_EPS = 1e-6
T_RTOL = 1e-5
TRI = 0xFFFFFFFF


def _seg_dist(p, a, b):
    ab = b - a
    L = np.dot(ab, ab)
    s = 0.0 if L == 0 else np.clip(np.dot(p - a, ab) / L, 0.0, 1.0)
    return np.linalg.norm(p - (a + s * ab))


def edge_distance(verts, face, point):
    """Distance from point to the nearest edge of a face; a quad's diagonal
    (0,2) counts as an edge (its two triangles meet there)."""
    idx = [int(face[k]) for k in range(3)] + ([] if face[3] == TRI else [int(face[3])])
    P = [verts[i].astype(np.float64) for i in idx]
    edges = [(0, 1), (1, 2), (2, 0)] if len(P) == 3 else [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)]
    return min(_seg_dist(point, P[a], P[b]) for a, b in edges)


def near_edge(verts, faces, ray, prim, t):
    if prim < 0:
        return False
    o = ray[:3].astype(np.float64)
    d = ray[4:7].astype(np.float64)
    p = o + float(t) * d
    scale = max(1.0, float(np.abs(p).max()))
    slack = 8.0 * float(np.finfo(np.float32).eps) * abs(float(t)) * float(np.linalg.norm(d))
    return edge_distance(verts, faces[prim], p) <= EDGE_EPS * scale + slack


def compare_closest(verts, faces, rays, got, ref):
    """got/ref: (prim, t, u, v).  Returns dict with counts and the indices of
    unexplained mismatches."""
    gp, gt, gu, gv = got
    rp, rt, ru, rv = ref
    mism = np.where(gp != rp)[0]
    edge, tie, bad = [], [], []
    for i in mism:
        if gp[i] >= 0 and rp[i] >= 0 and gt[i] == rt[i]:
            tie.append(int(i))
        elif near_edge(verts, faces, rays[i], gp[i], gt[i]) or near_edge(verts, faces, rays[i], rp[i], rt[i]):
            edge.append(int(i))
        else:
            bad.append(int(i))
    same = (gp == rp) & (rp >= 0)
    t_ok = np.allclose(gt[same], rt[same], rtol=T_RTOL, atol=0.0)
    uv_ok = np.allclose(gu[same], ru[same], rtol=T_RTOL, atol=1e-6) and np.allclose(gv[same], rv[same], rtol=T_RTOL, atol=1e-6)
    t_exact = bool(np.array_equal(gt[same], rt[same]))
    return {"n": len(rays), "hits": int((rp >= 0).sum()), "mismatch": len(mism), "edge": len(edge),
            "tie": len(tie), "bad": bad, "t_ok": bool(t_ok), "uv_ok": bool(uv_ok), "t_exact": t_exact}


def _segment_edge_hit(verts, faces, ray):
    """True if any primitive that the shadow segment of `ray` (the
    Accelerator::isShadowed set-up) crosses is crossed within EDGE_EPS of an
    edge."""
    import ctypes
    from oracle import orc
    L = orc.lib()
    o = ray[:3].astype(np.float32) + ray[4:7].astype(np.float32) * np.float32(ray[3])
    d = ray[4:7].astype(np.float32)
    t_max = np.float32(ray[7] - 2 * ray[3]) if ray[7] >= 0 else np.float32(np.finfo(np.float32).max)
    fp = ctypes.POINTER(ctypes.c_float)
    u = ctypes.c_float(); v = ctypes.c_float()
    for k, f in enumerate(faces):
        n = 3 if f[3] == TRI else 4
        q = np.zeros(12, np.float32)
        for j in range(n):
            q[3 * j:3 * j + 3] = verts[f[j]]
        t = L.orc_mt_intersect(q.ctypes.data_as(fp), n, o.ctypes.data_as(fp), d.ctypes.data_as(fp),
                               ctypes.byref(u), ctypes.byref(v))
        if 0.0 < t < t_max:
            p = o.astype(np.float64) + t * d.astype(np.float64)
            slack = 8.0 * float(np.finfo(np.float32).eps) * float(t) * float(np.linalg.norm(d))
            if edge_distance(verts, f, p) <= EDGE_EPS * max(1.0, float(np.abs(p).max())) + slack:
                return True
    return False


def compare_shadow(verts, faces, rays, got_occ, ref_hit):
    """got_occ: occluder ID or -1; ref_hit: 0/1.  A mismatch is explained
    when the shadow segment crosses some primitive within EDGE_EPS of an
    edge."""
    gh = (got_occ >= 0).astype(np.uint8)
    mism = np.where(gh != ref_hit)[0]
    bad = [int(i) for i in mism if not _segment_edge_hit(verts, faces, rays[i])]
    return {"n": len(rays), "occluded": int(ref_hit.sum()), "mismatch": len(mism), "edge": len(mism) - len(bad),
            "bad": bad}


def photon_hash(ph):
    """64-bit hash of each photon row (dir, pos, colour: 9 float32 bits)."""
    w = np.ascontiguousarray(ph, np.float32).view(np.uint32).astype(np.uint64)
    h = np.full(len(w), 0x9E3779B97F4A7C15, np.uint64)
    with np.errstate(over="ignore"):
        for j in range(w.shape[1]):
            h = (h ^ w[:, j]) * np.uint64(0xBF58476D1CE4E5B9)
            h ^= h >> np.uint64(31)
    return h


def photon_buckets(ph, nb=4096):
    """Order-free digest of a photon multiset: per hash bucket the photon
    count and the wrapping sum of the photons' hashes."""
    h = photon_hash(ph)
    b = (h >> np.uint64(52)).astype(np.int64) % nb
    counts = np.bincount(b, minlength=nb).astype(np.int64)
    sums = np.zeros(nb, np.uint64)
    with np.errstate(over="ignore"):
        np.add.at(sums, b, h)
    return counts, sums
