"""Structural validation of an exported GPU hierarchy (gbrt_bvh_export):
every primitive slot is reached exactly once, every child box (as stored,
grown) contains its subtree's primitives, primitive records reproduce the
faces (v0 and float32 edge differences exactly), and IDs are a permutation.
Returns a list of problems (empty = valid)."""
import numpy as np

LEAF = 0x80000000
QUAD = 0x80000000
TRI = 0xFFFFFFFF


def check_bvh(nodes, prims, ids, verts, faces):
    problems = []
    n = len(faces)
    if n == 0:
        return problems
    verts = np.asarray(verts, np.float32)
    faces = np.asarray(faces, np.uint32)
    pid = ids & ~np.uint32(QUAD)
    if not np.array_equal(np.sort(pid), np.arange(n, dtype=np.uint32)):
        problems.append("ids are not a permutation of the primitive IDs")
        return problems
    # primitive records
    f = faces[pid]
    v0 = verts[f[:, 0]]
    quad = f[:, 3] != TRI
    if not np.array_equal((ids & QUAD) != 0, quad):
        problems.append("quad flags differ from faces")
    if not np.array_equal(prims[:, 0:3], v0):
        problems.append("v0 differs")
    if not np.array_equal(prims[:, 4:7], (verts[f[:, 1]] - v0).astype(np.float32)):
        problems.append("e1 differs")
    if not np.array_equal(prims[:, 8:11], (verts[f[:, 2]] - v0).astype(np.float32)):
        problems.append("e2 differs")
    # per-slot primitive boxes from the original vertices
    idx = f.astype(np.int64).copy()
    idx[~quad, 3] = idx[~quad, 2]
    P = verts[idx]  # [n, 4, 3]
    plo, phi = P.min(1), P.max(1)
    u32 = nodes.view(np.uint32)
    seen = np.zeros(n, np.int32)
    stack = [(0, None, None)]

    def subtree_box(ref):
        """box of all prims below ref (iterative)"""
        lo = np.full(3, np.inf, np.float32); hi = np.full(3, -np.inf, np.float32)
        st = [ref]
        while st:
            r = st.pop()
            if r & LEAF:
                first, cnt = r & ((1 << 27) - 1), ((r >> 27) & 15) + 1
                lo = np.minimum(lo, plo[first:first + cnt].min(0)); hi = np.maximum(hi, phi[first:first + cnt].max(0))
            else:
                st += [int(u32[r, 12]), int(u32[r, 13])]
        return lo, hi

    visited = 0
    st = [0]
    while st:
        r = st.pop()
        visited += 1
        if visited > 4 * n + 8:
            problems.append("cycle or runaway traversal")
            break
        row = nodes[r]
        boxes = [(row[[0, 2, 8]], row[[1, 3, 9]]), (row[[4, 6, 10]], row[[5, 7, 11]])]
        for k in range(2):
            c = int(u32[r, 12 + k])
            if n == 1 and k == 1:
                continue
            lo, hi = subtree_box(c)
            blo, bhi = boxes[k]
            if (blo > lo).any() or (bhi < hi).any():
                problems.append(f"node {r} child {k} box does not contain its subtree")
            if c & LEAF:
                first, cnt = c & ((1 << 27) - 1), ((c >> 27) & 15) + 1
                seen[first:first + cnt] += 1
            else:
                st.append(c)
    if n == 1:
        seen[0] = 1
    if not (seen == 1).all():
        problems.append(f"{int((seen == 0).sum())} slots unreached, {int((seen > 1).sum())} reached twice")
    return problems
