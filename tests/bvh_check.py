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


def _byte(word, k):
    return (int(word) >> (8 * k)) & 0xFF


def check_wide(wnodes, prims, ids, verts, faces, depth):
    """Structural validation of the 8-wide compressed hierarchy
    (gbrt_bvh_export_wide): every node is reached once from the root, slot
    metadata agree with imask, every primitive slot is in exactly one leaf,
    every primitive lies inside the decoded (origin + q 2^e) box of every
    slot on its path, primitive records reproduce the faces, and the depth
    matches.  Returns a list of problems (empty = valid)."""
    problems = []
    n = len(faces)
    if n == 0:
        return problems
    verts = np.asarray(verts, np.float32)
    faces = np.asarray(faces, np.uint32)
    pid = ids & ~np.uint32(QUAD)
    if not np.array_equal(np.sort(pid), np.arange(n, dtype=np.uint32)):
        return ["ids are not a permutation of the primitive IDs"]
    f = faces[pid]
    v0 = verts[f[:, 0]]
    quad = f[:, 3] != TRI
    if not np.array_equal(prims[:, 0:3], v0) or not np.array_equal(prims[:, 4:7], (verts[f[:, 1]] - v0).astype(np.float32)):
        problems.append("primitive records differ from faces")
    idx = f.astype(np.int64).copy()
    idx[~quad, 3] = idx[~quad, 2]
    P = verts[idx].astype(np.float64)
    plo, phi = P.min(1), P.max(1)
    nn = len(wnodes)
    seen = np.zeros(n, np.int32)
    node_seen = np.zeros(nn, np.int32)
    max_depth = 0
    st = [(0, np.full(3, -np.inf), np.full(3, np.inf), 1)]
    while st:
        r, clo, chi, d = st.pop()
        if r >= nn:
            problems.append(f"node index {r} >= {nn}")
            continue
        node_seen[r] += 1
        if node_seen[r] > 1:
            problems.append(f"node {r} reached twice")
            continue
        max_depth = max(max_depth, d)
        w = wnodes[r]
        org = w[0:3].view(np.float32).astype(np.float64)
        e = [(int(w[3]) >> (8 * a)) & 0xFF for a in range(3)]
        scale = np.array([2.0 ** (x - 127) for x in e])
        imask = int(w[3]) >> 24
        child_base, prim_base = int(w[4]), int(w[5])
        for slot in range(8):
            mw = w[6] if slot < 4 else w[7]
            mb = _byte(mw, slot & 3)
            inner = (imask >> slot) & 1
            if mb == 0:
                if inner:
                    problems.append(f"node {r} slot {slot}: imask set on an empty slot")
                continue
            hi_word = 1 if slot >= 4 else 0
            ql = np.array([_byte(w[8 + hi_word], slot & 3), _byte(w[10 + hi_word], slot & 3), _byte(w[12 + hi_word], slot & 3)])
            qh = np.array([_byte(w[14 + hi_word], slot & 3), _byte(w[16 + hi_word], slot & 3), _byte(w[18 + hi_word], slot & 3)])
            blo, bhi = org + ql * scale, org + qh * scale
            nlo, nhi = np.maximum(clo, blo), np.minimum(chi, bhi)
            if (mb & 31) >= 24:
                if not inner or (mb & 7) != slot:
                    problems.append(f"node {r} slot {slot}: internal meta {mb:#x} disagrees with imask {imask:#x}")
                    continue
                c = child_base + bin(imask & ((1 << slot) - 1)).count("1")
                st.append((c, nlo, nhi, d + 1))
            else:
                if inner:
                    problems.append(f"node {r} slot {slot}: leaf meta with imask bit set")
                u = mb >> 5
                if u not in (1, 3, 7):
                    problems.append(f"node {r} slot {slot}: bad unary count {u}")
                    continue
                cnt, off = bin(u).count("1"), mb & 31
                a, b = prim_base + off, prim_base + off + cnt
                if off + cnt > 24 or b > n:
                    problems.append(f"node {r} slot {slot}: primitives {a}..{b} out of range")
                    continue
                seen[a:b] += 1
                if (plo[a:b] < nlo).any() or (phi[a:b] > nhi).any():
                    problems.append(f"node {r} slot {slot}: a primitive lies outside a box on its path")
    if (node_seen == 0).any():
        problems.append(f"{int((node_seen == 0).sum())} nodes unreached")
    if not (seen == 1).all():
        problems.append(f"{int((seen == 0).sum())} slots unreached, {int((seen > 1).sum())} reached twice")
    if max_depth != depth:
        problems.append(f"depth {max_depth} != reported {depth}")
    return problems
