"""Seeded synthetic workloads (numpy PCG64 generators).

Each generator returns plain arrays in the layout the C ABI takes:
vertices float32 [nv,3]; faces uint32 [nf,4] with column 3 == 0xFFFFFFFF for
a triangle (a quad keeps 4 indices and stays ONE primitive, as in
src/geometry/object/object_mesh.cc:96-112); rays float32 [n,8] in the
gbrt_ray layout (ox, oy, oz, tmin, dx, dy, dz, tmax) with tmax < 0 meaning
unbounded (include/geometry/ray.h:43-48, accelerator.h:91).
"""
import math

import numpy as np

TRI = 0xFFFFFFFF


def random_triangles(n, seed=1, spread=0.01):
    """Triangle soup: centroids uniform in the unit cube, each vertex offset
    from its centroid by U[-spread, spread] per axis (1,048,576 triangles in
    the traversal micro-benchmark)."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3), dtype=np.float64)
    off = rng.uniform(-spread, spread, size=(n, 3, 3))
    verts = (c + off).astype(np.float32).reshape(-1, 3)
    faces = np.empty((n, 4), np.uint32)
    faces[:, :3] = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    faces[:, 3] = TRI
    return verts, faces


def random_rays(n, seed=2, lo=-0.2, hi=1.2, tmin=0.0, tmax=-1.0):
    """Incoherent rays: origins uniform in [lo,hi]^3, directions uniform on
    the sphere (z = 1-2u, phi = 2 pi v)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    u = rng.random(n)
    v = rng.random(n)
    z = 1.0 - 2.0 * u
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * math.pi * v
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = tmin
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays


def _box_quads(corner_lo, corner_hi, yaw_deg=0.0, center=None):
    """Axis-aligned (optionally yawed about +y) box as 6 quads."""
    x0, y0, z0 = corner_lo
    x1, y1, z1 = corner_hi
    p = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float64)
    if yaw_deg:
        cx = center if center is not None else p.mean(axis=0)
        a = math.radians(yaw_deg)
        R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
        p = (p - cx) @ R.T + cx
    q = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [3, 7, 6, 2], [0, 4, 7, 3], [1, 2, 6, 5]]
    return p, np.array(q, np.uint32)


def cornell_mesh(as_quads=True):
    """Cornell-style box [-1,1]x[0,2]x[-1,1] (floor, ceiling, back, left, right
    walls) with two yawed boxes (0.6 m at +17 deg, 1.2 m at -20 deg).
    Returns (verts, faces, face_group) with groups 0 grey walls, 1 red,
    2 green, 3 short box, 4 tall box."""
    V, F, G = [], [], []

    def add(pts, quads, g):
        base = sum(len(v) for v in V)
        V.append(np.asarray(pts, np.float64))
        for q in quads:
            if as_quads:
                F.append([base + q[0], base + q[1], base + q[2], base + q[3]]); G.append(g)
            else:
                F.append([base + q[0], base + q[1], base + q[2], TRI]); G.append(g)
                F.append([base + q[0], base + q[2], base + q[3], TRI]); G.append(g)

    walls = {
        "floor": ([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], 0),
        "ceiling": ([[-1, 2, -1], [-1, 2, 1], [1, 2, 1], [1, 2, -1]], 0),
        "back": ([[-1, 0, -1], [-1, 2, -1], [1, 2, -1], [1, 0, -1]], 0),
        "left": ([[-1, 0, -1], [-1, 0, 1], [-1, 2, 1], [-1, 2, -1]], 1),
        "right": ([[1, 0, -1], [1, 2, -1], [1, 2, 1], [1, 0, 1]], 2),
    }
    for pts, g in walls.values():
        add(pts, [[0, 1, 2, 3]], g)
    p, q = _box_quads((0.05, 0.0, -0.05), (0.65, 0.6, 0.55), 17.0)
    add(p, q, 3)
    p, q = _box_quads((-0.7, 0.0, -0.7), (-0.1, 1.2, -0.1), -20.0)
    add(p, q, 4)
    verts = np.concatenate(V).astype(np.float32)
    faces = np.array(F, np.uint32)
    return verts, faces, np.array(G, np.int32)


def perlin_noise(p, seed=3):
    """Improved Perlin gradient noise (Perlin 2002: quintic fade, 12 edge
    gradients, seeded permutation) at points p [n, 3]; values in about [-1, 1]."""
    perm = np.random.default_rng(seed).permutation(256)
    perm = np.concatenate([perm, perm])
    grads = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                      [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], np.float64)
    p = np.asarray(p, np.float64)
    pi = np.floor(p).astype(np.int64)
    f = p - pi
    pi &= 255
    fade = f * f * f * (f * (f * 6.0 - 15.0) + 10.0)

    def grad(ix, iy, iz, dx, dy, dz):
        h = perm[perm[perm[ix] + iy] + iz] % 12
        g = grads[h]
        return g[:, 0] * dx + g[:, 1] * dy + g[:, 2] * dz
    x, y, z = pi[:, 0], pi[:, 1], pi[:, 2]
    fx, fy, fz = f[:, 0], f[:, 1], f[:, 2]
    c = {}
    for a in (0, 1):
        for b in (0, 1):
            for d in (0, 1):
                c[a, b, d] = grad(x + a, y + b, z + d, fx - a, fy - b, fz - d)
    lerp = lambda t, u, v: u + t * (v - u)
    x00 = lerp(fade[:, 0], c[0, 0, 0], c[1, 0, 0]); x10 = lerp(fade[:, 0], c[0, 1, 0], c[1, 1, 0])
    x01 = lerp(fade[:, 0], c[0, 0, 1], c[1, 0, 1]); x11 = lerp(fade[:, 0], c[0, 1, 1], c[1, 1, 1])
    return lerp(fade[:, 2], lerp(fade[:, 1], x00, x10), lerp(fade[:, 1], x01, x11))


def perlin_sphere(nu=2048, nv=512, amplitude=0.05, frequency=4.0, seed=3):
    """Unit sphere tessellated into nu x nv quads (2 nu nv triangles: 2,097,152
    at the defaults) displaced along the normal by amplitude x Perlin noise.
    Returns (vertices float32 [n, 3], faces uint32 [m, 4] TRI-marked)."""
    P, F = uv_sphere((0.0, 0.0, 0.0), 1.0, nu, nv)
    n = P / np.maximum(np.linalg.norm(P, axis=1, keepdims=True), 1e-12)
    P = n * (1.0 + amplitude * perlin_noise(n * frequency + 17.0, seed))[:, None]
    return P.astype(np.float32), np.concatenate([F, np.full((len(F), 1), TRI)], 1).astype(np.uint32)


def camera_rays(width, height, eye, target, up=(0.0, 1.0, 0.0), fov_deg=40.0, seed=None):
    """Pinhole primary rays through pixel centres (or jittered when seed is
    given), one per pixel, row-major from the top-left."""
    eye = np.asarray(eye, np.float64)
    w = np.asarray(target, np.float64) - eye
    w /= np.linalg.norm(w)
    r = np.cross(w, np.asarray(up, np.float64)); r /= np.linalg.norm(r)
    u = np.cross(r, w)
    th = math.tan(math.radians(fov_deg) * 0.5)
    aspect = height / width
    jy, jx = np.mgrid[0:height, 0:width].astype(np.float64)
    if seed is not None:
        rng = np.random.default_rng(seed)
        jx += rng.random(jx.shape); jy += rng.random(jy.shape)
    else:
        jx += 0.5; jy += 0.5
    px = (2.0 * jx / width - 1.0) * th
    py = (1.0 - 2.0 * jy / height) * th * aspect
    d = w[None, None, :] + px[..., None] * r[None, None, :] + py[..., None] * u[None, None, :]
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    rays = np.empty((height * width, 8), np.float32)
    rays[:, 0:3] = eye
    rays[:, 3] = 0.0
    rays[:, 4:7] = d.reshape(-1, 3)
    rays[:, 7] = -1.0
    return rays


# ---- scene descriptions for the renderers -------------------------------
# A scene is a plain dict: materials (ordered), objects (name, material,
# vertices, faces), lights, camera and integrator parameters, in the
# vocabulary of the reference's ParamMaps (shinydiffusemat "color",
# light_mat "color"/"power", arealight "corner"/"point1"/"point2"/"color"/
# "power"/"samples", perspective camera "from"/"to"/"up"/"focal",
# pathtracing "path_samples"/"bounces"/"russian_roulette_min_bounces").

def glossy_material(diffuse_color, glossy_color=(0.9, 0.9, 0.9), exponent=100.0, glossy_reflect=0.5,
                    diffuse_reflect=1.0):
    """A "glossy" material tuple: (type, diffuse_color, color, exponent,
    glossy_reflect, diffuse_reflect); as_diffuse keeps its default (true)."""
    return ("glossy", tuple(diffuse_color), tuple(glossy_color), float(exponent), float(glossy_reflect),
            float(diffuse_reflect))


def glass_material(ior=1.5, filter_color=(1.0, 1.0, 1.0), transmit_filter=0.0, mirror_color=(1.0, 1.0, 1.0), fake_shadows=False):
    """A "glass" material tuple: (type, IOR, filter_color, transmit_filter,
    mirror_color[, {"fake_shadows": True}]); the filter colour acts in
    proportion to transmit_filter; fake_shadows makes it transparent to
    shadow rays of integrators with transpShad."""
    m = ("glass", float(ior), tuple(filter_color), float(transmit_filter), tuple(mirror_color))
    return m + ({"fake_shadows": True},) if fake_shadows else m


def rough_glass_material(ior=1.5, alpha=0.1, filter_color=(1.0, 1.0, 1.0), transmit_filter=0.0, mirror_color=(1.0, 1.0, 1.0),
                         fake_shadows=False):
    """A "rough_glass" material tuple: (type, IOR, alpha, filter_color,
    transmit_filter, mirror_color[, {"fake_shadows": True}])."""
    m = ("rough_glass", float(ior), float(alpha), tuple(filter_color), float(transmit_filter), tuple(mirror_color))
    return m + ({"fake_shadows": True},) if fake_shadows else m


def icosphere(center, radius, subdiv):
    """Sphere mesh from a subdivided icosahedron: 20 * 4**subdiv outward-facing
    triangles.  Returns (vertices float32 [n,3], faces uint32 [m,4] TRI-marked)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.asarray(v, np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                mid[key] = len(V) - 1
            return mid[key]
        nf = []
        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    P = np.asarray(V) * float(radius) + np.asarray(center, np.float64)
    out = []
    for a, b, c in F:
        n = np.cross(P[b] - P[a], P[c] - P[a])
        if np.dot(n, (P[a] + P[b] + P[c]) / 3.0 - np.asarray(center)) < 0:
            b, c = c, b
        out.append([a, b, c, TRI])
    return P.astype(np.float32), np.asarray(out, np.uint32)


def cornell_scene(res=512, light_samples=4, bounces=5, rr_min=3, path_samples=1, glossy=False, glass=False, point_light=False,
                  shiny=False, transparent_shadows=None):
    """The Cornell-box configuration: 34 triangles of walls and boxes
    (shinydiffuse, grey 0.75 / red / green), a 0.5 x 0.5 m ceiling area light
    of colour (17,12,4) at y = 1.999 with a 2-triangle light_mat emitter,
    40-degree pinhole camera (focal 1.3737) from (0,1,3.7).  glossy=True
    makes the tall box glossy (exponent 100) and the floor glossy (exponent 20).
    glass=True adds a glass sphere (IOR 1.5, r 0.25, 320 triangles) on the
    short box and a rough-glass sphere (IOR 1.5, alpha 0.2, r 0.3) at the
    front left, both rendered through the recursive split.  point_light=True
    replaces the area light (and its emitter) by a pointlight at (0, 1.8, 0.2)
    of power 3.  shiny=True gives the shinydiffuse layers work: the tall box
    a Fresnel mirror (specular_reflect 0.8, IOR 1.5), the short box
    transparency 0.5 (transmit_filter 0.7) with translucency 0.3, the green
    wall a plain 0.4 mirror over its diffuse layer, the red wall emit 0.3.
    transparent_shadows=D turns on the integrator's transparent shadows
    ("transpShad", "shadowDepth" D); with glass the balls then take
    fake_shadows (the glass ball tinted: filter colour (0.9, 0.7, 0.4),
    transmit_filter 0.5)."""
    verts, faces, groups = cornell_mesh(as_quads=False)
    mats = {"grey": ("shinydiffusemat", (0.75, 0.75, 0.75)),
            "red": ("shinydiffusemat", (0.63, 0.065, 0.05)),
            "green": ("shinydiffusemat", (0.14, 0.45, 0.09)),
            "emitter": ("light_mat", (17.0, 12.0, 4.0), 1.0)}
    gmat = {0: "grey", 1: "red", 2: "green", 3: "grey", 4: "grey"}
    if shiny:
        feats = {"mirror", "fresnel", "transparent", "translucent", "emit"} if shiny is True else set(shiny)
        if "emit" in feats:
            mats["red"] = ("shinydiffusemat", (0.63, 0.065, 0.05), {"emit": 0.3})
        if "mirror" in feats:
            mats["green"] = ("shinydiffusemat", (0.14, 0.45, 0.09), {"specular_reflect": 0.4, "mirror_color": (0.8, 1.0, 0.8)})
        if "fresnel" in feats:
            mats["fresnel_box"] = ("shinydiffusemat", (0.75, 0.75, 0.75),
                                   {"specular_reflect": 0.8, "fresnel_effect": True, "IOR": 1.5, "mirror_color": (0.9, 0.95, 1.0)})
            gmat[4] = "fresnel_box"
        clear = {}
        if "transparent" in feats:
            clear.update({"transparency": 0.5, "transmit_filter": 0.7})
        if "translucent" in feats:
            clear.update({"translucency": 0.3, "diffuse_reflect": 0.8})
        if clear:
            mats["clear_box"] = ("shinydiffusemat", (0.2, 0.6, 0.9), clear)
            gmat[3] = "clear_box"
    if glossy:
        mats["glossy_box"] = glossy_material((0.75, 0.75, 0.75), exponent=100.0)
        mats["glossy_floor"] = glossy_material((0.75, 0.75, 0.75), exponent=20.0, glossy_reflect=0.4)
        gmat[4] = "glossy_box"
    if glossy:
        groups = groups.copy()
        groups[0:2] = 5          # the floor's two triangles get their own object
        gmat[5] = "glossy_floor"
    objects = []
    for g in sorted(set(groups.tolist())):
        sel = np.where(groups == g)[0]
        f = faces[sel]
        used = np.unique(f[:, :3])
        remap = {int(u): i for i, u in enumerate(used)}
        ff = np.array([[remap[int(x)] for x in row[:3]] + [TRI] for row in f], np.uint32)
        v = verts[used]
        if g == 3 and transparent_shadows is not None:
            # the short box 2 mm above the floor: its bottom face would be
            # coplanar with the floor, and a camera path through the
            # transparent box would then land on an exact closest-hit tie
            v = v + np.array([0.0, 0.002, 0.0], v.dtype)
        objects.append({"name": f"group{g}", "material": gmat[g], "vertices": v, "faces": ff})
    if glass:
        fake = transparent_shadows is not None
        mats["glass"] = glass_material(1.5, filter_color=(0.9, 0.7, 0.4), transmit_filter=0.5 if fake else 0.0,
                                       fake_shadows=fake) if fake else glass_material(1.5)
        mats["rough_glass"] = rough_glass_material(1.5, 0.2, fake_shadows=fake)
        v, f = icosphere((0.35, 0.85, 0.25), 0.25, 2)
        objects.append({"name": "glass_ball", "material": "glass", "vertices": v, "faces": f})
        v, f = icosphere((-0.5, 0.3, 0.55), 0.3, 2)
        objects.append({"name": "rough_ball", "material": "rough_glass", "vertices": v, "faces": f})
    c = np.array([-0.25, 1.999, -0.25])
    x = np.array([0.5, 0.0, 0.0])
    z = np.array([0.0, 0.0, 0.5])
    if point_light:
        del mats["emitter"]
        lights = [{"type": "pointlight", "from": (0.0, 1.8, 0.2), "color": (1.0, 0.9, 0.8), "power": 3.0}]
    else:
        lv = np.array([c, c + x, c + x + z, c + z], np.float32)
        objects.append({"name": "lamp", "material": "emitter", "vertices": lv,
                        "faces": np.array([[0, 1, 2, TRI], [0, 2, 3, TRI]], np.uint32)})
        lights = [{"type": "arealight", "corner": tuple(c), "point1": tuple(c + x), "point2": tuple(c + z),
                   "color": (17.0, 12.0, 4.0), "power": 1.0, "samples": light_samples}]
    camera = {"from": (0.0, 1.0, 3.7), "to": (0.0, 1.0, 0.0), "up": (0.0, 2.0, 3.7),
              "resx": res, "resy": res, "focal": 1.3737}
    integ = {"type": "pathtracing", "path_samples": path_samples, "bounces": bounces,
             "russian_roulette_min_bounces": rr_min}
    if transparent_shadows is not None:
        # transparent_shadows = shadowDepth; the glass balls get fake_shadows
        integ.update({"transpShad": True, "shadowDepth": int(transparent_shadows)})
    return {"materials": mats, "objects": objects, "lights": lights, "camera": camera, "integrator": integ}


def flatten(scene):
    """Concatenate objects in order into one mesh: (vertices, faces,
    per-face material index, material names).  Face order = primitive IDs
    (objects in creation order, faces in insertion order)."""
    names = list(scene["materials"].keys())
    V, F, M = [], [], []
    base = 0
    for o in scene["objects"]:
        v = np.asarray(o["vertices"], np.float32)
        f = np.asarray(o["faces"], np.uint32).copy()
        tri = f[:, 3] == TRI
        f[:, :3] += base
        f[~tri, 3] += base
        V.append(v); F.append(f)
        M.append(np.full(len(f), names.index(o["material"]), np.int32))
        base += len(v)
    return np.concatenate(V), np.concatenate(F), np.concatenate(M), names


def flatten_uvs(scene):
    """Texture coordinates of the flattened mesh: (uv [n, 2] float32, face uv
    indices [faces, 4] uint32), or (None, None) when no object has "uvs".
    An object's "face_uvs" index its own "uvs" (4th unused for triangles);
    objects without uvs get their faces' first uv indices pointing at a
    (0, 0) entry, which only an untextured material reads."""
    if not any("uvs" in o for o in scene["objects"]):
        return None, None
    U, FU = [np.zeros((1, 2), np.float32)], []
    base = 1
    for o in scene["objects"]:
        nf = len(o["faces"])
        if "uvs" in o:
            uv = np.asarray(o["uvs"], np.float32).reshape(-1, 2)
            fu = np.asarray(o["face_uvs"], np.uint32).reshape(nf, 4).copy()
            tri = np.asarray(o["faces"], np.uint32)[:, 3] == TRI
            fu[:, :3] += base
            fu[~tri, 3] += base
            fu[tri, 3] = 0
            U.append(uv)
            FU.append(fu)
            base += len(uv)
        else:
            FU.append(np.zeros((nf, 4), np.uint32))
    return np.concatenate(U), np.concatenate(FU)


def checker_image(w=16, h=16, c0=(0.9, 0.2, 0.1), c1=(0.1, 0.3, 0.8), seed=7):
    """A w x h RGBA float32 image: a 4 x 4 checker of two colours with a
    seeded per-texel tint (so the bilinear weights matter)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    sel = ((x * 4 // w) + (y * 4 // h)) % 2 == 0
    img = np.where(sel[..., None], np.asarray(c0, np.float32), np.asarray(c1, np.float32))
    img = img * rng.uniform(0.7, 1.0, (h, w, 1)).astype(np.float32)
    return np.concatenate([img, np.ones((h, w, 1), np.float32)], -1).astype(np.float32)


def textured_cornell_scene(res=64, **kw):
    """The Cornell box with image textures: the back wall carries uvs
    (0..1 across it) and a UV-mapped checker texture (bilinear, repeat
    x 2 / y 1, mirror_x); the tall box takes a second texture through global
    coordinates with cube mapping (scale 1.5, offset, clip extend, no
    interpolation) through a layer node (multiply, colfac 0.8 over the
    material colour); the short box a checker-clipped texture (odd tiles,
    checker_dist 0.2) in global coordinates.  Everything else is the plain
    Cornell box.  interpolate (e.g. "bicubic") replaces the interpolation
    of all three textures."""
    interpolate = kw.pop("interpolate", None)
    sc = cornell_scene(res=res, **kw)
    sc["textures"] = {
        "checker": {"image": checker_image(16, 16), "interpolate": "bilinear", "clipping": "repeat",
                    "xrepeat": 2, "yrepeat": 1, "mirror_x": True, "texco": "uv", "mapping": "plain"},
        "tiles": {"image": checker_image(8, 8, (0.8, 0.8, 0.3), (0.2, 0.7, 0.3), seed=11), "interpolate": "none",
                  "clipping": "extend", "texco": "global", "mapping": "cube", "scale": (1.5, 1.5, 1.5),
                  "offset": (0.1, 0.0, 0.2), "adj_intensity": 1.1, "adj_contrast": 0.9,
                  "layer": {"blend_mode": "multiply", "colfac": 0.8, "upper_color": (0.75, 0.75, 0.75, 1.0)}},
        "checks": {"image": checker_image(8, 8, (0.9, 0.5, 0.2), (0.3, 0.3, 0.9), seed=13), "interpolate": "bilinear",
                   "clipping": "checker", "checker_dist": 0.2, "texco": "global", "mapping": "plain",
                   "scale": (2.0, 2.0, 2.0)},
    }
    if interpolate:
        for t in sc["textures"].values():
            t["interpolate"] = interpolate
    sc["materials"]["back_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75), {"diffuse_texture": "checker"})
    sc["materials"]["box_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75), {"diffuse_texture": "tiles"})
    sc["materials"]["box2_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75), {"diffuse_texture": "checks"})
    objs = []
    for o in sc["objects"]:
        v = np.asarray(o["vertices"], np.float32)
        f = np.asarray(o["faces"], np.uint32)
        if o["name"] == "group0":
            # the back wall's triangles (z = -1 plane) get their own textured object
            back = np.all(np.abs(v[f[:, :3]][:, :, 2] + 1.0) < 1e-6, axis=1)
            rest = f[~back]
            fb = f[back]
            used = np.unique(fb[:, :3])
            remap = {int(u): i for i, u in enumerate(used)}
            vb = v[used]
            fbb = np.array([[remap[int(x)] for x in row[:3]] + [TRI] for row in fb], np.uint32)
            uvs = np.stack([(vb[:, 0] + 1.0) * 0.5, vb[:, 1] * 0.5], -1).astype(np.float32)
            fuv = np.concatenate([fbb[:, :3], np.zeros((len(fbb), 1), np.uint32)], 1)
            objs.append({"name": "group0", "material": o["material"], "vertices": v, "faces": rest})
            objs.append({"name": "back_wall", "material": "back_tex", "vertices": vb, "faces": fbb,
                         "uvs": uvs, "face_uvs": fuv})
        elif o["name"] == "group4":
            objs.append({**o, "material": "box_tex"})
        elif o["name"] == "group3":
            objs.append({**o, "material": "box2_tex"})
        else:
            objs.append(o)
    sc["objects"] = objs
    return sc


def procedural_cornell_scene(noise_tables, res=64, **kw):
    """The Cornell box with procedural textures on every surface
    (noise_tables: the reference's noise tables, as gbrt.noise_tables
    takes them): marble over the floor / ceiling / back wall (global
    coordinates, scale 2), blender-noise clouds through an HSV colour ramp
    on the red wall, voronoi position-outline colour cells on the green
    wall, wood rings (saw) on the short box through a multiply layer node
    over the material colour, a ridged Musgrave fractal on the tall box
    through tube mapping with colour adjustments, and distorted noise on
    the light's emitter surround.  Everything else is the plain Cornell
    box."""
    sc = cornell_scene(res=res, **kw)
    sc["noise_tables"] = noise_tables
    sc["textures"] = {
        "marble": {"type": "marble", "noise_type": "newperlin", "depth": 3, "turbulence": 4.0, "sharpness": 2.0,
                   "color1": (0.85, 0.82, 0.75), "color2": (0.35, 0.3, 0.28), "mapper": {"scale": (2.0, 2.0, 2.0)}},
        "clouds": {"type": "clouds", "noise_type": "blender", "depth": 3, "size": 0.6, "hard": True,
                   "ramp_num_items": 3, "ramp_color_mode": "HSV", "ramp_item_0_color": (0.7, 0.05, 0.05, 1.0),
                   "ramp_item_0_position": 0.2, "ramp_item_1_color": (0.9, 0.5, 0.1, 1.0), "ramp_item_1_position": 0.5,
                   "ramp_item_2_color": (0.5, 0.1, 0.4, 1.0), "ramp_item_2_position": 0.8},
        "cells": {"type": "voronoi", "color_mode": "position-outline", "distance_metric": "manhattan", "size": 4.0,
                  "weight1": 1.0, "weight2": -0.4, "adj_mult_factor_green": 1.2, "adj_saturation": 0.7},
        "wood": {"type": "wood", "wood_type": "rings", "shape": "saw", "noise_type": "stdperlin", "turbulence": 0.4,
                 "depth": 2, "color1": (0.6, 0.35, 0.15), "color2": (0.95, 0.75, 0.45), "mapper": {"scale": (3.0, 3.0, 3.0)},
                 "layer": {"blend_mode": "multiply", "colfac": 0.9, "upper_color": (0.75, 0.75, 0.75, 1.0)}},
        "fractal": {"type": "musgrave", "musgrave_type": "ridgedmf", "noise_type": "newperlin", "octaves": 3.5, "H": 0.9,
                    "lacunarity": 2.1, "offset": 1.0, "gain": 1.6, "intensity": 0.55, "size": 1.7,
                    "color1": (0.2, 0.3, 0.6), "color2": (0.95, 0.95, 0.8), "adj_contrast": 1.2, "adj_clamp": True,
                    "mapper": {"mapping": "tube", "scale": (1.0, 1.0, 1.0), "offset": (0.1, 0.0, 0.0)}},
    }
    for name, tex in (("grey", "marble"), ("red", "clouds"), ("green", "cells")):
        m = sc["materials"][name]
        sc["materials"][name] = ("shinydiffusemat", m[1], {"diffuse_texture": tex})
    sc["materials"]["short_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75), {"diffuse_texture": "wood"})
    sc["materials"]["tall_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75), {"diffuse_texture": "fractal"})
    for o in sc["objects"]:
        if o["name"] == "group3":
            o["material"] = "short_tex"
        elif o["name"] == "group4":
            o["material"] = "tall_tex"
    return sc


def node_cornell_scene(noise_tables, res=64, **kw):
    """The glass and glossy Cornell box with shader node trees on every
    colour slot: mix nodes in each blend mode (multiply with a texture's
    scalar as factor, overlay, darken, lighten, screen, subtract,
    difference, add), value nodes, a chain of two layer nodes (the second
    stencilled over the first through upper_layer), texture mappers over
    procedural and image textures; slots: shinydiffuse and glossy diffuse,
    glossy colour, glass and rough-glass filter and mirror colours."""
    sc = cornell_scene(res=res, glass=True, glossy=True, **kw)
    sc["noise_tables"] = noise_tables
    sc["textures"] = {
        "marble": {"type": "marble", "noise_type": "newperlin", "depth": 2, "turbulence": 3.0, "color1": (0.9, 0.85, 0.8),
                   "color2": (0.3, 0.25, 0.2)},
        "clouds": {"type": "clouds", "noise_type": "blender", "depth": 3, "size": 0.7, "color1": (0.2, 0.3, 0.5),
                   "color2": (0.9, 0.8, 0.6)},
        "cells": {"type": "voronoi", "color_mode": "position", "size": 3.0, "weight1": 1.0, "weight2": -0.3},
        "checker": {"image": checker_image(8, 8, (0.9, 0.9, 0.2), (0.2, 0.4, 0.9), seed=17), "interpolate": "bilinear",
                    "clipping": "repeat"},
    }
    sc["nodes"] = {
        "m_marble": {"type": "texture_mapper", "texture": "marble", "scale": (2.0, 2.0, 2.0)},
        "m_clouds": {"type": "texture_mapper", "texture": "clouds"},
        "m_cells": {"type": "texture_mapper", "texture": "cells", "scale": (1.5, 1.5, 1.5)},
        "m_check": {"type": "texture_mapper", "texture": "checker", "mapping": "cube", "scale": (1.5, 1.5, 1.5)},
        "v_tint": {"type": "value", "color": (0.9, 0.6, 0.3), "alpha": 0.8, "scalar": 0.4},
        "mix_grey": {"type": "mix", "blend_mode": "multiply", "input1": "m_marble", "input2": "v_tint", "input_factor": "m_clouds"},
        "lay1": {"type": "layer", "input": "m_cells", "upper_color": (0.63, 0.065, 0.05, 1.0), "blend_mode": "mix", "colfac": 0.7},
        "lay2": {"type": "layer", "input": "m_check", "upper_layer": "lay1", "blend_mode": "difference", "colfac": 0.5,
                 "stencil": True},
        "ov": {"type": "mix", "blend_mode": "overlay", "input1": "m_clouds", "color2": (0.2, 0.5, 0.9, 1.0), "cfactor": 0.6},
        "dk": {"type": "mix", "blend_mode": "darken", "input1": "m_cells", "input2": "v_tint", "cfactor": 0.8},
        "lt": {"type": "mix", "blend_mode": "lighten", "input1": "v_tint", "input2": "m_cells", "cfactor": 0.7},
        "scr": {"type": "mix", "blend_mode": "screen", "color1": (0.9, 0.9, 1.0, 1.0), "input2": "m_marble", "cfactor": 0.3},
        "sub": {"type": "mix", "blend_mode": "subtract", "color1": (1.0, 1.0, 1.0, 1.0), "input2": "m_clouds", "cfactor": 0.25},
        "diff": {"type": "mix", "blend_mode": "difference", "input1": "m_check", "input2": "m_cells", "cfactor": 0.5},
        "add": {"type": "mix", "blend_mode": "add", "input1": "v_tint", "input2": "m_marble", "cfactor": 0.2},
    }
    sc["material_shaders"] = {
        "grey": {"diffuse_shader": "mix_grey"},
        "red": {"diffuse_shader": "lay2"},
        "green": {"diffuse_shader": "lt"},
        "glossy_box": {"diffuse_shader": "m_clouds", "glossy_shader": "ov"},
        "glossy_floor": {"diffuse_shader": "diff"},
        "glass": {"filter_color_shader": "scr", "mirror_color_shader": "dk"},
        "rough_glass": {"filter_color_shader": "sub", "mirror_color_shader": "add"},
    }
    return sc


def bump_cornell_scene(noise_tables, res=64, **kw):
    """Bump mapping (bump_shader): the back wall (uv-mapped) bumped by a
    noisy image through uv coordinates (the image branch of the mapper's
    derivative: slopes in texture space through dP/du, dP/dv), the short box
    by a marble texture in global coordinates, the tall box, glossy, by a
    stencilled, negated layer over clouds with a voronoi upper layer, and
    the glass ball by blender-noise clouds; the floor, ceiling and side
    walls stay flat."""
    sc = textured_cornell_scene(res=res, **kw)
    sc["noise_tables"] = noise_tables
    rng = np.random.default_rng(23)
    bumps = rng.random((16, 16, 1)).astype(np.float32)
    img = np.concatenate([bumps, bumps, bumps, np.ones((16, 16, 1), np.float32)], -1)
    sc["textures"] = {
        "bumps": {"image": img, "interpolate": "bilinear", "clipping": "repeat"},
        "marble": {"type": "marble", "noise_type": "newperlin", "depth": 2, "turbulence": 2.0},
        "clouds": {"type": "clouds", "noise_type": "newperlin", "depth": 3, "size": 0.5},
        "cells": {"type": "voronoi", "size": 2.0},
        "noise": {"type": "clouds", "noise_type": "blender", "depth": 2, "size": 0.3},
    }
    sc["nodes"] = {
        "b_img": {"type": "texture_mapper", "texture": "bumps", "texco": "uv", "bump_strength": 2.0},
        "b_marble": {"type": "texture_mapper", "texture": "marble", "scale": (3.0, 3.0, 3.0), "bump_strength": 4.0},
        "b_clouds": {"type": "texture_mapper", "texture": "clouds", "bump_strength": 3.0},
        "b_cells": {"type": "texture_mapper", "texture": "cells", "bump_strength": 1.5},
        "b_up": {"type": "layer", "input": "b_cells"},
        "b_layer": {"type": "layer", "input": "b_clouds", "upper_layer": "b_up", "negative": True, "stencil": True},
        "b_noise": {"type": "texture_mapper", "texture": "noise", "bump_strength": 2.5},
    }
    sc["materials"]["back_tex"] = ("shinydiffusemat", (0.75, 0.75, 0.75))
    sc["materials"]["box2_tex"] = ("shinydiffusemat", (0.8, 0.7, 0.4))
    sc["materials"]["box_tex"] = glossy_material((0.6, 0.65, 0.75), exponent=80.0, glossy_reflect=0.6)
    sc["materials"]["glass"] = glass_material(1.5)
    v, f = icosphere((0.35, 0.85, 0.25), 0.25, 2)
    sc["objects"].insert(-1, {"name": "glass_ball", "material": "glass", "vertices": v, "faces": f})
    sc["material_shaders"] = {
        "back_tex": {"bump_shader": "b_img"},
        "box2_tex": {"bump_shader": "b_marble"},
        "box_tex": {"bump_shader": "b_layer"},
        "glass": {"bump_shader": "b_noise"},
    }
    return sc


def cornell_sppm_scene(res=48, photons=100000, passes=8, bounces=5, pm_ire=False, photon_radius=0.1, search_num=10):
    """The glass Cornell box (a glass and a rough-glass ball) rendered by the
    "SPPM" integrator: caustics under the balls come from the photon
    gathers, the rest from direct light and the specular split."""
    sc = cornell_scene(res=res, glass=True)
    sc["integrator"] = {"type": "SPPM", "photons": int(photons), "passNums": int(passes), "bounces": int(bounces),
                        "raydepth": 5}
    if pm_ire:
        sc["integrator"].update({"pmIRE": True, "photonRadius": float(photon_radius), "searchNum": int(search_num)})
    return sc


def _box_tris(center, size, yaw, subdiv=1):
    """Triangles of a yawed box, each face subdivided into subdiv x subdiv
    quads (2 triangles each), outward-facing.  Returns (vertices, tri indices)."""
    h = 0.5 * np.asarray(size, np.float64)
    c, s = math.cos(yaw), math.sin(yaw)
    R = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    # (origin corner, u edge, v edge) per face with u x v pointing outwards
    faces = [((-1, -1, -1), (0, 2, 0), (2, 0, 0)), ((-1, -1, 1), (2, 0, 0), (0, 2, 0)),
             ((-1, -1, -1), (2, 0, 0), (0, 0, 2)), ((-1, 1, -1), (0, 0, 2), (2, 0, 0)),
             ((-1, -1, -1), (0, 0, 2), (0, 2, 0)), ((1, -1, -1), (0, 2, 0), (0, 0, 2))]
    V, T = [], []
    n = subdiv
    g = np.linspace(0.0, 1.0, n + 1)
    for o, u, v in faces:
        o, u, v = (np.asarray(x, np.float64) * h for x in (o, u, v))
        base = len(V) * 0
        pts = o[None, None, :] + g[:, None, None] * u[None, None, :] + g[None, :, None] * v[None, None, :]
        off = sum(len(x) for x in V)
        V.append(pts.reshape(-1, 3))
        for i in range(n):
            for j in range(n):
                a = off + i * (n + 1) + j
                b, cc, d = a + (n + 1), a + (n + 1) + 1, a + 1
                T.append([a, b, cc]); T.append([a, cc, d])
    P = np.concatenate(V) @ R.T + np.asarray(center, np.float64)
    return P, np.array(T)


def indoor_scene(n_boxes=463, subdiv=6, res=(960, 540), seed=5, bounces=12, rr_min=4, light_samples=2):
    """Indoor scene lit through a gap: a closed 10 x 4 x 6 m room whose
    1 x 2 m door (in the wall z = 6, x in [4.5, 5.5]) stands ajar by 0.1 m,
    an outdoor 2 x 2 m area light of radiance 200 facing the door 3 m beyond
    it (z = 9), and n_boxes seeded furniture boxes (edges U[0.1, 0.6] m,
    faces tessellated subdiv x subdiv: 463 boxes x 432 = 200,016 triangles)
    with shinydiffuse albedo U[0.2, 0.8] per channel (palette of 32) or, for
    20 % of the boxes, glossy exponent 100 (palette of 8).  Camera inside
    looking at the door wall; max depth 12."""
    rng = np.random.default_rng(seed)
    mats = {}
    for i in range(32):
        mats[f"diff{i}"] = ("shinydiffusemat", tuple(float(x) for x in rng.uniform(0.2, 0.8, 3)))
    for i in range(8):
        mats[f"glossy{i}"] = glossy_material(tuple(float(x) for x in rng.uniform(0.2, 0.8, 3)), exponent=100.0)
    mats["wall"] = ("shinydiffusemat", (0.7, 0.7, 0.7))
    mats["emitter"] = ("light_mat", (1.0, 1.0, 1.0), 200.0)
    objects = []

    def quad_obj(name, mat, pts):
        objects.append({"name": name, "material": mat, "vertices": np.asarray(pts, np.float32),
                        "faces": np.array([[0, 1, 2, TRI], [0, 2, 3, TRI]], np.uint32)})

    W, H, D = 10.0, 4.0, 6.0
    quad_obj("floor", "wall", [[0, 0, 0], [0, 0, D], [W, 0, D], [W, 0, 0]])
    quad_obj("ceiling", "wall", [[0, H, 0], [W, H, 0], [W, H, D], [0, H, D]])
    quad_obj("wall_front", "wall", [[0, 0, 0], [W, 0, 0], [W, H, 0], [0, H, 0]])
    quad_obj("wall_left", "wall", [[0, 0, 0], [0, H, 0], [0, H, D], [0, 0, D]])
    quad_obj("wall_right", "wall", [[W, 0, 0], [W, 0, D], [W, H, D], [W, H, 0]])
    # back wall z = D with a 1 x 2 m door opening at x in [4.5, 5.5]
    quad_obj("wall_back_l", "wall", [[0, 0, D], [0, H, D], [4.5, H, D], [4.5, 0, D]])
    quad_obj("wall_back_r", "wall", [[5.5, 0, D], [5.5, H, D], [W, H, D], [W, 0, D]])
    quad_obj("wall_back_t", "wall", [[4.5, 2, D], [4.5, H, D], [5.5, H, D], [5.5, 2, D]])
    # door leaf hinged at x = 4.5, opened outwards so its free edge leaves a 0.1 m gap
    ang = math.asin(0.1)
    ex, ez = 4.5 + math.cos(ang), D + math.sin(ang)
    quad_obj("door", "wall", [[4.5, 0, D], [4.5, 2, D], [ex, 2, ez], [ex, 0, ez]])
    # furniture boxes, kept out of the door's light path
    V, F, M = [], [], []
    names_d = [f"diff{i}" for i in range(32)]
    names_g = [f"glossy{i}" for i in range(8)]
    for b in range(n_boxes):
        size = rng.uniform(0.1, 0.6, 3)
        while True:
            c = np.array([rng.uniform(0.3, W - 0.3), rng.uniform(0.0, 3.2), rng.uniform(0.3, D - 0.4)])
            if not (3.5 < c[0] < 6.5 and c[2] > 4.2):
                break
        c[1] += 0.5 * size[1]
        p, t = _box_tris(c, size, rng.uniform(0, 2 * math.pi), subdiv)
        V.append(p); F.append(t)
        M.append(names_g[rng.integers(8)] if rng.random() < 0.2 else names_d[rng.integers(32)])
    by_mat = {}
    for v, f, m in zip(V, F, M):
        by_mat.setdefault(m, []).append((v, f))
    for m, lst in sorted(by_mat.items()):
        vv = np.concatenate([v for v, _ in lst]).astype(np.float32)
        offs = np.cumsum([0] + [len(v) for v, _ in lst[:-1]])
        ff = np.concatenate([f + o for o, (_, f) in zip(offs, lst)]).astype(np.uint32)
        faces = np.empty((len(ff), 4), np.uint32); faces[:, :3] = ff; faces[:, 3] = TRI
        objects.append({"name": f"boxes_{m}", "material": m, "vertices": vv, "faces": faces})
    # outdoor light 3 m beyond the gap, facing -z, with its light_mat emitter
    c = (4.0, 0.0, D + 3.0)
    lights = [{"type": "arealight", "corner": c, "point1": (4.0, 2.0, D + 3.0), "point2": (6.0, 0.0, D + 3.0),
               "color": (1.0, 1.0, 1.0), "power": 200.0, "samples": light_samples}]
    quad_obj("lamp", "emitter", [[4, 0, D + 3], [4, 2, D + 3], [6, 2, D + 3], [6, 0, D + 3]])
    camera = {"from": (5.0, 1.6, 0.4), "to": (5.0, 1.1, 6.0), "up": (5.0, 2.6, 0.4),
              "resx": res[0], "resy": res[1], "focal": 1.0}
    integ = {"type": "pathtracing", "path_samples": 1, "bounces": bounces, "russian_roulette_min_bounces": rr_min}
    return {"materials": mats, "objects": objects, "lights": lights, "camera": camera, "integrator": integ}


def caustic_scene(res=(1024, 1024), subdiv=7, diffuse_photons=10_000_000, caustic_photons=10_000_000, final_gather=True,
                  fg_samples=32, radius=0.02, search=50, fg_bounces=2, bounces=3, geodesic=None):
    """Photon-mapping configuration: a glass icosphere (r 0.5, IOR 1.5,
    20 * 4**subdiv triangles; geodesic=freq instead makes a geodesic sphere
    of 20 freq^2 triangles, 200,000 at freq 100) resting on a 4 x 4 m
    shinydiffuse plane (albedo 0.8), lit by a pointlight at (1, 3, 1) of power
    1000; `photonmapping` with caustics, diffuse_search = caustic_mix =
    search, diffuse_radius = caustic_radius = radius, finalGather."""
    mats = {"floor": ("shinydiffusemat", (0.8, 0.8, 0.8)), "glass": glass_material(1.5)}
    plane = np.array([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]], np.float32)
    objects = [{"name": "floor", "material": "floor", "vertices": plane,
                "faces": np.array([[0, 2, 1, TRI], [0, 3, 2, TRI]], np.uint32)}]
    v, f = geodesic_sphere((0.0, 0.5, 0.0), 0.5, geodesic) if geodesic else icosphere((0.0, 0.5, 0.0), 0.5, subdiv)
    objects.append({"name": "ball", "material": "glass", "vertices": v, "faces": f})
    lights = [{"type": "pointlight", "from": (1.0, 3.0, 1.0), "color": (1.0, 1.0, 1.0), "power": 1000.0}]
    rx, ry = (res, res) if isinstance(res, int) else res
    camera = {"from": (0.0, 2.2, 3.6), "to": (0.0, 0.3, 0.0), "up": (0.0, 3.2, 3.6), "resx": rx, "resy": ry, "focal": 1.3737}
    integ = {"type": "photonmapping", "diffuse_photons": int(diffuse_photons), "caustic_photons": int(caustic_photons),
             "caustics": True, "diffuse_search": int(search), "caustic_mix": int(search), "diffuse_radius": float(radius),
             "caustic_radius": float(radius), "finalGather": bool(final_gather), "fg_samples": int(fg_samples),
             "fg_bounces": int(fg_bounces), "bounces": int(bounces), "threads_photons": 1}
    return {"materials": mats, "objects": objects, "lights": lights, "camera": camera, "integrator": integ}


def caustic_scene_small(final_gather):
    """The photon-mapping configuration at test size: 1280-triangle glass
    ball, 200k diffuse and 200k caustic photon paths, 48x48.  Without final
    gather diffuse_radius = 0.01 (the reference takes it as the squared
    radius); with it diffuse_radius = 0.05 and fg_samples 8."""
    kw = dict(res=48, subdiv=3, diffuse_photons=200000, caustic_photons=200000, radius=0.05, search=50, bounces=3)
    if final_gather:
        return caustic_scene(final_gather=True, fg_samples=8, **kw)
    sc = caustic_scene(final_gather=False, **kw)
    sc["integrator"]["diffuse_radius"] = 0.01
    return sc


def cornell_pm_scene(res, final_gather, diffuse_photons=100000):
    """The Cornell box rendered by `photonmapping` (no caustic map): direct
    photon estimate with diffuse_radius 0.005 (the reference takes it as the
    squared radius), or final gather with diffuse_radius 0.1, fg_samples 8,
    fg_bounces 2; diffuse_search 50, photon bounces 3."""
    sc = cornell_scene(res=res)
    sc["integrator"] = {"type": "photonmapping", "diffuse_photons": int(diffuse_photons), "caustic_photons": 0,
                        "caustics": False, "diffuse_search": 50, "diffuse_radius": 0.1 if final_gather else 0.005,
                        "finalGather": bool(final_gather), "fg_samples": 8, "fg_bounces": 2, "bounces": 3,
                        "threads_photons": 1}
    return sc


def geodesic_sphere(center, radius, freq):
    """Class-I geodesic sphere: every icosahedron face cut into freq^2
    triangles (20 freq^2 in all: 200,000 at freq 100), vertices projected
    onto the sphere and shared along the face edges, faces outward."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    n = int(freq)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = ii + jj <= n
    ii, jj = ii[keep], jj[keep]
    local = {(int(a), int(b)): k for k, (a, b) in enumerate(zip(ii, jj))}
    # the freq^2 triangles of one face in local vertex numbers
    tris = []
    for a in range(n):
        for b in range(n - a):
            tris.append((local[(a, b)], local[(a + 1, b)], local[(a, b + 1)]))
            if a + b + 1 < n:
                tris.append((local[(a + 1, b)], local[(a + 1, b + 1)], local[(a, b + 1)]))
    tris = np.asarray(tris, np.int64)
    P, T = [], []
    for f, (A, B, C) in enumerate(F):
        pts = V[A] + np.outer(ii / n, V[B] - V[A]) + np.outer(jj / n, V[C] - V[A])
        P.append(pts / np.linalg.norm(pts, axis=1, keepdims=True))
        T.append(tris + f * len(ii))
    P, T = np.concatenate(P), np.concatenate(T)
    # shared edge vertices: merge points that agree to 1e-9
    key = np.round(P * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)
    remap = np.empty(len(order), np.int64)
    remap[order] = np.arange(len(order))
    P = P[first[order]] * float(radius) + np.asarray(center, np.float64)
    T = remap[inv.reshape(-1)][T]
    # outward orientation
    n_ = np.cross(P[T[:, 1]] - P[T[:, 0]], P[T[:, 2]] - P[T[:, 0]])
    out = np.einsum("ij,ij->i", n_, P[T].mean(1) - np.asarray(center, np.float64)) >= 0
    T[~out] = T[~out][:, [0, 2, 1]]
    faces = np.empty((len(T), 4), np.uint32)
    faces[:, :3] = T
    faces[:, 3] = TRI
    return P.astype(np.float32), faces


def uv_sphere(center, radius, nu, nv):
    """Latitude-longitude sphere: nu x nv quads as 2 nu nv outward triangles."""
    th = np.linspace(0.0, math.pi, nv + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, nu + 1)[:-1]
    P = np.stack([np.outer(np.sin(th), np.cos(ph)), np.repeat(np.cos(th)[:, None], nu, 1), np.outer(np.sin(th), np.sin(ph))], -1)
    P = P.reshape(-1, 3) * radius + np.asarray(center, np.float64)
    i, j = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    a, b = i * nu + j, i * nu + (j + 1) % nu
    c, d = a + nu, b + nu
    F = np.stack([np.stack([a, d, c], -1), np.stack([a, b, d], -1)], 2).reshape(-1, 3)
    return P, F


def torus(center, R, r, nu, nv):
    """Torus around +y: nu x nv quads as 2 nu nv outward triangles."""
    u = np.linspace(0.0, 2.0 * math.pi, nu + 1)[:-1]
    v = np.linspace(0.0, 2.0 * math.pi, nv + 1)[:-1]
    U, V = np.meshgrid(u, v, indexing="ij")
    P = np.stack([(R + r * np.cos(V)) * np.cos(U), r * np.sin(V), (R + r * np.cos(V)) * np.sin(U)], -1).reshape(-1, 3)
    P = P + np.asarray(center, np.float64)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a, b = i * nv + j, i * nv + (j + 1) % nv
    c, d = ((i + 1) % nu) * nv + j, ((i + 1) % nu) * nv + (j + 1) % nv
    F = np.stack([np.stack([a, b, d], -1), np.stack([a, d, c], -1)], 2).reshape(-1, 3)
    return P, F


def torus_quads(center, R, r, nu, nv):
    """Torus around +y as nu x nv quads (one primitive each)."""
    P, F = torus(center, R, r, nu, nv)
    T = F.reshape(-1, 2, 3)
    Q = np.stack([T[:, 0, 0], T[:, 0, 1], T[:, 0, 2], T[:, 1, 2]], -1)   # (a, b, d, c)
    return P.astype(np.float32), Q.astype(np.uint32)


def smooth_cornell_scene(res=64, glass=True):
    """The Cornell box with shading normals: a coarse shinydiffuse icosphere
    (80 triangles) averaged at every vertex (smooth 181), a glossy torus of
    quads smoothed across faces within 40 degrees, the short box smoothed at
    30 degrees (its coplanar triangles share normals, its 90-degree edges stay
    sharp) and, with glass, a glass icosphere (320 triangles, smooth 181) on
    the short box through the recursive split."""
    sc = cornell_scene(res=res)
    sc["materials"]["ball"] = ("shinydiffusemat", (0.8, 0.7, 0.3))
    sc["materials"]["ring"] = glossy_material((0.3, 0.5, 0.8), exponent=60.0, glossy_reflect=0.5)
    v, f = icosphere((-0.45, 0.3, 0.45), 0.3, 1)
    sc["objects"].insert(-1, {"name": "smooth_ball", "material": "ball", "vertices": v, "faces": f, "smooth": 181.0})
    v, f = torus_quads((0.55, 0.08, 0.82), 0.2, 0.08, 16, 10)
    sc["objects"].insert(-1, {"name": "ring", "material": "ring", "vertices": v, "faces": f, "smooth": 40.0})
    for o in sc["objects"]:
        if o["name"] == "group3":
            o["smooth"] = 30.0
    if glass:
        sc["materials"]["glass"] = glass_material(1.5)
        v, f = icosphere((0.35, 0.85, 0.25), 0.25, 2)
        sc["objects"].insert(-1, {"name": "glass_ball", "material": "glass", "vertices": v, "faces": f, "smooth": 181.0})
    return sc


def cornell_pt_variant_scene(res=48, caustic_type="path", caustic_photons=100000, caustic_radius=0.08, caustic_mix=40,
                             no_recursive=False, clamp_indirect=0.0):
    """The glass Cornell box through `pathtracing` with the integrator's
    caustic options: caustic_type path / photon / both / none (photon: a
    caustic photon map of caustic_photons paths, estimated with caustic_mix
    photons within caustic_radius at diffuse camera hits), no_recursive (the
    path loop at every first hit), and the film's AA_clamp_indirect."""
    sc = cornell_scene(res=res, glass=True)
    it = sc["integrator"]
    it["caustic_type"] = caustic_type
    if caustic_type in ("photon", "both"):
        it.update({"caustic_photons": int(caustic_photons), "caustic_radius": float(caustic_radius),
                   "caustic_mix": int(caustic_mix)})
    if no_recursive:
        it["no_recursive"] = True
    if clamp_indirect:
        sc["film"] = {"filter_type": "pixel", "AA_clamp_indirect": float(clamp_indirect)}
    return sc


def batch_scene(i, res=None, spp_scale=1.0):
    """Scene i of the 64-scene batch (seed 1000 + i): about
    round(10^U[3, log10 2e6]) triangles of tessellated spheres and tori under
    random rotations, scales and translations on a ground plane; each object
    50 % shinydiffuse, 30 % glossy (exponent U[50, 500]), 20 % rough_glass
    (IOR 1.5, alpha 0.1); 1-4 quad area lights (power U[5, 50]) with their
    light_mat emitters; resolution from {256, 512, 1024}; pathtracing,
    bounces 8.  res overrides the resolution (tests)."""
    rng = np.random.default_rng(1000 + i)
    n_tris = int(round(10 ** rng.uniform(3.0, math.log10(2e6))))
    n_obj = int(rng.integers(1, 6))
    mats = {"ground": ("shinydiffusemat", (0.6, 0.6, 0.6))}
    objects = [{"name": "ground", "material": "ground",
                "vertices": np.array([[-8, 0, -8], [8, 0, -8], [8, 0, 8], [-8, 0, 8]], np.float32),
                "faces": np.array([[0, 2, 1, TRI], [0, 3, 2, TRI]], np.uint32)}]
    per = max(200, n_tris // n_obj)
    for k in range(n_obj):
        u = rng.uniform()
        if u < 0.5:
            mats[f"m{k}"] = ("shinydiffusemat", tuple(float(x) for x in rng.uniform(0.2, 0.8, 3)))
        elif u < 0.8:
            mats[f"m{k}"] = glossy_material(tuple(float(x) for x in rng.uniform(0.2, 0.8, 3)), exponent=float(rng.uniform(50, 500)))
        else:
            mats[f"m{k}"] = rough_glass_material(1.5, 0.1)
        size = float(rng.uniform(0.4, 1.2))
        q = max(4, int(math.sqrt(per / 2.0)))
        if rng.uniform() < 0.5:
            P, F = uv_sphere((0, 0, 0), size, q, q)
        else:
            P, F = torus((0, 0, 0), size, size * float(rng.uniform(0.2, 0.45)), q, q)
        a, b = rng.uniform(0, 2 * math.pi, 2)
        Ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
        Rx = np.array([[1, 0, 0], [0, math.cos(b), -math.sin(b)], [0, math.sin(b), math.cos(b)]])
        S = np.diag(rng.uniform(0.7, 1.3, 3))
        M = Ry @ Rx @ S
        t = np.array([rng.uniform(-3, 3), 0.0, rng.uniform(-3, 3)])
        P = P @ M.T + t
        P[:, 1] += -P[:, 1].min() + 0.001                # rest on the ground
        objects.append({"name": f"o{k}", "material": f"m{k}", "vertices": P.astype(np.float32),
                        "faces": np.concatenate([F, np.full((len(F), 1), TRI)], 1).astype(np.uint32)})
    lights = []
    for k in range(int(rng.integers(1, 5))):
        c = np.array([rng.uniform(-3, 3), rng.uniform(4, 6), rng.uniform(-3, 3)])
        w = float(rng.uniform(0.5, 1.5))
        x, z = np.array([w, 0, 0]), np.array([0, 0, w])
        power = float(rng.uniform(5, 50))
        mats[f"lamp{k}"] = ("light_mat", (1.0, 1.0, 1.0), power)
        lv = np.array([c, c + x, c + x + z, c + z], np.float32)
        objects.append({"name": f"lamp{k}", "material": f"lamp{k}", "vertices": lv,
                        "faces": np.array([[0, 1, 2, TRI], [0, 2, 3, TRI]], np.uint32)})
        lights.append({"type": "arealight", "corner": tuple(c), "point1": tuple(c + x), "point2": tuple(c + z),
                       "color": (1.0, 1.0, 1.0), "power": power, "samples": 1})
    if res is None:
        res = int(rng.choice([256, 512, 1024]))
    cam_a = rng.uniform(0, 2 * math.pi)
    camera = {"from": (9.0 * math.cos(cam_a), 4.0, 9.0 * math.sin(cam_a)), "to": (0.0, 0.5, 0.0),
              "up": (9.0 * math.cos(cam_a), 5.0, 9.0 * math.sin(cam_a)), "resx": res, "resy": res, "focal": 1.3737}
    integ = {"type": "pathtracing", "path_samples": 1, "bounces": 8, "russian_roulette_min_bounces": 3}
    return {"materials": mats, "objects": objects, "lights": lights, "camera": camera, "integrator": integ}


def cornell_dl_scene(res, caustics=True, caustic_photons=200000):
    """The glass Cornell box (glass + rough-glass balls) rendered by
    `directlighting` with a caustic photon map (caustic_radius 0.05,
    caustic_mix 50)."""
    sc = cornell_scene(res=res, glass=True)
    sc["integrator"] = {"type": "directlighting", "caustics": bool(caustics), "caustic_photons": int(caustic_photons),
                        "caustic_radius": 0.05, "caustic_mix": 50, "caustic_depth": 10, "threads_photons": 1}
    return sc
