"""TEST ORACLE bindings (test infrastructure, never the product path).

``OracleScene`` wraps liborc.so, the C restatement of libYafaRay's
ray/primitive acceleration semantics (oracle/traverse_oracle.c).
``run_reference_kdtree`` drives oracle/_ref/kdtree_dump, the reference's own
kd-tree (src/accelerator/accelerator_kdtree_original.cc) compiled from its
sources by oracle/ref/Makefile; it exists only where the reference sources
were available at build time and is used to make and check golden vectors.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_KDTREE = os.path.join(HERE, "_ref", "kdtree_dump")
TRI_MARK = 0xFFFFFFFF

_lib = None


def build():
    """Compile liborc.so (plain C, gcc)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        up = ctypes.POINTER(ctypes.c_uint32)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.orc_scene_create.restype = ctypes.c_void_p
        L.orc_scene_create.argtypes = [fp, ctypes.c_uint32, up, ctypes.c_uint32]
        L.orc_scene_destroy.argtypes = [ctypes.c_void_p]
        L.orc_scene_bound.argtypes = [ctypes.c_void_p, fp]
        L.orc_trace.argtypes = [ctypes.c_void_p, fp, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ip, fp, fp, fp]
        L.orc_mt_intersect.restype = ctypes.c_float
        L.orc_mt_intersect.argtypes = [fp, ctypes.c_int, fp, fp, fp, fp]
        L.orc_bound_cross.restype = ctypes.c_int
        L.orc_bound_cross.argtypes = [fp, fp, fp, ctypes.c_float, fp, fp]
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class OracleScene:
    """CPU restatement of an accelerator over one mesh (faces: uint32 [n,4],
    column 3 == 0xFFFFFFFF for triangles)."""

    def __init__(self, verts, faces):
        self.verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 4)
        L = lib()
        self._h = L.orc_scene_create(_f(self.verts), len(self.verts),
                                     self.faces.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                     len(self.faces))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_scene_destroy(self._h)
            self._h = None

    def bound(self):
        out = np.zeros(6, np.float32)
        lib().orc_scene_bound(self._h, _f(out))
        return out

    def trace(self, rays, mode=0, bruteforce=False, threads=None):
        """rays: float32 [n,8] (ox oy oz tmin dx dy dz tmax).  mode 0 closest
        (Accelerator::intersect), 1 shadow (Accelerator::isShadowed).
        Returns (prim int32, t, u, v)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(rays)
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        if threads is None:
            threads = os.cpu_count() or 1
        lib().orc_trace(self._h, _f(rays), n, int(mode), int(bool(bruteforce)), int(threads),
                        prim.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _f(t), _f(u), _f(v))
        return prim, t, u, v


def reference_available():
    return os.path.exists(REF_KDTREE)


def run_reference_kdtree(verts, faces, rays, mode=0, accel="yafaray-kdtree-original"):
    """Run the compiled reference kd-tree ray by ray.  Returns
    (bound[6], build_s, trace_s, prim, t, u, v)."""
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 4)
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(b"GBRTKD01")
            f.write(struct.pack("<I", len(verts))); f.write(verts.tobytes())
            f.write(struct.pack("<I", len(faces))); f.write(faces.tobytes())
            f.write(struct.pack("<I", len(rays))); f.write(rays.tobytes())
            f.write(struct.pack("<I", mode))
            a = accel.encode()
            f.write(struct.pack("<I", len(a))); f.write(a)
        subprocess.run([REF_KDTREE, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
    bound = np.frombuffer(raw[:24], np.float32).copy()
    build_s, trace_s = struct.unpack("<dd", raw[24:40])
    rec = np.frombuffer(raw[40:], dtype=np.dtype([("id", "<i4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")]))
    return bound, build_s, trace_s, rec["id"].copy(), rec["t"].copy(), rec["u"].copy(), rec["v"].copy()


REF_NORMALS = os.path.join(HERE, "_ref", "normals_dump")


def run_reference_normals(verts, faces, angle):
    """The reference's yafaray_smoothObjectMesh(angle) on one mesh: per face
    corner (4 per face) the normal index (-1 = none) and the normal."""
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 4)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(b"GBRTNM01")
            f.write(struct.pack("<I", len(verts))); f.write(verts.tobytes())
            f.write(struct.pack("<I", len(faces))); f.write(faces.tobytes())
            f.write(struct.pack("<f", angle))
        subprocess.run([REF_NORMALS, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
    nf = struct.unpack("<I", raw[:4])[0]
    rec = np.frombuffer(raw[4:], dtype=np.dtype([("idx", "<i4"), ("n", "<f4", 3)])).reshape(nf, 4)
    return rec["idx"].copy(), rec["n"].copy()


REF_RENDER = os.path.join(HERE, "_ref", "render_dump")


def reference_scene_text(scene, spp, batches, threads=-1, offset_stride=None):
    """Scene dict (libyafaray_gb300.scenes) -> render_dump input text."""
    out = []
    tex_keys = ("interpolate", "clipping", "xrepeat", "yrepeat", "cropmin_x", "cropmin_y", "cropmax_x", "cropmax_y",
                "rot90", "mirror_x", "mirror_y", "even_tiles", "odd_tiles", "checker_dist", "adj_intensity", "adj_contrast", "adj_mult_factor_red", "adj_mult_factor_green",
                "adj_mult_factor_blue", "adj_clamp")

    def fmt(v):
        if isinstance(v, bool):
            return str(v).lower()
        if isinstance(v, str):
            return v
        if isinstance(v, (tuple, list)):
            return ",".join(repr(float(x)) for x in v)
        return repr(v)
    for tname, tx in scene.get("textures", {}).items():
        if tx.get("type", "image") != "image":
            out.append(f"texture {tname} {texture_spec({k: v for k, v in tx.items() if k != 'mapper'})}")
            continue
        img = np.asarray(tx["image"], np.float32)
        h, w = img.shape[:2]
        out.append(f"image {tname}_img {w} {h}")
        out += [" ".join(repr(float(x)) for x in row.reshape(-1)) for row in img]
        out.append(f"texture {tname} type=image image_name={tname}_img "
                   + " ".join(f"{k}={fmt(tx[k])}" for k in tex_keys if k in tx))
    shaders = scene.get("material_shaders", {})
    for name, m in scene["materials"].items():
        t = m[0]
        slot_extra = ""
        if name in shaders:
            # the material's node trees: every node its slots read, then the slots
            nodes = scene["nodes"]
            need, todo = [], list(shaders[name].values())
            while todo:
                n = todo.pop()
                if n in need:
                    continue
                need.append(n)
                todo += [nodes[n][k] for k in ("input1", "input2", "input_factor", "input", "upper_layer") if nodes[n].get(k)]
            for n in need:
                nd = dict(nodes[n])
                kv = [f"name={n}", f"type={nd.pop('type')}"]
                for k, v in nd.items():
                    if k in ("color", "color1", "color2", "upper_color", "def_col") and isinstance(v, (tuple, list)):
                        v = [float(x) for x in v]
                        v = v + [1.0 if k in ("color", "def_col") else 0.0] if len(v) == 3 else v
                        kv.append(f"{k}=" + ",".join(repr(x) for x in v[:4]))
                    else:
                        kv.append(f"{k}={fmt(v)}")
                out.append("node " + " ".join(kv))
            slot_extra = "".join(f" {k}={v}" for k, v in shaders[name].items())
        if t == "shinydiffusemat":
            extra = ""
            for k, v in (m[2] if len(m) > 2 else {}).items():
                if k == "diffuse_texture":
                    tx = scene["textures"][v]
                    mp = tx.get("mapper", tx if tx.get("type", "image") == "image" else {})
                    node = f"{name}_dtex"
                    proj = mp.get("proj", (1, 2, 3))
                    out.append(f"node name={node} type=texture_mapper texture={v} texco={mp.get('texco', 'global')} "
                               f"mapping={mp.get('mapping', 'plain')} scale={fmt(mp.get('scale', (1.0, 1.0, 1.0)))} "
                               f"offset={fmt(mp.get('offset', (0.0, 0.0, 0.0)))} proj_x={proj[0]} proj_y={proj[1]} proj_z={proj[2]}")
                    lay = tx.get("layer")
                    if lay is not None:
                        layer = f"{name}_dlayer"
                        up = lay.get("upper_color", (0.0, 0.0, 0.0, 0.0))
                        dc = (*lay.get("def_col", (1.0, 1.0, 1.0)), 1.0)
                        out.append(f"node name={layer} type=layer input={node} blend_mode={lay.get('blend_mode', 'mix')} "
                                   f"colfac={float(lay.get('colfac', 1.0))!r} upper_color={fmt(up)} def_col={fmt(dc)} "
                                   f"negative={fmt(bool(lay.get('negative', False)))} noRGB={fmt(bool(lay.get('noRGB', False)))} "
                                   f"stencil={fmt(bool(lay.get('stencil', False)))} do_color=true color_input=true")
                        node = layer
                    extra += f" diffuse_shader={node}"
                    continue
                if isinstance(v, bool):
                    extra += f" {k}={str(v).lower()}"
                elif isinstance(v, (tuple, list)):
                    extra += f" {k}=" + ",".join(repr(float(x)) for x in v)
                else:
                    extra += f" {k}={float(v)!r}"
            out.append(f"material {name} shinydiffusemat {m[1][0]!r} {m[1][1]!r} {m[1][2]!r}{extra}" + slot_extra)
        elif t == "light_mat":
            out.append(f"material {name} light_mat {m[1][0]!r} {m[1][1]!r} {m[1][2]!r} {m[2]!r}" + slot_extra)
        elif t == "glossy":
            _, dc, gc, e, gr, dr = m
            vals = [*dc, *gc, e, gr, dr]
            out.append(f"material {name} glossy " + " ".join(repr(float(x)) for x in vals) + slot_extra)
        elif t == "glass":
            _, ior, fc, tf, mc = m[:5]
            vals = [ior, tf, *fc, *mc]
            fake = " fake_shadows=true" if len(m) > 5 and m[5].get("fake_shadows") else ""
            out.append(f"material {name} glass " + " ".join(repr(float(x)) for x in vals) + fake + slot_extra)
        elif t == "rough_glass":
            _, ior, alpha, fc, tf, mc = m[:6]
            vals = [ior, alpha, tf, *fc, *mc]
            fake = " fake_shadows=true" if len(m) > 6 and m[6].get("fake_shadows") else ""
            out.append(f"material {name} rough_glass " + " ".join(repr(float(x)) for x in vals) + fake + slot_extra)
        else:
            out.append(f"material {name} {t} " + " ".join(repr(float(x)) for x in m[1]) + slot_extra)
    for o in scene["objects"]:
        v = np.asarray(o["vertices"], np.float32)
        f = np.asarray(o["faces"], np.uint32)
        if "uvs" in o:
            uv = np.asarray(o["uvs"], np.float32).reshape(-1, 2)
            fu = np.asarray(o["face_uvs"], np.uint32).reshape(len(f), 4)
            out.append(f"object {o['name']} {o['material']} {len(v)} {len(f)} {len(uv)}")
            out += [f"{float(a)!r} {float(b)!r} {float(c)!r}" for a, b, c in v]
            out += [f"{float(a)!r} {float(b)!r}" for a, b in uv]
            out += [" ".join(str(int(x)) for x in ((*row[:3], *fr[:3]) if row[3] == TRI_MARK else (*row, *fr)))
                    for row, fr in zip(f, fu)]
        else:
            out.append(f"object {o['name']} {o['material']} {len(v)} {len(f)}")
            out += [f"{float(a)!r} {float(b)!r} {float(c)!r}" for a, b, c in v]
            out += [" ".join(str(int(x)) for x in (row[:3] if row[3] == TRI_MARK else row)) for row in f]
        if "smooth" in o:
            out.append(f"smooth {o['name']} {float(o['smooth'])!r}")
    for L in scene["lights"]:
        if L["type"] == "arealight":
            vals = [*L["corner"], *L["point1"], *L["point2"], *L["color"], L["power"]]
            out.append("arealight " + " ".join(repr(float(x)) for x in vals) + f" {int(L['samples'])}")
        elif L["type"] == "pointlight":
            vals = [*L["from"], *L["color"], L["power"]]
            out.append("pointlight " + " ".join(repr(float(x)) for x in vals))
    c = scene["camera"]
    vals = [*c["from"], *c["to"], *c["up"]]
    out.append("camera " + " ".join(repr(float(x)) for x in vals) + f" {c['resx']} {c['resy']} {float(c['focal'])!r}")
    integ = dict(scene["integrator"])
    t = integ.pop("type")
    out.append(f"integrator {t} " + " ".join(f"{k}={str(v).lower() if isinstance(v, bool) else v}" for k, v in integ.items()))
    film = scene.get("film")
    if film:
        if film["filter_type"] == "pixel":      # the single-pixel splat: the reference's box filter of width 1
            out.append("film box 1.0")
        else:
            out.append(f"film {film['filter_type']} {float(film.get('AA_pixelwidth', 1.5))!r}")
        aa = {k: v for k, v in film.items() if k.startswith("AA_") and k not in ("AA_pixelwidth", "AA_minsamples")}
        if aa:
            def fmt(v):
                return str(v).lower() if isinstance(v, (bool, str)) else repr(v)
            out.append("aa " + " ".join(f"{k}={fmt(v)}" for k, v in aa.items()))
    out.append(f"render {spp} {batches} {threads}" + (f" {int(offset_stride)}" if offset_stride is not None else ""))
    return "\n".join(out) + "\n"


def run_reference_aa(scene, spp, batches, offset_stride, threads=-1):
    """Adaptive-AA renders with the compiled reference (the scene's "film"
    AA_* entries): (rgb [K,H,W,3], seconds per batch, passes of batch 0 =
    [{pass, threshold, sums [H,W,4], weights [H,W], flagged (y W + x)}])."""
    text = reference_scene_text(scene, spp, batches, threads, offset_stride)
    with tempfile.TemporaryDirectory() as d:
        fin, fout, faa = os.path.join(d, "scene.txt"), os.path.join(d, "out.bin"), os.path.join(d, "aa.bin")
        open(fin, "w").write(text)
        subprocess.run([REF_RENDER, fin, fout, faa], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
        rawa = open(faa, "rb").read()
    K, H, W = struct.unpack("<iii", raw[:12])
    secs = np.frombuffer(raw[12:12 + 8 * K], np.float64).copy()
    rgb = np.frombuffer(raw[12 + 8 * K:], np.float32).reshape(K, H, W, 3).copy()
    passes = []
    n_pass = struct.unpack("<i", rawa[:4])[0]
    o = 4
    for _ in range(n_pass):
        pno, thr, n = struct.unpack("<ifi", rawa[o:o + 12]); o += 12
        sums = np.frombuffer(rawa, np.float32, 4 * H * W, o).reshape(H, W, 4).copy(); o += 16 * H * W
        w = np.frombuffer(rawa, np.float32, H * W, o).reshape(H, W).copy(); o += 4 * H * W
        fl = np.frombuffer(rawa, np.int32, n, o).copy(); o += 4 * n
        passes.append({"pass": pno, "threshold": thr, "sums": sums, "weights": w, "flagged": fl})
    return rgb, secs, passes


def run_reference_render(scene, spp, batches, threads=-1, offset_stride=None):
    """Render with the compiled reference; returns (rgb [K,H,W,3] float32,
    seconds per batch).  Batch k renders at adv_base_sampling_offset
    k x offset_stride (default spp)."""
    text = reference_scene_text(scene, spp, batches, threads, offset_stride)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "scene.txt"), os.path.join(d, "out.bin")
        open(fin, "w").write(text)
        subprocess.run([REF_RENDER, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
    K, H, W = struct.unpack("<iii", raw[:12])
    secs = np.frombuffer(raw[12:12 + 8 * K], np.float64).copy()
    rgb = np.frombuffer(raw[12 + 8 * K:], np.float32).reshape(K, H, W, 3).copy()
    return rgb, secs


def run_reference_photons(scene):
    """Diffuse and caustic photon maps of the reference's photonmapping
    preprocess: [(photons [n, 9] = dir, pos, col; n_paths), (caustic ...)]."""
    text = reference_scene_text(scene, 1, 1, 1)
    with tempfile.TemporaryDirectory() as d:
        fin, fout, fph = os.path.join(d, "scene.txt"), os.path.join(d, "out.bin"), os.path.join(d, "ph.bin")
        open(fin, "w").write(text)
        subprocess.run([REF_RENDER, fin, fout, fph], check=True, stdout=subprocess.DEVNULL)
        raw = open(fph, "rb").read()
    out, o = [], 0
    for _ in range(2):
        n, paths = struct.unpack("<ii", raw[o:o + 8]); o += 8
        ph = np.frombuffer(raw, np.float32, 9 * n, o).reshape(n, 9).copy(); o += 36 * n
        out.append((ph, paths))
    return out


REF_BINDING = os.path.join(HERE, "_ref", "binding_dump")


def binding_available():
    return os.path.exists(REF_BINDING)


def run_reference_translation(scene, spp=1):
    """The scene as the reference-side binding (oracle/ref/gb300_binding.cc)
    hands it to the GPU library: gb300::translate of the reference's own
    Scene and camera, gb300::pt_params of the integrator's ParamMap and
    gb300::film_params of the film's.  Returns a dict of numpy arrays and
    ctypes structures (libyafaray_gb300.gbrt layouts), with "ok" and
    "error" for a scene the binding refuses."""
    from libyafaray_gb300 import gbrt
    text = reference_scene_text(scene, spp, 1)
    with tempfile.TemporaryDirectory() as d:
        fin, fout, ftr = os.path.join(d, "scene.txt"), os.path.join(d, "out.bin"), os.path.join(d, "tr.bin")
        open(fin, "w").write(text)
        env = {k: v for k, v in os.environ.items() if k != "GB300_INTEGRATOR"}
        # the render itself is the reference's own (a short one): only the translation is read
        subprocess.run([REF_BINDING, fin, fout, ftr], check=True, stdout=subprocess.DEVNULL, env=env)
        raw = open(ftr, "rb").read()
    nv, nf, nm, nl, nn, hn = struct.unpack("<6i", raw[:24])
    o = 24

    def take(dtype, count, shape):
        nonlocal o
        a = np.frombuffer(raw, dtype, count, o).reshape(shape).copy()
        o += a.nbytes
        return a

    def take_struct(cls, count):
        nonlocal o
        arr = (cls * max(1, count))()
        n = ctypes.sizeof(cls) * count
        ctypes.memmove(arr, raw[o:o + n], n)
        o += n
        return arr[:count]

    out = {"vertices": take(np.float32, 3 * nv, (nv, 3)), "faces": take(np.uint32, 4 * nf, (nf, 4)),
           "face_material": take(np.int32, nf, (nf,))}
    out["materials"] = take_struct(gbrt.MaterialDesc, nm)
    out["lights"] = take_struct(gbrt.LightDesc, nl)
    if hn:
        out["normals"] = take(np.float32, 3 * nn, (nn, 3))
        out["face_normals"] = take(np.uint32, 4 * nf, (nf, 4))
    out["camera"] = take_struct(gbrt.CameraDesc, 1)[0]
    out["params"] = take_struct(gbrt.PtParams, 1)[0]
    out["aa"] = take_struct(gbrt.AaParams, 1)[0]
    out["caustic"] = take_struct(gbrt.PmParams, 1)[0]
    out["ok"] = struct.unpack("<i", raw[o:o + 4])[0] == 0
    out["error"] = raw[o + 4:].decode()
    return out


REF_NOISE = os.path.join(HERE, "_ref", "noise_dump")


def _tex_value(k, v):
    if isinstance(v, bool):
        return str(v).lower()
    if isinstance(v, str):
        return v
    if isinstance(v, (tuple, list)):
        vals = [float(x) for x in v]
        if k in ("color1", "color2") and len(vals) == 3:
            vals.append(1.0)                      # a colour parameter, not a vector
        return ",".join(repr(x) for x in vals)
    return repr(v)


def texture_spec(t):
    """A procedural texture dict as a noise_dump / render_dump "texture"
    statement's key=value list."""
    return " ".join(f"{k}={_tex_value(k, v)}" for k, v in t.items() if k not in ("mapper", "layer"))


def run_reference_textures(textures, points, noises=(), turbulences=()):
    """The reference's noise tables, and its procedural textures evaluated at
    texture-space points (oracle/_ref/noise_dump): returns (tables dict,
    [(status, rgba [n, 4], value [n]) per texture], [noise values [n] per
    noise type], [turbulence values [n] per (type, oct, size, hard)])."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    lines = [f"points {len(pts)}"] + [f"{float(a)!r} {float(b)!r} {float(c)!r}" for a, b, c in pts] + ["tables"]
    lines += [f"noise {n}" for n in noises]
    lines += [f"turbulence {n} {int(o)} {float(s)!r} {int(h)}" for n, o, s, h in turbulences]
    lines += [f"texture {texture_spec(t)}" for t in textures]
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "spec.txt"), os.path.join(d, "out.bin")
        open(fin, "w").write("\n".join(lines) + "\n")
        subprocess.run([REF_NOISE, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
    n = len(pts)
    o = 0
    tables = {}
    for key, dt, cnt in (("hash", np.uint8, 512), ("hashpntf", np.float32, 768), ("hashvectf", np.float32, 768),
                         ("stdp_p", np.uint8, 514), ("stdp_g", np.float32, 514 * 3)):
        a = np.frombuffer(raw, dt, cnt, o).copy()
        o += a.nbytes
        tables[key] = a
    nz = []
    for _ in noises:
        nz.append(np.frombuffer(raw, np.float32, n, o).copy()); o += 4 * n
    tb = []
    for _ in turbulences:
        tb.append(np.frombuffer(raw, np.float32, n, o).copy()); o += 4 * n
    tex = []
    for _ in textures:
        status = struct.unpack("<i", raw[o:o + 4])[0]; o += 4
        rgba = np.frombuffer(raw, np.float32, 4 * n, o).reshape(n, 4).copy(); o += 16 * n
        val = np.frombuffer(raw, np.float32, n, o).copy(); o += 4 * n
        tex.append((status, rgba, val))
    return tables, tex, nz, tb
