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


BUILD_NO_TREELETS = 1
BUILD_GREEDY_WIDE = 2


def _build_flags(treelets, greedy_wide):
    return (0 if treelets else BUILD_NO_TREELETS) | (BUILD_GREEDY_WIDE if greedy_wide else 0)


class BuildParams(ctypes.Structure):
    _fields_ = [("max_leaf_size", ctypes.c_uint32), ("traversal_cost", ctypes.c_float),
                ("intersect_cost", ctypes.c_float), ("flags", ctypes.c_uint32)]


class BvhInfo(ctypes.Structure):
    _fields_ = [("n_prims", ctypes.c_uint32), ("n_nodes", ctypes.c_uint32), ("n_leaves", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32), ("sah_cost", ctypes.c_float), ("bound", ctypes.c_float * 6),
                ("device_bytes", ctypes.c_uint64)]


class MaterialDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("color", ctypes.c_float * 3), ("color2", ctypes.c_float * 3),
                ("power", ctypes.c_float), ("params", ctypes.c_float * 8)]


class LightDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("corner", ctypes.c_float * 3), ("point1", ctypes.c_float * 3),
                ("point2", ctypes.c_float * 3), ("color", ctypes.c_float * 3), ("power", ctypes.c_float),
                ("samples", ctypes.c_int32)]


class CameraDesc(ctypes.Structure):
    _fields_ = [("from_", ctypes.c_float * 3), ("to", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("resx", ctypes.c_int32), ("resy", ctypes.c_int32), ("focal", ctypes.c_float)]


class PtParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_int32), ("path_samples", ctypes.c_int32), ("bounces", ctypes.c_int32),
                ("russian_roulette_min_bounces", ctypes.c_int32), ("base_sampling_offset", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("wave_paths", ctypes.c_uint32),
                ("guide", ctypes.c_void_p), ("guide_alpha", ctypes.c_float), ("guide_train_steps", ctypes.c_uint32),
                ("guide_batch", ctypes.c_uint32), ("guide_max_vertex", ctypes.c_uint32), ("raydepth", ctypes.c_int32),
                ("filter_type", ctypes.c_uint32), ("aa_pixel_width", ctypes.c_float), ("film_weight_dev", ctypes.c_void_p),
                ("transparent_shadows", ctypes.c_int32), ("shadow_depth", ctypes.c_int32),
                ("caustic_type", ctypes.c_uint32), ("no_recursive", ctypes.c_int32), ("caustic", ctypes.c_void_p),
                ("clamp_indirect", ctypes.c_float)]


# PathIntegrator "caustic_type" names -> gbrt_pt_params.caustic_type
CAUSTIC_TYPES = {"path": 0, "none": 1, "photon": 2, "both": 3}


# ImageFilm "filter_type" names -> gbrt_pt_params.filter_type ("pixel": single-pixel splat, plain sums)
FILTERS = {"pixel": 0, "box": 1, "gauss": 2, "mitchell": 3, "lanczos": 4}


class AaParams(ctypes.Structure):
    _fields_ = [("passes", ctypes.c_int32), ("inc_samples", ctypes.c_int32), ("threshold", ctypes.c_float),
                ("resampled_floor", ctypes.c_float), ("sample_multiplier_factor", ctypes.c_float),
                ("light_sample_multiplier_factor", ctypes.c_float), ("indirect_sample_multiplier_factor", ctypes.c_float),
                ("detect_color_noise", ctypes.c_int32), ("dark_detection_type", ctypes.c_int32),
                ("dark_threshold_factor", ctypes.c_float), ("variance_edge_size", ctypes.c_int32),
                ("variance_pixels", ctypes.c_int32)]


class SppmParams(ctypes.Structure):
    _fields_ = [("photons", ctypes.c_int32), ("passes", ctypes.c_int32), ("bounces", ctypes.c_int32),
                ("pm_ire", ctypes.c_int32), ("photon_radius", ctypes.c_float), ("search_num", ctypes.c_int32)]


def sppm_params(it):
    """gbrt_sppm_params from an "SPPM" integrator dict (SppmIntegrator's
    parameter names and defaults, integrator_sppm.h:79-86)."""
    return SppmParams(int(it.get("photons", 500000)), int(it.get("passNums", 1000)), int(it.get("bounces", 5)),
                      int(bool(it.get("pmIRE", False))), float(it.get("photonRadius", 1.0)), int(it.get("searchNum", 10)))


RAMP_MAX = 16


class ProceduralDesc(ctypes.Structure):
    _fields_ = [("noise_type", ctypes.c_uint32), ("noise_type2", ctypes.c_uint32), ("color1", ctypes.c_float * 3),
                ("color2", ctypes.c_float * 3), ("size", ctypes.c_float), ("depth", ctypes.c_int32), ("hard", ctypes.c_int32),
                ("bias", ctypes.c_uint32), ("shape", ctypes.c_uint32), ("wood_type", ctypes.c_uint32),
                ("blend_type", ctypes.c_uint32), ("use_flip_axis", ctypes.c_int32), ("sharpness", ctypes.c_float),
                ("turbulence", ctypes.c_float), ("distance_metric", ctypes.c_uint32), ("color_mode", ctypes.c_uint32),
                ("weight", ctypes.c_float * 4), ("mk_exponent", ctypes.c_float), ("intensity", ctypes.c_float),
                ("musgrave_type", ctypes.c_uint32), ("h", ctypes.c_float), ("lacunarity", ctypes.c_float),
                ("octaves", ctypes.c_float), ("offset", ctypes.c_float), ("gain", ctypes.c_float), ("distort", ctypes.c_float),
                ("ramp_n", ctypes.c_int32), ("ramp_mode", ctypes.c_uint32), ("ramp_interpolation", ctypes.c_uint32),
                ("ramp_hue_interpolation", ctypes.c_uint32), ("ramp", (ctypes.c_float * 5) * RAMP_MAX)]


class NoiseTablesDesc(ctypes.Structure):
    _fields_ = [("hash", ctypes.c_void_p), ("hashpntf", ctypes.c_void_p), ("hashvectf", ctypes.c_void_p),
                ("stdp_p", ctypes.c_void_p), ("stdp_g", ctypes.c_void_p)]


class ShaderNode(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("texture", ctypes.c_int32), ("do_scalar", ctypes.c_int32), ("input1", ctypes.c_int32),
                ("input2", ctypes.c_int32), ("input_factor", ctypes.c_int32), ("color1", ctypes.c_float * 4),
                ("color2", ctypes.c_float * 4), ("value1", ctypes.c_float), ("value2", ctypes.c_float), ("factor", ctypes.c_float),
                ("mode", ctypes.c_uint32), ("def_col", ctypes.c_float * 4), ("def_val", ctypes.c_float), ("colfac", ctypes.c_float),
                ("valfac", ctypes.c_float), ("do_color", ctypes.c_int32), ("color_input", ctypes.c_int32), ("use_alpha", ctypes.c_int32),
                ("no_rgb", ctypes.c_int32), ("stencil", ctypes.c_int32), ("negative", ctypes.c_int32), ("bump_strength", ctypes.c_float)]


NODE_TYPES = {"texture_mapper": 0, "value": 1, "mix": 2, "layer": 3}
MIX_MODES = {"mix": 0, "add": 1, "multiply": 2, "subtract": 3, "screen": 4, "difference": 5, "darken": 6, "lighten": 7, "overlay": 8}
SLOTS = {"diffuse_shader": 0, "glossy_shader": 1, "mirror_color_shader": 2, "filter_color_shader": 3, "bump_shader": 4}
N_SLOTS = 5


def _rgba(v, alpha=1.0):
    v = [float(x) for x in v]
    return v + [alpha] if len(v) == 3 else v[:4]


def shader_nodes(scene, texture_base=0):
    """The scene's shader node trees ("nodes": name -> node dict with the
    reference's parameter names; "material_shaders": material name ->
    {slot parameter name: node name}) as gbrt_shader_node entries in an
    order where every node follows its inputs, the textures their
    texture_mapper nodes read (texture dict + the node's mapper
    parameters; their texture indices start at texture_base), and the node
    index of each name."""
    nodes = scene.get("nodes", {})
    order, seen = [], set()

    def visit(name):
        if name in seen:
            return
        seen.add(name)
        nd = nodes[name]
        for k in ("input1", "input2", "input_factor", "input", "upper_layer"):
            if nd.get(k):
                visit(nd[k])
        order.append(name)

    for name in nodes:
        visit(name)
    index = {n: i for i, n in enumerate(order)}
    arr = (ShaderNode * max(1, len(order)))()
    textures = []
    for i, name in enumerate(order):
        nd = nodes[name]
        d = arr[i]
        d.type = NODE_TYPES[nd["type"]]
        d.texture = -1
        d.input1 = d.input2 = d.input_factor = -1
        d.bump_strength = float(nd.get("bump_strength", 1.0))
        if nd["type"] == "texture_mapper":
            tx = dict(scene["textures"][nd["texture"]])
            mp = {k: nd[k] for k in ("texco", "mapping", "scale", "offset") if k in nd}
            mp["proj"] = tuple(int(nd.get(f"proj_{a}", d0)) for a, d0 in (("x", 1), ("y", 2), ("z", 3)))
            tx["mapper"] = mp
            tx.pop("layer", None)
            d.texture = texture_base + len(textures)
            textures.append(tx)
            d.do_scalar = int(bool(nd.get("do_scalar", True)))
        elif nd["type"] == "value":
            d.color1[:] = [*[float(x) for x in nd.get("color", (1.0, 1.0, 1.0))][:3], float(nd.get("alpha", 1.0))]
            d.value1 = float(nd.get("scalar", 1.0))
        elif nd["type"] == "mix":
            d.input1 = index[nd["input1"]] if nd.get("input1") else -1
            d.input2 = index[nd["input2"]] if nd.get("input2") else -1
            d.input_factor = index[nd["input_factor"]] if nd.get("input_factor") else -1
            d.color1[:] = _rgba(nd.get("color1", (0.0, 0.0, 0.0, 0.0)), 0.0)
            d.color2[:] = _rgba(nd.get("color2", (0.0, 0.0, 0.0, 0.0)), 0.0)
            d.value1, d.value2 = float(nd.get("value1", 0.0)), float(nd.get("value2", 0.0))
            d.factor = float(nd.get("cfactor", 0.5))
            d.mode = MIX_MODES[nd.get("blend_mode", "mix")]
        else:
            d.input1 = index[nd["input"]]
            d.input2 = index[nd["upper_layer"]] if nd.get("upper_layer") else -1
            d.color1[:] = _rgba(nd.get("upper_color", (0.0, 0.0, 0.0, 0.0)), 0.0)
            d.value1 = float(nd.get("upper_value", 0.0))
            d.def_col[:] = _rgba(nd.get("def_col", (1.0, 1.0, 1.0, 1.0)), 1.0)
            d.def_val, d.colfac, d.valfac = float(nd.get("def_val", 1.0)), float(nd.get("colfac", 1.0)), float(nd.get("valfac", 1.0))
            d.do_color = int(bool(nd.get("do_color", True)))
            d.do_scalar = int(bool(nd.get("do_scalar", False)))
            d.color_input = int(bool(nd.get("color_input", True)))
            d.use_alpha = int(bool(nd.get("use_alpha", False)))
            d.no_rgb, d.stencil, d.negative = (int(bool(nd.get(k, False))) for k in ("noRGB", "stencil", "negative"))
            d.mode = BLEND_MODES[nd.get("blend_mode", "mix")]
    return arr, len(order), textures, index


class TextureDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("rgba", ctypes.c_void_p),
                ("interpolate", ctypes.c_uint32), ("clipping", ctypes.c_uint32), ("xrepeat", ctypes.c_int32),
                ("yrepeat", ctypes.c_int32), ("crop", ctypes.c_float * 4), ("rot90", ctypes.c_int32),
                ("adj_intensity", ctypes.c_float), ("adj_contrast", ctypes.c_float),
                ("adj_mult_factor", ctypes.c_float * 3), ("adj_clamp", ctypes.c_int32), ("texco", ctypes.c_uint32),
                ("mapping", ctypes.c_uint32), ("scale", ctypes.c_float * 3), ("offset", ctypes.c_float * 3),
                ("proj", ctypes.c_int32 * 3), ("layer", ctypes.c_int32), ("blend_mode", ctypes.c_uint32),
                ("colfac", ctypes.c_float), ("upper_color", ctypes.c_float * 4), ("def_col", ctypes.c_float * 3),
                ("negative", ctypes.c_int32), ("no_rgb", ctypes.c_int32), ("stencil", ctypes.c_int32),
                ("mirror_x", ctypes.c_int32), ("mirror_y", ctypes.c_int32), ("even_tiles", ctypes.c_int32),
                ("odd_tiles", ctypes.c_int32), ("checker_dist", ctypes.c_float), ("kind", ctypes.c_uint32),
                ("adj_saturation", ctypes.c_float), ("adj_hue", ctypes.c_float), ("proc", ProceduralDesc)]


# ImageTexture / TextureMapperNode enum names (texture_image.h, shader_node_texture.h)
TEXCO = {"global": 0, "uv": 1}
MAPPING = {"plain": 0, "cube": 1, "tube": 2, "sphere": 3}
# Texture::Type and the procedural textures' enum names (include/texture/*.h,
# include/noise/*.h, include/color/color_ramp.h)
TEX_KINDS = {"image": 0, "blend": 1, "clouds": 2, "marble": 3, "wood": 4, "voronoi": 5, "musgrave": 6, "distorted_noise": 7,
             "rgb_cube": 8}
NOISE_TYPES = {"blender": 0, "stdperlin": 1, "newperlin": 2, "cellnoise": 3, "voronoi_f1": 4, "voronoi_f2": 5, "voronoi_f3": 6,
               "voronoi_f4": 7, "voronoi_f2f1": 8, "voronoi_crackle": 9}
DISTANCE_METRICS = {"real": 0, "squared": 1, "manhattan": 2, "chebychev": 3, "minkovsky_half": 4, "minkovsky_four": 5,
                    "minkovsky": 6}
PROGRESSIONS = {"linear": 0, "quadratic": 1, "easing": 2, "diagonal": 3, "sphere": 4, "quad_sphere": 5, "radial": 6}
BIASES = {"none": 0, "positive": 1, "negative": 2}
SHAPES = {"sin": 0, "saw": 1, "tri": 2}
WOOD_TYPES = {"bands": 0, "rings": 1}
VORONOI_COLOR_MODES = {"intensity-without-color": 0, "position": 1, "position-outline": 2, "position-outline-intensity": 3}
MUSGRAVE_TYPES = {"fBm": 0, "multifractal": 1, "heteroterrain": 2, "hybridmf": 3, "ridgedmf": 4}
RAMP_MODES = {"RGB": 0, "HSV": 1, "HSL": 2}
RAMP_INTERPOLATIONS = {"LINEAR": 0, "CONSTANT": 1}
HUE_INTERPOLATIONS = {"NEAR": 0, "FAR": 1, "CW": 2, "CCW": 3}


def procedural_desc(t):
    """gbrt_procedural_desc of a procedural texture dict (the reference's
    parameter names; missing ones take its defaults)."""
    p = ProceduralDesc()
    load().gbrt_procedural_defaults(ctypes.byref(p))
    kind = t["type"]
    p.noise_type = NOISE_TYPES[t.get("noise_type1" if kind == "distorted_noise" else "noise_type", "newperlin")]
    p.noise_type2 = NOISE_TYPES[t.get("noise_type2", "newperlin")]
    p.color1[:] = [float(x) for x in t.get("color1", (0.0, 0.0, 0.0))][:3]
    p.color2[:] = [float(x) for x in t.get("color2", (1.0, 1.0, 1.0))][:3]
    p.size = float(t.get("size", 1.0))
    p.depth = int(t.get("depth", 2))
    p.hard = int(bool(t.get("hard", False)))
    p.bias = BIASES[t.get("bias", "none")]
    p.shape = SHAPES[t.get("shape", "sin")]
    p.wood_type = WOOD_TYPES[t.get("wood_type", "bands")]
    p.blend_type = PROGRESSIONS[t.get("blend_type", "linear")]
    p.use_flip_axis = int(bool(t.get("use_flip_axis", False)))
    p.sharpness = float(t.get("sharpness", 1.0))
    p.turbulence = float(t.get("turbulence", 1.0))
    p.distance_metric = DISTANCE_METRICS[t.get("distance_metric", "real")]
    p.color_mode = VORONOI_COLOR_MODES[t.get("color_mode", "intensity-without-color")]
    p.weight[:] = [float(t.get(f"weight{i}", 1.0 if i == 1 else 0.0)) for i in range(1, 5)]
    p.mk_exponent = float(t.get("mk_exponent", 2.5))
    p.intensity = float(t.get("intensity", 1.0))
    p.musgrave_type = MUSGRAVE_TYPES[t.get("musgrave_type", "fBm")]
    p.h, p.lacunarity, p.octaves = float(t.get("H", 1.0)), float(t.get("lacunarity", 2.0)), float(t.get("octaves", 2.0))
    p.offset, p.gain = float(t.get("offset", 1.0)), float(t.get("gain", 1.0))
    p.distort = float(t.get("distort", 1.0))
    n = int(t.get("ramp_num_items", 0))
    if n > RAMP_MAX:
        raise ValueError(f"at most {RAMP_MAX} ramp items")
    p.ramp_n = n
    p.ramp_mode = RAMP_MODES[t.get("ramp_color_mode", "RGB")]
    p.ramp_interpolation = RAMP_INTERPOLATIONS[t.get("ramp_interpolation", "LINEAR")]
    p.ramp_hue_interpolation = HUE_INTERPOLATIONS[t.get("ramp_hue_interpolation", "NEAR")]
    for i in range(n):
        c = [float(x) for x in t.get(f"ramp_item_{i}_color", (0.0, 0.0, 0.0, 1.0))]
        p.ramp[i][:] = [*c[:4], float(t.get(f"ramp_item_{i}_position", 0.0))]
    return p
CLIPPING = {"extend": 0, "clip": 1, "clipcube": 2, "repeat": 3, "checker": 4}
INTERPOLATE = {"none": 0, "bilinear": 1, "bicubic": 2}
BLEND_MODES = {"mix": 0, "add": 1, "multiply": 2, "subtract": 3, "screen": 4, "divide": 5, "difference": 6, "darken": 7,
               "lighten": 8}


def mapper_of(t):
    """The texture-mapper node parameters of a scene texture entry (texco,
    mapping, scale, offset, proj): its "mapper" dict, or, for an image
    texture, the entry itself (musgrave's own "offset" would clash)."""
    if "mapper" in t:
        return t["mapper"]
    return t if t.get("type", "image") == "image" else {}


def texture_desc(t):
    """gbrt_texture_desc of a scene "textures" entry (image [h, w, 4] float32
    plus the reference's texture and texture-mapper parameter names); the
    image array must stay alive until the call that takes the desc.  A
    procedural texture ("type" other than "image", no image) carries its
    parameters in the desc's proc part (procedural_desc)."""
    d = TextureDesc()
    kind = t.get("type", "image")
    d.kind = TEX_KINDS[kind]
    d.adj_saturation, d.adj_hue = float(t.get("adj_saturation", 1.0)), float(t.get("adj_hue", 0.0))
    if kind == "image":
        img = np.ascontiguousarray(t["image"], np.float32)
        d.height, d.width = int(img.shape[0]), int(img.shape[1])
        d.rgba = img.ctypes.data
    else:
        img = None
        d.proc = procedural_desc(t)
    d.interpolate = INTERPOLATE[t.get("interpolate", "bilinear")]
    d.clipping = CLIPPING[t.get("clipping", "repeat")]
    d.xrepeat, d.yrepeat = int(t.get("xrepeat", 1)), int(t.get("yrepeat", 1))
    d.crop[:] = [float(t.get("cropmin_x", 0.0)), float(t.get("cropmin_y", 0.0)), float(t.get("cropmax_x", 1.0)),
                 float(t.get("cropmax_y", 1.0))]
    d.rot90 = int(bool(t.get("rot90", False)))
    d.mirror_x, d.mirror_y = int(bool(t.get("mirror_x", False))), int(bool(t.get("mirror_y", False)))
    d.even_tiles, d.odd_tiles = int(bool(t.get("even_tiles", False))), int(bool(t.get("odd_tiles", True)))
    d.checker_dist = float(t.get("checker_dist", 0.0))
    d.adj_intensity, d.adj_contrast = float(t.get("adj_intensity", 1.0)), float(t.get("adj_contrast", 1.0))
    d.adj_mult_factor[:] = [float(t.get("adj_mult_factor_red", 1.0)), float(t.get("adj_mult_factor_green", 1.0)),
                            float(t.get("adj_mult_factor_blue", 1.0))]
    d.adj_clamp = int(bool(t.get("adj_clamp", False)))
    mp = mapper_of(t)
    d.texco = TEXCO[mp.get("texco", "global")]
    d.mapping = MAPPING[mp.get("mapping", "plain")]
    d.scale[:] = [float(x) for x in mp.get("scale", (1.0, 1.0, 1.0))]
    d.offset[:] = [float(x) for x in mp.get("offset", (0.0, 0.0, 0.0))]
    d.proj[:] = [int(x) for x in mp.get("proj", (1, 2, 3))]
    lay = t.get("layer")
    d.layer = int(lay is not None)
    lay = lay or {}
    d.blend_mode = BLEND_MODES[lay.get("blend_mode", "mix")]
    d.colfac = float(lay.get("colfac", 1.0))
    d.upper_color[:] = [float(x) for x in lay.get("upper_color", (0.0, 0.0, 0.0, 0.0))]
    d.def_col[:] = [float(x) for x in lay.get("def_col", (1.0, 1.0, 1.0))]
    d.negative, d.no_rgb, d.stencil = (int(bool(lay.get(k, False))) for k in ("negative", "noRGB", "stencil"))
    return d, img


# AaNoiseParams::DarkDetectionType names (include/common/aa_noise_params.h:30-37)
DARK_DETECTION = {"none": 0, "linear": 1, "curve": 2}


def aa_params(film):
    """gbrt_aa_params from a film dict with the reference's ImageFilm
    parameter names and defaults (include/render/imagefilm.h:212-225)."""
    film = film or {}
    return AaParams(int(film.get("AA_passes", 1)), int(film.get("AA_inc_samples", 1)),
                    float(film.get("AA_threshold", 0.05)), float(film.get("AA_resampled_floor", 0.0)),
                    float(film.get("AA_sample_multiplier_factor", 1.0)),
                    float(film.get("AA_light_sample_multiplier_factor", 1.0)),
                    float(film.get("AA_indirect_sample_multiplier_factor", 1.0)),
                    int(bool(film.get("AA_detect_color_noise", False))),
                    DARK_DETECTION[film.get("AA_dark_detection_type", "none")],
                    float(film.get("AA_dark_threshold_factor", 0.0)), int(film.get("AA_variance_edge_size", 10)),
                    int(film.get("AA_variance_pixels", 0)))


class PmParams(ctypes.Structure):
    _fields_ = [("diffuse_photons", ctypes.c_int32), ("caustic_photons", ctypes.c_int32), ("diffuse_radius", ctypes.c_float),
                ("diffuse_search", ctypes.c_int32), ("caustic_radius", ctypes.c_float), ("caustic_mix", ctypes.c_int32),
                ("caustic_depth", ctypes.c_int32), ("bounces", ctypes.c_int32), ("caustics", ctypes.c_int32),
                ("diffuse", ctypes.c_int32), ("final_gather", ctypes.c_int32), ("fg_samples", ctypes.c_int32),
                ("fg_bounces", ctypes.c_int32), ("fg_min_pathlen", ctypes.c_float)]


# photonmapping parameter names of the reference -> PmParams fields
PM_KEYS = {"diffuse_photons": "diffuse_photons", "caustic_photons": "caustic_photons", "diffuse_radius": "diffuse_radius",
           "diffuse_search": "diffuse_search", "caustic_radius": "caustic_radius", "caustic_mix": "caustic_mix",
           "caustic_depth": "caustic_depth", "bounces": "bounces", "caustics": "caustics", "diffuse": "diffuse",
           "finalGather": "final_gather", "fg_samples": "fg_samples", "fg_bounces": "fg_bounces",
           "fg_min_pathlen": "fg_min_pathlen"}


def pm_params(integrator):
    """PmParams from a photonmapping integrator dict (reference names)."""
    p = PmParams()
    check(load().gbrt_pm_default_params(ctypes.byref(p)))
    for k, v in integrator.items():
        if k in PM_KEYS:
            setattr(p, PM_KEYS[k], type(getattr(p, PM_KEYS[k]))(v))
    return p


class PtStats(ctypes.Structure):
    _fields_ = [("camera_samples", ctypes.c_uint64), ("extension_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("ms", ctypes.c_float), ("photon_paths", ctypes.c_uint64),
                ("photons_stored", ctypes.c_uint64), ("radiance_photons", ctypes.c_uint64), ("photon_ms", ctypes.c_float)]


class GuideParams(ctypes.Structure):
    _fields_ = [("log2_table", ctypes.c_uint32), ("base_resolution", ctypes.c_float),
                ("max_resolution", ctypes.c_float), ("learning_rate", ctypes.c_float), ("seed", ctypes.c_uint32)]


MAT_TYPES = {"shinydiffusemat": 0, "light_mat": 1, "glossy": 2, "rough_glass": 3, "glass": 4}
PT_FP64_FILM = 1
PT_GUIDE_RADIANCE = 2

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
    "gbrt_bvh_export_wide": (_I, [_VP, ctypes.POINTER(_U32), ctypes.POINTER(_U32), _VP, ctypes.c_size_t, _VP, ctypes.c_size_t,
                                  _VP, ctypes.c_size_t]),
    "gbrt_bvh_build_static": (_I, [_VP, _U32, _VP, _U32, ctypes.POINTER(BuildParams), _VP, ctypes.c_size_t, _VP,
                                   ctypes.c_size_t, _VP, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float), _VP]),
    "gbrt_trace_closest": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "gbrt_trace_shadow": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "gbrt_trace_closest_host": (_I, [_VP, _VP, _U32, _VP]),
    "gbrt_trace_shadow_host": (_I, [_VP, _VP, _U32, _VP]),
    "gbrt_host_path": (_I, [_VP, _U32, _VP, ctypes.c_int, _VP]),
    "gbrt_scene_create": (_I, [_VP, _VP, _U32, _VP, _U32, _VP, ctypes.POINTER(MaterialDesc), _U32,
                               ctypes.POINTER(LightDesc), _U32, ctypes.POINTER(_VP)]),
    "gbrt_scene_destroy": (_I, [_VP]),
    "gbrt_sampler_eval": (_I, [_I, _I, _VP, _U32, _VP, _I]),
    "gbrt_guide_create": (_I, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(GuideParams), ctypes.POINTER(_VP)]),
    "gbrt_guide_destroy": (_I, [_VP]),
    "gbrt_guide_info": (_I, [_VP, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64)]),
    "gbrt_guide_get_params": (_I, [_VP, _VP, _VP]),
    "gbrt_guide_set_params": (_I, [_VP, _VP, _VP]),
    "gbrt_guide_eval": (_I, [_VP, _VP, _U32, _VP, _VP]),
    "gbrt_guide_grad": (_I, [_VP, _VP, _U32, ctypes.POINTER(ctypes.c_float), _VP]),
    "gbrt_guide_get_grads": (_I, [_VP, _VP, _VP]),
    "gbrt_guide_step": (_I, [_VP, _VP, _U32, ctypes.POINTER(ctypes.c_float), _VP]),
    "gbrt_guide_forward_host": (_I, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(GuideParams), _VP, _VP, _VP, _U32, _VP]),
    "gbrt_guide_set_eval_mode": (_I, [_VP, ctypes.c_int]),
    "gbrt_guide_status": (_I, [_VP, ctypes.POINTER(ctypes.c_uint32)]),
    "gbrt_tc_selftest": (_I, [_VP, _VP, _U32, _U32, _VP]),
    "gbrt_pm_default_params": (_I, [_VP]),
    "gbrt_pt_render_batch": (_I, [_VP, _VP, _VP, _VP, _U32, _U32, _VP]),
    "gbrt_pt_render_multi": (_I, [_VP, _VP, _VP, _VP, _U32, _VP, _VP, _VP]),
    "gbrt_pm_render": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "gbrt_pm_render_host": (_I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "gbrt_dl_render": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "gbrt_dl_render_host": (_I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "gbrt_pm_photons": (_I, [_VP, _VP, ctypes.c_int, _VP, _U32, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "gbrt_knn_gather": (_I, [_VP, _U32, _VP, _U32, ctypes.c_float, ctypes.c_int, ctypes.c_float, _VP, _VP, _VP]),
    "gbrt_grid_buckets": (_I, [_VP, _U32, ctypes.c_double, _U32, _VP, _VP]),
    "gbrt_pt_render": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), _VP, _VP,
                            ctypes.POINTER(PtStats), _VP]),
    "gbrt_pt_render_host": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), _VP,
                                 ctypes.POINTER(PtStats)]),
    "gbrt_pt_render_aa": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), ctypes.POINTER(AaParams), _VP,
                               ctypes.POINTER(PtStats), _VP, _VP]),
    "gbrt_pt_render_aa_host": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), ctypes.POINTER(AaParams),
                                    _VP, ctypes.POINTER(PtStats), _VP]),
    "gbrt_aa_flags": (_I, [_VP, _VP, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(AaParams), ctypes.c_float, _VP,
                           ctypes.POINTER(ctypes.c_uint32)]),
    "gbrt_scene_set_textures": (_I, [_VP, _VP, _U32, _VP, ctypes.POINTER(TextureDesc), _U32, _VP, _U32]),
    "gbrt_mesh_smooth_normals": (_I, [_VP, _U32, _VP, _U32, ctypes.c_float, _VP, _U32, ctypes.POINTER(_U32), _VP]),
    "gbrt_scene_set_normals": (_I, [_VP, _VP, _U32, _VP]),
    "gbrt_procedural_defaults": (None, [ctypes.POINTER(ProceduralDesc)]),
    "gbrt_scene_set_noise_tables": (_I, [_VP, ctypes.POINTER(NoiseTablesDesc)]),
    "gbrt_scene_set_shader_nodes": (_I, [_VP, ctypes.POINTER(ShaderNode), _U32, _VP, _U32]),
    "gbrt_texture_eval": (_I, [ctypes.POINTER(TextureDesc), ctypes.POINTER(NoiseTablesDesc), _VP, _U32, _VP, _VP, ctypes.c_int]),
    "gbrt_pm_render_aa_host": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), _VP, ctypes.POINTER(AaParams),
                                    _VP, ctypes.POINTER(PtStats), _VP]),
    "gbrt_dl_render_aa_host": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), _VP, ctypes.POINTER(AaParams),
                                    _VP, ctypes.POINTER(PtStats), _VP]),
    "gbrt_sppm_render": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), ctypes.POINTER(SppmParams), _VP,
                              ctypes.POINTER(PtStats), _VP]),
    "gbrt_sppm_render_host": (_I, [_VP, ctypes.POINTER(CameraDesc), ctypes.POINTER(PtParams), ctypes.POINTER(SppmParams), _VP,
                                   ctypes.POINTER(PtStats)]),
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
    def build_host(cls, vertices, faces, max_leaf_size=0, traversal_cost=0.0, intersect_cost=0.0, treelets=True,
                   greedy_wide=False):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 4)
        p = BuildParams(max_leaf_size, traversal_cost, intersect_cost, _build_flags(treelets, greedy_wide))
        h = ctypes.c_void_p()
        check(load().gbrt_bvh_build_host(_ptr(v), len(v), _ptr(f), len(f), ctypes.byref(p), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def build_device(cls, vertices_ptr, n_vertices, faces_ptr, n_faces, stream=0, max_leaf_size=0,
                     traversal_cost=0.0, intersect_cost=0.0, treelets=True, greedy_wide=False):
        p = BuildParams(max_leaf_size, traversal_cost, intersect_cost, _build_flags(treelets, greedy_wide))
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

    def export_wide(self):
        """(nodes uint32 [n_nodes, 20], prims float32 [n,12], ids uint32 [n], depth): the 8-wide
        compressed hierarchy the traversal walks."""
        n = self.info()["n_prims"]
        nn, depth = _U32(), _U32()
        check(load().gbrt_bvh_export_wide(self._h, ctypes.byref(nn), ctypes.byref(depth), None, 0, None, 0, None, 0))
        nodes = np.empty((max(nn.value, 1), 20), np.uint32)
        prims = np.empty((max(n, 1), 12), np.float32)
        ids = np.empty(max(n, 1), np.uint32)
        check(load().gbrt_bvh_export_wide(self._h, None, None, _ptr(nodes), nodes.nbytes, _ptr(prims), prims.nbytes,
                                          _ptr(ids), ids.nbytes))
        return nodes[:nn.value], prims[:n], ids[:n], depth.value

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


def _material_desc(m):
    d = MaterialDesc()
    kind = m[0]
    d.type = MAT_TYPES[kind]
    if kind == "shinydiffusemat":
        # ("shinydiffusemat", color[, {reference parameter name: value}])
        d.color[:] = [float(x) for x in m[1]]
        opt = m[2] if len(m) > 2 else {}
        d.color2[:] = [float(x) for x in opt.get("mirror_color", (1.0, 1.0, 1.0))]
        d.power = float(opt.get("emit", 0.0))
        d.params[:5] = [float(opt.get("diffuse_reflect", 1.0)), float(opt.get("specular_reflect", 0.0)),
                        float(opt.get("transparency", 0.0)), float(opt.get("translucency", 0.0)),
                        float(opt.get("transmit_filter", 1.0))]
        d.params[6] = 1.0 if opt.get("fresnel_effect", False) else 0.0
        d.params[7] = float(opt.get("IOR", 1.33))
    elif kind == "light_mat":
        d.color[:] = [float(x) for x in m[1]]
        d.power = float(m[2])
    elif kind == "glossy":
        _, dc, gc, e, gr, dr = m[:6]
        d.color[:] = [float(x) for x in gc]
        d.color2[:] = [float(x) for x in dc]
        d.params[:4] = [float(e), float(gr), float(dr), float(m[6]) if len(m) > 6 else 1.0]
    elif kind in ("glass", "rough_glass"):
        # ("glass", IOR, filter_color, transmit_filter, mirror_color[, {"fake_shadows": bool}])
        # ("rough_glass", IOR, alpha, filter_color, transmit_filter, mirror_color[, {...}])
        ior, rest = float(m[1]), m[2:]
        alpha = 0.0
        if kind == "rough_glass":
            alpha, rest = float(rest[0]), rest[1:]
        fc, tf, mc = rest[:3]
        opt = rest[3] if len(rest) > 3 else {}
        d.color[:] = [float(x) for x in fc]
        d.color2[:] = [float(x) for x in mc]
        d.params[:4] = [ior, float(tf), alpha, 1.0 if opt.get("fake_shadows", False) else 0.0]
    else:
        vals = [float(x) for x in m[1]]
        d.color[:] = vals[0:3]
        d.params[:len(vals[3:9])] = vals[3:9]
    return d


NO_NORMAL = 0xFFFFFFFF
FLAT_FACE = 0xFFFFFFFE


def noise_tables(tables):
    """gbrt_noise_tables of a dict of the reference's noise tables (hash
    uint8 [512], hashpntf float32 [768], hashvectf float32 [768], stdp_p
    uint8 [514], stdp_g float32 [514, 3]); returns (desc, arrays to keep)."""
    keep = [np.ascontiguousarray(tables["hash"], np.uint8).reshape(512),
            np.ascontiguousarray(tables["hashpntf"], np.float32).reshape(768),
            np.ascontiguousarray(tables["hashvectf"], np.float32).reshape(768),
            np.ascontiguousarray(tables["stdp_p"], np.uint8).reshape(514),
            np.ascontiguousarray(tables["stdp_g"], np.float32).reshape(514 * 3)]
    return NoiseTablesDesc(*[a.ctypes.data for a in keep]), keep


def texture_eval(texture, tables, points, on_device=False):
    """gbrt_texture_eval: a procedural texture dict's getColor (RGBA [n, 4])
    and getFloat ([n]) at texture-space points [n, 3]."""
    d, _ = texture_desc(texture)
    nt, keep = noise_tables(tables)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    rgba = np.empty((max(1, len(pts)), 4), np.float32)
    val = np.empty(max(1, len(pts)), np.float32)
    check(load().gbrt_texture_eval(ctypes.byref(d), ctypes.byref(nt), _ptr(pts), len(pts), _ptr(rgba), _ptr(val), int(bool(on_device))))
    return rgba[:len(pts)], val[:len(pts)]


def smooth_normals(vertices, faces, angle):
    """The reference's yafaray_smoothObjectMesh(angle) on one mesh object,
    by gbrt_mesh_smooth_normals: (normals float32 [n, 3], face normal
    indices uint32 [faces, 4], NO_NORMAL where a vertex keeps the face's
    geometric normal)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 4)
    fn = np.empty((max(1, len(f)), 4), np.uint32)
    n = _U32()
    L = load()
    check(L.gbrt_mesh_smooth_normals(_ptr(v), len(v), _ptr(f), len(f), float(angle), None, 0, ctypes.byref(n), _ptr(fn)))
    out = np.empty((max(1, n.value), 3), np.float32)
    check(L.gbrt_mesh_smooth_normals(_ptr(v), len(v), _ptr(f), len(f), float(angle), _ptr(out), len(out), ctypes.byref(n),
                                     _ptr(fn)))
    return out[:n.value], fn[:len(f)]


class Renderer:
    """A scene dict (libyafaray_gb300.scenes) on the GPU: BVH + materials +
    lights, rendered by the wavefront path tracer (gbrt_pt_render)."""

    def __init__(self, scene):
        from . import scenes as _scenes
        self.scene = scene
        self.vertices, self.faces, self.face_mat, self.mat_names = _scenes.flatten(scene)
        self.bvh = Bvh.build_host(self.vertices, self.faces)
        mats = (MaterialDesc * max(1, len(self.mat_names)))()
        for i, name in enumerate(self.mat_names):
            mats[i] = _material_desc(scene["materials"][name])
        lights = (LightDesc * max(1, len(scene["lights"])))()
        for i, L in enumerate(scene["lights"]):
            if L["type"] == "pointlight":
                lights[i].type = 1
                lights[i].corner[:] = [float(x) for x in L["from"]]
                lights[i].color[:] = [float(x) for x in L["color"]]
                lights[i].power = float(L["power"])
                lights[i].samples = 1
                continue
            if L["type"] != "arealight":
                raise ValueError(f"unsupported light type {L['type']}")
            lights[i].type = 0
            lights[i].corner[:] = [float(x) for x in L["corner"]]
            lights[i].point1[:] = [float(x) for x in L["point1"]]
            lights[i].point2[:] = [float(x) for x in L["point2"]]
            lights[i].color[:] = [float(x) for x in L["color"]]
            lights[i].power = float(L["power"])
            lights[i].samples = int(L["samples"])
        h = ctypes.c_void_p()
        fm = np.ascontiguousarray(self.face_mat, np.int32)
        check(load().gbrt_scene_create(self.bvh.handle, _ptr(self.vertices), len(self.vertices), _ptr(self.faces),
                                       len(self.faces), _ptr(fm), mats, len(self.mat_names), lights,
                                       len(scene["lights"]), ctypes.byref(h)))
        self._h = h
        if scene.get("textures") or scene.get("nodes"):
            self._set_textures()
        if any("smooth" in o or "normals" in o for o in scene["objects"]):
            self._set_normals()

    def _set_normals(self):
        """Shading normals of the objects with "smooth" (an angle, as
        yafaray_smoothObjectMesh) or explicit per-vertex "normals" (as
        yafaray_addNormal, one per vertex); other objects stay flat."""
        N, FN = [], []
        base = 0
        for o in self.scene["objects"]:
            v = np.asarray(o["vertices"], np.float32)
            f = np.asarray(o["faces"], np.uint32)
            tri = f[:, 3] == TRIANGLE
            if "normals" in o:
                n = np.asarray(o["normals"], np.float32).reshape(-1, 3)
                fn = f.copy()
                fn[tri, 3] = NO_NORMAL
            elif "smooth" in o:
                n, fn = smooth_normals(v, f, float(o["smooth"]))
            else:
                FN.append(np.full((len(f), 4), FLAT_FACE, np.uint32))
                continue
            fn = fn.copy()
            live = fn != NO_NORMAL
            fn[live] += base
            N.append(n)
            FN.append(fn)
            base += len(n)
        normals = np.ascontiguousarray(np.concatenate(N) if N else np.zeros((0, 3), np.float32), np.float32)
        face_normals = np.ascontiguousarray(np.concatenate(FN), np.uint32)
        check(load().gbrt_scene_set_normals(self._h, _ptr(normals), len(normals), _ptr(face_normals)))

    def _set_textures(self):
        """Image and procedural textures of the scene's "textures" entry on
        the shinydiffuse materials whose options name one
        ("diffuse_texture"), then the shader node trees ("nodes",
        "material_shaders"; shader_nodes); procedural textures need the
        scene's "noise_tables" (the reference's NoiseGenerator tables)."""
        from . import scenes as _scenes
        names = list(self.scene.get("textures", {}).keys())
        nodes, n_nodes, node_tex, index = shader_nodes(self.scene, len(names))
        all_tex = [self.scene["textures"][n] for n in names] + node_tex
        if any(t.get("type", "image") != "image" for t in all_tex):
            nt, self._noise_keep = noise_tables(self.scene["noise_tables"])
            check(load().gbrt_scene_set_noise_tables(self._h, ctypes.byref(nt)))
        descs, keep = (TextureDesc * max(1, len(all_tex)))(), []
        for i, t in enumerate(all_tex):
            d, img = texture_desc(t)
            descs[i] = d
            keep.append(img)
        mt = np.full(len(self.mat_names), -1, np.int32)
        for i, n in enumerate(self.mat_names):
            m = self.scene["materials"][n]
            if m[0] == "shinydiffusemat" and len(m) > 2 and m[2].get("diffuse_texture"):
                mt[i] = names.index(m[2]["diffuse_texture"])
        uv, fuv = _scenes.flatten_uvs(self.scene)
        if uv is not None:
            uv = np.ascontiguousarray(uv, np.float32)
            fuv = np.ascontiguousarray(fuv, np.uint32)
        check(load().gbrt_scene_set_textures(self._h, _ptr(uv), 0 if uv is None else len(uv), _ptr(fuv), descs, len(all_tex),
                                             _ptr(mt), len(mt)))
        if n_nodes:
            slots = np.full((len(self.mat_names), N_SLOTS), -1, np.int32)
            for i, n in enumerate(self.mat_names):
                for key, node in self.scene.get("material_shaders", {}).get(n, {}).items():
                    slots[i, SLOTS[key]] = index[node]
            check(load().gbrt_scene_set_shader_nodes(self._h, nodes, n_nodes, _ptr(slots), len(self.mat_names)))

    def close(self):
        if getattr(self, "_h", None):
            load().gbrt_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def kind(self):
        return self.scene["integrator"].get("type", "pathtracing")

    @property
    def is_pm(self):
        return self.kind == "photonmapping"

    def photons(self, which):
        """One photon map of this scene's photonmapping parameters (which =
        "diffuse" or "caustic"): (photons [n, 9] = dir, pos, col; n_paths)."""
        pm = pm_params(self.scene["integrator"])
        w = {"diffuse": 0, "caustic": 1}[which]
        n, paths = ctypes.c_uint32(), ctypes.c_uint32()
        check(load().gbrt_pm_photons(self._h, ctypes.byref(pm), w, None, 0, ctypes.byref(n), ctypes.byref(paths)))
        out = np.empty((max(1, n.value), 9), np.float32)
        check(load().gbrt_pm_photons(self._h, ctypes.byref(pm), w, _ptr(out), len(out), ctypes.byref(n), ctypes.byref(paths)))
        return out[:n.value], paths.value

    def make_guide(self, **kw):
        """A guiding network over this scene's tree bound."""
        return Guide(self.bvh.bound(), **kw)

    def camera_desc(self):
        c = self.scene["camera"]
        d = CameraDesc()
        d.from_[:] = [float(x) for x in c["from"]]
        d.to[:] = [float(x) for x in c["to"]]
        d.up[:] = [float(x) for x in c["up"]]
        d.resx, d.resy, d.focal = int(c["resx"]), int(c["resy"]), float(c["focal"])
        return d

    def params(self, spp, base_offset=0, seed=1, fp64=False, wave_paths=0, guide=None, alpha=0.0, train_steps=0,
               batch=0, max_vertex=0, weight_ptr=0):
        """gbrt_pt_params; the film filter comes from the scene's optional
        "film" entry ({"filter_type": ..., "AA_pixelwidth": ...}; default the
        single-pixel splat)."""
        it = self.scene["integrator"]
        film = self.scene.get("film", {})
        p = PtParams(int(spp), int(it.get("path_samples", 1)), int(it.get("bounces", 5)),
                     int(it.get("russian_roulette_min_bounces", 0)), int(base_offset), int(seed),
                     PT_FP64_FILM if fp64 else 0, int(wave_paths), guide.handle if guide is not None else None,
                     float(alpha), int(train_steps), int(batch), int(max_vertex), int(it.get("raydepth", 5)),
                     FILTERS[film.get("filter_type", "pixel")], float(film.get("AA_pixelwidth", 0.0)),
                     int(weight_ptr) or None, int(bool(it.get("transpShad", False))), int(it.get("shadowDepth", 4)))
        if self.kind == "pathtracing":
            p.caustic_type = CAUSTIC_TYPES[it.get("caustic_type", "path")]
            p.no_recursive = int(bool(it.get("no_recursive", False)))
            if p.caustic_type in (2, 3):
                self._caustic = pm_params(it)          # caustic_photons / _mix / _radius / _depth
                p.caustic = ctypes.addressof(self._caustic)
        p.clamp_indirect = float(film.get("AA_clamp_indirect", 0.0))
        return p

    def render(self, spp, base_offset=0, seed=1, fp64=False, guide=None, alpha=0.0, train_steps=0, batch=0,
               max_vertex=0):
        """Per-pixel mean image [resy, resx, 3] and stats dict."""
        cam = self.camera_desc()
        p = self.params(spp, base_offset, seed, fp64, 0, guide, alpha, train_steps, batch, max_vertex)
        img = np.empty((cam.resy, cam.resx, 3), np.float32)
        st = PtStats()
        if self.kind in ("photonmapping", "directlighting"):
            pm = pm_params(self.scene["integrator"])
            fn = load().gbrt_pm_render_host if self.kind == "photonmapping" else load().gbrt_dl_render_host
            check(fn(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(pm), _ptr(img), ctypes.byref(st)))
        elif self.kind == "SPPM":
            sp = sppm_params(self.scene["integrator"])
            check(load().gbrt_sppm_render_host(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(sp), _ptr(img),
                                               ctypes.byref(st)))
        else:
            check(load().gbrt_pt_render_host(self._h, ctypes.byref(cam), ctypes.byref(p), _ptr(img), ctypes.byref(st)))
        return img, {"camera_samples": st.camera_samples, "extension_rays": st.extension_rays,
                     "shadow_rays": st.shadow_rays, "ms": st.ms}

    def render_aa(self, spp=None, base_offset=0, seed=1):
        """Adaptive anti-aliasing render (TiledIntegrator::render's passes)
        with the scene's "film" AA parameters: (mean image [resy, resx, 3],
        stats dict, pixels rendered per pass).  spp: AA_minsamples."""
        if self.kind not in ("pathtracing", "photonmapping", "directlighting"):
            raise ValueError(f"adaptive AA passes are not built for the {self.kind} integrator")
        film = self.scene.get("film", {})
        spp = int(film.get("AA_minsamples", 1)) if spp is None else int(spp)
        aa = aa_params(film)
        cam = self.camera_desc()
        p = self.params(spp, base_offset, seed)
        img = np.empty((cam.resy, cam.resx, 3), np.float32)
        res = np.zeros(max(1, aa.passes), np.uint32)
        st = PtStats()
        if self.kind == "pathtracing":
            check(load().gbrt_pt_render_aa_host(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(aa), _ptr(img),
                                                ctypes.byref(st), _ptr(res)))
        else:
            pm = pm_params(self.scene["integrator"])
            fn = load().gbrt_pm_render_aa_host if self.kind == "photonmapping" else load().gbrt_dl_render_aa_host
            check(fn(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(pm), ctypes.byref(aa), _ptr(img),
                     ctypes.byref(st), _ptr(res)))
        return img, {"camera_samples": st.camera_samples, "extension_rays": st.extension_rays,
                     "shadow_rays": st.shadow_rays, "ms": st.ms}, res.tolist()

    def render_aa_device(self, film_ptr, weight_ptr, spp=None, base_offset=0, seed=1, stream=0):
        """Adaptive AA passes into a device film (float RGB sums) and its
        filter weights; returns the pixels rendered per pass."""
        film = self.scene.get("film", {})
        spp = int(film.get("AA_minsamples", 1)) if spp is None else int(spp)
        aa = aa_params(film)
        cam = self.camera_desc()
        p = self.params(spp, base_offset, seed, weight_ptr=weight_ptr)
        res = np.zeros(max(1, aa.passes), np.uint32)
        check(load().gbrt_pt_render_aa(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(aa),
                                       ctypes.c_void_p(film_ptr), None, _ptr(res), ctypes.c_void_p(stream)))
        return res.tolist()

    def render_device(self, spp, film_ptr, film64_ptr=0, base_offset=0, seed=1, stream=0, stats=False, wave_paths=0,
                      guide=None, alpha=0.0, train_steps=0, batch=0, max_vertex=0, radiance_target=False, weight_ptr=0):
        """Adds sample sums into a device film (float or double RGB); with a
        filtered film (scene "film" entry) the filter weights go to weight_ptr."""
        cam = self.camera_desc()
        p = self.params(spp, base_offset, seed, bool(film64_ptr), wave_paths, guide, alpha, train_steps, batch,
                        max_vertex, weight_ptr)
        if radiance_target:
            p.flags |= PT_GUIDE_RADIANCE
        st = PtStats()
        if self.kind in ("photonmapping", "directlighting"):
            pm = pm_params(self.scene["integrator"])
            fn = load().gbrt_pm_render if self.kind == "photonmapping" else load().gbrt_dl_render
            check(fn(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.byref(pm), ctypes.c_void_p(film_ptr or None),
                     ctypes.c_void_p(film64_ptr or None), ctypes.byref(st) if stats else None, ctypes.c_void_p(stream)))
        else:
            check(load().gbrt_pt_render(self._h, ctypes.byref(cam), ctypes.byref(p), ctypes.c_void_p(film_ptr or None),
                                        ctypes.c_void_p(film64_ptr or None), ctypes.byref(st) if stats else None,
                                        ctypes.c_void_p(stream)))
        if stats:
            out = {"camera_samples": st.camera_samples, "extension_rays": st.extension_rays,
                   "shadow_rays": st.shadow_rays, "ms": st.ms}
            if self.is_pm:
                out.update(photon_paths=st.photon_paths, photons_stored=st.photons_stored,
                           radiance_photons=st.radiance_photons, photon_ms=st.photon_ms)
            return out
        return None


def host_path_direct(rays_ptr, n, out_ptr, shadow=False):
    """True when gbrt_trace_*_host would trace these host buffers in place
    (one launch), False when it would stage them in chunks."""
    d = ctypes.c_int(0)
    check(load().gbrt_host_path(ctypes.c_void_p(rays_ptr), int(n), ctypes.c_void_p(out_ptr), 1 if shadow else 0, ctypes.byref(d)))
    return bool(d.value)


def aa_flags(film_ptr, weight_ptr, resx, resy, aa, threshold, flags_ptr):
    """ImageFilm::nextPass's resample flags of a device film (float RGB sums
    and filter weights) into a device uint8 buffer; returns the flagged count."""
    n = ctypes.c_uint32()
    check(load().gbrt_aa_flags(ctypes.c_void_p(film_ptr), ctypes.c_void_p(weight_ptr), int(resx), int(resy),
                               ctypes.byref(aa), float(threshold), ctypes.c_void_p(flags_ptr), ctypes.byref(n)))
    return n.value


def sampler_eval(kind, dim, inputs, on_device):
    x = np.ascontiguousarray(inputs, np.uint32)
    out = np.empty(len(x), np.float64)
    check(load().gbrt_sampler_eval(int(kind), int(dim), _ptr(x), len(x), _ptr(out), int(bool(on_device))))
    return out


class Guide:
    """Path-guiding network handle (gbrt_guide)."""

    def __init__(self, bound, log2_table=19, base_resolution=16.0, max_resolution=2048.0, learning_rate=5e-3, seed=1):
        b = (ctypes.c_float * 6)(*[float(x) for x in bound])
        p = GuideParams(log2_table, base_resolution, max_resolution, learning_rate, seed)
        h = ctypes.c_void_p()
        check(load().gbrt_guide_create(b, ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        n_mlp, n_tab = ctypes.c_uint32(), ctypes.c_uint64()
        check(load().gbrt_guide_info(h, ctypes.byref(n_mlp), ctypes.byref(n_tab)))
        self.n_mlp, self.n_table = n_mlp.value, n_tab.value
        self.log2_table = log2_table

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            load().gbrt_guide_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        mlp = np.empty(self.n_mlp, np.float32)
        tab = np.empty(self.n_table, np.float32)
        check(load().gbrt_guide_get_params(self._h, _ptr(mlp), _ptr(tab)))
        return mlp, tab.reshape(16, 1 << self.log2_table, 2)

    def set_params(self, mlp=None, table=None):
        m = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        check(load().gbrt_guide_set_params(self._h, _ptr(m), _ptr(t)))

    def grads(self):
        mlp = np.empty(self.n_mlp, np.float32)
        tab = np.empty(self.n_table, np.float32)
        check(load().gbrt_guide_get_grads(self._h, _ptr(mlp), _ptr(tab)))
        return mlp, tab.reshape(16, 1 << self.log2_table, 2)

    EVAL_TENSOR, EVAL_FP32 = 0, 1

    def set_eval_mode(self, mode):
        """EVAL_TENSOR (tcgen05, BF16 operands, the default) or EVAL_FP32."""
        check(load().gbrt_guide_set_eval_mode(self._h, int(mode)))

    def status(self):
        """Reads and clears the device status flags (bit 0: an MMA wait timed out)."""
        f = ctypes.c_uint32()
        check(load().gbrt_guide_status(self._h, ctypes.byref(f)))
        return f.value

    def eval_device(self, pos_ptr, n, lobes_ptr, stream=0):
        check(load().gbrt_guide_eval(self._h, ctypes.c_void_p(pos_ptr), n, ctypes.c_void_p(lobes_ptr), ctypes.c_void_p(stream)))

    def grad_device(self, rec_ptr, n, stream=0):
        loss = ctypes.c_float()
        check(load().gbrt_guide_grad(self._h, ctypes.c_void_p(rec_ptr), n, ctypes.byref(loss), ctypes.c_void_p(stream)))
        return loss.value

    def step_device(self, rec_ptr, n, stream=0):
        loss = ctypes.c_float()
        check(load().gbrt_guide_step(self._h, ctypes.c_void_p(rec_ptr), n, ctypes.byref(loss), ctypes.c_void_p(stream)))
        return loss.value


def tc_selftest(a, b):
    """D = A B^T through one tcgen05 MMA chain (BF16 operands, FP32
    accumulation); A [128, K], B [N, K]."""
    A = np.ascontiguousarray(a, np.float32)
    B = np.ascontiguousarray(b, np.float32)
    n, k = B.shape
    assert A.shape == (128, k)
    D = np.empty((128, n), np.float32)
    check(load().gbrt_tc_selftest(_ptr(A), _ptr(B), n, k, _ptr(D)))
    return D


def guide_forward_host(bound, mlp, table, pos, log2_table=19, base_resolution=16.0, max_resolution=2048.0):
    """Host build of the guide's forward pass: lobes [n, 40]."""
    b = (ctypes.c_float * 6)(*[float(x) for x in bound])
    p = GuideParams(log2_table, base_resolution, max_resolution, 0.0, 0)
    m = np.ascontiguousarray(mlp, np.float32)
    t = np.ascontiguousarray(table, np.float32)
    x = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    out = np.empty((len(x), 40), np.float32)
    check(load().gbrt_guide_forward_host(b, ctypes.byref(p), _ptr(m), _ptr(t), _ptr(x), len(x), _ptr(out)))
    return out


def knn_gather(points, queries, cell, k, r2):
    """PhotonMap::gather semantics on the device grid: (count [m], final r2
    [m], indices [m, k] of the found points, unordered; -1 past count)."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    Q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    m = len(Q)
    cnt = np.empty(m, np.int32)
    rr = np.empty(m, np.float32)
    idx = np.full((m, k), 0xFFFFFFFF, np.uint32)
    check(load().gbrt_knn_gather(_ptr(P), len(P), _ptr(Q), m, float(cell), int(k), float(r2), _ptr(cnt), _ptr(rr), _ptr(idx)))
    return cnt, rr, idx.astype(np.int64) - np.where(idx == 0xFFFFFFFF, 1 << 32, 0)


class BatchTuning(ctypes.Structure):
    _fields_ = [("wave_paths", ctypes.c_uint32), ("shade_block", ctypes.c_uint32), ("trace_blocks_per_sm", ctypes.c_uint32),
                ("streams", ctypes.c_uint32), ("tune_ms", ctypes.c_float)]


def render_multi(renderers, spp, film_ptrs, tuning=None, base_offset=0, seed=1, stream=0):
    """gbrt_pt_render_multi: every Renderer's scene into its device float film
    (pointer) in one wavefront.  tuning: None (autotune) or a dict with
    wave_paths / shade_block / trace_blocks_per_sm / streams (missing or 0 =
    tuned).
    Returns (stats dict of the batch, the tuning used incl. tune_ms)."""
    n = len(renderers)
    S = (ctypes.c_void_p * n)(*[r._h.value for r in renderers])
    cams = (CameraDesc * n)(*[r.camera_desc() for r in renderers])
    ps = (PtParams * n)(*[r.params(spp, base_offset, seed) for r in renderers])
    F = (ctypes.c_void_p * n)(*[int(f) for f in film_ptrs])
    t = BatchTuning()
    for k, v in (tuning or {}).items():
        if k != "tune_ms":
            setattr(t, k, int(v))
    st = PtStats()
    check(load().gbrt_pt_render_multi(S, cams, ps, F, n, ctypes.byref(t), ctypes.byref(st), ctypes.c_void_p(stream)))
    return ({"camera_samples": st.camera_samples, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
             "ms": st.ms},
            {"wave_paths": t.wave_paths, "shade_block": t.shade_block, "trace_blocks_per_sm": t.trace_blocks_per_sm,
             "streams": t.streams, "tune_ms": t.tune_ms})


def render_batch(renderers, spp, film_ptrs, concurrency=8, base_offset=0, seed=1):
    """gbrt_pt_render_batch: renders every Renderer's scene into its device
    float film (pointer), all in one wavefront (autotuned).  Returns the
    per-scene stats (rays and device time of the batch in entry 0)."""
    n = len(renderers)
    S = (ctypes.c_void_p * n)(*[r._h.value for r in renderers])
    cams = (CameraDesc * n)(*[r.camera_desc() for r in renderers])
    ps = (PtParams * n)(*[r.params(spp, base_offset, seed) for r in renderers])
    F = (ctypes.c_void_p * n)(*[int(f) for f in film_ptrs])
    st = (PtStats * n)()
    check(load().gbrt_pt_render_batch(S, cams, ps, F, n, int(concurrency), st))
    return [{"camera_samples": x.camera_samples, "extension_rays": x.extension_rays, "shadow_rays": x.shadow_rays,
             "ms": x.ms} for x in st]


def grid_buckets(points, cell_size, grid_size, box_lo):
    """Bucket of each point under the reference HashGrid's cell assignment."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    lo = (ctypes.c_float * 3)(*[float(x) for x in box_lo])
    out = np.empty(len(P), np.uint32)
    check(load().gbrt_grid_buckets(_ptr(P), len(P), float(cell_size), int(grid_size), lo, _ptr(out)))
    return out
