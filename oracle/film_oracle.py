"""CPU restatement of the reference's image-film splat, for tests only.

Test infrastructure: imported by tests/ to check the GPU film; never part of
the product path.

Follows
  * sample positions: TiledIntegrator::renderTile (src/integrator/surface/
    integrator_tiled.cc:297, 316-323): pixel offset fnv32ABuf(y *
    fnv32ABuf(x)); one sample -> (0.5, 0.5); n > 1 samples ->
    ((0.5 + s) / n, riLp(s + offset)); sample::riLp and sample::fnv32ABuf
    (include/sampler/sample.h:118-148);
  * the filter table: ImageFilm::ImageFilm (src/render/imagefilm.cc:231-264)
    with math::filter::box / gauss / mitchell / lanczos2
    (include/math/filter.h:30-86) and FAST_MATH exp = exp2(log2e x)
    (include/math/math.h:116-127, 200-206);
  * the splat: ImageFilm::addSample (imagefilm.cc:771-822) with
    roundToIntWithBias (include/render/imagefilm.h:344-348);
  * normalisation: Rgba::normalized (include/color/color.h:538-542);
  * adaptive anti-aliasing: the resample flags of ImageFilm::nextPass
    (imagefilm.cc:399-512) with Rgba::colorDifference / col2Bri / abscol2Bri
    (color.h:57-58, 434-452) and darkThresholdCurveInterpolate
    (imagefilm.cc:882-899); multipass sample positions (riVdC, riS of
    pass offset + sample, integrator_tiled.cc:316-319; sample.h:99-114).

The sampler functions are pinned bit for bit against the reference's own
values in tests/golden/sampler.npz (made by the compiled reference).
"""
import numpy as np

F32 = np.float32
TABLE = 16
MAX_FILTER = 8


def fnv32a(values):
    """sample::fnv32ABuf over the 4 little-endian bytes of each uint32."""
    v = np.asarray(values, np.uint32).astype(np.uint64)
    h = np.full(v.shape, 0x811C9DC5, np.uint64)
    for k in range(4):
        h ^= (v >> np.uint64(8 * k)) & np.uint64(0xFF)
        h = (h * np.uint64(0x01000193)) & np.uint64(0xFFFFFFFF)
    return h.astype(np.uint32)


def ri_lp(values, r=0):
    """sample::riLp: Larcher-Pillichshammer radical inverse, float32."""
    i = np.asarray(values, np.uint32).astype(np.uint64).copy()
    acc = np.full(i.shape, r, np.uint64)
    v = np.full(i.shape, 1 << 31, np.uint64)
    while (i != 0).any():
        acc = np.where(i & np.uint64(1), acc ^ v, acc)
        i >>= np.uint64(1)
        v |= v >> np.uint64(1)
    return np.clip((acc.astype(np.float64) * 2.0 ** -32).astype(F32), F32(0), F32(1))


def ri_vdc(values, r=0):
    """sample::riVdC: bit-reversed radical inverse xor r, float32."""
    b = np.asarray(values, np.uint32).astype(np.uint64)
    rev = np.zeros_like(b)
    for k in range(32):
        rev |= ((b >> np.uint64(k)) & np.uint64(1)) << np.uint64(31 - k)
    v = (rev ^ np.asarray(r, np.uint64)).astype(np.float64) * 2.0 ** -32
    return np.clip(v.astype(F32), F32(0), F32(1))


def ri_s(values, r=0):
    """sample::riS: Sobol second dimension xor r, float32."""
    i = np.asarray(values, np.uint32).astype(np.uint64).copy()
    acc = (np.zeros(i.shape, np.uint64) + np.asarray(r, np.uint64)).astype(np.uint64)
    v = np.full(i.shape, 1 << 31, np.uint64)
    while (i != 0).any():
        acc = np.where(i & np.uint64(1), acc ^ v, acc)
        i >>= np.uint64(1)
        v ^= v >> np.uint64(1)
    return np.clip((acc.astype(np.float64) * 2.0 ** -32).astype(F32), F32(0), F32(1))


def pixel_offset(x, y):
    """fnv32ABuf(y * fnv32ABuf(x)) (integrator_tiled.cc:297; x = column j, y = row i)."""
    inner = fnv32a(np.asarray(x, np.uint32))
    return fnv32a((np.asarray(y, np.uint64) * inner.astype(np.uint64)).astype(np.uint32))


def sample_positions(x, y, sample, n_samples, multipass=False, pass_offset=0):
    """(dx, dy) of camera sample `sample` of n in pixel (x, y); with AA_passes
    > 1 every pass takes riVdC / riS of sample_ = pass offset + sample,
    scrambled by the pixel offset."""
    if multipass:
        off = pixel_offset(x, y)
        s_ = (np.asarray(sample, np.uint64) + np.uint64(pass_offset)).astype(np.uint32)
        return ri_vdc(s_, off), ri_s(s_, off)
    if n_samples <= 1:
        z = np.full(np.shape(sample), F32(0.5))
        return z, z.copy()
    d1 = F32(1) / F32(n_samples)
    dx = ((F32(0.5) + np.asarray(sample, np.float32)) * d1).astype(F32)
    dy = ri_lp((np.asarray(sample, np.uint64) + pixel_offset(x, y).astype(np.uint64)).astype(np.uint32))
    return dx, dy


def _exp2(x):
    """FAST_MATH exp2 (math.h:116-127), float32."""
    x = np.asarray(x, F32)
    xl = np.maximum(np.minimum(x, F32(129.0)), F32(-126.99999))
    ipart = (xl - F32(0.5)).astype(np.int32)
    fpart = (xl - ipart.astype(F32)).astype(F32)
    p = fpart * F32(1.8775767e-3) + F32(8.9893397e-3)
    p = fpart * p + F32(5.5826318e-2)
    p = fpart * p + F32(2.4015361e-1)
    p = fpart * p + F32(6.9315308e-1)
    p = fpart * p + F32(9.9999994e-1)
    scale = ((ipart + 127).astype(np.int64) << 23).astype(np.uint32).view(F32)
    return (scale * p).astype(F32)


def _log2(x):
    """FAST_MATH log2 (math.h:129-146), float32 (used to pin _exp2 through the
    reference's pow values: pow(a, b) = exp2(log2(a) b))."""
    x = np.asarray(x, F32)
    i = x.view(np.int32)
    m = ((i & 0x7FFFFF) | np.int32(0x3F800000)).view(F32)
    e = (((i & 0x7F800000) >> 23) - 127).astype(F32)
    p = m * F32(-3.4436006e-2) + F32(3.1821337e-1)
    p = m * p + F32(-1.2315303)
    p = m * p + F32(2.5988452)
    p = m * p + F32(-3.3241990)
    p = m * p + F32(3.1157899)
    return (p * (m - F32(1)) + e).astype(F32)


def filter_table(kind, pixel_width=1.5):
    """(table [16,16] float32, filter width, table scale) for "box" / "gauss" / "mitchell"."""
    width = F32(F32(pixel_width) * F32(0.5))
    if kind == "mitchell":
        width = F32(width * F32(2.6))
    elif kind == "gauss":
        width = F32(width * F32(2.0))
    width = F32(min(max(F32(0.501), width), F32(0.5 * MAX_FILTER)))
    c = ((np.arange(TABLE, dtype=F32) + F32(0.5)) * F32(1.0 / TABLE)).astype(F32)
    dx, dy = np.meshgrid(c, c)          # [y, x]
    r2 = (dx * dx + dy * dy).astype(F32)
    if kind == "box":
        t = np.ones((TABLE, TABLE), F32)
    elif kind == "gauss":
        e = _exp2(F32(1.4426950408889634) * (F32(-6.0) * r2))
        t = np.maximum(F32(0), (e - F32(0.00247875)).astype(F32))
    elif kind == "mitchell":
        x = (F32(2) * np.sqrt(r2)).astype(F32)
        far = x * (x * (x * F32(-0.38888889) + F32(2.0)) - F32(3.33333333)) + F32(1.77777778)
        near = x * x * (F32(1.16666666) * x - F32(2.0)) + F32(0.88888889)
        t = np.where(x >= F32(2), F32(0), np.where(x >= F32(1), far, near)).astype(F32)
    else:
        raise ValueError(kind)
    scale = F32(F32(0.9999) * F32(TABLE) / width)
    return t.astype(F32), float(width), float(scale)


def _round_bias(v):
    return np.trunc(np.asarray(v, np.float64) + (0.5 - 1.4e-11)).astype(np.int64)


def splat_weights(resx, resy, n_samples, kind, pixel_width=1.5, multipass=False, pass_offset=0, pixels=None):
    """Weight image [resy, resx] (float64 sums) of every camera sample of
    every pixel (or of the pixels y resx + x listed in `pixels`)."""
    table, width, scale = filter_table(kind, pixel_width)
    if pixels is None:
        ys, xs = np.mgrid[0:resy, 0:resx]
        xs, ys = xs.ravel(), ys.ravel()
    else:
        pixels = np.asarray(pixels, np.int64)
        xs, ys = pixels % resx, pixels // resx
    npx = len(xs)
    xs = np.repeat(xs, n_samples)
    ys = np.repeat(ys, n_samples)
    ss = np.tile(np.arange(n_samples), npx)
    dx, dy = sample_positions(xs, ys, ss, n_samples, multipass, pass_offset)
    dx = dx.astype(np.float64)
    dy = dy.astype(np.float64)
    dx0 = np.maximum(-xs, _round_bias(dx - width))
    dx1 = np.minimum(resx - 1 - xs, _round_bias(dx + width - 1.0))
    dy0 = np.maximum(-ys, _round_bias(dy - width))
    dy1 = np.minimum(resy - 1 - ys, _round_bias(dy + width - 1.0))
    out = np.zeros((resy, resx), np.float64)
    for j in range(-MAX_FILTER, MAX_FILTER + 1):
        yi = np.floor(np.abs((j - (dy - 0.5)) * scale)).astype(np.int64)
        okj = (j >= dy0) & (j <= dy1)
        for i in range(-MAX_FILTER, MAX_FILTER + 1):
            ok = okj & (i >= dx0) & (i <= dx1)
            if not ok.any():
                continue
            xi = np.floor(np.abs((i - (dx - 0.5)) * scale)).astype(np.int64)
            w = table[np.minimum(yi[ok], TABLE - 1), np.minimum(xi[ok], TABLE - 1)].astype(np.float64)
            np.add.at(out, (ys[ok] + j, xs[ok] + i), w)
    return out


# ---- adaptive anti-aliasing: ImageFilm::nextPass ----

def _bri(r, g, b):
    """Rgb::col2Bri in float32, unfused, left to right."""
    return ((F32(0.2126) * r + F32(0.7152) * g).astype(F32) + (F32(0.0722) * b)).astype(F32)


_CURVE_B = np.array([0.10, 0.20, 0.30, 0.40, 0.50, 0.60, 0.70, 0.80, 0.90, 1.00, 1.20, 1.40, 1.80], F32)
_CURVE_T = np.array([0.0001, 0.0010, 0.0020, 0.0035, 0.0055, 0.0075, 0.0100, 0.0150, 0.0250, 0.0400, 0.0800,
                     0.0950, 0.1000], F32)
_CURVE_W = np.array([0.0, 0.10, 0.10, 0.10, 0.10, 0.10, 0.10, 0.10, 0.10, 0.10, 0.20, 0.20, 0.40], F32)


def dark_curve(b):
    """darkThresholdCurveInterpolate: piecewise linear in brightness, float32."""
    b = np.asarray(b, F32)
    out = np.full(b.shape, _CURVE_T[-1], F32)
    done = np.zeros(b.shape, bool)
    m = b <= _CURVE_B[0]
    out[m] = _CURVE_T[0]
    done |= m
    for k in range(1, len(_CURVE_B)):
        m = ~done & (b <= _CURVE_B[k])
        dt = F32(_CURVE_T[k] - _CURVE_T[k - 1])
        seg = (((b - _CURVE_B[k - 1]).astype(F32) * dt).astype(F32) / _CURVE_W[k]).astype(F32)
        out[m] = (_CURVE_T[k - 1] + seg[m]).astype(F32)
        done |= m
    return out


def normalized(sums, weights):
    """Rgba::normalized of film sums [H, W, 4] (rgba) by weights [H, W]: x (1 / w), 0 where w is 0."""
    w = np.asarray(weights, F32)
    nz = w != F32(0)
    inv = np.where(nz, F32(1) / np.where(nz, w, F32(1)), F32(0)).astype(F32)
    return (np.asarray(sums, F32) * inv[..., None]).astype(F32) * nz[..., None]


def aa_flags(sums, weights, threshold, detect_color_noise=False, dark_detection="none", dark_threshold_factor=0.0,
             variance_edge_size=10, variance_pixels=0):
    """Resample flags [H, W] of one ImageFilm::nextPass with threshold > 0.

    sums: combined-layer sums [H, W, 4] (rgba; with opaque samples a = the
    weight sum), weights: filter weights [H, W]."""
    w = np.asarray(weights, F32)
    H, W = w.shape
    c = normalized(sums, w)
    flags = ~(w > F32(0))
    if W < 2 or H < 2:
        return flags
    thr0 = F32(threshold)
    core = c[:H - 1, :W - 1]
    bri_abs = _bri(np.abs(core[..., 0]), np.abs(core[..., 1]), np.abs(core[..., 2]))
    if dark_detection == "linear" and dark_threshold_factor > 0:
        f = F32(dark_threshold_factor)
        thr = (thr0 * ((F32(1) - f) + (bri_abs * f).astype(F32)).astype(F32)).astype(F32)
    elif dark_detection == "curve":
        thr = dark_curve(bri_abs)
    else:
        thr = np.full((H - 1, W - 1), thr0, F32)
    bri = _bri(c[..., 0], c[..., 1], c[..., 2])

    def diff(a_yx, b_yx):
        d = np.abs((bri[b_yx] - bri[a_yx]).astype(F32))
        if detect_color_noise:
            for ch in range(4):
                d = np.maximum(d, np.abs((c[b_yx][..., ch] - c[a_yx][..., ch]).astype(F32)))
        return d

    ys, xs = np.mgrid[0:H - 1, 0:W - 1]
    here = (ys, xs)
    for dy, dx in ((0, 1), (1, 0), (1, 1), (1, -1)):
        ny, nx = ys + dy, xs + dx
        ok = nx >= 0
        nxc = np.maximum(nx, 0)
        m = ok & (diff(here, (ny, nxc)) >= thr)
        flags[ys[m], xs[m]] = True
        flags[ny[m], nxc[m]] = True
    if variance_pixels > 0:
        h = variance_edge_size // 2
        vx = np.zeros((H - 1, W - 1), np.int64)
        vy = np.zeros((H - 1, W - 1), np.int64)
        for d in range(-h, h - 1):
            xi = np.clip(xs + d, 0, W - 2)
            vx += diff((ys, xi), (ys, xi + 1)) >= thr
            yi = np.clip(ys + d, 0, H - 2)
            vy += diff((yi, xs), (yi + 1, xs)) >= thr
        m = (vx + vy) >= variance_pixels
        for ddx in range(-h, h):
            for ddy in range(-h, h):
                flags[np.clip(ys[m] + ddy, 0, H - 1), np.clip(xs[m] + ddx, 0, W - 1)] = True
    return flags
