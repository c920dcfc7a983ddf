// Procedural textures of the reference, host and device: the noise
// generators (src/noise/generator/*.cc), turbulence and cell colour
// (src/noise/noise_generator.cc), the Musgrave fractals
// (src/noise/musgrave/*.cc), the blend / clouds / marble / wood / voronoi /
// musgrave / distorted_noise / rgb_cube textures (src/texture/texture_*.cc),
// the colour ramp (src/color/color_ramp.cc) and Texture's colour
// adjustments (src/texture/texture.cc:219-287).
//
// The float operations follow the reference's order (its FAST_MATH pow and
// FAST_TRIG sin, std::floor / sqrt / fmod, which are exact or correctly
// rounded on both sides), so a texture evaluates bit for bit like the
// reference's.  Translation units that include this compile without
// floating-point contraction (--fmad=false on the device, -ffp-contract=off
// on the host).
//
// The permutation and gradient tables the generators index are the host
// application's (libYafaRay's NoiseGenerator tables): the library carries no
// copy and takes them through gbrt_scene_set_noise_tables / gbrt_texture_eval.
#pragma once

#include "gbrt.h"
#include "sampling.cuh"

#include <cmath>
#include <cstdint>

namespace gbrt {

// The reference's noise tables (gbrt_noise_tables).
struct NoiseTables {
	const uint8_t *hash;        // 512 entries
	const float *hashpntf;      // 768
	const float *hashvectf;     // 768
	const uint8_t *stdp_p;      // 514
	const float *stdp_g;        // 514 x 3
};

// A procedural texture as the kernels read it (gbrt_procedural_desc with the
// reference's derived members precomputed).
struct ProcTex {
	uint32_t kind;
	uint32_t noise1, noise2;
	float c1[3], c2[3];
	float size;
	int32_t depth, hard;
	uint32_t bias, shape, wood_type, blend_type;
	int32_t flip_axis;
	float sharpness;            // marble: 1 / sharpness when sharpness > 1, else 1 (texture_marble.h)
	float turbulence;
	uint32_t metric, color_mode;
	float w[4], aw[4];          // voronoi weights and |weights|
	float mk_exp, intensity, iscale;   // iscale: intensity / sum |w| (0 when that sum is 0)
	uint32_t musgrave_type;
	float h, lacunarity, octaves, offset, gain;
	float distort;
	// adjustments (Texture::Params) and the colour ramp
	int32_t adj;                // adjustments_set_
	float intensity_adj, contrast, saturation, hue6;   // hue6 = adj_hue / 60 (adj_hue_radians_)
	float mult[3];
	int32_t adj_clamp;
	int32_t ramp_n;
	uint32_t ramp_mode, ramp_interp, ramp_hue;
	float ramp[GBRT_RAMP_MAX][5];   // sorted by position: r, g, b, a, position
};

GBRT_HD float lerp_f(float y1, float y2, float x) { return y1 * (1.f - x) + y2 * x; }

// math::lerpSegment (include/math/interpolation.h:47-58)
GBRT_HD float lerp_segment(float x, float y1, float x1, float y2, float x2)
{
	if(x == x1 || x1 == x2) return y1;
	if(x == x2) return y2;
	const float dy = y2 - y1;
	const float dx = x2 - x1;
	const float da = x - x1;
	return y1 + ((da / dx) * dy);
}

// math::pow with FAST_MATH (include/math/math.h:177-184)
GBRT_HD float fpow(float a, float b) { return fast_exp2(fast_log2(a) * b); }

// ---- noise generators -------------------------------------------------------

// BlenderNoiseGenerator::operator() (noise_blender.cc:25-92)
GBRT_HD float noise_blender(const NoiseTables &T, float x, float y, float z)
{
	const int ix = static_cast<int>(floorf(x)), iy = static_cast<int>(floorf(y)), iz = static_cast<int>(floorf(z));
	const float ox = x - ix, oy = y - iy, oz = z - iz;
	const float jx = ox - 1.f, jy = oy - 1.f, jz = oz - 1.f;
	float cn1 = ox * ox, cn2 = oy * oy, cn3 = oz * oz, cn4 = jx * jx, cn5 = jy * jy, cn6 = jz * jz;
	cn1 = 1.f - 3.f * cn1 + 2.f * cn1 * ox;
	cn2 = 1.f - 3.f * cn2 + 2.f * cn2 * oy;
	cn3 = 1.f - 3.f * cn3 + 2.f * cn3 * oz;
	cn4 = 1.f - 3.f * cn4 - 2.f * cn4 * jx;
	cn5 = 1.f - 3.f * cn5 - 2.f * cn5 * jy;
	cn6 = 1.f - 3.f * cn6 - 2.f * cn6 * jz;
	const uint8_t *H = T.hash;
	const int b00 = H[H[ix & 255] + (iy & 255)];
	const int b10 = H[H[(ix + 1) & 255] + (iy & 255)];
	const int b01 = H[H[ix & 255] + ((iy + 1) & 255)];
	const int b11 = H[H[(ix + 1) & 255] + ((iy + 1) & 255)];
	const int b20 = iz & 255, b21 = (iz + 1) & 255;
	float n = 0.5f;
	auto corner = [&](float i, int hidx, float a, float b, float c) {
		const float *h = T.hashvectf + 3 * H[hidx];
		n += i * (h[0] * a + h[1] * b + h[2] * c);
	};
	corner(cn1 * cn2 * cn3, b20 + b00, ox, oy, oz);
	corner(cn1 * cn2 * cn6, b21 + b00, ox, oy, jz);
	corner(cn1 * cn5 * cn3, b20 + b01, ox, jy, oz);
	corner(cn1 * cn5 * cn6, b21 + b01, ox, jy, jz);
	corner(cn4 * cn2 * cn3, b20 + b10, jx, oy, oz);
	corner(cn4 * cn2 * cn6, b21 + b10, jx, oy, jz);
	corner(cn4 * cn5 * cn3, b20 + b11, jx, jy, oz);
	corner(cn4 * cn5 * cn6, b21 + b11, jx, jy, jz);
	if(n < 0.f) n = 0.f;
	else if(n > 1.f) n = 1.f;
	return n;
}

// StdPerlinNoiseGenerator::operator() (noise_perlin_standard.cc:37-96)
GBRT_HD float noise_stdperlin(const NoiseTables &T, float x, float y, float z)
{
	auto setup = [](float v, int &b0, int &b1, float &r0, float &r1) {
		const float t = v + 10000.f;
		b0 = static_cast<int>(t) & 255;
		b1 = (b0 + 1) & 255;
		r0 = t - static_cast<int>(t);
		r1 = r0 - 1.f;
	};
	int bx0, bx1, by0, by1, bz0, bz1;
	float rx0, rx1, ry0, ry1, rz0, rz1;
	setup(x, bx0, bx1, rx0, rx1);
	setup(y, by0, by1, ry0, ry1);
	setup(z, bz0, bz1, rz0, rz1);
	const uint8_t *P = T.stdp_p;
	const int i = P[bx0], j = P[bx1];
	const int b00 = P[i + by0], b10 = P[j + by0], b01 = P[i + by1], b11 = P[j + by1];
	auto surve = [](float t) { return t * t * (3.f - 2.f * t); };
	const float sx = surve(rx0), sy = surve(ry0), sz = surve(rz0);
	auto at = [&](float a, float b, float c, int g) { const float *q = T.stdp_g + 3 * g; return a * q[0] + b * q[1] + c * q[2]; };
	float u = at(rx0, ry0, rz0, b00 + bz0), v = at(rx1, ry0, rz0, b10 + bz0);
	float a = lerp_f(u, v, sx);
	u = at(rx0, ry1, rz0, b01 + bz0); v = at(rx1, ry1, rz0, b11 + bz0);
	float b = lerp_f(u, v, sx);
	const float c = lerp_f(a, b, sy);
	u = at(rx0, ry0, rz1, b00 + bz1); v = at(rx1, ry0, rz1, b10 + bz1);
	a = lerp_f(u, v, sx);
	u = at(rx0, ry1, rz1, b01 + bz1); v = at(rx1, ry1, rz1, b11 + bz1);
	b = lerp_f(u, v, sx);
	const float d = lerp_f(a, b, sy);
	return 0.5f + 0.75f * lerp_f(c, d, sz);
}

// NewPerlinNoiseGenerator::grad (noise_perlin_improved.h) and operator()
// (noise_perlin_improved.cc:24-61)
GBRT_HD float perlin_grad(int hash, float x, float y, float z)
{
	const int h = hash & 15;
	const float u = h < 8 ? x : y;
	const float v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
	return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}

GBRT_HD float noise_newperlin(const NoiseTables &T, float x, float y, float z)
{
	float u = floorf(x), v = floorf(y), w = floorf(z);
	const int xi = static_cast<int>(u) & 255, yi = static_cast<int>(v) & 255, zi = static_cast<int>(w) & 255;
	x -= u; y -= v; z -= w;
	auto fade = [](float t) { return t * t * t * (t * (t * 6 - 15) + 10); };
	u = fade(x); v = fade(y); w = fade(z);
	const uint8_t *H = T.hash;
	const int a = H[xi] + yi, aa = H[a] + zi, ab = H[a + 1] + zi;
	const int b = H[xi + 1] + yi, ba = H[b] + zi, bb = H[b + 1] + zi;
	const float l00 = lerp_f(perlin_grad(H[ab + 1], x, y - 1, z - 1), perlin_grad(H[bb + 1], x - 1, y - 1, z - 1), u);
	const float l01 = lerp_f(perlin_grad(H[aa + 1], x, y, z - 1), perlin_grad(H[ba + 1], x - 1, y, z - 1), u);
	const float l02 = lerp_f(l01, l00, v);
	const float l03 = lerp_f(perlin_grad(H[ab], x, y - 1, z), perlin_grad(H[bb], x - 1, y - 1, z), u);
	const float l04 = lerp_f(perlin_grad(H[aa], x, y, z), perlin_grad(H[ba], x - 1, y, z), u);
	const float l05 = lerp_f(l04, l03, v);
	const float nv = lerp_f(l05, l02, w);
	return 0.5f + 0.5f * nv;
}

// CellNoiseGenerator::operator() (noise_cell.cc:22-31)
GBRT_HD float noise_cell(float x, float y, float z)
{
	const int xi = static_cast<int>(floorf(x)), yi = static_cast<int>(floorf(y)), zi = static_cast<int>(floorf(z));
	uint32_t n = static_cast<uint32_t>(xi) + static_cast<uint32_t>(yi) * 1301u + static_cast<uint32_t>(zi) * 314159u;
	n ^= (n << 13);
	// float(n ...) / 2^32 in double, then float: the power-of-two scaling is exact
	return static_cast<float>(n * (n * n * 15731u + 789221u) + 1376312589u) * 2.3283064365386962890625e-10f;
}

// NoiseGenerator::hashPnt (noise_generator.cc:48-53)
GBRT_HD void hash_pnt(const NoiseTables &T, int x, int y, int z, float out[3])
{
	const uint8_t *H = T.hash;
	const int index = 3 * H[(H[(H[z & 255] + y) & 255] + x) & 255];
	if(index < 0 || index > 768 - 3) { out[0] = out[1] = out[2] = 0.f; return; }
	out[0] = T.hashpntf[index]; out[1] = T.hashpntf[index + 1]; out[2] = T.hashpntf[index + 2];
}

// VoronoiNoiseGenerator distance metrics (noise_voronoi.cc:23-63)
GBRT_HD float voronoi_dist(uint32_t metric, float x, float y, float z, float e)
{
	switch(metric)
	{
		case GBRT_DIST_SQUARED: return x * x + y * y + z * z;
		case GBRT_DIST_MANHATTAN: return fabsf(x) + fabsf(y) + fabsf(z);
		case GBRT_DIST_CHEBYCHEV:
		{
			x = fabsf(x); y = fabsf(y); z = fabsf(z);
			const float t = (x > y) ? x : y;
			return (z > t) ? z : t;
		}
		case GBRT_DIST_MINKOVSKY_HALF:
		{
			const float d = sqrtf(fabsf(x)) + sqrtf(fabsf(y)) + sqrtf(fabsf(z));
			return d * d;
		}
		case GBRT_DIST_MINKOVSKY_FOUR:
		{
			x *= x; y *= y; z *= z;
			return sqrtf(sqrtf(x * x + y * y + z * z));
		}
		case GBRT_DIST_MINKOVSKY: return fpow(fpow(fabsf(x), e) + fpow(fabsf(y), e) + fpow(fabsf(z), e), 1.0f / e);
		default: return sqrtf(x * x + y * y + z * z);
	}
}

// VoronoiNoiseGenerator::getFeatures (noise_voronoi.cc:82-123): the four
// nearest feature points of the 27 cells around p, nearest first.
GBRT_HD void voronoi_features(const NoiseTables &T, uint32_t metric, float e, const float p[3], float da[4], float pa[4][3])
{
	const int xi = static_cast<int>(floorf(p[0])), yi = static_cast<int>(floorf(p[1])), zi = static_cast<int>(floorf(p[2]));
	for(int k = 0; k < 4; ++k) { da[k] = 1e10f; pa[k][0] = pa[k][1] = pa[k][2] = 0.f; }
	for(int xx = xi - 1; xx <= xi + 1; ++xx)
		for(int yy = yi - 1; yy <= yi + 1; ++yy)
			for(int zz = zi - 1; zz <= zi + 1; ++zz)
			{
				float h[3];
				hash_pnt(T, xx, yy, zz, h);
				const float xd = p[0] - (h[0] + xx), yd = p[1] - (h[1] + yy), zd = p[2] - (h[2] + zz);
				const float d = voronoi_dist(metric, xd, yd, zd, e);
				const float q[3] = {h[0] + xx, h[1] + yy, h[2] + zz};
				int at = 4;
				if(d < da[0]) at = 0;
				else if(d < da[1]) at = 1;
				else if(d < da[2]) at = 2;
				else if(d < da[3]) at = 3;
				if(at < 4)
				{
					for(int k = 3; k > at; --k)
					{
						da[k] = da[k - 1];
						pa[k][0] = pa[k - 1][0]; pa[k][1] = pa[k - 1][1]; pa[k][2] = pa[k - 1][2];
					}
					da[at] = d;
					pa[at][0] = q[0]; pa[at][1] = q[1]; pa[at][2] = q[2];
				}
			}
}

// NoiseGenerator::newNoise + operator(): the voronoi types measure the real
// distance with exponent 2.5 (noise_generator.cc:29-45).
GBRT_HD float noise_eval(const NoiseTables &T, uint32_t type, float x, float y, float z)
{
	switch(type)
	{
		case GBRT_NOISE_BLENDER: return noise_blender(T, x, y, z);
		case GBRT_NOISE_STDPERLIN: return noise_stdperlin(T, x, y, z);
		case GBRT_NOISE_CELL: return noise_cell(x, y, z);
		case GBRT_NOISE_VORONOI_F1: case GBRT_NOISE_VORONOI_F2: case GBRT_NOISE_VORONOI_F3: case GBRT_NOISE_VORONOI_F4:
		case GBRT_NOISE_VORONOI_F2F1: case GBRT_NOISE_VORONOI_CRACKLE:
		{
			const float p[3] = {x, y, z};
			float da[4], pa[4][3];
			voronoi_features(T, GBRT_DIST_REAL, 2.5f, p, da, pa);
			switch(type)
			{
				case GBRT_NOISE_VORONOI_F2: return da[1];
				case GBRT_NOISE_VORONOI_F3: return da[2];
				case GBRT_NOISE_VORONOI_F4: return da[3];
				case GBRT_NOISE_VORONOI_F2F1: return da[1] - da[0];
				case GBRT_NOISE_VORONOI_CRACKLE: { const float t = 10.f * (da[1] - da[0]); return (t > 1.f) ? 1.f : t; }
				default: return da[0];
			}
		}
		default: return noise_newperlin(T, x, y, z);
	}
}

GBRT_HD float signed_noise(const NoiseTables &T, uint32_t type, float x, float y, float z) { return 2.f * noise_eval(T, type, x, y, z) - 1.f; }

// NoiseGenerator::turbulence (noise_generator.cc:67-78); blender noise
// offsets the point by one (noise_blender.h:33).
GBRT_HD float turbulence(const NoiseTables &T, uint32_t type, const float p[3], int oct, float size, bool hard)
{
	float amp = 1.f, sum = 0.f;
	float tp[3] = {p[0] * size, p[1] * size, p[2] * size};
	if(type == GBRT_NOISE_BLENDER) { tp[0] = (p[0] + 1.f) * size; tp[1] = (p[1] + 1.f) * size; tp[2] = (p[2] + 1.f) * size; }
	for(int i = 0; i <= oct; i++, amp *= 0.5f)
	{
		float val = noise_eval(T, type, tp[0], tp[1], tp[2]);
		if(hard) val = fabsf(2.f * val - 1.f);
		sum += amp * val;
		tp[0] *= 2.f; tp[1] *= 2.f; tp[2] *= 2.f;
	}
	return sum * (static_cast<float>(1 << oct) / static_cast<float>((1 << (oct + 1)) - 1));
}

// ---- Musgrave fractals (src/noise/musgrave/*.cc) ----------------------------
GBRT_HD float musgrave(const NoiseTables &T, const ProcTex &t, const float p[3])
{
	const uint32_t nt = t.noise1;
	const float pw_hl = fpow(t.lacunarity, -t.h);
	float tp[3] = {p[0], p[1], p[2]};
	auto scale_tp = [&]() { tp[0] *= t.lacunarity; tp[1] *= t.lacunarity; tp[2] *= t.lacunarity; };
	auto sn = [&]() { return signed_noise(T, nt, tp[0], tp[1], tp[2]); };
	const int oct = static_cast<int>(t.octaves);
	const float rmd = t.octaves - floorf(t.octaves);
	switch(t.musgrave_type)
	{
		case GBRT_MUSGRAVE_MULTIFRACTAL:
		{
			float value = 1, pwr = 1;
			for(int i = 0; i < oct; i++)
			{
				value *= (pwr * sn() + 1.0f);
				pwr *= pw_hl;
				scale_tp();
			}
			if(rmd != 0.0f) value *= (rmd * sn() * pwr + 1.0f);
			return value;
		}
		case GBRT_MUSGRAVE_RIDGED:
		{
			float pwr = pw_hl;
			float signal = t.offset - fabsf(sn());
			signal *= signal;
			float result = signal, weight = 1.0f;
			for(int i = 1; i < oct; i++)
			{
				scale_tp();
				weight = signal * t.gain;
				if(weight > 1.0f) weight = 1.0f;
				else if(weight < 0.0f) weight = 0.0f;
				signal = t.offset - fabsf(sn());
				signal *= signal;
				signal *= weight;
				result += signal * pwr;
				pwr *= pw_hl;
			}
			return result;
		}
		case GBRT_MUSGRAVE_HYBRID:
		{
			float pwr = pw_hl;
			float result = sn() + t.offset;
			float weight = t.gain * result;
			scale_tp();
			for(int i = 1; (weight > 0.001f) && (i < oct); i++)
			{
				if(weight > 1.0f) weight = 1.0f;
				const float signal = (sn() + t.offset) * pwr;
				pwr *= pw_hl;
				result += weight * signal;
				weight *= t.gain * signal;
				scale_tp();
			}
			if(rmd != 0.0f) result += rmd * ((sn() + t.offset) * pwr);
			return result;
		}
		case GBRT_MUSGRAVE_HETERO:
		{
			float pwr = pw_hl;
			float value = t.offset + sn();
			scale_tp();
			for(int i = 1; i < oct; i++)
			{
				const float increment = (sn() + t.offset) * pwr * value;
				value += increment;
				pwr *= pw_hl;
				scale_tp();
			}
			if(rmd != 0.0f)
			{
				const float increment = (sn() + t.offset) * pwr * value;
				value += rmd * increment;
			}
			return value;
		}
		default:   // fBm
		{
			float value = 0, pwr = 1;
			for(int i = 0; i < oct; i++)
			{
				value += sn() * pwr;
				pwr *= pw_hl;
				scale_tp();
			}
			if(rmd != 0.f) value += rmd * sn() * pwr;
			return value;
		}
	}
}

// ---- colour helpers (include/color/color.h:90-104, 452-545) -----------------
GBRT_HD void rgb_to_hsv(const float c[3], float &h, float &s, float &v)
{
	const float r1 = fmaxf(c[0], 0.f), g1 = fmaxf(c[1], 0.f), b1 = fmaxf(c[2], 0.f);
	const float mx = fmaxf(fmaxf(r1, g1), b1), mn = fminf(fminf(r1, g1), b1);
	const float range = mx - mn;
	v = mx;
	if(fabsf(range) < 1.0e-6f) { h = 0.f; s = 0.f; }
	else if(mx == r1) { h = fmodf((g1 - b1) / range, 6.f); s = range / fmaxf(v, 1.0e-6f); }
	else if(mx == g1) { h = ((b1 - r1) / range) + 2.f; s = range / fmaxf(v, 1.0e-6f); }
	else if(mx == b1) { h = ((r1 - g1) / range) + 4.f; s = range / fmaxf(v, 1.0e-6f); }
	else { h = 0.f; s = 0.f; v = 0.f; }
	if(h < 0.f) h += 6.f;
}

GBRT_HD void rgb_to_hsl(const float c[3], float &h, float &s, float &l)
{
	const float r1 = fmaxf(c[0], 0.f), g1 = fmaxf(c[1], 0.f), b1 = fmaxf(c[2], 0.f);
	const float mx = fmaxf(fmaxf(r1, g1), b1), mn = fminf(fminf(r1, g1), b1);
	const float range = mx - mn;
	l = 0.5f * (mx + mn);
	const float den = fmaxf((1.f - fabsf((2.f * l) - 1)), 1.0e-6f);
	if(fabsf(range) < 1.0e-6f) { h = 0.f; s = 0.f; }
	else if(mx == r1) { h = fmodf((g1 - b1) / range, 6.f); s = range / den; }
	else if(mx == g1) { h = ((b1 - r1) / range) + 2.f; s = range / den; }
	else if(mx == b1) { h = ((r1 - g1) / range) + 4.f; s = range / den; }
	else { h = 0.f; s = 0.f; l = 0.f; }
	if(h < 0.f) h += 6.f;
}

GBRT_HD void hsv_to_rgb(float h, float s, float v, float out[3])
{
	const float c = v * s;
	const float x = c * (1.f - fabsf(fmodf(h, 2.f) - 1.f));
	const float m = v - c;
	float r1 = 0.f, g1 = 0.f, b1 = 0.f;
	if(h >= 0.f && h < 1.f) { r1 = c; g1 = x; }
	else if(h >= 1.f && h < 2.f) { r1 = x; g1 = c; }
	else if(h >= 2.f && h < 3.f) { g1 = c; b1 = x; }
	else if(h >= 3.f && h < 4.f) { g1 = x; b1 = c; }
	else if(h >= 4.f && h < 5.f) { r1 = x; b1 = c; }
	else if(h >= 5.f && h < 6.f) { r1 = c; b1 = x; }
	out[0] = r1 + m; out[1] = g1 + m; out[2] = b1 + m;
}

GBRT_HD void clamp_rgb0(float c[3]) { for(int k = 0; k < 3; ++k) if(c[k] < 0.f) c[k] = 0.f; }

// Texture::applyIntensityContrastAdjustments (texture.cc:238-256, 272-287)
GBRT_HD float adjust_float(const ProcTex &t, float v)
{
	if(!t.adj) return v;
	float r = v;
	if(t.intensity_adj != 1.f || t.contrast != 1.f) r = (v - 0.5f) * t.contrast + t.intensity_adj - 0.5f;
	if(t.adj_clamp) { if(r < 0.f) r = 0.f; else if(r > 1.f) r = 1.f; }
	return r;
}

GBRT_HD void adjust_ic(const ProcTex &t, float c[4])
{
	if(!t.adj) return;
	if(t.intensity_adj != 1.f || t.contrast != 1.f)
		for(int k = 0; k < 3; ++k) c[k] = (c[k] - 0.5f) * t.contrast + t.intensity_adj - 0.5f;
	if(t.adj_clamp) clamp_rgb0(c);
}

// Texture::applyColorAdjustments (texture.cc:258-270)
GBRT_HD void adjust_color(const ProcTex &t, float c[4])
{
	if(!t.adj) return;
	for(int k = 0; k < 3; ++k) if(t.mult[k] != 1.f) c[k] *= t.mult[k];
	if(t.adj_clamp) clamp_rgb0(c);
	if(t.saturation != 1.f || t.hue6 != 0.f)
	{
		float h = 0.f, s = 0.f, v = 0.f;
		rgb_to_hsv(c, h, s, v);
		s *= t.saturation;
		h += t.hue6;
		if(h < 0.f) h += 6.f;
		else if(h > 6.f) h -= 6.f;
		hsv_to_rgb(h, s, v, c);
		if(t.adj_clamp) clamp_rgb0(c);
	}
}

// ColorRamp::getColorInterpolated (color_ramp.cc:32-119).  The reference
// reads the item before the first when pos equals the first position; here
// that item is the first itself.
GBRT_HD void ramp_color(const ProcTex &t, float pos, float out[4])
{
	const int n = t.ramp_n;
	auto set = [&](int i) { for(int k = 0; k < 4; ++k) out[k] = t.ramp[i][k]; };
	if(pos < t.ramp[0][4]) { set(0); return; }
	if(pos > t.ramp[n - 1][4]) { set(n - 1); return; }
	int cur = 0;
	while(cur < n && t.ramp[cur][4] < pos) ++cur;       // std::lower_bound
	const int prv = cur > 0 ? cur - 1 : 0;
	const float *ic = t.ramp[cur], *ip = t.ramp[prv];
	const float p1 = ic[4], p2 = ip[4];
	if(t.ramp_mode == GBRT_RAMP_HSV || t.ramp_mode == GBRT_RAMP_HSL)
	{
		float h1, s1, v1, h2, s2, v2;
		if(t.ramp_mode == GBRT_RAMP_HSV) { rgb_to_hsv(ic, h1, s1, v1); rgb_to_hsv(ip, h2, s2, v2); }
		else { rgb_to_hsl(ic, h1, s1, v1); rgb_to_hsl(ip, h2, s2, v2); }
		const float s = lerp_segment(pos, s1, p1, s2, p2);
		const float v = lerp_segment(pos, v1, p1, v2, p2);
		const float a = lerp_segment(pos, ic[3], p1, ip[3], p2);
		const uint32_t hi = t.ramp_hue;
		if(hi == GBRT_HUE_CLOCKWISE && h1 < h2) h1 += 6.f;
		else if(hi == GBRT_HUE_COUNTERCLOCKWISE && h1 > h2) h2 += 6.f;
		else if(hi == GBRT_HUE_NEAR && h1 < h2 && (h2 - h1) > 3.f) h1 += 6.f;
		else if(hi == GBRT_HUE_NEAR && h1 > h2 && (h2 - h1) < -3.f) h2 += 6.f;
		else if(hi == GBRT_HUE_FAR && h1 < h2 && (h2 - h1) < 3.f) h1 += 6.f;
		else if(hi == GBRT_HUE_FAR && h1 > h2 && (h2 - h1) > -3.f) h2 += 6.f;
		float h = lerp_segment(pos, h1, p1, h2, p2);
		if(h < 0.f) h += 6.f;
		else if(h > 6.f) h -= 6.f;
		// the HSL mode converts back as HSV too (color_ramp.cc:107)
		hsv_to_rgb(h, s, v, out);
		out[3] = a;
		return;
	}
	if(t.ramp_interp == GBRT_RAMP_CONSTANT) { set(cur); return; }
	for(int k = 0; k < 4; ++k) out[k] = lerp_segment(pos, ic[k], p1, ip[k], p2);
}

// ---- the textures -----------------------------------------------------------

// getFloat of each procedural texture at a texture-space point.
GBRT_HD float proc_float(const NoiseTables &T, const ProcTex &t, const float p[3])
{
	switch(t.kind)
	{
		case GBRT_TEX_BLEND:
		{
			// BlendTexture::getFloat (texture_blend.cc:63-108)
			const float c1 = t.flip_axis ? p[1] : p[0], c2 = t.flip_axis ? p[0] : p[1];
			float blend;
			switch(t.blend_type)
			{
				case GBRT_PROGRESSION_QUADRATIC:
					blend = 0.5f * (c1 + 1.f);
					if(blend < 0.f) blend = 0.f;
					else blend *= blend;
					break;
				case GBRT_PROGRESSION_EASING:
					blend = 0.5f * (c1 + 1.f);
					if(blend <= 0.f) blend = 0.f;
					else if(blend >= 1.f) blend = 1.f;
					else blend = (3.f * blend * blend - 2.f * blend * blend * blend);
					break;
				case GBRT_PROGRESSION_DIAGONAL: blend = 0.25f * (2.f + c1 + c2); break;
				case GBRT_PROGRESSION_SPHERE:
				case GBRT_PROGRESSION_QUAD_SPHERE:
					blend = 1.f - sqrtf(c1 * c1 + c2 * c2 + p[2] * p[2]);
					if(blend < 0.f) blend = 0.f;
					if(t.blend_type == GBRT_PROGRESSION_QUAD_SPHERE) blend *= blend;
					break;
				case GBRT_PROGRESSION_RADIAL: blend = (atan2f(c2, c1) / (2.f * 3.14159265358979323846f) + 0.5f); break;
				default: blend = 0.5f * (c1 + 1.f); break;
			}
			blend = fmaxf(0.f, fminf(blend, 1.f));
			return adjust_float(t, blend);
		}
		case GBRT_TEX_CLOUDS:
		{
			// CloudsTexture::getFloat (texture_clouds.cc:76-85)
			float v = turbulence(T, t.noise1, p, t.depth, t.size, t.hard != 0);
			if(t.bias != GBRT_BIAS_NONE)
			{
				v *= v;
				if(t.bias == GBRT_BIAS_POSITIVE) return -v;
			}
			return adjust_float(t, v);
		}
		case GBRT_TEX_MARBLE:
		case GBRT_TEX_WOOD:
		{
			// MarbleTexture / WoodTexture::getFloat (texture_marble.cc:80-98,
			// texture_wood.cc:79-100)
			float w;
			if(t.kind == GBRT_TEX_MARBLE) w = (p[0] + p[1] + p[2]) * 5.f;
			else if(t.wood_type == GBRT_WOOD_RINGS) w = sqrtf(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) * 20.f;
			else w = (p[0] + p[1] + p[2]) * 10.f;
			w += (t.turbulence == 0.f) ? 0.f : t.turbulence * turbulence(T, t.noise1, p, t.depth, t.size, t.hard != 0);
			const float k = 0.5f * 0.318309886183790671537767526745f;
			switch(t.shape)
			{
				case GBRT_SHAPE_SAW: w *= k; w -= floorf(w); break;
				case GBRT_SHAPE_TRI: w *= k; w = fabsf(2.f * (w - floorf(w)) - 1.f); break;
				default: w = 0.5f + 0.5f * fast_sin(w); break;
			}
			return adjust_float(t, t.kind == GBRT_TEX_MARBLE ? fpow(w, t.sharpness) : w);
		}
		case GBRT_TEX_VORONOI:
		{
			// VoronoiTexture::getFloat (texture_voronoi.cc:90-94)
			const float q[3] = {p[0] * t.size, p[1] * t.size, p[2] * t.size};
			float da[4], pa[4][3];
			voronoi_features(T, t.metric, t.mk_exp, q, da, pa);
			return adjust_float(t, t.iscale * fabsf(t.w[0] * da[0] + t.w[1] * da[1] + t.w[2] * da[2] + t.w[3] * da[3]));
		}
		case GBRT_TEX_MUSGRAVE:
		{
			// MusgraveTexture::getFloat (texture_musgrave.cc:91-94)
			const float q[3] = {p[0] * t.size, p[1] * t.size, p[2] * t.size};
			return adjust_float(t, t.intensity * musgrave(T, t, q));
		}
		case GBRT_TEX_DISTORTED_NOISE:
		{
			// DistortedNoiseTexture::getFloat (texture_distorted_noise.cc:70-78)
			const float tp[3] = {p[0] * t.size, p[1] * t.size, p[2] * t.size};
			const float rv[3] = {signed_noise(T, t.noise1, tp[0] + 13.5f, tp[1] + 13.5f, tp[2] + 13.5f),
			                     signed_noise(T, t.noise1, tp[0], tp[1], tp[2]),
			                     signed_noise(T, t.noise1, tp[0] - 13.5f, tp[1] - 13.5f, tp[2] - 13.5f)};
			return adjust_float(t, signed_noise(T, t.noise2, tp[0] + rv[0] * t.distort, tp[1] + rv[1] * t.distort, tp[2] + rv[2] * t.distort));
		}
		case GBRT_TEX_RGB_CUBE:
		{
			// RgbCubeTexture::getFloat (texture_rgb_cube.cc:67-72)
			float c[3] = {p[0], p[1], p[2]};
			for(int k = 0; k < 3; ++k) c[k] = c[k] < 0.f ? 0.f : (c[k] > 1.f ? 1.f : c[k]);
			return adjust_float(t, (c[0] + c[1] + c[2]) * 0.333333f);
		}
		default: return 0.f;
	}
}

// getColor of each procedural texture (RGBA).
GBRT_HD void proc_color(const NoiseTables &T, const ProcTex &t, const float p[3], float out[4])
{
	if(t.kind == GBRT_TEX_RGB_CUBE)
	{
		// RgbCubeTexture::getColor (texture_rgb_cube.cc:59-65)
		out[0] = p[0]; out[1] = p[1]; out[2] = p[2]; out[3] = 1.f;
		for(int k = 0; k < 3; ++k) out[k] = out[k] < 0.f ? 0.f : (out[k] > 1.f ? 1.f : out[k]);
		if(t.adj) { adjust_ic(t, out); adjust_color(t, out); }
		return;
	}
	if(t.kind == GBRT_TEX_VORONOI)
	{
		// VoronoiTexture::getColor (texture_voronoi.cc:96-120)
		const float q[3] = {p[0] * t.size, p[1] * t.size, p[2] * t.size};
		float da[4], pa[4][3];
		voronoi_features(T, t.metric, t.mk_exp, q, da, pa);
		const float inte = t.iscale * fabsf(t.w[0] * da[0] + t.w[1] * da[1] + t.w[2] * da[2] + t.w[3] * da[3]);
		if(t.ramp_n > 0) { ramp_color(t, inte, out); adjust_color(t, out); return; }
		if(t.color_mode != GBRT_VORONOI_INTENSITY)
		{
			out[0] = out[1] = out[2] = out[3] = 0.f;
			for(int f = 0; f < 4; ++f)
			{
				// NoiseGenerator::cellNoiseColor (noise_generator.cc:56-64), alpha 1
				float cl[3];
				hash_pnt(T, static_cast<int>(floorf(pa[f][0])), static_cast<int>(floorf(pa[f][1])), static_cast<int>(floorf(pa[f][2])), cl);
				out[0] += t.aw[f] * cl[0]; out[1] += t.aw[f] * cl[1]; out[2] += t.aw[f] * cl[2]; out[3] += t.aw[f] * 1.f;
			}
			float m;
			if(t.color_mode == GBRT_VORONOI_POSITION_OUTLINE || t.color_mode == GBRT_VORONOI_POSITION_OUTLINE_INTENSITY)
			{
				float t1 = (da[1] - da[0]) * 10.f;
				if(t1 > 1) t1 = 1;
				if(t.color_mode == GBRT_VORONOI_POSITION_OUTLINE_INTENSITY) t1 *= inte;
				else t1 *= t.iscale;
				m = t1;
			}
			else m = t.iscale;
			for(int k = 0; k < 4; ++k) out[k] *= m;
			if(t.adj) { adjust_ic(t, out); adjust_color(t, out); }
			return;
		}
		out[0] = out[1] = out[2] = out[3] = inte;
		adjust_color(t, out);
		return;
	}
	const float f = proc_float(T, t, p);
	if(t.ramp_n > 0) { ramp_color(t, f, out); adjust_color(t, out); return; }
	if(t.kind == GBRT_TEX_BLEND)
	{
		out[0] = out[1] = out[2] = out[3] = f;            // Rgba(float): grey with alpha f
		adjust_color(t, out);
		return;
	}
	// Rgba{color1} + f Rgba{color2 - color1}: alpha 1 + f
	for(int k = 0; k < 3; ++k) out[k] = t.c1[k] + f * (t.c2[k] - t.c1[k]);
	out[3] = 1.f + f * 1.f;
	adjust_color(t, out);
}

// gbrt_texture_desc (procedural kind) -> ProcTex, with the reference's
// derived members: marble's sharpness, voronoi's |weights| and intensity
// scale, Texture's adjustments_set_ and hue / 60, the ramp sorted by
// position (ColorRamp::addItem).  Returns false for an out-of-range ramp.
inline bool proc_from_desc(const gbrt_texture_desc &d, ProcTex &t)
{
	const gbrt_procedural_desc &p = d.proc;
	t = ProcTex{};
	t.kind = d.kind;
	t.noise1 = p.noise_type; t.noise2 = p.noise_type2;
	for(int k = 0; k < 3; ++k) { t.c1[k] = p.color1[k]; t.c2[k] = p.color2[k]; }
	t.size = p.size; t.depth = p.depth; t.hard = p.hard;
	t.bias = p.bias; t.shape = p.shape; t.wood_type = p.wood_type; t.blend_type = p.blend_type; t.flip_axis = p.use_flip_axis;
	t.sharpness = p.sharpness > 1.f ? 1.f / p.sharpness : 1.f;
	t.turbulence = p.turbulence;
	t.metric = p.distance_metric; t.color_mode = p.color_mode;
	float sum = 0.f;
	for(int k = 0; k < 4; ++k) { t.w[k] = p.weight[k]; t.aw[k] = fabsf(p.weight[k]); }
	sum = t.aw[0] + t.aw[1] + t.aw[2] + t.aw[3];
	t.mk_exp = p.mk_exponent; t.intensity = p.intensity;
	t.iscale = sum != 0.f ? p.intensity / sum : sum;
	t.musgrave_type = p.musgrave_type;
	t.h = p.h; t.lacunarity = p.lacunarity; t.octaves = p.octaves; t.offset = p.offset; t.gain = p.gain;
	t.distort = p.distort;
	t.intensity_adj = d.adj_intensity; t.contrast = d.adj_contrast; t.saturation = d.adj_saturation;
	t.hue6 = d.adj_hue / 60.f;
	for(int k = 0; k < 3; ++k) t.mult[k] = d.adj_mult_factor[k];
	t.adj_clamp = d.adj_clamp;
	t.adj = d.adj_mult_factor[0] != 1.f || d.adj_mult_factor[1] != 1.f || d.adj_mult_factor[2] != 1.f || d.adj_intensity != 1.f ||
	        d.adj_contrast != 1.f || d.adj_saturation != 1.f || d.adj_hue != 0.f || d.adj_clamp != 0;
	if(p.ramp_n < 0 || p.ramp_n > GBRT_RAMP_MAX) return false;
	t.ramp_n = p.ramp_n;
	t.ramp_mode = p.ramp_mode; t.ramp_interp = p.ramp_interpolation; t.ramp_hue = p.ramp_hue_interpolation;
	for(int i = 0; i < p.ramp_n; ++i)
		for(int k = 0; k < 5; ++k) t.ramp[i][k] = p.ramp[i][k];
	// insertion sort by position, stable like repeated sorted insertion
	for(int i = 1; i < t.ramp_n; ++i)
		for(int j = i; j > 0 && t.ramp[j][4] < t.ramp[j - 1][4]; --j)
			for(int k = 0; k < 5; ++k) { const float x = t.ramp[j][k]; t.ramp[j][k] = t.ramp[j - 1][k]; t.ramp[j - 1][k] = x; }
	return true;
}

} // namespace gbrt
