// Wavefront path tracer: the `pathtracing` integrator's per-sample work
// (PathIntegrator::integrate, src/integrator/surface/integrator_path_tracer.cc:138-314,
// with MonteCarloIntegrator's light estimation, integrator_montecarlo.cc:92-440)
// as a sequence of kernels over queues:
//
//   k_camera  camera rays (TiledIntegrator::renderTile sample positions,
//             integrator_tiled.cc:296-325; PerspectiveCamera::shootRay,
//             camera_perspective.cc:165-180)
//   k_extend  closest hit of every queued ray (traverse_core.cuh)
//   k_shade   one path vertex: emission, light estimation (shadow rays are
//             appended to the shadow queue with their would-be contribution),
//             Russian roulette and BSDF sampling of the continuation ray
//             (appended to the next ray queue, warp-ballot compacted)
//   k_shadow  any hit of every shadow ray; unoccluded ones add their
//             contribution to the film (ImageFilm::addSample with a box
//             filter of width 1, imagefilm.cc:771-822)
//
// The vertex logic, sample dimensions and weights follow the reference
// line by line (cited at each step); quirks are kept, e.g. the first-bounce
// vertex adds emission unconditionally, later vertices use the first-bounce
// material's flags (integrator_path_tracer.cc:214-283), light sampling uses
// an area of 1 (light_area.h:79) and the 0.99 pdf + 0.01 weight
// (material_shiny_diffuse.cc:432).
#include "traverse_core.cuh"
#include "sampling.cuh"
#include "procedural.cuh"
#include "guide_device.cuh"
#include "photon_map.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <string>
#include <thread>
#include <type_traits>
#include <functional>
#include <mutex>
#include <vector>

namespace {

using gbrt::xa;
using gbrt::xm;
using gbrt::xs;

// BsdfFlags subset (include/material/material.h), own bit assignment.
enum : uint32_t {
	BF_SPECULAR = 1u, BF_GLOSSY = 2u, BF_DIFFUSE = 4u, BF_DISPERSIVE = 8u, BF_REFLECT = 16u,
	BF_TRANSMIT = 32u, BF_FILTER = 64u, BF_EMIT = 128u, BF_ALL = 255u
};

struct DevMaterial {
	uint32_t type;
	uint32_t flags;
	float col[3];      // shinydiffuse: diffuse colour; light_mat: colour x power; glossy: glossy colour;
	                   // glass, rough_glass: filter colour
	float col2[3];     // shinydiffuse, glass, rough_glass: mirror colour; glossy: diffuse colour
	float exponent, m_glossy, m_diffuse, p_diffuse;
	uint32_t as_diffuse, with_diffuse, double_sided, addl_depth;
	float ior, a2;     // glass, rough_glass: IOR; shinydiffuse: IOR^2; rough_glass: GGX alpha^2
	uint32_t sd;       // shinydiffuse components present (SD_*)
	uint32_t transparent;   // Material::isTransparent: shinydiffuse with a transparency layer, glass / rough_glass with fake_shadows
	float sdc[4];      // shinydiffuse component strengths: mirror, transparency, translucency, diffuse
	float tcol[3];     // shinydiffuse: transmit_filter x colour + (1 - transmit_filter)
	float ecol[3];     // shinydiffuse: emit x colour
	int32_t dtex;      // shinydiffuse: texture driving the diffuse colour ("diffuse_shader"), -1 none
	float tf, emit;    // shinydiffuse: transmit_filter, emit (for a textured diffuse colour)
	// shader node trees of the colour slots (gbrt_scene_set_shader_nodes):
	// root node and the lowest node index of its tree, -1 for none
	int32_t nroot[GBRT_SLOTS], nfirst[GBRT_SLOTS];
	uint32_t nmask[GBRT_SLOTS];   // the nodes of the tree (bit i: node nfirst + i)
	uint32_t has_nodes;
};

// ShinyDiffuseMaterial components (material_shiny_diffuse.cc:146-189)
enum : uint32_t { SD_MIRROR = 1u, SD_TRANSPARENT = 2u, SD_TRANSLUCENT = 4u, SD_DIFFUSE = 8u, SD_FRESNEL = 16u };

// An image texture and its texture-mapper node (gbrt_texture_desc).
struct DevTexture {
	uint32_t off;               // first texel in the scene's texel array
	int w, h;
	uint32_t interp, clip, texco, mapping;
	int xrep, yrep, rot90, crop_x, crop_y;
	int adj, adj_ic, adj_clamp; // adjustments_set_, intensity / contrast set, adj_clamp
	float crop[4];
	float intensity, contrast, mult[3];
	float scale[3], offset2[3]; // offset2 = 2 x offset (shader_node_texture.h:108)
	int proj[3];
	int layer, blend, negative, no_rgb, stencil;   // LayerNode over the mapper
	int mirror_x, mirror_y;
	float colfac, upper[4], def_col[3];
	int even_tiles, odd_tiles;  // clipping checker
	float checker_dist;
	float saturation, hue6;     // adj_saturation, adj_hue / 60 (HSV adjustment when either is set)
	uint32_t kind;              // GBRT_TEX_*: image, or a procedural texture in proc
	gbrt::ProcTex proc;
};

struct DevLight {
	float c[3], tx[3], ty[3], nflip[3], col[3];   // area light (light_area.h:70-78); point light: c = from, col
	float e1[3], e2[3], e3[3];                    // quad edges from the corner, for intersect
	int samples;
	uint32_t type;                                // GBRT_LIGHT_AREA / GBRT_LIGHT_POINT
	float pad;
};

constexpr int kThreads = 128;
constexpr uint32_t kDead = 0xFFFFFFFFu;
constexpr uint32_t kMaxBatch = 1u << 18;   // largest guide training batch
constexpr float kRayMinDist = 0.00005f;   // Accelerator::min_raydist_ (accelerator.h:85)
constexpr float kShadowBias = 0.0005f;    // Accelerator::shadow_bias_ (accelerator.h:86)
constexpr uint32_t kSppmMaxGather = 1000u; // SppmIntegrator::n_max_gather_ (integrator_sppm.h:118)
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;

struct Camera {
	float from[3], vright[3], vup[3], vto[3];
	int resx, resy;
};

struct Params {
	int spp, path_samples, bounces, rr_min;
	int raydepth;         // MonteCarloIntegrator raydepth: last ray level of the recursive glossy / specular split
	uint32_t base_offset, seed;
	uint32_t wave_start, wave_n;
	float d1;
	uint32_t n_lights;
	int fp64;
	int guiding;          // sample continuation directions with the guide (one-sample MIS)
	float alpha;          // probability of the guide technique
	int record;           // write training records
	uint32_t rec_stride;  // record slots per path (= bounces)
	int radiance_target;  // train on incident radiance instead of the product with the BSDF
	// photonmapping integrator (PhotonIntegrator::integrate / finalGathering)
	int pm;                    // 1: photonmapping, 2: directlighting (DirectLightIntegrator::integrate)
	int pm_fg;                 // final gathering (path_samples then holds fg_samples)
	int pm_fg_bounces;
	float pm_gather_dist;      // fg_min_pathlen
	int pm_diffuse;            // non-FG diffuse estimate from the diffuse map
	int pm_caustics;
	float pm_diffuse_r2;       // diffuse_radius, used as the squared radius (integrator_photon_mapping.cc:772)
	int pm_diffuse_k;
	float pm_caustic_r2;       // caustic_radius^2
	int pm_caustic_k;
	float pm_diffuse_paths, pm_caustic_paths;
	float pm_lookup_r2;        // 4 diffuse_radius^2 (integrator_photon_mapping.h:90)
	gbrt::PhotonGrid g_diffuse, g_caustic, g_radiance;
	// film filter (ImageFilm::addSample): film_w = per-pixel weight sums, or
	// NULL for the single-pixel splat whose weights are the sample counts
	float *film_w;
	const float *filter_tab;   // 16 x 16 filter table
	float filter_width;        // filter_width_ (pixels)
	float filter_scale;        // filter_table_scale_
	int film_resx, film_resy;
	// adaptive anti-aliasing (TiledIntegrator::render / renderTile)
	float lmult;               // aa_light_sample_multiplier
	int aa_multipass;          // AA_passes > 1: sample positions (riVdC, riS)
	const uint32_t *pix_list;  // pixels of this pass (resampled ones), or NULL for all
	uint32_t n_list;
	// transparent shadows (MonteCarloIntegrator "transpShad", "shadowDepth")
	int tshadow, shadow_depth;
	// SPPM (pm == 3): per-pixel squared gather radius and this pass's
	// photon flux (xyz) and photon count (w)
	float *sppm_r2;
	float4 *sppm_pass;
	uint8_t *sppm_ire;         // pmIRE: per-pixel "radius set" flags, or null (no estimate this pass)
	float sppm_ire_r2;         // photonRadius^2
	int sppm_ire_k;            // searchNum
	// pathtracing (PathIntegrator): caustic_type has "path" (emission after
	// specular / glossy / filter samples counts at later vertices), and
	// no_recursive (the path loop starts at every first hit, all components)
	int pt_caustic_path;
	int no_recursive;
	float clamp_indirect;      // AA_clamp_indirect (0: off)
};

struct Work {
	uint32_t *p_pixel, *p_si, *p_state;
	uint32_t *p_scene;          // batch renders: the path's entry of the scene table
	float4 *p_thr;
	uint4 *p_task;              // integrate() call of the path: {level | addl << 8 | division << 16, branch, deco1, deco2}
	float4 *p_pm;               // final gathering: path length, colour of the last lookup
	// spawned integrate() calls of the recursive split (5 float4 each:
	// origin+tmin, dir+tmax, weight, {pixel, si, task.x, branch}, {deco1, deco2})
	float4 *sp_out;
	uint32_t *sp_count;
	uint32_t sp_cap;
	float4 *q_ray[2];
	uint32_t *q_path[2];
	float4 *hits;
	float4 *s_ray;
	float4 *s_col;
	uint32_t *s_pix;
	uint32_t *s_path;
	uint32_t *count;            // [0],[1] ray queues, [2] shadow queue, [3] training records
	unsigned long long *stats;  // [0] extension rays, [1] shadow rays traced
	// path guiding (allocated only when a guide is attached)
	float *hitpos;              // [queue][3] hit points for the network
	float *lobes;               // [queue][40] mixture parameters
	float4 *p_sum;              // [path] contributions added so far (recording)
	float4 *r_pos;              // [path * stride + vertex] position xyz, mixture pdf
	float4 *r_dir;              // direction xyz
	float4 *r_thr;              // throughput after sampling
	float4 *r_pre;              // contributions before the next vertex
	uint32_t *r_valid;
	float *train;               // [n][8] training records
	uint32_t train_cap;
};

struct SceneDev {
	gbrt::BvhView bv;
	const float4 *prim_ng;      // geometric normal xyz, material index in w (bits)
	const DevMaterial *mats;
	const DevLight *lights;
	gbrt::LdsTables lds;
	// textures (gbrt_scene_set_textures); null without
	const DevTexture *tex;
	const float4 *texels;
	const float2 *uv;
	const uint4 *face_uv;       // uv indices per face; x = kNoIdx: no uvs; w = kNoIdx: triangle
	// shading normals (gbrt_scene_set_normals); null without
	const float4 *vnrm;         // vertex normals
	const uint4 *face_nrm;      // normal indices per face; x = kFlatFace: geometric normal; w = kTriFace: triangle
	gbrt::NoiseTables nt;       // the host's noise tables (gbrt_scene_set_noise_tables); null without
	const gbrt_shader_node *nodes;   // shader node trees (gbrt_scene_set_shader_nodes); null without
	const uint32_t *prim_slot;  // primitive -> its record in the BVH's leaf order (bump mapping); null without
};

__device__ __forceinline__ float dot3(const float a[3], const float b[3]) { return xa(xa(xm(a[0], b[0]), xm(a[1], b[1])), xm(a[2], b[2])); }

__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
	x ^= x >> 16; x *= 0x7feb352du;
	x ^= x >> 15; x *= 0x846ca68bu;
	x ^= x >> 16;
	return x;
}
__device__ __forceinline__ float rng01(uint32_t a, uint32_t b, uint32_t c, uint32_t seed)
{
	const uint32_t h = hash32(a ^ hash32(b ^ hash32(c ^ hash32(seed))));
	return static_cast<float>(h >> 8) * (1.f / 16777216.f);
}

// Vec3::createCoordsSystem (include/geometry/vector.h:399-420)
__device__ __forceinline__ void coords_system(const float n[3], float u[3], float v[3])
{
	if(n[0] == 0.f && n[1] == 0.f)
	{
		u[0] = n[2] < 0.f ? -1.f : 1.f; u[1] = 0.f; u[2] = 0.f;
		v[0] = 0.f; v[1] = 1.f; v[2] = 0.f;
		return;
	}
	const float d = __fdiv_rn(1.f, sqrtf(xa(xm(n[1], n[1]), xm(n[0], n[0]))));
	u[0] = xm(n[1], d); u[1] = xm(-n[0], d); u[2] = 0.f;
	v[0] = xs(xm(n[1], u[2]), xm(n[2], u[1]));
	v[1] = xs(xm(n[2], u[0]), xm(n[0], u[2]));
	v[2] = xs(xm(n[0], u[1]), xm(n[1], u[0]));
}

// sample::cosHemisphere (include/sampler/sample.h:43-52) with FAST_TRIG.
// kExact: the accurate sine and cosine, so the directions follow the cosine
// density exactly (guided vertices: the one-sample MIS weights need the true
// density of the BSDF technique; the FAST_TRIG parabola bends the azimuth by
// up to about 1 %).
template <bool kExact = false>
__device__ __forceinline__ void cos_hemisphere(const float n[3], const float u[3], const float v[3], float s1, float s2, float out[3])
{
	if(s1 >= 1.f) { out[0] = n[0]; out[1] = n[1]; out[2] = n[2]; return; }
	const float z2 = xm(s2, 6.28318530717958647692f);
	float cz, sz;
	if constexpr(kExact) sincosf(z2, &sz, &cz);
	else { cz = gbrt::fast_cos(z2); sz = gbrt::fast_sin(z2); }
	const float a = sqrtf(xs(1.f, s1)), b = sqrtf(s1);
	for(int k = 0; k < 3; ++k) out[k] = xa(xm(xa(xm(u[k], cz), xm(v[k], sz)), a), xm(n[k], b));
}

struct Surface {
	float p[3], ng[3], n[3], u[3], v[3];
	float dcol[3];              // the diffuse colour here (the material's, or its texture's)
	const DevMaterial *m;
};

// SurfacePoint::normalFaceForward (include/geometry/surface.h:202-205)
__device__ __forceinline__ void face_forward(const Surface &s, const float wo[3], float out[3])
{
	const bool flip = dot3(s.ng, wo) < 0.f;
	for(int k = 0; k < 3; ++k) out[k] = flip ? -s.n[k] : s.n[k];
}

__device__ __forceinline__ void normalize3(float v[3])
{
	const float l2 = dot3(v, v);
	if(l2 != 0.f)
	{
		const float inv = __fdiv_rn(1.f, sqrtf(l2));
		for(int k = 0; k < 3; ++k) v[k] = xm(v[k], inv);
	}
}

// microfacet helpers (include/material/material_utils_microfacet.h:26-34, 87-104, 181-198)
__device__ __forceinline__ float blinn_d(float cos_h, float e) { return xm(xa(e, 1.f), gbrt::fast_pow(cos_h, e)); }
__device__ __forceinline__ float pdf_divisor(float c) { return xm(xm(8.f, kPi), xa(xm(c, 0.99f), 0.04f)); }
__device__ __forceinline__ float blinn_pdf(float cos_theta, float cos_w_h, float e) { return __fdiv_rn(blinn_d(cos_theta, e), pdf_divisor(cos_w_h)); }
__device__ __forceinline__ float as_divisor(float c1, float ci, float co)
{
	return xm(xm(8.f, kPi), xa(xm(xm(c1, fmaxf(ci, co)), 0.99f), 0.04f));
}
__device__ __forceinline__ float schlick(float c, float r)
{
	const float c1 = xs(1.f, c), c2 = xm(c1, c1);
	return xa(r, xm(xm(xm(xs(1.f, r), c1), c2), c2));
}
__device__ __forceinline__ float diffuse_reflect_factor(float wi_n, float wo_n, float glossy, float diffuse)
{
	float f_wi = xs(1.f, xm(0.5f, wi_n));
	float t = xm(f_wi, f_wi);
	f_wi = xm(xm(t, t), f_wi);
	float f_wo = xs(1.f, xm(0.5f, wo_n));
	t = xm(f_wo, f_wo);
	f_wo = xm(xm(t, t), f_wo);
	const double r = 0.387507688 * diffuse * static_cast<double>(xs(1.f, glossy)) * static_cast<double>(xs(1.f, f_wi)) * static_cast<double>(xs(1.f, f_wo));
	return static_cast<float>(r);
}

// GlossyMaterial::eval (material_glossy.cc:200-242)
__device__ __forceinline__ void glossy_eval(const Surface &s, const float wo[3], const float wl[3], uint32_t bsdfs, float out[3])
{
	const DevMaterial &m = *s.m;
	out[0] = out[1] = out[2] = 0.f;
	if(!(bsdfs & BF_DIFFUSE) || xm(dot3(s.ng, wl), dot3(s.ng, wo)) < 0.f) return;
	const bool diffuse_flag = (bsdfs & BF_DIFFUSE) != 0u;
	float n[3];
	face_forward(s, wo, n);
	const float wi_n = fabsf(dot3(wl, n)), wo_n = fabsf(dot3(wo, n));
	if((m.as_diffuse && diffuse_flag) || (!m.as_diffuse && (bsdfs & BF_GLOSSY)))
	{
		float h[3] = {xa(wo[0], wl[0]), xa(wo[1], wl[1]), xa(wo[2], wl[2])};
		normalize3(h);
		const float cos_wi_h = fmaxf(0.f, dot3(wl, h));
		const float glossy = __fdiv_rn(xm(blinn_d(dot3(h, n), m.exponent), schlick(cos_wi_h, m.m_glossy)), as_divisor(cos_wi_h, wo_n, wi_n));
		for(int k = 0; k < 3; ++k) out[k] = xm(glossy, m.col[k]);
	}
	if(m.with_diffuse && diffuse_flag)
		for(int k = 0; k < 3; ++k) out[k] = xa(out[k], xm(xm(m.m_diffuse, xs(1.f, m.m_glossy)), m.col2[k]));
}

// GlossyMaterial::pdf (material_glossy.cc:404-444)
__device__ __forceinline__ float glossy_pdf(const Surface &s, const float wo[3], const float wi[3], uint32_t flags)
{
	const DevMaterial &m = *s.m;
	if(xm(dot3(s.ng, wo), dot3(s.ng, wi)) < 0.f) return 0.f;
	float n[3];
	face_forward(s, wo, n);
	const float pd = m.p_diffuse;
	const bool use_glossy = m.as_diffuse ? (flags & BF_DIFFUSE) != 0u : (flags & BF_GLOSSY) != 0u;
	const bool use_diffuse = m.with_diffuse && (flags & BF_DIFFUSE);
	float h[3] = {xa(wi[0], wo[0]), xa(wi[1], wo[1]), xa(wi[2], wo[2])};
	normalize3(h);
	if(use_diffuse)
	{
		float pdf = fabsf(dot3(wi, n));
		if(use_glossy) pdf = xa(xm(pdf, pd), xm(blinn_pdf(dot3(n, h), dot3(wo, h), m.exponent), xs(1.f, pd)));
		return pdf;
	}
	if(use_glossy) return blinn_pdf(dot3(n, h), dot3(wo, h), m.exponent);
	return 0.f;
}

// GlossyMaterial::sample (material_glossy.cc:245-402), isotropic Blinn.
// kExact: the directions drawn with the accurate pow / sine / cosine (see
// cos_hemisphere); the sample weight is the same function of the direction.
template <bool kExact = false>
__device__ __forceinline__ void glossy_sample(const Surface &s, const float wo[3], float s1, float s2, uint32_t flags,
                                              float wi[3], float col[3], float &w, float &pdf, uint32_t &sampled)
{
	const DevMaterial &m = *s.m;
	const float cos_ng_wo = dot3(s.ng, wo);
	float n[3];
	face_forward(s, wo, n);
	pdf = 0.f;
	float wi_n = 0.f;
	const float wo_n = fabsf(dot3(wo, n));
	col[0] = col[1] = col[2] = 0.f;
	sampled = 0u;
	wi[0] = n[0]; wi[1] = n[1]; wi[2] = n[2];
	const float pd = m.p_diffuse;
	const bool use_glossy = m.as_diffuse ? (flags & BF_DIFFUSE) != 0u : (flags & BF_GLOSSY) != 0u;
	const bool use_diffuse = m.with_diffuse && (flags & BF_DIFFUSE);
	if(use_diffuse)
	{
		const float s_pd = use_glossy ? pd : 1.f;
		if(s1 < s_pd)
		{
			s1 = __fdiv_rn(s1, s_pd);
			cos_hemisphere<kExact>(n, s.u, s.v, s1, s2, wi);
			if(xm(dot3(s.ng, wi), cos_ng_wo) < 0.f) { w = 0.f; return; }
			wi_n = fabsf(dot3(wi, n));
			pdf = wi_n;
			float glossy = 0.f;
			if(use_glossy)
			{
				float h[3] = {xa(wi[0], wo[0]), xa(wi[1], wo[1]), xa(wi[2], wo[2])};
				normalize3(h);
				const float cos_wo_h = dot3(wo, h), cos_wi_h = fabsf(dot3(wi, h)), cos_n_h = dot3(n, h);
				pdf = xa(xm(pdf, pd), xm(blinn_pdf(cos_n_h, cos_wo_h, m.exponent), xs(1.f, pd)));
				glossy = __fdiv_rn(xm(blinn_d(cos_n_h, m.exponent), schlick(cos_wi_h, m.m_glossy)), as_divisor(cos_wi_h, wo_n, wi_n));
			}
			sampled = BF_DIFFUSE | BF_REFLECT;
			if(!(flags & BF_REFLECT)) { w = 0.f; return; }
			const float dr = diffuse_reflect_factor(wi_n, wo_n, m.m_glossy, m.m_diffuse);
			for(int k = 0; k < 3; ++k) col[k] = xa(xm(glossy, m.col[k]), xm(dr, m.col2[k]));
			w = __fdiv_rn(wi_n, xa(xm(pdf, 0.99f), 0.01f));
			return;
		}
		s1 = __fdiv_rn(xs(s1, pd), xs(1.f, pd));
	}
	if(use_glossy)
	{
		// microfacet::blinnSample (material_utils_microfacet.h:96-104)
		const float e1 = __fdiv_rn(1.f, xa(m.exponent, 1.f));
		const float cos_theta = kExact ? powf(xs(1.f, s2), e1) : gbrt::fast_pow(xs(1.f, s2), e1);
		const float sin_theta = sqrtf(xs(1.f, xm(cos_theta, cos_theta)));
		const float phi = xm(s1, 6.28318530717958647692f);
		float cphi, sphi;
		if constexpr(kExact) sincosf(phi, &sphi, &cphi);
		else { cphi = gbrt::fast_cos(phi); sphi = gbrt::fast_sin(phi); }
		const float hs[3] = {xm(sin_theta, cphi), xm(sin_theta, sphi), cos_theta};
		float h[3];
		for(int k = 0; k < 3; ++k) h[k] = xa(xa(xm(hs[0], s.u[k]), xm(hs[1], s.v[k])), xm(hs[2], n[k]));
		float cos_wo_h = dot3(wo, h);
		if(cos_wo_h < 0.f)
		{
			const float vn = xm(2.f, dot3(h, n));   // Vec::reflect (vector.h:358-362)
			for(int k = 0; k < 3; ++k) h[k] = xs(xm(vn, n[k]), h[k]);
			cos_wo_h = dot3(wo, h);
		}
		const float vn = dot3(wo, h);               // Vec::reflectDir (vector.h:391-396)
		for(int k = 0; k < 3; ++k) wi[k] = vn < 0.f ? -wo[k] : xs(xm(xm(2.f, vn), h[k]), wo[k]);
		if(xm(cos_ng_wo, dot3(s.ng, wi)) < 0.f) { w = 0.f; return; }
		wi_n = fabsf(dot3(wi, n));
		const float cos_hn = dot3(h, n);
		pdf = blinn_pdf(cos_hn, cos_wo_h, m.exponent);
		const float glossy = __fdiv_rn(xm(blinn_d(cos_hn, m.exponent), schlick(cos_wo_h, m.m_glossy)), as_divisor(cos_wo_h, wo_n, wi_n));
		for(int k = 0; k < 3; ++k) col[k] = xm(glossy, m.col[k]);
		sampled = m.as_diffuse ? (BF_DIFFUSE | BF_REFLECT) : (BF_GLOSSY | BF_REFLECT);
	}
	if(use_diffuse)
	{
		const float dr = diffuse_reflect_factor(wi_n, wo_n, m.m_glossy, m.m_diffuse);
		for(int k = 0; k < 3; ++k) col[k] = xa(col[k], xm(dr, m.col2[k]));
		pdf = xa(xm(wi_n, pd), xm(pdf, xs(1.f, pd)));
	}
	w = __fdiv_rn(wi_n, xa(xm(pdf, 0.99f), 0.01f));
}

// ---- glass and rough glass ---------------------------------------------------

// Vec3::refract (include/geometry/vector.h:484-503): directions point away
// from the surface; false on total internal reflection.
__device__ __forceinline__ bool vec_refract(const float n_in[3], const float wi[3], float wo[3], float ior)
{
	float n[3] = {n_in[0], n_in[1], n_in[2]};
	float eta, cos_v_n = dot3(wi, n);
	if(cos_v_n < 0.f) { eta = ior; n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; cos_v_n = -cos_v_n; }
	else eta = 1.f / ior;
	const float k = 1.f - eta * eta * (1.f - cos_v_n * cos_v_n);
	if(k <= 0.f) return false;
	const float a = eta * cos_v_n - sqrtf(k);
	for(int c = 0; c < 3; ++c) wo[c] = eta * -wi[c] + a * n[c];
	normalize3(wo);
	return true;
}

// Vec3::fresnel (vector.h:505-518)
__device__ __forceinline__ void vec_fresnel(const float i[3], const float n[3], float ior, float &kr, float &kt)
{
	const float d = dot3(i, n);
	const float c = d < 0.f ? -d : d;
	float g = ior * ior + c * c - 1.f;
	g = g <= 0.f ? 0.f : sqrtf(g);
	const float aux = c * (g + c);
	kr = ((0.5f * (g - c) * (g - c)) / ((g + c) * (g + c))) * (1.f + ((aux - 1.f) * (aux - 1.f)) / ((aux + 1.f) * (aux + 1.f)));
	kt = kr < 1.f ? 1.f - kr : 0.f;
}

// Vec3::reflect: 2 (v.n) n - v (vector.h:358-362)
__device__ __forceinline__ void vec_reflect(const float v[3], const float n[3], float out[3])
{
	const float vn = 2.f * dot3(v, n);
	for(int c = 0; c < 3; ++c) out[c] = vn * n[c] - v[c];
}

// Normal used by GlassMaterial::sample / getSpecular (material_glass.cc:173-177,
// 320-330): the shading normal, bent towards wo when it faces away.
__device__ __forceinline__ void glass_normal(const Surface &s, const float wo[3], float n[3], bool &outside)
{
	outside = dot3(s.ng, wo) > 0.f;
	const float c = dot3(s.n, wo);
	if(outside ? c >= 0.f : c <= 0.f) { n[0] = s.n[0]; n[1] = s.n[1]; n[2] = s.n[2]; return; }
	for(int k = 0; k < 3; ++k) n[k] = s.n[k] - (1.00001f * c) * wo[k];
	normalize3(n);
}

// GlassMaterial::sample without dispersion (material_glass.cc:164-176, 235-300).
// Note the weight: the chosen branch returns its colour with w = 1 (no
// division by the branch probability).
__device__ __forceinline__ bool glass_sample(const Surface &s, const float wo[3], float s1, uint32_t req, float wi[3], float col[3],
                                             float &w, float &pdf, uint32_t &sampled)
{
	const DevMaterial &m = *s.m;
	col[0] = col[1] = col[2] = 0.f; w = 0.f; pdf = 0.f; sampled = 0u;
	if(!(req & BF_SPECULAR)) return false;
	float n[3];
	bool outside;
	glass_normal(s, wo, n, outside);
	pdf = 1.f;
	float refdir[3];
	if(vec_refract(n, wo, refdir, m.ior))
	{
		float kr, kt;
		vec_fresnel(wo, n, m.ior, kr, kt);
		const float p_kr = 0.01f + 0.99f * kr, p_kt = 0.01f + 0.99f * kt;
		// transmit_flags_: Filter | Transmit with fake_shadows (material_glass.cc:147, 244-248)
		const uint32_t tflags = m.transparent ? (BF_FILTER | BF_TRANSMIT) : (BF_SPECULAR | BF_TRANSMIT);
		if(s1 < p_kt && (req & tflags))
		{
			for(int k = 0; k < 3; ++k) { wi[k] = refdir[k]; col[k] = m.col[k]; }
			pdf = p_kt; w = 1.f; sampled = tflags;
			return true;
		}
		if(req & (BF_SPECULAR | BF_REFLECT))
		{
			vec_reflect(wo, n, wi);
			for(int k = 0; k < 3; ++k) col[k] = m.col2[k];
			pdf = p_kr; w = 1.f; sampled = BF_SPECULAR | BF_REFLECT;
			return true;
		}
	}
	else if(req & (BF_SPECULAR | BF_REFLECT))   // total internal reflection
	{
		vec_reflect(wo, n, wi);
		col[0] = col[1] = col[2] = 1.f;
		w = 1.f; sampled = BF_SPECULAR | BF_REFLECT;
		return true;
	}
	pdf = 0.f;
	return false;
}

// GlassMaterial::getSpecular without dispersion (material_glass.cc:313-370):
// refraction (kt x filter colour) and reflection (kr x mirror colour; for
// rays leaving the glass only below ray level 3); TIR: mirror colour.
__device__ __forceinline__ void glass_specular(const Surface &s, const float wo[3], int ray_level, bool &has_refract, float rdir[3],
                                               float rcol[3], bool &has_reflect, float ldir[3], float lcol[3])
{
	const DevMaterial &m = *s.m;
	float n[3];
	bool outside;
	glass_normal(s, wo, n, outside);
	has_refract = has_reflect = false;
	if(vec_refract(n, wo, rdir, m.ior))
	{
		float kr, kt;
		vec_fresnel(wo, n, m.ior, kr, kt);
		has_refract = true;
		for(int k = 0; k < 3; ++k) rcol[k] = kt * m.col[k];
		if(outside || ray_level < 3)
		{
			has_reflect = true;
			vec_reflect(wo, n, ldir);
			for(int k = 0; k < 3; ++k) lcol[k] = m.col2[k] * kr;
		}
	}
	else
	{
		has_reflect = true;
		vec_reflect(wo, n, ldir);
		for(int k = 0; k < 3; ++k) lcol[k] = m.col2[k];
	}
}

// GGX helpers (include/material/material_utils_microfacet.h:109-179)
__device__ __forceinline__ void ggx_sample(float a2, float s1, float s2, float h[3])
{
	const float tan_theta_2 = a2 * (s1 / (1.00001f - s1));
	const float cos_theta = 1.f / sqrtf(1.f + tan_theta_2);
	const float sin_theta = sqrtf(1.00001f - cos_theta * cos_theta);
	const float phi = 6.28318530717958647692f * s2;
	h[0] = sin_theta * gbrt::fast_cos(phi); h[1] = sin_theta * gbrt::fast_sin(phi); h[2] = cos_theta;
}
__device__ __forceinline__ float ggx_d(float a2, float ct2, float tt2)
{
	const float ct4 = ct2 * ct2, a_tan = a2 + tt2;
	return a2 / (kPi * ct4 * a_tan * a_tan);
}
__device__ __forceinline__ float ggx_g(float a2, float wo_n, float wi_n)
{
	const float wo2 = wo_n * wo_n, wi2 = wi_n * wi_n;
	const float t1 = sqrtf(1.f + a2 * ((1.f - wo2) / wo2)), t2 = sqrtf(1.f + a2 * ((1.f - wi2) / wi2));
	return (2.f / (1.f + t1)) * (2.f / (1.f + t2));
}
__device__ __forceinline__ float mf_fresnel(float wo_h, float ior)
{
	const float c = fabsf(wo_h);
	float g = ior * ior - 1.f + c * c;
	if(g > 0.f)
	{
		g = sqrtf(g);
		const float a = (g - c) / (g + c), b = (c * (g + c) - 1.f) / (c * (g - c) + 1.f);
		return 0.5f * a * a * (1.f + b * b);
	}
	return 1.f;
}
__device__ __forceinline__ bool mf_refract(float eta, const float wo[3], float wi[3], const float h[3], float wo_h, float &kr, float &kt)
{
	wi[0] = wi[1] = wi[2] = 0.f;
	const float c = -dot3(wo, h);
	const float sign = c > 0.f ? 1.f : -1.f;
	const float t1 = 1.f - (eta * eta * (1.f - c * c));
	if(t1 < 0.f) return false;
	const float a = eta * c - sign * sqrtf(t1);
	for(int k = 0; k < 3; ++k) wi[k] = -(eta * wo[k] + a * h[k]);
	kt = 0.f;
	kr = mf_fresnel(wo_h, 1.f / eta);
	if(kr == 1.f) return false;
	kt = 1.f - kr;
	return true;
}

// Shared set-up of RoughGlassMaterial::sample (material_rough_glass.cc:165-190):
// GGX half vector in the shading frame, D term.
struct RoughFrame {
	float n[3], h[3];
	bool outside;
	float cos_theta, d, wo_h, wo_n;
};
__device__ __forceinline__ void rough_frame(const Surface &s, const float wo[3], float s1, float s2, RoughFrame &f)
{
	face_forward(s, wo, f.n);
	f.outside = dot3(s.ng, wo) > 0.f;
	float hs[3];
	ggx_sample(s.m->a2, s1, s2, hs);
	for(int k = 0; k < 3; ++k) f.h[k] = hs[0] * s.u[k] + hs[1] * s.v[k] + hs[2] * f.n[k];
	normalize3(f.h);
	f.cos_theta = dot3(f.h, f.n);
	const float ct2 = f.cos_theta * f.cos_theta;
	const float tt2 = (1.f - ct2) / fmaxf(1.0e-8f, ct2);
	f.d = f.cos_theta > 0.f ? ggx_d(s.m->a2, ct2, tt2) : 0.f;
	f.wo_h = dot3(wo, f.h);
	f.wo_n = dot3(wo, f.n);
}
__device__ __forceinline__ void rough_transmit(const Surface &s, const RoughFrame &f, const float wi[3], float kt, float col[3], float &w, float &pdf)
{
	const DevMaterial &m = *s.m;
	const float wi_n = dot3(wi, f.n), wi_h = dot3(wi, f.h);
	const float g = (wi_h * wi_n > 0.f && f.wo_h * f.wo_n > 0.f) ? ggx_g(m.a2, wi_n, f.wo_n) : 0.f;
	const float ior_wi = f.outside ? m.ior : 1.f, ior_wo = f.outside ? 1.f : m.ior;
	const float ht = ior_wo * f.wo_h + ior_wi * wi_h;
	const float jac = (ior_wi * ior_wi) / fmaxf(1.0e-8f, ht * ht);
	const float glossy = fabsf((f.wo_h * wi_h) / (wi_n * f.wo_n)) * kt * g * f.d * jac;
	pdf = f.d * f.cos_theta * (jac * fabsf(wi_h));
	for(int k = 0; k < 3; ++k) col[k] = glossy * m.col[k];
	w = fabsf(wi_n) / fmaxf(0.1f, pdf);
}
__device__ __forceinline__ void rough_reflect(const Surface &s, const RoughFrame &f, const float wo[3], float kr, float wi[3], float col[3],
                                              float &w, float &pdf)
{
	const DevMaterial &m = *s.m;
	const float hw = 2.f * dot3(f.h, wo);       // microfacet::reflect (material_utils_microfacet.h:175-179)
	for(int k = 0; k < 3; ++k) wi[k] = hw * f.h[k] - wo[k];
	const float wi_n = dot3(wi, f.n), wi_h = dot3(wi, f.h);
	const float g = ggx_g(m.a2, wi_n, f.wo_n);
	const float jac = 1.f / fmaxf(1.0e-8f, 4.f * fabsf(wi_h));
	const float glossy = (kr * g * f.d) / fmaxf(1.0e-8f, 4.f * fabsf(f.wo_n * wi_n));
	pdf = f.d * f.cos_theta * jac;
	for(int k = 0; k < 3; ++k) col[k] = glossy * m.col2[k];
	w = fabsf(wi_n) / fmaxf(0.1f, pdf);
}

// RoughGlassMaterial::sample, one direction (material_rough_glass.cc:165-245):
// transmission when s1 < kt, else reflection; TIR reflects with weight 1.
__device__ __forceinline__ bool rough_sample(const Surface &s, const float wo[3], float s1, float s2, uint32_t req, float wi[3], float col[3],
                                             float &w, float &pdf, uint32_t &sampled)
{
	col[0] = col[1] = col[2] = 0.f; w = 0.f; pdf = 1.f; sampled = 0u;
	RoughFrame f;
	rough_frame(s, wo, s1, s2, f);
	float kr, kt;
	if(mf_refract(f.outside ? 1.f / s.m->ior : s.m->ior, wo, wi, f.h, f.wo_h, kr, kt))
	{
		if(s1 < kt && (req & BF_TRANSMIT))
		{
			rough_transmit(s, f, wi, kt, col, w, pdf);
			sampled = BF_GLOSSY | BF_TRANSMIT;
			return true;
		}
		if(req & BF_REFLECT)
		{
			rough_reflect(s, f, wo, kr, wi, col, w, pdf);
			sampled = BF_GLOSSY | BF_REFLECT;
			return true;
		}
		return false;
	}
	const float hw = 2.f * dot3(wo, f.h);     // TIR: wo reflected about h
	for(int k = 0; k < 3; ++k) wi[k] = hw * f.h[k] - wo[k];
	col[0] = col[1] = col[2] = 1.f;
	w = 1.f;
	sampled = BF_GLOSSY | BF_REFLECT;
	return true;
}

// RoughGlassMaterial::sample, both directions (material_rough_glass.cc:247-347),
// as MonteCarloIntegrator::glossy calls it for transmissive materials with
// flags Glossy | AllGlossy: slot 0 = transmission (TIR: the reflection,
// colour 1, weight 1), slot 1 = reflection; n = slots filled.
__device__ __forceinline__ int rough_sample2(const Surface &s, const float wo[3], float s1, float s2, float dir[2][3], float col[2][3], float w[2])
{
	RoughFrame f;
	rough_frame(s, wo, s1, s2, f);
	float kr, kt, wi[3], pdf;
	if(mf_refract(f.outside ? 1.f / s.m->ior : s.m->ior, wo, wi, f.h, f.wo_h, kr, kt))
	{
		rough_transmit(s, f, wi, kt, col[0], w[0], pdf);
		for(int k = 0; k < 3; ++k) dir[0][k] = wi[k];
		rough_reflect(s, f, wo, kr, dir[1], col[1], w[1], pdf);
		return 2;
	}
	const float hw = 2.f * dot3(wo, f.h);
	for(int k = 0; k < 3; ++k) { dir[0][k] = hw * f.h[k] - wo[k]; col[0][k] = 1.f; }
	w[0] = 1.f;
	return 1;
}


// ---- image textures (TextureMapperNode -> ImageTexture) --------------------
constexpr uint32_t kNoIdx = 0xFFFFFFFFu;

// Texture coordinates of a hit (PrimitivePolygon::getSurfacePolygon,
// primitive_polygon.cc:70-101): a triangle's uvs at the barycentric weights
// (1 - u - v, u, v), a quad's by ShapePolygon::interpolate (shape_polygon.h:
// 94-100); a face without uvs takes the implicit (1 - u - v, u), a quad (u, v).
__device__ __forceinline__ void hit_uv(const SceneDev &sc, int prim, float bu, float bv, float uv[2])
{
	const uint4 f = __ldg(sc.face_uv + prim);
	const bool quad = f.w != kNoIdx;
	const float w0 = xs(xs(1.f, bu), bv);
	if(f.x == kNoIdx)
	{
		uv[0] = quad ? bu : w0;
		uv[1] = quad ? bv : bu;
		return;
	}
	const float2 a = __ldg(sc.uv + f.x), b = __ldg(sc.uv + f.y), c = __ldg(sc.uv + f.z);
	if(!quad)
	{
		uv[0] = xa(xa(xm(w0, a.x), xm(bu, b.x)), xm(bv, c.x));
		uv[1] = xa(xa(xm(w0, a.y), xm(bu, b.y)), xm(bv, c.y));
		return;
	}
	const float2 d = __ldg(sc.uv + f.w);
	const float iu = xs(1.f, bu), iv = xs(1.f, bv);
	uv[0] = xa(xm(iv, xa(xm(iu, a.x), xm(bu, b.x))), xm(bv, xa(xm(iu, d.x), xm(bu, c.x))));
	uv[1] = xa(xm(iv, xa(xm(iu, a.y), xm(bu, b.y))), xm(bv, xa(xm(iu, d.y), xm(bu, c.y))));
}

// ---- shading normals --------------------------------------------------------
constexpr uint32_t kFlatFace = 0xFFFFFFFEu;   // face_nrm.x: the face shades with its geometric normal
constexpr uint32_t kTriFace = 0xFFFFFFFDu;    // face_nrm.w: the face is a triangle

// Shading normal of a hit (PrimitivePolygon::getSurfacePolygon,
// primitive_polygon.cc:49-56): a face of a mesh with vertex normals takes
// its vertices' normals (a vertex without one contributes the geometric
// normal, FacePrimitive::getVertexNormal, primitive_face.h:106-110) at the
// barycentric weights (1 - u - v, u, v), a quad's by ShapePolygon::interpolate
// (shape_polygon.h:94-100), normalised; other faces the geometric normal.
__device__ __forceinline__ void shading_normal(const SceneDev &sc, int prim, float bu, float bv, const float ng[3], float n[3])
{
	n[0] = ng[0]; n[1] = ng[1]; n[2] = ng[2];
	if(!sc.face_nrm) return;
	const uint4 f = __ldg(sc.face_nrm + prim);
	if(f.x == kFlatFace) return;
	auto vn = [&](uint32_t i) {
		if(i == GBRT_NO_NORMAL) return make_float3(ng[0], ng[1], ng[2]);
		const float4 q = __ldg(sc.vnrm + i);
		return make_float3(q.x, q.y, q.z);
	};
	const float3 a = vn(f.x), b = vn(f.y), c = vn(f.z);
	if(f.w == kTriFace)
	{
		const float w0 = xs(xs(1.f, bu), bv);
		n[0] = xa(xa(xm(w0, a.x), xm(bu, b.x)), xm(bv, c.x));
		n[1] = xa(xa(xm(w0, a.y), xm(bu, b.y)), xm(bv, c.y));
		n[2] = xa(xa(xm(w0, a.z), xm(bu, b.z)), xm(bv, c.z));
	}
	else
	{
		const float3 d = vn(f.w);
		const float iu = xs(1.f, bu), iv = xs(1.f, bv);
		n[0] = xa(xm(iv, xa(xm(iu, a.x), xm(bu, b.x))), xm(bv, xa(xm(iu, d.x), xm(bu, c.x))));
		n[1] = xa(xm(iv, xa(xm(iu, a.y), xm(bu, b.y))), xm(bv, xa(xm(iu, d.y), xm(bu, c.y))));
		n[2] = xa(xm(iv, xa(xm(iu, a.z), xm(bu, b.z))), xm(bv, xa(xm(iu, d.z), xm(bu, c.z))));
	}
	normalize3(n);
}

// ImageTexture::findTextureInterpolationCoordinates (texture_image.cc:
// 264-341): the texel pair along one axis and the weight.
__device__ __forceinline__ void tex_axis(float cf, int res, bool repeat, bool mirror, int &c1, int &c2, float &d, int *c0 = nullptr,
                                         int *c3 = nullptr)
{
	int o0, o3;
	if(repeat && mirror)
	{
		c1 = static_cast<int>(cf) % res;
		if(cf < 0.f) { o0 = 1 % res; c2 = c1; o3 = o0; d = -cf; }
		else if(cf >= static_cast<float>(res - 1))
		{
			o0 = (2 * res - 1) % res; c2 = c1; o3 = o0;
			d = xs(cf, static_cast<float>(static_cast<int>(cf)));
		}
		else
		{
			o0 = (res + c1 - 1) % res;
			c2 = c1 + 1;
			if(c2 >= res) c2 = (2 * res - c2) % res;
			o3 = c1 + 2;
			if(o3 >= res) o3 = (2 * res - o3) % res;
			d = xs(cf, static_cast<float>(static_cast<int>(cf)));
		}
	}
	else if(repeat)
	{
		c1 = static_cast<int>(cf) % res;
		if(cf > 0.f)
		{
			o0 = (res + c1 - 1) % res; c2 = (c1 + 1) % res; o3 = (c1 + 2) % res;
			d = xs(cf, static_cast<float>(static_cast<int>(cf)));
		}
		else { o0 = 1 % res; c2 = (res - 1) % res; o3 = (res - 2) % res; d = -cf; }
	}
	else
	{
		c1 = max(0, min(res - 1, static_cast<int>(cf)));
		c2 = cf > 0.f ? min(res - 1, c1 + 1) : 0;
		o0 = max(0, c1 - 1);
		o3 = min(res - 1, c2 + 1);
		d = xs(cf, floorf(cf));
	}
	if(c0) *c0 = o0;
	if(c3) *c3 = o3;
}

// math::cubicInterpolate (include/math/interpolation.h:70-80) on one channel,
// the reference's operation order.
__device__ __forceinline__ float cubic_interp(float y0, float y1, float y2, float y3, float x)
{
	const float x2 = xm(x, x), x3 = xm(x, x2);
	const float a0 = xa(xs(xs(y3, y2), y0), y1);
	const float a1 = xs(xs(y0, y1), a0);
	const float a2 = xs(y2, y0);
	return xa(xa(xa(xm(a0, x3), xm(a1, x2)), xm(a2, x)), y1);
}

// LayerNode::eval, colour part (shader_node_layer.cc:110-171) with the
// mapper's colour as input and no upper layer, and textureRgbBlend
// (:264-316): rgb = the mapper's colour in, the layer's colour out.
__device__ void tex_layer(const DevTexture &T, float ta, float rgb[3])
{
	if(!T.layer) return;
	float tex[3] = {rgb[0], rgb[1], rgb[2]};
	float stencil_tin = T.upper[3];
	float tin = 0.f;
	bool tex_rgb = true;
	if(T.no_rgb) { tin = xa(xa(xm(0.2126f, tex[0]), xm(0.7152f, tex[1])), xm(0.0722f, tex[2])); tex_rgb = false; }
	if(T.negative)
	{
		if(tex_rgb) for(int k = 0; k < 3; ++k) tex[k] = xs(1.f, tex[k]);
		tin = xs(1.f, tin);
	}
	if(T.stencil)
	{
		if(tex_rgb) { const float f = ta; ta = xm(ta, stencil_tin); stencil_tin = xm(stencil_tin, f); }
		else { const float f = tin; tin = xm(tin, stencil_tin); stencil_tin = xm(stencil_tin, f); }
	}
	if(!tex_rgb) for(int k = 0; k < 3; ++k) tex[k] = T.def_col[k];
	else tin = ta;
	const float tt = tin > 1.f ? 1.f : (tin < 0.f ? 0.f : tin);
	const float facg = xm(stencil_tin, T.colfac);
	const float fact = xm(tt, facg);
	for(int k = 0; k < 3; ++k)
	{
		const float t = tex[k], o = T.upper[k];
		float v;
		switch(T.blend)
		{
			case GBRT_BLEND_MULTIPLY: v = xm(xa(xs(1.f, facg), xm(fact, t)), o); break;
			case GBRT_BLEND_SCREEN: v = xs(1.f, xm(xa(xs(1.f, facg), xm(fact, xs(1.f, t))), xs(1.f, o))); break;
			case GBRT_BLEND_SUBTRACT: v = xs(o, xm(fact, t)); break;
			case GBRT_BLEND_ADD: v = xa(o, xm(fact, t)); break;
			case GBRT_BLEND_DIVIDE: v = xa(xm(xs(1.f, fact), o), xm(xm(fact, o), t != 0.f ? __fdiv_rn(1.f, t) : 0.f)); break;
			case GBRT_BLEND_DIFFERENCE: v = xa(xm(xs(1.f, fact), o), xm(fact, fabsf(xs(t, o)))); break;
			case GBRT_BLEND_DARKEN: v = xm(fact, t) > o ? o : xm(fact, t); break;
			case GBRT_BLEND_LIGHTEN: v = xm(fact, t) < o ? o : xm(fact, t); break;
			default: v = xa(xm(fact, t), xm(xs(1.f, fact), o)); break;
		}
		rgb[k] = v < 0.f ? 0.f : v;
	}
}

// A procedural texture's colour, out of line so the shading kernels keep
// their registers for the common path.
__device__ __noinline__ void tex_procedural(const SceneDev &sc, const DevTexture &T, const float p[3], float c4[4], float *scalar)
{
	gbrt::proc_color(sc.nt, T.proc, p, c4);
	if(scalar) *scalar = gbrt::proc_float(sc.nt, T.proc, p);
}

// Texture::applyIntensityContrastAdjustments(float) of an image texture
// (texture.cc:272-287).
__device__ __forceinline__ float image_adjust_float(const DevTexture &T, float v)
{
	if(!T.adj) return v;
	float r = v;
	if(T.adj_ic) r = xs(xa(xm(xs(v, 0.5f), T.contrast), T.intensity), 0.5f);
	if(T.adj_clamp) r = r < 0.f ? 0.f : (r > 1.f ? 1.f : r);
	return r;
}

// TextureMapperNode::getCoords / doMapping (shader_node_texture.cc:153-230),
// ImageTexture::getColor / doMapping / noInterpolation /
// bilinearInterpolation / bicubicInterpolation (texture_image.cc:180-262,
// 343-427) and
// Texture::applyAdjustments (texture.cc:219-253): the texture's RGBA at a
// hit (getColor); with scalar, also its getFloat (for an image,
// applyIntensityContrastAdjustments of the colour's brightness, texture.h:52).
__device__ void tex_domap(const DevTexture &T, const float c[3], const float ng[3], float t[3])
{
	float q[3];
	if(T.texco == GBRT_TEXCO_UV) { q[0] = xs(xm(2.f, c[0]), 1.f); q[1] = xs(xm(2.f, c[1]), 1.f); q[2] = c[2]; }
	else { q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; }
	const float tm[4] = {0.f, q[0], q[1], q[2]};
	t[0] = tm[T.proj[0]]; t[1] = tm[T.proj[1]]; t[2] = tm[T.proj[2]];
	if(T.mapping == GBRT_MAPPING_CUBE)
	{
		// cubeMap: axis of the largest normal component (ties to z, then y)
		const float ax = fabsf(ng[0]), ay = fabsf(ng[1]), az = fabsf(ng[2]);
		float r[3];
		if(az >= ax && az >= ay) { r[0] = t[0]; r[1] = t[1]; r[2] = t[2]; }
		else if(ay >= ax && ay >= az) { r[0] = t[0]; r[1] = t[2]; r[2] = t[1]; }
		else { r[0] = t[1]; r[1] = t[2]; r[2] = t[0]; }
		t[0] = r[0]; t[1] = r[1]; t[2] = r[2];
	}
	else if(T.mapping == GBRT_MAPPING_TUBE)
	{
		// TextureMapperNode::tubeMap (shader_node_texture.cc:125-137)
		float r[3];
		r[1] = t[2];
		const float d = xa(xm(t[0], t[0]), xm(t[1], t[1]));
		if(d > 0.f) { r[2] = __fdiv_rn(1.f, sqrtf(d)); r[0] = xm(-atan2f(t[0], t[1]), kInvPi); }
		else r[0] = r[2] = 0.f;
		t[0] = r[0]; t[1] = r[1]; t[2] = r[2];
	}
	else if(T.mapping == GBRT_MAPPING_SPHERE)
	{
		// TextureMapperNode::sphereMap (:139-151) with math::acos's clamp
		float r[3] = {0.f, 0.f, 0.f};
		const float d = xa(xa(xm(t[0], t[0]), xm(t[1], t[1])), xm(t[2], t[2]));
		if(d > 0.f)
		{
			r[2] = sqrtf(d);
			if(t[0] != 0.f && t[1] != 0.f) r[0] = xm(-atan2f(t[0], t[1]), kInvPi);
			const float c = __fdiv_rn(t[2], r[2]);
			const float ac = c <= -1.f ? kPi : (c >= 1.f ? 0.f : acosf(c));
			r[1] = xs(1.f, xm(2.f, xm(ac, kInvPi)));
		}
		t[0] = r[0]; t[1] = r[1]; t[2] = r[2];
	}
	for(int k = 0; k < 3; ++k) t[k] = xa(xm(t[k], T.scale[k]), T.offset2[k]);
}

// TextureMapperNode::getCoords (shader_node_texture.cc:203-230): the hit
// position, or (u, v, 0) for uv coordinates.
__device__ __forceinline__ void tex_coords(const DevTexture &T, const float p[3], const float uv[2], float c[3])
{
	if(T.texco == GBRT_TEXCO_UV) { c[0] = uv[0]; c[1] = uv[1]; c[2] = 0.f; }
	else { c[0] = p[0]; c[1] = p[1]; c[2] = p[2]; }
}

// The texture's getColor and (with scalar) getFloat at a texture-space point.
__device__ void tex_eval_at(const SceneDev &sc, const DevTexture &T, const float t[3], float out[4], float *scalar)
{
	if(T.kind != GBRT_TEX_IMAGE)
	{
		// a procedural texture at the mapped point
		tex_procedural(sc, T, t, out, scalar);
		return;
	}
	// the image's own mapping of (x, -y, z)
	float mx = xa(xm(0.5f, t[0]), 0.5f), my = xa(xm(0.5f, -t[1]), 0.5f);
	const float mz = xa(xm(0.5f, t[2]), 0.5f);
	if(T.clip == GBRT_CLIP_REPEAT)
	{
		if(T.xrep > 1) mx = xm(mx, static_cast<float>(T.xrep));
		if(T.yrep > 1) my = xm(my, static_cast<float>(T.yrep));
		if(T.mirror_x && static_cast<int>(ceilf(mx)) % 2 == 0) mx = -mx;
		if(T.mirror_y && static_cast<int>(ceilf(my)) % 2 == 0) my = -my;
		if(mx > 1.f) mx = xs(mx, truncf(mx));
		else if(mx < 0.f) mx = xa(mx, xs(1.f, truncf(mx)));
		if(my > 1.f) my = xs(my, truncf(my));
		else if(my < 0.f) my = xa(my, xs(1.f, truncf(my)));
	}
	if(T.crop_x) mx = xa(T.crop[0], xm(mx, xs(T.crop[2], T.crop[0])));
	if(T.crop_y) my = xa(T.crop[1], xm(my, xs(T.crop[3], T.crop[1])));
	if(T.rot90) { const float tmp = mx; mx = my; my = tmp; }
	bool outside = false;
	if(T.clip == GBRT_CLIP_CLIPCUBE) outside = mx < 0.f || mx > 1.f || my < 0.f || my > 1.f || mz < -1.f || mz > 1.f;
	else if(T.clip == GBRT_CLIP_CHECKER)
	{
		const float fx = floorf(mx), fy = floorf(my);
		mx = xs(mx, fx);
		my = xs(my, fy);
		const bool odd = (static_cast<int>(xa(fx, fy)) & 1) != 0;
		if(!T.odd_tiles && !odd) outside = true;
		else if(!T.even_tiles && odd) outside = true;
		else
		{
			// scaled about the tile centre, then the clip test
			if(T.checker_dist < 1.f)
			{
				mx = xa(__fdiv_rn(xs(mx, 0.5f), xs(1.f, T.checker_dist)), 0.5f);
				my = xa(__fdiv_rn(xs(my, 0.5f), xs(1.f, T.checker_dist)), 0.5f);
			}
			outside = mx < 0.f || mx > 1.f || my < 0.f || my > 1.f;
		}
	}
	else if(T.clip == GBRT_CLIP_CLIP) outside = mx < 0.f || mx > 1.f || my < 0.f || my > 1.f;
	else if(T.clip == GBRT_CLIP_EXTEND)
	{
		mx = mx > 0.99999f ? 0.99999f : (mx < 0.f ? 0.f : mx);
		my = my > 0.99999f ? 0.99999f : (my < 0.f ? 0.f : my);
	}
	if(outside)
	{
		out[0] = out[1] = out[2] = out[3] = 0.f;
		if(scalar) *scalar = image_adjust_float(T, 0.f);
		return;
	}
	const bool rep = T.clip == GBRT_CLIP_REPEAT;
	const float4 *tx = sc.texels + T.off;
	float4 c;
	if(T.interp == GBRT_INTERP_NONE)
	{
		const float xf = xm(static_cast<float>(T.w), xs(mx, floorf(mx)));
		const float yf = xm(static_cast<float>(T.h), xs(my, floorf(my)));
		int x1, x2, y1, y2;
		float dx, dy;
		tex_axis(xf, T.w, rep, T.mirror_x != 0, x1, x2, dx);
		tex_axis(yf, T.h, rep, T.mirror_y != 0, y1, y2, dy);
		c = __ldg(tx + y1 * T.w + x1);
	}
	else if(T.interp == GBRT_INTERP_BICUBIC)
	{
		// ImageTexture::bicubicInterpolation (texture_image.cc:387-427): rows
		// along x first, then the four row results along y
		const float xf = xs(xm(static_cast<float>(T.w), xs(mx, floorf(mx))), 0.5f);
		const float yf = xs(xm(static_cast<float>(T.h), xs(my, floorf(my))), 0.5f);
		int xs4[4], ys4[4];
		float dx, dy;
		tex_axis(xf, T.w, rep, T.mirror_x != 0, xs4[1], xs4[2], dx, &xs4[0], &xs4[3]);
		tex_axis(yf, T.h, rep, T.mirror_y != 0, ys4[1], ys4[2], dy, &ys4[0], &ys4[3]);
		float4 row[4];
		for(int j = 0; j < 4; ++j)
		{
			const float4 *t = tx + static_cast<size_t>(ys4[j]) * T.w;
			const float4 a = __ldg(t + xs4[0]), b = __ldg(t + xs4[1]), cc = __ldg(t + xs4[2]), e = __ldg(t + xs4[3]);
			row[j] = make_float4(cubic_interp(a.x, b.x, cc.x, e.x, dx), cubic_interp(a.y, b.y, cc.y, e.y, dx),
			                     cubic_interp(a.z, b.z, cc.z, e.z, dx), cubic_interp(a.w, b.w, cc.w, e.w, dx));
		}
		c = make_float4(cubic_interp(row[0].x, row[1].x, row[2].x, row[3].x, dy), cubic_interp(row[0].y, row[1].y, row[2].y, row[3].y, dy),
		                cubic_interp(row[0].z, row[1].z, row[2].z, row[3].z, dy), cubic_interp(row[0].w, row[1].w, row[2].w, row[3].w, dy));
	}
	else
	{
		const float xf = xs(xm(static_cast<float>(T.w), xs(mx, floorf(mx))), 0.5f);
		const float yf = xs(xm(static_cast<float>(T.h), xs(my, floorf(my))), 0.5f);
		int x1, x2, y1, y2;
		float dx, dy;
		tex_axis(xf, T.w, rep, T.mirror_x != 0, x1, x2, dx);
		tex_axis(yf, T.h, rep, T.mirror_y != 0, y1, y2, dy);
		const float4 c11 = __ldg(tx + y1 * T.w + x1), c21 = __ldg(tx + y1 * T.w + x2);
		const float4 c12 = __ldg(tx + y2 * T.w + x1), c22 = __ldg(tx + y2 * T.w + x2);
		const float w11 = xm(xs(1.f, dx), xs(1.f, dy)), w12 = xm(xs(1.f, dx), dy);
		const float w21 = xm(dx, xs(1.f, dy)), w22 = xm(dx, dy);
		c.x = xa(xa(xa(xm(w11, c11.x), xm(w12, c12.x)), xm(w21, c21.x)), xm(w22, c22.x));
		c.y = xa(xa(xa(xm(w11, c11.y), xm(w12, c12.y)), xm(w21, c21.y)), xm(w22, c22.y));
		c.z = xa(xa(xa(xm(w11, c11.z), xm(w12, c12.z)), xm(w21, c21.z)), xm(w22, c22.z));
		c.w = xa(xa(xa(xm(w11, c11.w), xm(w12, c12.w)), xm(w21, c21.w)), xm(w22, c22.w));
	}
	const float alpha = c.w;
	float r[3] = {c.x, c.y, c.z};
	if(T.adj)
	{
		if(T.adj_ic)
			for(int k = 0; k < 3; ++k) r[k] = xs(xa(xm(xs(r[k], 0.5f), T.contrast), T.intensity), 0.5f);
		if(T.adj_clamp) for(int k = 0; k < 3; ++k) r[k] = r[k] < 0.f ? 0.f : r[k];
		for(int k = 0; k < 3; ++k) if(T.mult[k] != 1.f) r[k] = xm(r[k], T.mult[k]);
		if(T.adj_clamp) for(int k = 0; k < 3; ++k) r[k] = r[k] < 0.f ? 0.f : r[k];
		if(T.saturation != 1.f || T.hue6 != 0.f)
		{
			// the HSV step of Texture::applyColorAdjustments (texture.cc:260-269)
			float h = 0.f, sat = 0.f, v = 0.f;
			gbrt::rgb_to_hsv(r, h, sat, v);
			sat = xm(sat, T.saturation);
			h = xa(h, T.hue6);
			if(h < 0.f) h = xa(h, 6.f);
			else if(h > 6.f) h = xs(h, 6.f);
			gbrt::hsv_to_rgb(h, sat, v, r);
			if(T.adj_clamp) for(int k = 0; k < 3; ++k) r[k] = r[k] < 0.f ? 0.f : r[k];
		}
	}
	out[0] = r[0]; out[1] = r[1]; out[2] = r[2]; out[3] = alpha;
	if(scalar) *scalar = image_adjust_float(T, xa(xa(xm(0.2126f, r[0]), xm(0.7152f, r[1])), xm(0.0722f, r[2])));
}

__device__ void tex_eval(const SceneDev &sc, const DevTexture &T, const float p[3], const float ng[3], const float uv[2], float out[4],
                         float *scalar)
{
	float c[3], t[3];
	tex_coords(T, p, uv, c);
	tex_domap(T, c, ng, t);
	tex_eval_at(sc, T, t, out, scalar);
}

// A diffuse shader of gbrt_scene_set_textures: the texture through its
// mapper and optional layer node.
__device__ __noinline__ void tex_color(const SceneDev &sc, const DevTexture &T, const float p[3], const float ng[3], const float uv[2],
                                       float out[3])
{
	float c4[4];
	tex_eval(sc, T, p, ng, uv, c4, nullptr);
	out[0] = c4[0]; out[1] = c4[1]; out[2] = c4[2];
	tex_layer(T, c4[3], out);
}

// Evaluates the shader node tree [first, root] at a surface point
// (Material::evalNodes over the nodes of src/shader/): every node's colour
// (RGBA) and scalar, in index order (each reads only lower indices); returns
// the root's.
__device__ __noinline__ void node_tree(const SceneDev &sc, int first, int root, uint32_t mask, const float p[3], const float ng[3],
                                       const float uv[2], float out[4], float &scalar)
{
	float R[GBRT_TREE_MAX][5];
	for(int i = first; i <= root; ++i)
	{
		if(!((mask >> (i - first)) & 1u)) continue;      // a node the root does not read
		const gbrt_shader_node &N = sc.nodes[i];
		float *r = R[i - first];
		auto col_of = [&](int j, const float def[4], float c[4]) {
			for(int k = 0; k < 4; ++k) c[k] = j >= 0 ? R[j - first][k] : def[k];
		};
		auto val_of = [&](int j, float def) { return j >= 0 ? R[j - first][4] : def; };
		switch(N.type)
		{
			case GBRT_NODE_TEXTURE:
			{
				// TextureMapperNode::eval (shader_node_texture.cc:232-251)
				float f = 0.f;
				tex_eval(sc, sc.tex[N.texture], p, ng, uv, r, N.do_scalar ? &f : nullptr);
				r[4] = f;
				break;
			}
			case GBRT_NODE_VALUE:
				// ValueNode::eval (shader_node_value.cc:71-74): colour with its alpha, scalar
				for(int k = 0; k < 4; ++k) r[k] = N.color1[k];
				r[4] = N.value1;
				break;
			case GBRT_NODE_MIX:
			{
				// MixNode::getInputs / eval and the blend-mode nodes (shader_node_mix.cc:143-175, mix/*.h)
				const float f = val_of(N.input_factor, N.factor);
				float c1[4], c2[4];
				col_of(N.input1, N.color1, c1);
				col_of(N.input2, N.color2, c2);
				float f1 = val_of(N.input1, N.value1), f2 = val_of(N.input2, N.value2);
				switch(N.mode)
				{
					case GBRT_MIX_ADD:
						for(int k = 0; k < 4; ++k) c1[k] = xa(c1[k], xm(f, c2[k]));
						f1 = xa(f1, xm(f, f2));
						break;
					case GBRT_MIX_MULTIPLY:
						for(int k = 0; k < 4; ++k) c1[k] = xm(c1[k], xa(xm(1.f, xs(1.f, f)), xm(c2[k], f)));
						f1 = xm(f1, xa(xm(1.f, xs(1.f, f)), xm(f2, f)));
						break;
					case GBRT_MIX_SUBTRACT:
						for(int k = 0; k < 4; ++k) c1[k] = xs(c1[k], xm(f, c2[k]));
						f1 = xs(f1, xm(f, f2));
						break;
					case GBRT_MIX_SCREEN:
					{
						const float fr = xs(1.f, f);
						for(int k = 0; k < 4; ++k) c1[k] = xs(1.f, xm(xa(fr, xm(f, xs(1.f, c2[k]))), xs(1.f, c1[k])));
						f1 = xs(1.f, xm(xa(fr, xm(f, xs(1.f, f2))), xs(1.f, f1)));
						break;
					}
					case GBRT_MIX_DIFFERENCE:
						for(int k = 0; k < 4; ++k) c1[k] = xa(xm(c1[k], xs(1.f, f)), xm(fabsf(xs(c1[k], c2[k])), f));
						f1 = xa(xm(f1, xs(1.f, f)), xm(fabsf(xs(f1, f2)), f));
						break;
					case GBRT_MIX_DARKEN:
					case GBRT_MIX_LIGHTEN:
					{
						const bool dark = N.mode == GBRT_MIX_DARKEN;
						for(int k = 0; k < 4; ++k)
						{
							const float v = xm(c2[k], f);
							if(dark ? v < c1[k] : v > c1[k]) c1[k] = v;
						}
						const float v = xm(f2, f);
						if(dark ? v < f1 : v > f1) f1 = v;
						break;
					}
					case GBRT_MIX_OVERLAY:
					{
						auto ov = [&](float a, float b) {
							if(a < 0.5f) return xm(a, xa(xs(1.f, f), xm(xm(2.f, f), b)));
							return xs(1.f, xm(xa(xs(1.f, f), xm(xm(2.f, f), xs(1.f, b))), xs(1.f, a)));
						};
						for(int k = 0; k < 4; ++k) c1[k] = ov(c1[k], c2[k]);
						f1 = ov(f1, f2);
						break;
					}
					default:   // mix: math::lerp
						for(int k = 0; k < 4; ++k) c1[k] = xa(xm(c1[k], xs(1.f, f)), xm(c2[k], f));
						f1 = xa(xm(f1, xs(1.f, f)), xm(f2, f));
						break;
				}
				for(int k = 0; k < 4; ++k) r[k] = c1[k];
				r[4] = f1;
				break;
			}
			default:
			{
				// LayerNode::eval (shader_node_layer.cc:110-194) with textureRgbBlend /
				// textureValueBlend (:264-366)
				float rcol[4], tex[4] = {0.f, 0.f, 0.f, 1.f};
				col_of(N.input2, N.color1, rcol);
				float rval = val_of(N.input2, N.value1);
				float stencil_tin = rcol[3];
				float tin = 0.f, ta = 1.f;
				bool tex_rgb = N.color_input != 0;
				if(N.color_input) { for(int k = 0; k < 4; ++k) tex[k] = R[N.input1 - first][k]; ta = tex[3]; }
				else tin = R[N.input1 - first][4];
				if(N.no_rgb) { tin = xa(xa(xm(0.2126f, tex[0]), xm(0.7152f, tex[1])), xm(0.0722f, tex[2])); tex_rgb = false; }
				if(N.negative)
				{
					if(tex_rgb) for(int k = 0; k < 4; ++k) tex[k] = xs(1.f, tex[k]);
					tin = xs(1.f, tin);
				}
				if(N.stencil)
				{
					if(tex_rgb) { const float fact = ta; ta = xm(ta, stencil_tin); stencil_tin = xm(stencil_tin, fact); }
					else { const float fact = tin; tin = xm(tin, stencil_tin); stencil_tin = xm(stencil_tin, fact); }
				}
				if(N.do_color)
				{
					if(!tex_rgb) for(int k = 0; k < 4; ++k) tex[k] = N.def_col[k];
					else tin = ta;
					const float tt = tin > 1.f ? 1.f : (tin < 0.f ? 0.f : tin);
					const float facg = xm(stencil_tin, N.colfac);
					const float fact = xm(tt, facg);
					for(int k = 0; k < 3; ++k)
					{
						const float t = tex[k], o = rcol[k];
						float v;
						switch(N.mode)
						{
							case GBRT_BLEND_MULTIPLY: v = xm(xa(xs(1.f, facg), xm(fact, t)), o); break;
							case GBRT_BLEND_SCREEN: v = xs(1.f, xm(xa(xs(1.f, facg), xm(fact, xs(1.f, t))), xs(1.f, o))); break;
							case GBRT_BLEND_SUBTRACT: v = xs(o, xm(fact, t)); break;
							case GBRT_BLEND_ADD: v = xa(o, xm(fact, t)); break;
							case GBRT_BLEND_DIVIDE: v = xa(xm(xs(1.f, fact), o), xm(xm(fact, o), t != 0.f ? __fdiv_rn(1.f, t) : 0.f)); break;
							case GBRT_BLEND_DIFFERENCE: v = xa(xm(xs(1.f, fact), o), xm(fact, fabsf(xs(t, o)))); break;
							case GBRT_BLEND_DARKEN: v = xm(fact, t) > o ? o : xm(fact, t); break;
							case GBRT_BLEND_LIGHTEN: v = xm(fact, t) < o ? o : xm(fact, t); break;
							default: v = xa(xm(fact, t), xm(xs(1.f, fact), o)); break;
						}
						rcol[k] = v < 0.f ? 0.f : v;
					}
				}
				if(N.do_scalar)
				{
					if(tex_rgb)
					{
						if(N.use_alpha) { tin = ta; if(N.negative) tin = xs(1.f, tin); }
						else tin = xa(xa(xm(0.2126f, tex[0]), xm(0.7152f, tex[1])), xm(0.0722f, tex[2]));
					}
					const float facg = xm(stencil_tin, N.valfac);
					float fact = xm(tin, facg);
					float facm = xs(1.f, fact);
					const float t = N.def_val, o = rval;
					float v;
					switch(N.mode)
					{
						case GBRT_BLEND_MULTIPLY: facm = xs(1.f, facg); v = xm(xa(facm, xm(fact, t)), o); break;
						case GBRT_BLEND_SCREEN: facm = xs(1.f, facg); v = xs(1.f, xm(xa(facm, xm(fact, xs(1.f, t))), xs(1.f, o))); break;
						case GBRT_BLEND_SUBTRACT: v = xs(o, xm(fact, t)); break;
						case GBRT_BLEND_ADD: v = xa(o, xm(fact, t)); break;
						case GBRT_BLEND_DIVIDE: v = t == 0.f ? 0.f : xa(xm(facm, o), __fdiv_rn(xm(fact, o), t)); break;
						case GBRT_BLEND_DIFFERENCE: v = xa(xm(facm, o), xm(fact, fabsf(xs(t, o)))); break;
						case GBRT_BLEND_DARKEN: { const float c = xm(fact, t); v = c < o ? c : o; break; }
						case GBRT_BLEND_LIGHTEN: { const float c = xm(fact, t); v = c > o ? c : o; break; }
						default: v = xa(xm(fact, t), xm(facm, o)); break;
					}
					rval = v < 0.f ? 0.f : v;
				}
				rcol[3] = stencil_tin;
				for(int k = 0; k < 4; ++k) r[k] = rcol[k];
				r[4] = rval;
				break;
			}
		}
	}
	for(int k = 0; k < 4; ++k) out[k] = R[root - first][k];
	scalar = R[root - first][4];
}

// The diffuse colour of a surface point (the material's, or its diffuse
// shader's texture at the hit's coordinates).
// TextureMapperNode::evalDerivative (shader_node_texture.cc:255-355) of a
// texture node: the texture's getFloat differences along the surface frame
// (s.u, s.v: createCoordsSystem of the shading normal) around the point, or,
// for an image through uv coordinates of a uv-mapped mesh, its slopes in
// texture space carried into shading space by dP/du, dP/dv
// (PrimitivePolygon::getSurfacePolygon, primitive_polygon.cc:70-114).
__device__ void tex_derivative(const SceneDev &sc, const DevTexture &T, float bump_strength, const Surface &s, int prim, const float uv[2],
                               float &du, float &dv)
{
	const bool image = T.kind == GBRT_TEX_IMAGE;
	const float d_u = image ? __fdiv_rn(1.f, static_cast<float>(T.w)) : 0.0002f;
	const float d_v = image ? __fdiv_rn(1.f, static_cast<float>(T.h)) : 0.0002f;
	// bump_strength / |scale| / 100 (the mapper's constructor)
	const float len = sqrtf(xa(xa(xm(T.scale[0], T.scale[0]), xm(T.scale[1], T.scale[1])), xm(T.scale[2], T.scale[2])));
	const float bs = __fdiv_rn(__fdiv_rn(bump_strength, len), 100.f);
	const uint4 fu = __ldg(sc.face_uv + prim);
	float c[3], f0, f1, g0, g1, col[4];
	tex_coords(T, s.p, uv, c);
	if(image && fu.x != kNoIdx && T.texco == GBRT_TEXCO_UV)
	{
		float t[3], q[3];
		tex_domap(T, c, s.ng, t);
		q[0] = xs(t[0], d_u); q[1] = t[1]; q[2] = t[2]; tex_eval_at(sc, T, q, col, &f0);
		q[0] = xa(t[0], d_u); tex_eval_at(sc, T, q, col, &f1);
		q[0] = t[0]; q[1] = xs(t[1], d_v); tex_eval_at(sc, T, q, col, &g0);
		q[1] = xa(t[1], d_v); tex_eval_at(sc, T, q, col, &g1);
		const float dfdu = __fdiv_rn(xs(f0, f1), d_u), dfdv = __fdiv_rn(xs(g0, g1), d_v);
		// dP/du, dP/dv of the face from its first three corners and uvs
		const uint32_t slot = __ldg(sc.prim_slot + prim);
		const float4 B = __ldg(sc.bv.tris + 3ull * slot + 1), C = __ldg(sc.bv.tris + 3ull * slot + 2);
		const float e1[3] = {B.x, B.y, B.z}, e2[3] = {C.x, C.y, C.z};
		const float2 a = __ldg(sc.uv + fu.x), b = __ldg(sc.uv + fu.y), cc = __ldg(sc.uv + fu.z);
		const float d1u = xs(b.x, a.x), d1v = xs(b.y, a.y), d2u = xs(cc.x, a.x), d2v = xs(cc.y, a.y);
		const float det = xs(xm(d1u, d2v), xm(d1v, d2u));
		float dpu[3], dpv[3];
		if(fabsf(det) > 1e-30f)
		{
			const float inv = __fdiv_rn(1.f, det);
			for(int k = 0; k < 3; ++k)
			{
				dpu[k] = xm(xs(xm(d2v, e1[k]), xm(d1v, e2[k])), inv);
				dpv[k] = xm(xs(xm(d1u, e2[k]), xm(d2u, e1[k])), inv);
			}
		}
		else for(int k = 0; k < 3; ++k) { dpu[k] = e1[k]; dpv[k] = e2[k]; }
		normalize3(dpu);
		normalize3(dpv);
		float vu[3] = {dot3(s.u, dpu), dot3(s.v, dpu), dfdu};
		float vv[3] = {dot3(s.u, dpv), dot3(s.v, dpv), dfdv};
		float nrm[3] = {xs(xm(vu[1], vv[2]), xm(vu[2], vv[1])), xs(xm(vu[2], vv[0]), xm(vu[0], vv[2])), xs(xm(vu[0], vv[1]), xm(vu[1], vv[0]))};
		normalize3(nrm);
		if(fabsf(nrm[2]) > 1e-30f)
		{
			const float nf = xm(__fdiv_rn(1.f, nrm[2]), bs);
			du = xm(nrm[0], nf);
			dv = xm(nrm[1], nf);
		}
		else du = dv = 0.f;
		return;
	}
	float q[3], t[3];
	for(int k = 0; k < 3; ++k) q[k] = xs(c[k], xm(d_u, s.u[k]));
	tex_domap(T, q, s.ng, t); tex_eval_at(sc, T, t, col, &f0);
	for(int k = 0; k < 3; ++k) q[k] = xa(c[k], xm(d_u, s.u[k]));
	tex_domap(T, q, s.ng, t); tex_eval_at(sc, T, t, col, &f1);
	for(int k = 0; k < 3; ++k) q[k] = xs(c[k], xm(d_v, s.v[k]));
	tex_domap(T, q, s.ng, t); tex_eval_at(sc, T, t, col, &g0);
	for(int k = 0; k < 3; ++k) q[k] = xa(c[k], xm(d_v, s.v[k]));
	tex_domap(T, q, s.ng, t); tex_eval_at(sc, T, t, col, &g1);
	du = xm(__fdiv_rn(xs(f0, f1), d_u), bs);
	dv = xm(__fdiv_rn(xs(g0, g1), d_v), bs);
	if(T.texco != GBRT_TEXCO_UV) { du = -du; dv = -dv; }
}

// NodeMaterial::evalBump (material_node.cc:95-100): the bump tree's
// evalDerivative results (texture nodes above; LayerNode::evalDerivative,
// shader_node_layer.cc:196-225; other nodes zero) and Material::applyBump
// (material.cc:218-225) on the shading frame.
__device__ __noinline__ void surface_bump(const SceneDev &sc, Surface &s, int first, int root, uint32_t mask, int prim, const float uv[2])
{
	float R[GBRT_TREE_MAX][4];
	for(int i = first; i <= root; ++i)
	{
		if(!((mask >> (i - first)) & 1u)) continue;
		const gbrt_shader_node &N = sc.nodes[i];
		float *r = R[i - first];
		if(N.type == GBRT_NODE_TEXTURE)
		{
			tex_derivative(sc, sc.tex[N.texture], N.bump_strength, s, prim, uv, r[0], r[1]);
			r[2] = 0.f; r[3] = 0.f;
		}
		else if(N.type == GBRT_NODE_LAYER)
		{
			float rdu = 0.f, rdv = 0.f, stencil = 1.f;
			if(N.input2 >= 0) { const float *u = R[N.input2 - first]; rdu = u[0]; rdv = u[1]; stencil = u[3]; }
			const float *t = R[N.input1 - first];
			float tdu = t[0], tdv = t[1];
			if(N.negative) { tdu = -tdu; tdv = -tdv; }
			r[0] = xa(rdu, tdu); r[1] = xa(rdv, tdv); r[2] = 0.f; r[3] = stencil;
		}
		else { r[0] = r[1] = r[2] = 0.f; r[3] = 1.f; }
	}
	const float du = R[root - first][0], dv = R[root - first][1];
	for(int k = 0; k < 3; ++k) { s.u[k] = xa(s.u[k], xm(du, s.n[k])); s.v[k] = xa(s.v[k], xm(dv, s.n[k])); }
	s.n[0] = xs(xm(s.u[1], s.v[2]), xm(s.u[2], s.v[1]));
	s.n[1] = xs(xm(s.u[2], s.v[0]), xm(s.u[0], s.v[2]));
	s.n[2] = xs(xm(s.u[0], s.v[1]), xm(s.u[1], s.v[0]));
	normalize3(s.n);
	normalize3(s.u);
	s.v[0] = xs(xm(s.n[1], s.u[2]), xm(s.n[2], s.u[1]));
	s.v[1] = xs(xm(s.n[2], s.u[0]), xm(s.n[0], s.u[2]));
	s.v[2] = xs(xm(s.n[0], s.u[1]), xm(s.n[1], s.u[0]));
	normalize3(s.v);
}

// With shader node trees on its slots the material is copied to mloc with
// the slot colours of this point (the reference's getShaderColor of each
// slot) and s.m points there: the diffuse colour of shinydiffuse (s.dcol)
// and glossy, the glossy colour, the mirror colour, the glass filter colour.
__device__ __noinline__ void surface_nodes(const SceneDev &sc, Surface &s, int prim, float bu, float bv, DevMaterial &mloc)
{
	mloc = *s.m;
	float uv[2];
	hit_uv(sc, prim, bu, bv, uv);
	// the bump first: the colour nodes see the bumped surface (initBsdf)
	if(mloc.nroot[GBRT_SLOT_BUMP] >= 0)
		surface_bump(sc, s, mloc.nfirst[GBRT_SLOT_BUMP], mloc.nroot[GBRT_SLOT_BUMP], mloc.nmask[GBRT_SLOT_BUMP], prim, uv);
	for(int slot = 0; slot < GBRT_SLOT_BUMP; ++slot)
	{
		if(mloc.nroot[slot] < 0) continue;
		float c[4], f;
		node_tree(sc, mloc.nfirst[slot], mloc.nroot[slot], mloc.nmask[slot], s.p, s.ng, uv, c, f);
		if(slot == GBRT_SLOT_DIFFUSE)
		{
			if(mloc.type == GBRT_MAT_SHINYDIFFUSE) { s.dcol[0] = c[0]; s.dcol[1] = c[1]; s.dcol[2] = c[2]; mloc.dtex = 0; }
			else for(int k = 0; k < 3; ++k) mloc.col2[k] = c[k];
		}
		else if(slot == GBRT_SLOT_MIRROR_COLOR) for(int k = 0; k < 3; ++k) mloc.col2[k] = c[k];
		else for(int k = 0; k < 3; ++k) mloc.col[k] = c[k];    // glossy colour, glass filter colour
	}
	s.m = &mloc;
}

// kTex false: the scene has no textured material and no node trees (the
// kernels instantiated so carry none of the texture code).
template <bool kTex = true>
__device__ __forceinline__ void surface_color(const SceneDev &sc, Surface &s, int prim, float bu, float bv, DevMaterial &mloc)
{
	const DevMaterial &m = *s.m;
	if(!kTex || m.dtex < 0) { s.dcol[0] = m.col[0]; s.dcol[1] = m.col[1]; s.dcol[2] = m.col[2]; }
	else
	{
		float uv[2];
		hit_uv(sc, prim, bu, bv, uv);
		tex_color(sc, sc.tex[m.dtex], s.p, s.ng, uv, s.dcol);
	}
	if(kTex && m.has_nodes) surface_nodes(sc, s, prim, bu, bv, mloc);
}

// ---- ShinyDiffuseMaterial layers (material_shiny_diffuse.cc:205-619) -------
// The transmit colour transmit_filter x diffuse colour + (1 - transmit_filter)
// (:410, 517, 562), precomputed for an untextured diffuse colour.
__device__ __forceinline__ float shiny_tcol(const Surface &s, int k)
{
	return s.m->dtex < 0 ? s.m->tcol[k] : s.m->tf * s.dcol[k] + (1.f - s.m->tf);
}

// getFresnelKr (:205-217): Fresnel reflectance with the fresnel_effect, else 1.
__device__ __forceinline__ float shiny_kr(const DevMaterial &m, const float wo[3], const float n[3])
{
	if(!(m.sd & SD_FRESNEL)) return 1.f;
	float N[3] = {n[0], n[1], n[2]};
	if(dot3(wo, n) < 0.f) { N[0] = -n[0]; N[1] = -n[1]; N[2] = -n[2]; }
	const float c = dot3(wo, N);
	float g = m.ior + c * c - 1.f;
	if(g < 0.f) g = 0.f;
	else g = sqrtf(g);
	const float aux = c * (g + c);
	return ((0.5f * (g - c) * (g - c)) / ((g + c) * (g + c))) * (1.f + ((aux - 1.f) * (aux - 1.f)) / ((aux + 1.f) * (aux + 1.f)));
}

// accumulate (:222-233): absolute component weights from the layer fractions.
__device__ __forceinline__ void shiny_accum(const DevMaterial &m, float kr, float a[4])
{
	a[0] = m.sdc[0] * kr;
	float acc = 1.f - a[0];
	a[1] = m.sdc[1] * acc;
	acc *= 1.f - m.sdc[1];
	a[2] = m.sdc[2] * acc;
	acc *= 1.f - m.sdc[2];
	a[3] = m.sdc[3] * acc;
}

// Component order and flags (config, :146-189): mirror Specular|Reflect,
// transparency Transmit|Filter, translucency Diffuse|Transmit, diffuse
// Diffuse|Reflect.
__device__ __forceinline__ uint32_t shiny_cflags(int i)
{
	return i == 0 ? (BF_SPECULAR | BF_REFLECT) : i == 1 ? (BF_TRANSMIT | BF_FILTER) : i == 2 ? (BF_DIFFUSE | BF_TRANSMIT) : (BF_DIFFUSE | BF_REFLECT);
}

// eval (:297-337) with bsdfs = All
__device__ __noinline__ void shiny_eval_layers(const Surface &s, const float wo[3], const float wl[3], float out[3])
{
	const DevMaterial &m = *s.m;
	out[0] = out[1] = out[2] = 0.f;
	const float cos_ng_wo = dot3(s.ng, wo), cos_ng_wl = dot3(s.ng, wl);
	float n[3];
	face_forward(s, wo, n);
	if(!(m.flags & BF_DIFFUSE)) return;
	const float kr = shiny_kr(m, wo, n);
	const float m_t = (1.f - kr * m.sdc[0]) * (1.f - m.sdc[1]);
	if(xm(cos_ng_wo, cos_ng_wl) < 0.f && (m.sd & SD_TRANSLUCENT))
	{
		const float f = m.sdc[2] * m_t;
		for(int k = 0; k < 3; ++k) out[k] = f * s.dcol[k];
		return;
	}
	if(dot3(n, wl) < 0.f) return;
	const float m_d = m_t * (1.f - m.sdc[2]) * m.sdc[3];
	for(int k = 0; k < 3; ++k) out[k] = m_d * s.dcol[k];
}

// pdf (:443-484): the components whose flags share a bit with bsdfs add
// their weights to the normalisation (mirror and transparency included).
__device__ __noinline__ float shiny_pdf_layers(const Surface &s, const float wo[3], const float wi[3], uint32_t bsdfs)
{
	const DevMaterial &m = *s.m;
	if(!(bsdfs & BF_DIFFUSE)) return 0.f;
	const float cos_ng_wo = dot3(s.ng, wo);
	float n[3];
	face_forward(s, wo, n);
	float a[4];
	shiny_accum(m, shiny_kr(m, wo, n), a);
	float sum = 0.f, pdf = 0.f;
	int n_match = 0;
	for(int i = 0; i < 4; ++i)
	{
		if(!((m.sd >> i) & 1u) || !(bsdfs & shiny_cflags(i))) continue;
		const float width = a[i];
		sum += width;
		if(i == 2) { if(xm(cos_ng_wo, dot3(s.ng, wi)) < 0.f) pdf += fabsf(dot3(wi, n)) * width; }
		else if(i == 3) pdf += fabsf(dot3(wi, n)) * width;
		++n_match;
	}
	if(!n_match || sum < 0.00001f) return 0.f;
	return pdf / sum;
}

// reflectDir (vector.h:391-396)
__device__ __forceinline__ void reflect_dir(const float n[3], const float v[3], float out[3])
{
	const float vn = dot3(v, n);
	if(vn < 0.f) { out[0] = -v[0]; out[1] = -v[1]; out[2] = -v[2]; return; }
	for(int c = 0; c < 3; ++c) out[c] = 2.f * vn * n[c] - v[c];
}

// sample (:346-440): pick a component among those whose flags are all in
// the request, by s1, then sample it; w = |wi . N| / (0.99 pdf + 0.01).
__device__ __noinline__ bool shiny_sample_layers(const Surface &s, const float wo[3], float s1, float s2, uint32_t req, float wi[3],
                                                 float col[3], float &w, float &pdf, uint32_t &sampled)
{
	const DevMaterial &m = *s.m;
	const float cos_ng_wo = dot3(s.ng, wo);
	float n[3];
	face_forward(s, wo, n);
	const float kr = shiny_kr(m, wo, n);
	float a[4];
	shiny_accum(m, kr, a);
	float sum = 0.f, val[4], width[4];
	int choice[4], n_match = 0, pick = -1;
	for(int i = 0; i < 4; ++i)
	{
		const uint32_t cf = shiny_cflags(i);
		if(!((m.sd >> i) & 1u) || (req & cf) != cf) continue;
		width[n_match] = a[i];
		sum += width[n_match];
		choice[n_match] = i;
		val[n_match] = sum;
		++n_match;
	}
	if(!n_match || sum < 0.00001f) { sampled = 0u; pdf = 0.f; return false; }
	const float inv_sum = 1.f / sum;
	for(int i = 0; i < n_match; ++i)
	{
		val[i] *= inv_sum;
		width[i] *= inv_sum;
		if(s1 <= val[i] && pick < 0) pick = i;
	}
	if(pick < 0) pick = n_match - 1;
	const float s_1 = pick > 0 ? (s1 - val[pick - 1]) / width[pick] : s1 / width[pick];
	const int c = choice[pick];
	col[0] = col[1] = col[2] = 0.f;
	if(c == 0)
	{
		reflect_dir(n, wo, wi);
		pdf = width[pick];
		const float f = 1.f / fmaxf(fabsf(dot3(s.n, wi)), 1.0e-6f);
		for(int k = 0; k < 3; ++k) col[k] = (m.col2[k] * a[0]) * f;
	}
	else if(c == 1)
	{
		wi[0] = -wo[0]; wi[1] = -wo[1]; wi[2] = -wo[2];
		for(int k = 0; k < 3; ++k) col[k] = a[1] * shiny_tcol(s, k);
		pdf = fabsf(dot3(wi, n)) < 1e-6f ? 0.f : width[pick];
	}
	else if(c == 2)
	{
		const float nn[3] = {-n[0], -n[1], -n[2]};
		cos_hemisphere(nn, s.u, s.v, s_1, s2, wi);
		if(xm(cos_ng_wo, dot3(s.ng, wi)) < 0.f) for(int k = 0; k < 3; ++k) col[k] = a[2] * s.dcol[k];
		pdf = fabsf(dot3(wi, n)) * width[pick];
	}
	else
	{
		cos_hemisphere(n, s.u, s.v, s_1, s2, wi);
		if(xm(cos_ng_wo, dot3(s.ng, wi)) > 0.f) for(int k = 0; k < 3; ++k) col[k] = a[3] * s.dcol[k];
		pdf = fabsf(dot3(wi, n)) * width[pick];
	}
	sampled = shiny_cflags(c);
	w = __fdiv_rn(fabsf(dot3(wi, s.n)), xa(xm(pdf, 0.99f), 0.01f));
	if(m.sd & SD_TRANSPARENT)
	{
		// getAlpha (:568-587): alpha = 1 - (1 - mirror kr) transparency, and
		// sample() returns w alpha + (1 - alpha) for every component
		const float alpha = 1.f - (1.f - m.sdc[0] * kr) * m.sdc[1];
		w = xa(xm(w, alpha), 1.f - alpha);
	}
	return true;
}

// The diffuse layer alone (no mirror, transparency, translucency or
// Fresnel): kr = 1 and the accumulated weight is the diffuse strength c, so
// eval = c colour, pdf = |wi.n| c / c and sample picks the one component
// with width c (1 / c) — the same float operations as the general code.
// kPlain: the caller knows the material is the diffuse layer alone.
template <bool kPlain = false>
__device__ __forceinline__ void shiny_eval(const Surface &s, const float wo[3], const float wl[3], float out[3])
{
	if(!kPlain && s.m->sd != SD_DIFFUSE) { shiny_eval_layers(s, wo, wl, out); return; }
	out[0] = out[1] = out[2] = 0.f;
	float n[3];
	face_forward(s, wo, n);
	if(dot3(n, wl) < 0.f) return;
	const float m_d = s.m->sdc[3];
	for(int k = 0; k < 3; ++k) out[k] = m_d * s.dcol[k];
}

template <bool kPlain = false>
__device__ __forceinline__ float shiny_pdf(const Surface &s, const float wo[3], const float wi[3], uint32_t bsdfs)
{
	if(!kPlain && s.m->sd != SD_DIFFUSE) return shiny_pdf_layers(s, wo, wi, bsdfs);
	if(!(bsdfs & BF_DIFFUSE)) return 0.f;
	const float c = s.m->sdc[3];
	if(c < 0.00001f) return 0.f;
	float n[3];
	face_forward(s, wo, n);
	return (fabsf(dot3(wi, n)) * c) / c;
}

template <bool kExact = false, bool kPlain = false>
__device__ __forceinline__ bool shiny_sample(const Surface &s, const float wo[3], float s1, float s2, uint32_t req, float wi[3], float col[3],
                                             float &w, float &pdf, uint32_t &sampled)
{
	if(!kPlain && s.m->sd != SD_DIFFUSE) return shiny_sample_layers(s, wo, s1, s2, req, wi, col, w, pdf, sampled);
	const float c = s.m->sdc[3];
	if((req & (BF_DIFFUSE | BF_REFLECT)) != (BF_DIFFUSE | BF_REFLECT) || c < 0.00001f) { sampled = 0u; pdf = 0.f; return false; }
	const float width = c * (1.f / c);
	float n[3];
	face_forward(s, wo, n);
	cos_hemisphere<kExact>(n, s.u, s.v, s1 / width, s2, wi);
	col[0] = col[1] = col[2] = 0.f;
	if(xm(dot3(s.ng, wo), dot3(s.ng, wi)) > 0.f) for(int k = 0; k < 3; ++k) col[k] = c * s.dcol[k];
	pdf = fabsf(dot3(wi, n)) * width;
	sampled = BF_DIFFUSE | BF_REFLECT;
	w = __fdiv_rn(fabsf(dot3(wi, s.n)), xa(xm(pdf, 0.99f), 0.01f));
	return true;
}

// getSpecular (:490-533): transparency straight through, mirror reflection
// lifted off the surface when it grazes (cos with Ng < 0.01).
__device__ __forceinline__ void shiny_specular(const Surface &s, const float wo[3], bool &has_refract, float rdir[3], float rcol[3],
                                               bool &has_reflect, float ldir[3], float lcol[3])
{
	const DevMaterial &m = *s.m;
	const bool backface = dot3(wo, s.ng) < 0.f;
	float n[3], ng[3];
	for(int k = 0; k < 3; ++k) { n[k] = backface ? -s.n[k] : s.n[k]; ng[k] = backface ? -s.ng[k] : s.ng[k]; }
	const float kr = shiny_kr(m, wo, n);
	has_refract = (m.sd & SD_TRANSPARENT) != 0u;
	has_reflect = (m.sd & SD_MIRROR) != 0u;
	if(has_refract)
	{
		const float f = (1.f - m.sdc[0] * kr) * m.sdc[1];
		for(int k = 0; k < 3; ++k) { rdir[k] = -wo[k]; rcol[k] = f * shiny_tcol(s, k); }
	}
	if(has_reflect)
	{
		vec_reflect(wo, n, ldir);
		const float cos_wi_ng = dot3(ldir, ng);
		if(cos_wi_ng < 0.01f)
		{
			const float lift = 0.01f - cos_wi_ng;
			for(int k = 0; k < 3; ++k) ldir[k] += lift * ng[k];
			normalize3(ldir);
		}
		const float f = m.sdc[0] * kr;
		for(int k = 0; k < 3; ++k) lcol[k] = m.col2[k] * f;
	}
}

// Material::eval dispatch; ShinyDiffuseMaterial::eval diffuse component
// (material_shiny_diffuse.cc:297-337).
__device__ __forceinline__ void mat_eval(const Surface &s, const float wo[3], const float wl[3], float out[3])
{
	out[0] = out[1] = out[2] = 0.f;
	if(s.m->type == GBRT_MAT_GLOSSY) { glossy_eval(s, wo, wl, BF_ALL, out); return; }
	if(s.m->type == GBRT_MAT_SHINYDIFFUSE) shiny_eval(s, wo, wl, out);
}

// Material::pdf dispatch; ShinyDiffuseMaterial::pdf lambertian part
// (material_shiny_diffuse.cc:443-484).  Flags of the MIS calls:
// Glossy | Diffuse | Dispersive | Reflect | Transmit.
__device__ __forceinline__ float mat_pdf(const Surface &s, const float wo[3], const float wi[3])
{
	if(s.m->type == GBRT_MAT_GLOSSY) return glossy_pdf(s, wo, wi, BF_GLOSSY | BF_DIFFUSE | BF_DISPERSIVE | BF_REFLECT | BF_TRANSMIT);
	if(s.m->type != GBRT_MAT_SHINYDIFFUSE) return 0.f;
	return shiny_pdf(s, wo, wi, BF_GLOSSY | BF_DIFFUSE | BF_DISPERSIVE | BF_REFLECT | BF_TRANSMIT);
}

// Material::sample dispatch; ShinyDiffuseMaterial::sample diffuse reflection
// branch (material_shiny_diffuse.cc:346-440); light_mat returns pdf 0
// (material_light.cc:75-80).
template <bool kExact = false>
__device__ __forceinline__ bool mat_sample(const Surface &s, const float wo[3], float s1, float s2, uint32_t req_flags,
                                           float wi[3], float col[3], float &w, float &pdf, uint32_t &sampled)
{
	col[0] = col[1] = col[2] = 0.f;
	w = 0.f; pdf = 0.f; sampled = 0u;
	if(s.m->type == GBRT_MAT_GLOSSY)
	{
		glossy_sample<kExact>(s, wo, s1, s2, req_flags, wi, col, w, pdf, sampled);
		return sampled != 0u;
	}
	if(s.m->type == GBRT_MAT_GLASS) return glass_sample(s, wo, s1, req_flags, wi, col, w, pdf, sampled);
	if(s.m->type == GBRT_MAT_ROUGH_GLASS) return rough_sample(s, wo, s1, s2, req_flags, wi, col, w, pdf, sampled);
	if(s.m->type != GBRT_MAT_SHINYDIFFUSE) return false;
	return shiny_sample<kExact>(s, wo, s1, s2, req_flags, wi, col, w, pdf, sampled);
}

// The dispatch for scenes whose materials are all plain: shinydiffuse with
// the diffuse layer alone and an untextured colour, or light_mat
// (kLean); the same float operations as the general dispatch for those.
template <bool kLean>
__device__ __forceinline__ void mat_eval_l(const Surface &s, const float wo[3], const float wl[3], float out[3])
{
	if constexpr(kLean)
	{
		out[0] = out[1] = out[2] = 0.f;
		if(s.m->type == GBRT_MAT_SHINYDIFFUSE) shiny_eval<true>(s, wo, wl, out);
	}
	else mat_eval(s, wo, wl, out);
}

template <bool kLean>
__device__ __forceinline__ float mat_pdf_l(const Surface &s, const float wo[3], const float wi[3])
{
	if constexpr(kLean)
	{
		if(s.m->type != GBRT_MAT_SHINYDIFFUSE) return 0.f;
		return shiny_pdf<true>(s, wo, wi, BF_GLOSSY | BF_DIFFUSE | BF_DISPERSIVE | BF_REFLECT | BF_TRANSMIT);
	}
	else return mat_pdf(s, wo, wi);
}

template <bool kLean>
__device__ __forceinline__ bool mat_sample_l(const Surface &s, const float wo[3], float s1, float s2, uint32_t req_flags, float wi[3],
                                             float col[3], float &w, float &pdf, uint32_t &sampled)
{
	if constexpr(kLean)
	{
		col[0] = col[1] = col[2] = 0.f;
		w = 0.f; pdf = 0.f; sampled = 0u;
		if(s.m->type != GBRT_MAT_SHINYDIFFUSE) return false;
		return shiny_sample<false, true>(s, wo, s1, s2, req_flags, wi, col, w, pdf, sampled);
	}
	else return mat_sample(s, wo, s1, s2, req_flags, wi, col, w, pdf, sampled);
}

// Sample colour x weight that Material::sample would return for a given
// direction wi (both sampling branches of glossy give the same function of
// wi), used for directions drawn from the guide.
__device__ __forceinline__ void bsdf_eval_at(const Surface &s, const float wo[3], const float wi[3], uint32_t flags, float fw[3])
{
	fw[0] = fw[1] = fw[2] = 0.f;
	float n[3];
	face_forward(s, wo, n);
	if(dot3(wi, n) <= 0.f) return;
	const float cos_ng_wo = dot3(s.ng, wo), cos_ng_wi = dot3(s.ng, wi);
	if(s.m->type == GBRT_MAT_SHINYDIFFUSE)
	{
		// guided only when the diffuse layer is the sole component (shiny_guidable)
		if(!(xm(cos_ng_wo, cos_ng_wi) > 0.f)) return;
		const float pdf = fabsf(dot3(wi, n));
		const float w = __fdiv_rn(fabsf(dot3(wi, s.n)), xa(xm(pdf, 0.99f), 0.01f));
		for(int k = 0; k < 3; ++k) fw[k] = xm(s.m->sdc[3] * s.dcol[k], w);
		return;
	}
	if(s.m->type != GBRT_MAT_GLOSSY || xm(cos_ng_wo, cos_ng_wi) < 0.f) return;
	const DevMaterial &m = *s.m;
	const float pd = m.p_diffuse;
	const bool use_glossy = m.as_diffuse ? (flags & BF_DIFFUSE) != 0u : (flags & BF_GLOSSY) != 0u;
	const bool use_diffuse = m.with_diffuse && (flags & BF_DIFFUSE);
	const float wi_n = fabsf(dot3(wi, n)), wo_n = fabsf(dot3(wo, n));
	float h[3] = {xa(wi[0], wo[0]), xa(wi[1], wo[1]), xa(wi[2], wo[2])};
	normalize3(h);
	const float cos_wo_h = dot3(wo, h), cos_wi_h = fabsf(dot3(wi, h)), cos_n_h = dot3(n, h);
	float pdf = use_diffuse ? wi_n : 0.f, glossy = 0.f;
	if(use_glossy)
	{
		const float bp = blinn_pdf(cos_n_h, cos_wo_h, m.exponent);
		pdf = use_diffuse ? xa(xm(pdf, pd), xm(bp, xs(1.f, pd))) : bp;
		glossy = __fdiv_rn(xm(blinn_d(cos_n_h, m.exponent), schlick(cos_wi_h, m.m_glossy)), as_divisor(cos_wi_h, wo_n, wi_n));
	}
	const float dr = use_diffuse ? diffuse_reflect_factor(wi_n, wo_n, m.m_glossy, m.m_diffuse) : 0.f;
	const float w = __fdiv_rn(wi_n, xa(xm(pdf, 0.99f), 0.01f));
	for(int k = 0; k < 3; ++k) fw[k] = xm(xa(xm(glossy, m.col[k]), xm(dr, m.col2[k])), w);
}

// Solid-angle density of the directions Material::sample draws: cosine
// hemisphere (1/pi normalised) and, for glossy, the Blinn half-vector
// density (e+1)/(2 pi) cos^e / (4 |wo.h|), mixed by the diffuse pick
// probability.
__device__ __forceinline__ float bsdf_true_pdf(const Surface &s, const float wo[3], const float wi[3], uint32_t flags)
{
	float n[3];
	face_forward(s, wo, n);
	const float c = dot3(wi, n);
	if(c <= 0.f) return 0.f;
	if(s.m->type == GBRT_MAT_SHINYDIFFUSE) return c * kInvPi;
	if(s.m->type != GBRT_MAT_GLOSSY) return 0.f;
	const DevMaterial &m = *s.m;
	const bool use_glossy = m.as_diffuse ? (flags & BF_DIFFUSE) != 0u : (flags & BF_GLOSSY) != 0u;
	const bool use_diffuse = m.with_diffuse && (flags & BF_DIFFUSE);
	const float pd = use_diffuse ? (use_glossy ? m.p_diffuse : 1.f) : 0.f;
	float pg = 0.f;
	if(use_glossy)
	{
		float h[3] = {wi[0] + wo[0], wi[1] + wo[1], wi[2] + wo[2]};
		normalize3(h);
		const float ch = dot3(h, n), woh = dot3(wo, h);
		if(ch > 0.f && woh > 0.f) pg = (m.exponent + 1.f) * (0.5f * kInvPi) * powf(ch, m.exponent) / (4.f * woh);
	}
	return pd * c * kInvPi + (1.f - pd) * pg;
}

// LightMaterial::emit (material_light.cc:82-87); ShinyDiffuseMaterial::emit
// (material_shiny_diffuse.cc:342-347): emit x colour, both sides.
__device__ __forceinline__ bool mat_emit(const Surface &s, const float wo[3], float out[3])
{
	if(s.m->type == GBRT_MAT_SHINYDIFFUSE)
	{
		if(!(s.m->flags & BF_EMIT)) return false;
		for(int k = 0; k < 3; ++k) out[k] = s.m->dtex < 0 ? s.m->ecol[k] : s.dcol[k] * s.m->emit;
		return true;
	}
	if(s.m->type != GBRT_MAT_LIGHT) return false;
	if(dot3(wo, s.n) <= 0.f && !s.m->double_sided) return false;
	for(int k = 0; k < 3; ++k) out[k] = s.m->col[k];
	return true;
}


__device__ __forceinline__ void path_sum_add(const Work &W, uint32_t path, float r, float g, float b)
{
	float *p = reinterpret_cast<float *>(W.p_sum + path);
	atomicAdd(p, r); atomicAdd(p + 1, g); atomicAdd(p + 2, b);
}

__device__ __forceinline__ void film_add(float *film, double *film64, uint32_t pixel, float r, float g, float b)
{
	if(film64)
	{
		atomicAdd(film64 + 3ull * pixel, static_cast<double>(r));
		atomicAdd(film64 + 3ull * pixel + 1, static_cast<double>(g));
		atomicAdd(film64 + 3ull * pixel + 2, static_cast<double>(b));
	}
	else
	{
		atomicAdd(film + 3ull * pixel, r);
		atomicAdd(film + 3ull * pixel + 1, g);
		atomicAdd(film + 3ull * pixel + 2, b);
	}
}

// Writes a lane's reserved run of shadow-queue slots; unused slots are
// marked dead so the shadow kernel skips them.
struct ShadowWriter {
	float4 *ray;
	float4 *col;
	uint32_t *pix;
	uint32_t *pth;
	uint32_t path;
	uint32_t slot, end;
	__device__ void put(const float o[3], float tmin, const float d[3], float tmax, uint32_t pixel, const float c[3])
	{
		if(slot >= end) return;
		ray[2ull * slot] = make_float4(o[0], o[1], o[2], tmin);
		ray[2ull * slot + 1] = make_float4(d[0], d[1], d[2], tmax);
		col[slot] = make_float4(c[0], c[1], c[2], 0.f);
		pix[slot] = pixel;
		pth[slot] = path;
		++slot;
	}
	__device__ void close()
	{
		for(; slot < end; ++slot) pix[slot] = kDead;
	}
};

// MonteCarloIntegrator::doLightEstimation for an area light
// (integrator_montecarlo.cc:417-440): num_samples light samples
// (areaLightSampleLight, :192-330) and num_samples BSDF samples that hit the
// light (areaLightSampleMaterial, :332-415), power-heuristic MIS, Halton
// bases 2/3 from offs = num_samples * sample + pixel offset + loffs * 4567.
__device__ __forceinline__ int light_samples(const DevLight &L, uint32_t division, float lmult)
{
	if(L.type == GBRT_LIGHT_POINT) return 1;
	// integrator_montecarlo.cc:428-429
	const int n = static_cast<int>(ceilf(static_cast<float>(L.samples) * lmult));
	return division > 1 ? max(1, n / static_cast<int>(division)) : n;
}

// Shadow rays one light estimation writes: 2 per area-light sample, 1 for a point light.
__device__ __forceinline__ uint32_t light_shadow_rays(const DevLight &L, uint32_t division, float lmult)
{
	return L.type == GBRT_LIGHT_POINT ? 1u : 2u * static_cast<uint32_t>(light_samples(L, division, lmult));
}

template <bool kLean = false>
__device__ void light_estimation(const SceneDev &sc, const Surface &s, const float wo[3], uint32_t li, uint32_t loffs,
                                 uint32_t sample_, uint32_t offset_, const float weight[3], uint32_t pixel, ShadowWriter &sw,
                                 uint32_t division, float lmult)
{
	const DevLight &L = sc.lights[li];
	if(L.type == GBRT_LIGHT_POINT)
	{
		// MonteCarloIntegrator::diracLight (integrator_montecarlo.cc:117-190) with
		// PointLight::illuminate (light_point.cc:71-82)
		float ldir[3];
		for(int k = 0; k < 3; ++k) ldir[k] = L.c[k] - s.p[k];
		const float dist_sqr = ldir[0] * ldir[0] + ldir[1] * ldir[1] + ldir[2] * ldir[2];
		const float dist = sqrtf(dist_sqr);
		if(dist == 0.f) return;
		const float idist_sqr = 1.f / dist_sqr, inv = 1.f / dist;
		for(int k = 0; k < 3; ++k) ldir[k] *= inv;
		const float sbias = kShadowBias * fmaxf(1.f, sqrtf(dot3(s.p, s.p)));
		float surf[3];
		mat_eval_l<kLean>(s, wo, ldir, surf);
		const float angle = fabsf(dot3(s.n, ldir));
		float c[3];
		for(int k = 0; k < 3; ++k) c[k] = surf[k] * (L.col[k] * idist_sqr) * angle * weight[k];
		if(c[0] != 0.f || c[1] != 0.f || c[2] != 0.f) sw.put(s.p, sbias, ldir, dist, pixel, c);
		return;
	}
	const int ns = light_samples(L, division, lmult);
	const float inv_ns = __fdiv_rn(1.f, static_cast<float>(ns));
	const uint32_t offs = static_cast<uint32_t>(ns) * sample_ + offset_ + loffs * 4567u;
	const float plen = sqrtf(dot3(s.p, s.p));
	const float sbias = xm(kShadowBias, fmaxf(1.f, plen));
	const float rbias = xm(kRayMinDist, fmaxf(1.f, plen));
	for(int i = 0; i < ns; ++i)
	{
		const float s1 = gbrt::radical_inverse(offs + static_cast<uint32_t>(i), 2);
		const float s2 = gbrt::radical_inverse3_f(sc.lds, offs + static_cast<uint32_t>(i));
		// light sample (AreaLight::illumSample, light_area.cc:99-124)
		{
			float lp[3], ldir[3];
			for(int k = 0; k < 3; ++k) lp[k] = xa(xa(L.c[k], xm(s1, L.tx[k])), xm(s2, L.ty[k]));
			for(int k = 0; k < 3; ++k) ldir[k] = xs(lp[k], s.p[k]);
			const float dist_sqr = dot3(ldir, ldir);
			const float dist = sqrtf(dist_sqr);
			if(dist > 0.f)
			{
				const float invd = __fdiv_rn(1.f, dist);
				for(int k = 0; k < 3; ++k) ldir[k] = xm(ldir[k], invd);
				const float cos_angle = dot3(ldir, L.nflip);
				if(cos_angle > 0.f)
				{
					const float pdf = __fdiv_rn(xm(dist_sqr, kPi), xm(1.f, cos_angle));
					if(pdf > 1e-6f)
					{
						float surf[3];
						mat_eval_l<kLean>(s, wo, ldir, surf);
						const float angle = fabsf(dot3(s.n, ldir));
						float w = 1.f;
						const float m_pdf = mat_pdf_l<kLean>(s, wo, ldir);
						if(m_pdf > 1e-6f)
						{
							const float l2 = xm(pdf, pdf), m2 = xm(m_pdf, m_pdf);
							w = __fdiv_rn(l2, xa(l2, m2));
						}
						float c[3];
						for(int k = 0; k < 3; ++k)
							c[k] = xm(xm(__fdiv_rn(xm(xm(xm(surf[k], L.col[k]), angle), w), pdf), inv_ns), weight[k]);
						if(c[0] != 0.f || c[1] != 0.f || c[2] != 0.f) sw.put(s.p, sbias, ldir, dist, pixel, c);
					}
				}
			}
		}
		// BSDF sample towards the light (Material::sample + AreaLight::intersect, light_area.cc:146-155)
		{
			float wi[3], scol[3], W, spdf;
			uint32_t sflags;
			mat_sample_l<kLean>(s, wo, s1, s2, BF_GLOSSY | BF_DIFFUSE | BF_DISPERSIVE | BF_REFLECT | BF_TRANSMIT, wi, scol, W, spdf, sflags);
			const float cos_angle = dot3(wi, L.nflip);
			if(cos_angle > 0.f && spdf > 1e-6f)
			{
				const float4 A = make_float4(L.c[0], L.c[1], L.c[2], L.e3[0]);
				const float4 B = make_float4(L.e1[0], L.e1[1], L.e1[2], L.e3[1]);
				const float4 C = make_float4(L.e2[0], L.e2[1], L.e2[2], L.e3[2]);
				float u, v;
				const float t = gbrt::mt_intersect(A, B, C, true, s.p, wi, u, v);
				if(t > 0.f)
				{
					const float ipdf = xm(xm(xm(__fdiv_rn(1.f, xm(t, t)), 1.f), cos_angle), kInvPi);
					if(ipdf > 1e-6f)
					{
						const float l_pdf = __fdiv_rn(1.f, ipdf);
						const float l2 = xm(l_pdf, l_pdf), m2 = xm(spdf, spdf);
						const float w = __fdiv_rn(m2, xa(l2, m2));
						float c[3];
						for(int k = 0; k < 3; ++k) c[k] = xm(xm(xm(xm(xm(scol[k], L.col[k]), w), W), inv_ns), weight[k]);
						if(c[0] != 0.f || c[1] != 0.f || c[2] != 0.f) sw.put(s.p, rbias, wi, t, pixel, c);
					}
				}
			}
		}
	}
}


// Writes a lane's reserved run of spawn slots (recursive split of
// MonteCarloIntegrator::recursiveRaytrace); unused slots are marked dead.
struct SpawnWriter {
	float4 *out;
	uint32_t slot, end, cap;
	uint32_t scene;               // the caller's entry of a batch's scene table (0 for one scene)
	__device__ void put(const float o[3], const float d[3], const float wt[3], uint32_t pixel, uint32_t si, uint32_t tx, uint32_t branch,
	                    float d1, float d2)
	{
		if(slot >= end) return;
		if(slot < cap)
		{
			float4 *r = out + 5ull * slot;
			r[0] = make_float4(o[0], o[1], o[2], kRayMinDist);
			r[1] = make_float4(d[0], d[1], d[2], -1.f);
			r[2] = make_float4(wt[0], wt[1], wt[2], 0.f);
			r[3] = make_float4(__uint_as_float(pixel), __uint_as_float(si), __uint_as_float(tx), __uint_as_float(branch));
			r[4] = make_float4(d1, d2, __uint_as_float(scene), 0.f);
		}
		++slot;
	}
	__device__ void close()
	{
		for(; slot < end; ++slot)
			if(slot < cap) reinterpret_cast<uint32_t *>(out + 5ull * slot + 3)[0] = kDead;
	}
};

// Upper bound of the integrate() calls recursiveRaytrace starts at a hit
// (each call as max(1, path_samples / division) paths).
__device__ __forceinline__ uint32_t spawn_bound(uint32_t flags, bool glossy, bool spec, uint32_t division, uint32_t ps)
{
	uint32_t n = 0;
	if(glossy)
	{
		const uint32_t rs = division > 1 ? max(1u, 8u / division) : 8u;
		n += rs * ((flags & BF_TRANSMIT) ? 2u : 1u) * max(1u, ps / (division * rs));
	}
	if(spec) n += 2u * max(1u, ps / division);
	return n;
}

// MonteCarloIntegrator::recursiveRaytrace at ray level nl
// (integrator_montecarlo.cc:698-748): glossy() (:506-589) splits into
// ray_samples_glossy = 8 / division directions (Halton 2/3 from
// ray_samples * sample + pixel offset, decorrelation from Faure dims
// 2 nl + 1, 2 nl + 2 at branch + pixel offset), each integrate() weighted by
// colour x w / ray_samples; getSpecular's reflection and refraction keep the
// parent's division.
__device__ void spawn_children(const SceneDev &sc, const Params &P, const Surface &s, const float wo[3], const float thr[3],
                               uint32_t pixel, uint32_t si, uint32_t sample_, uint32_t offset_, uint32_t nl, uint32_t addl,
                               uint32_t division, uint32_t branch, float deco1, float deco2, bool do_glossy, bool do_spec, SpawnWriter &sw)
{
	const uint32_t ps = static_cast<uint32_t>(P.path_samples);
	const uint32_t si0 = si - si % ps;
	auto emit = [&](const float d[3], const float wt[3], uint32_t div, uint32_t br, float d1, float d2) {
		if(wt[0] == 0.f && wt[1] == 0.f && wt[2] == 0.f) return;     // contributes nothing
		const uint32_t nsub = max(1u, ps / div);
		const uint32_t tx = nl | (addl << 8) | (div << 16);
		for(uint32_t j = 0; j < nsub; ++j) sw.put(s.p, d, wt, pixel, si0 + j, tx, br, d1, d2);
	};
	if(do_glossy)
	{
		const uint32_t rs = division > 1 ? max(1u, 8u / division) : 8u;
		const uint32_t ndiv = division * rs, branch0 = ndiv * branch, offs = rs * sample_ + offset_;
		const float inv_rs = 1.f / static_cast<float>(rs);
		for(uint32_t j = 0; j < rs; ++j)
		{
			const float d1 = gbrt::low_discrepancy_f(sc.lds, 2 * static_cast<int>(nl) + 1, branch0 + j + offset_);
			const float d2 = gbrt::low_discrepancy_f(sc.lds, 2 * static_cast<int>(nl) + 2, branch0 + j + offset_);
			const float s1 = gbrt::radical_inverse(offs + 1u + j, 2), s2 = gbrt::radical_inverse3_f(sc.lds, offs + 1u + j);
			if(s.m->flags & BF_TRANSMIT)
			{
				float dir[2][3], col[2][3], w[2];
				const int nd = rough_sample2(s, wo, s1, s2, dir, col, w);
				for(int c = 0; c < nd; ++c)
				{
					float wt[3];
					for(int k = 0; k < 3; ++k) wt[k] = thr[k] * col[c][k] * w[c] * inv_rs;
					emit(dir[c], wt, ndiv, branch0 + j, d1, d2);
				}
			}
			else
			{
				float wi[3], col[3], w, pdf, wt[3];
				uint32_t sf;
				mat_sample(s, wo, s1, s2, BF_GLOSSY | BF_REFLECT, wi, col, w, pdf, sf);
				for(int k = 0; k < 3; ++k) wt[k] = thr[k] * col[k] * w * inv_rs;
				emit(wi, wt, ndiv, branch0 + j, d1, d2);
			}
		}
	}
	if(do_spec && (s.m->type == GBRT_MAT_GLASS || s.m->type == GBRT_MAT_SHINYDIFFUSE))
	{
		bool hr, hl;
		float rdir[3], rcol[3], ldir[3], lcol[3], wt[3];
		if(s.m->type == GBRT_MAT_GLASS) glass_specular(s, wo, static_cast<int>(nl), hr, rdir, rcol, hl, ldir, lcol);
		else shiny_specular(s, wo, hr, rdir, rcol, hl, ldir, lcol);
		if(hl) { for(int k = 0; k < 3; ++k) wt[k] = thr[k] * lcol[k]; emit(ldir, wt, division, branch, deco1, deco2); }
		if(hr) { for(int k = 0; k < 3; ++k) wt[k] = thr[k] * rcol[k]; emit(rdir, wt, division, branch, deco1, deco2); }
	}
}

__device__ __forceinline__ uint32_t pixel_offset(uint32_t pixel, int resx)
{
	const uint32_t x = pixel % static_cast<uint32_t>(resx), y = pixel / static_cast<uint32_t>(resx);
	return gbrt::fnv32(y * gbrt::fnv32(x));      // integrator_tiled.cc:297
}

// ImageFilm::roundToIntWithBias (imagefilm.h:344-348): + (0.5 - 1.4e-11), truncated.
__device__ __forceinline__ int round_bias(double v) { return static_cast<int>(v + (0.5 - 1.4e-11)); }

// Sub-pixel position of camera sample si (TiledIntegrator::renderTile,
// integrator_tiled.cc:316-323): pixel centre for one sample, else
// ((0.5 + s) / n, riLp(s + pixel offset)).
__device__ __forceinline__ void sample_pos(const Params &P, uint32_t pixel, uint32_t si, float &dx, float &dy)
{
	dx = 0.5f; dy = 0.5f;
	if(P.aa_multipass)
	{
		// AA_passes > 1 (integrator_tiled.cc:316-319): sample index of the pass
		const uint32_t sample_ = P.base_offset + si / static_cast<uint32_t>(P.path_samples);
		const uint32_t off = pixel_offset(pixel, P.film_resx);
		dx = gbrt::ri_vdc(sample_, off);
		dy = gbrt::ri_s(sample_, off);
	}
	else if(P.spp > 1)
	{
		const uint32_t sample = si / static_cast<uint32_t>(P.path_samples);
		dx = xm(xa(0.5f, static_cast<float>(sample)), P.d1);
		dy = gbrt::ri_lp(sample + pixel_offset(pixel, P.film_resx));
	}
}

// ImageFilm::addSample (imagefilm.cc:771-822): the filter footprint of a
// sample (the reference's asymmetric rounding included), table indices from
// |(i - (dx - 0.5)) x table scale| in double, and colour x weight into every
// covered pixel; weight_only adds the filter weights (once per camera sample).
__device__ void film_splat(const Params &P, float *film, double *film64, uint32_t pixel, uint32_t si, float r, float g, float b,
                           bool weight_only)
{
	float dx, dy;
	sample_pos(P, pixel, si, dx, dy);
	const int x = static_cast<int>(pixel % static_cast<uint32_t>(P.film_resx));
	const int y = static_cast<int>(pixel / static_cast<uint32_t>(P.film_resx));
	const double fw = P.filter_width;
	const int dx0 = max(-x, round_bias(static_cast<double>(dx) - fw));
	const int dx1 = min(P.film_resx - 1 - x, round_bias(static_cast<double>(dx) + fw - 1.0));
	const int dy0 = max(-y, round_bias(static_cast<double>(dy) - fw));
	const int dy1 = min(P.film_resy - 1 - y, round_bias(static_cast<double>(dy) + fw - 1.0));
	const double xo = static_cast<double>(dx) - 0.5, yo = static_cast<double>(dy) - 0.5;
	const double sc = P.filter_scale;
	for(int j = dy0; j <= dy1; ++j)
	{
		const int yi = min(15, static_cast<int>(floor(fabs((static_cast<double>(j) - yo) * sc))));
		for(int i = dx0; i <= dx1; ++i)
		{
			const int xi = min(15, static_cast<int>(floor(fabs((static_cast<double>(i) - xo) * sc))));
			const float w = __ldg(P.filter_tab + yi * 16 + xi);
			const uint32_t q = static_cast<uint32_t>((y + j) * P.film_resx + (x + i));
			if(weight_only) atomicAdd(P.film_w + q, w);
			else film_add(film, film64, q, r * w, g * w, b * w);
		}
	}
}

// A contribution of camera sample si to the film.
__device__ __forceinline__ void film_put(const Params &P, float *film, double *film64, uint32_t pixel, uint32_t si, float r, float g, float b)
{
	if(P.film_w) film_splat(P, film, film64, pixel, si, r, g, b, false);
	else film_add(film, film64, pixel, r, g, b);
}

// Camera sample g (an index into the render's sample-major path order) into
// path slot s: sample-major order, so a wave holds whole sample indices of
// every pixel, each wave (and each guide training batch drawn from it)
// covers the full image, and neighbouring threads shoot neighbouring
// pixels; the path samples of one camera sample are adjacent (so a wave of
// W paths holds at most W / path_samples + 2 integrate() roots).
__device__ __forceinline__ void camera_path(const Camera &cam, const Params &P, const Work &W, uint32_t s, uint32_t g)
{
	const uint32_t n_pix = P.pix_list ? P.n_list : static_cast<uint32_t>(cam.resx) * static_cast<uint32_t>(cam.resy);
	const uint32_t ps = static_cast<uint32_t>(P.path_samples);
	const uint32_t rest = g / ps, sub = g % ps;
	const uint32_t pixel = P.pix_list ? P.pix_list[rest % n_pix] : rest % n_pix, si = (rest / n_pix) * ps + sub;
	float dx, dy;
	sample_pos(P, pixel, si, dx, dy);
	const float px = xa(static_cast<float>(pixel % static_cast<uint32_t>(cam.resx)), dx);
	const float py = xa(static_cast<float>(pixel / static_cast<uint32_t>(cam.resx)), dy);
	float d[3];
	for(int k = 0; k < 3; ++k) d[k] = xa(xa(xm(cam.vright[k], px), xm(cam.vup[k], py)), cam.vto[k]);
	const float l2 = dot3(d, d);
	if(l2 != 0.f)
	{
		const float inv = __fdiv_rn(1.f, sqrtf(l2));
		for(int k = 0; k < 3; ++k) d[k] = xm(d[k], inv);
	}
	W.p_pixel[s] = pixel;
	W.p_si[s] = si;
	W.p_thr[s] = make_float4(1.f, 1.f, 1.f, 0.f);
	W.p_state[s] = 0u;
	W.p_task[s] = make_uint4(1u << 16, 0u, 0u, 0u);       // ray level 0, division 1
	if(W.p_sum)
	{
		W.p_sum[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		for(uint32_t k = 0; k < P.rec_stride; ++k) W.r_valid[static_cast<size_t>(s) * P.rec_stride + k] = 0u;
	}
	W.q_ray[0][2ull * s] = make_float4(cam.from[0], cam.from[1], cam.from[2], 0.f);
	W.q_ray[0][2ull * s + 1] = make_float4(d[0], d[1], d[2], -1.f);
	W.q_path[0][s] = s;
	if(P.film_w && sub == 0) film_splat(P, nullptr, nullptr, pixel, si, 0.f, 0.f, 0.f, true);
}

__global__ void __launch_bounds__(kThreads) k_camera(Camera cam, Params P, Work W)
{
	for(uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < P.wave_n; s += gridDim.x * blockDim.x)
		camera_path(cam, P, W, s, P.wave_start + s);
	if(blockIdx.x == 0 && threadIdx.x == 0)
	{
		W.count[0] = P.wave_n;
		atomicAdd(W.stats, static_cast<unsigned long long>(P.wave_n));
	}
}

__global__ void __launch_bounds__(kThreads) k_extend(gbrt::BvhView bv, const float4 *__restrict__ rays, const uint32_t *__restrict__ count,
                                                     uint32_t *counter, float4 *__restrict__ hits, float *__restrict__ hitpos)
{
	__shared__ uint2 stack[gbrt::kStackShared * kThreads];
	gbrt::trace_persistent<false>(
		bv, *count, counter, stack + threadIdx.x, kThreads,
		[&](uint32_t i, float r[8]) {
			const float4 a = rays[2ull * i], b = rays[2ull * i + 1];
			r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
			return true;
		},
		[&](uint32_t i, const gbrt::Hit &h) {
			hits[i] = make_float4(__int_as_float(h.prim), h.t, h.u, h.v);
			if(hitpos)
			{
				const float4 a = rays[2ull * i], b = rays[2ull * i + 1];
				hitpos[3ull * i] = xa(a.x, xm(h.t, b.x));
				hitpos[3ull * i + 1] = xa(a.y, xm(h.t, b.y));
				hitpos[3ull * i + 2] = xa(a.z, xm(h.t, b.z));
			}
		});
}

// One batch scene as the batch kernels read it: the scene, its render
// parameters, camera and film, and its range of the batch's path indices.
struct BatchScene {
	SceneDev sc;
	Params P;
	Camera cam;
	float *film;
	uint32_t path_begin, paths;
};

// Where a queue entry's scene comes from: the launch's one scene (kernel
// parameters), or the batch's scene table indexed by the path's scene.
struct OneScene {
	SceneDev sc;
	Params P;
	float *film;
	double *film64;
	__device__ __forceinline__ uint32_t id(const Work &, uint32_t) const { return 0u; }
	__device__ __forceinline__ const SceneDev &scene(uint32_t) const { return sc; }
	__device__ __forceinline__ const Params &params(uint32_t) const { return P; }
	__device__ __forceinline__ float *film_of(uint32_t) const { return film; }
	__device__ __forceinline__ double *film64_of(uint32_t) const { return film64; }
};

struct SceneTable {
	const BatchScene *bs;
	__device__ __forceinline__ uint32_t id(const Work &W, uint32_t path) const { return W.p_scene[path]; }
	__device__ __forceinline__ const SceneDev &scene(uint32_t i) const { return bs[i].sc; }
	__device__ __forceinline__ const Params &params(uint32_t i) const { return bs[i].P; }
	__device__ __forceinline__ float *film_of(uint32_t i) const { return bs[i].film; }
	__device__ __forceinline__ double *film64_of(uint32_t) const { return nullptr; }
};

// Shading of one vertex level of the wavefront (see the kernels below).
// kLean: a pathtracing render without guiding, records or photon maps of a
// scene whose materials are all plain (mat_eval_l) and flat-shaded: the
// photonmapping, guiding, recording, recursive-split, texture and
// shading-normal code is compiled out, which roughly halves the kernel's
// registers and lets twice the warps stay resident.
// kGuide: a render with a path guide attached (guided sampling, training
// records); without it that code is compiled out.
template <typename Src, bool kLean = false, bool kTex = true, bool kGuide = false>
__device__ __forceinline__ void shade_queue(const Src &src, Work W, int cur, uint32_t shadow_cap)
{
	const uint32_t n = W.count[cur];
	const int nxt = cur ^ 1;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t lt_mask = (1u << lane) - 1u;
	for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
	{
		const uint32_t q = base + threadIdx.x;
		const bool live = q < n;
		const uint32_t path0 = live ? W.q_path[cur][q] : 0u;
		const uint32_t sid = live ? src.id(W, path0) : 0u;
		const SceneDev &sc = src.scene(sid);
		const Params &P = src.params(sid);
		float *const film = src.film_of(sid);
		double *const film64 = src.film64_of(sid);
		const int resx = P.film_resx;
		bool cont = false;
		float nray[8];
		uint32_t path = 0, n_shadow = 0;
		Surface s;
		DevMaterial mloc;           // the material with node-tree slot colours, when it has node trees
		float wo[3] = {0.f, 0.f, 0.f}, thr[3] = {0.f, 0.f, 0.f};
		uint32_t pixel = 0, sample_ = 0, offset_ = 0, sub = 0, k = 0, mat1 = 0, caustic = 0;
		uint32_t level = 0, addl = 0, division = 1, branch = 0, si = 0, tseed = P.seed;
		float deco1 = 0.f, deco2 = 0.f;
		bool hit = false;
		if(live)
		{
			path = path0;
			const float4 h = W.hits[q];
			const int32_t prim = __float_as_int(h.x);
			if(prim >= 0)
			{
				hit = true;
				const float4 ra = W.q_ray[cur][2ull * q], rb = W.q_ray[cur][2ull * q + 1];
				const float dir[3] = {rb.x, rb.y, rb.z};
				s.p[0] = xa(ra.x, xm(h.y, dir[0])); s.p[1] = xa(ra.y, xm(h.y, dir[1])); s.p[2] = xa(ra.z, xm(h.y, dir[2]));
				const float4 ng = __ldg(sc.prim_ng + prim);
				s.ng[0] = ng.x; s.ng[1] = ng.y; s.ng[2] = ng.z;
				s.m = sc.mats + __float_as_uint(ng.w);
				if constexpr(kLean)
				{
					s.n[0] = ng.x; s.n[1] = ng.y; s.n[2] = ng.z;
					s.dcol[0] = s.m->col[0]; s.dcol[1] = s.m->col[1]; s.dcol[2] = s.m->col[2];
					coords_system(s.n, s.u, s.v);
				}
				else
				{
					shading_normal(sc, prim, h.z, h.w, s.ng, s.n);
					coords_system(s.n, s.u, s.v);
					surface_color<kTex>(sc, s, prim, h.z, h.w, mloc);
				}
				wo[0] = -dir[0]; wo[1] = -dir[1]; wo[2] = -dir[2];
				pixel = W.p_pixel[path];
				si = W.p_si[path];
				const uint4 tk = W.p_task[path];
				level = tk.x & 0xffu; addl = (tk.x >> 8) & 0xffu; division = max(1u, tk.x >> 16); branch = tk.y;
				deco1 = __uint_as_float(tk.z); deco2 = __uint_as_float(tk.w);
				// random streams of a spawned integrate() call differ from its siblings'
				if(level) tseed = P.seed ^ hash32(tk.x * 0x9e3779b9u + branch * 0x85ebca6bu + 1u);
				sub = si % static_cast<uint32_t>(P.path_samples);
				sample_ = P.base_offset + si / static_cast<uint32_t>(P.path_samples);
				offset_ = pixel_offset(pixel, resx);
				const uint32_t st = W.p_state[path];
				k = st & 0xffu; mat1 = (st >> 8) & 0xffu; caustic = (st >> 16) & 1u;
				const float4 t4 = W.p_thr[path];
				thr[0] = t4.x; thr[1] = t4.y; thr[2] = t4.z;
			}
		}
		// the previous vertex's record: incident radiance along its sampled
		// direction = what the path adds from here on
		if(kGuide && hit && W.p_sum && k >= 1 && k - 1 < P.rec_stride && W.r_valid[static_cast<size_t>(path) * P.rec_stride + (k - 1)] == 2u)
		{
			const size_t slot = static_cast<size_t>(path) * P.rec_stride + (k - 1);
			W.r_pre[slot] = W.p_sum[path];
			W.r_valid[slot] = 1u;     // complete
		}
		// --- decide this vertex's work, count its shadow rays -----------------
		bool do_nee_all = false, do_nee_one = false, rr_dead = false, do_glossy = false, do_spec = false, pm_cont = false;
		float nee_weight[3] = {0.f, 0.f, 0.f};
		uint32_t nee_light = 0, n_spawn = 0;
		if(hit)
		{
			if(k == 0)
			{
				// root of an integrate() call: emission and all-light estimation
				// weighted by the call's weight (1 for camera rays)
				float e[3];
				if((s.m->flags & BF_EMIT) && sub == 0 && mat_emit(s, wo, e))
				{
					// photonmapping adds it twice (integrator_photon_mapping.cc:686-687, 713-721)
					const float em = P.pm == 1 ? 2.f : 1.f;
					film_put(P, film, film64, pixel, si, xm(thr[0], e[0]) * em, xm(thr[1], e[1]) * em, xm(thr[2], e[2]) * em);
					if(kGuide && W.p_sum) path_sum_add(W, path, xm(thr[0], e[0]), xm(thr[1], e[1]), xm(thr[2], e[2]));
				}
				do_nee_all = (s.m->flags & BF_DIFFUSE) && sub == 0;
				for(int c = 0; c < 3; ++c) nee_weight[c] = thr[c];
				if(do_nee_all)
					for(uint32_t l = 0; l < P.n_lights; ++l) n_shadow += light_shadow_rays(sc.lights[l], division, P.lmult);
				// recursiveRaytrace at ray level + 1 (integrator_path_tracer.cc:287,
				// integrator_montecarlo.cc:698-710)
				addl = max(addl, s.m->addl_depth);
				const uint32_t nl = level + 1u;
				if(!kLean && sub == 0 && W.sp_out && nl <= static_cast<uint32_t>(P.raydepth) + addl && nl < 20u)
				{
					const uint32_t f = s.m->flags;
					do_glossy = (f & BF_GLOSSY) && (f & BF_REFLECT);
					do_spec = (f & (BF_SPECULAR | BF_FILTER)) != 0u;
					n_spawn = spawn_bound(f, do_glossy, do_spec, division, static_cast<uint32_t>(P.path_samples));
				}
			}
			else if(!kLean && P.pm)
			{
				// PhotonIntegrator::finalGathering (integrator_photon_mapping.cc:547-668)
				// after its zero'th bounce: vertex k is the loop's depth k - 1
				const float4 pm4 = W.p_pm[path];
				float length = pm4.x;
				float lcol[3] = {pm4.y, pm4.z, pm4.w};
				const float tk = W.hits[q].y;
				bool fg_caustic = caustic != 0u;
				bool do_bounce;
				if(k == 1)
				{
					length = tk;
					mat1 = s.m->flags;
					fg_caustic = false;
					do_bounce = length < P.pm_gather_dist || (mat1 & BF_SPECULAR);
				}
				else
				{
					length += tk;
					fg_caustic = (fg_caustic || k == 2u) && ((W.p_state[path] >> 17) & 1u);
					do_bounce = fg_caustic || length < P.pm_gather_dist;
				}
				const bool close = length < P.pm_gather_dist;
				const int depth = static_cast<int>(k) - 1;
				float nf[3];
				face_forward(s, wo, nf);
				if(do_bounce && depth < P.pm_fg_bounces)
				{
					bool add = false;
					if(mat1 & BF_DIFFUSE)
					{
						if(close)
						{
							// estimateOneDirectLight: its value reaches the film through the
							// shadow rays and is not kept in lcol
							lcol[0] = lcol[1] = lcol[2] = 0.f;
							do_nee_one = P.n_lights > 0;
							if(do_nee_one)
							{
								const float r = rng01(pixel, sample_ * 64u + sub, k, tseed ^ 0x9e3779b9u);
								nee_light = min(static_cast<uint32_t>(r * static_cast<float>(P.n_lights)), P.n_lights - 1u);
								for(int c = 0; c < 3; ++c) nee_weight[c] = thr[c] * static_cast<float>(P.n_lights);
								n_shadow = light_shadow_rays(sc.lights[nee_light], division, P.lmult);
							}
						}
						else if(fg_caustic)
						{
							const int j = gbrt::find_nearest(P.g_radiance, s.p, nf, P.pm_lookup_r2);
							if(j >= 0) { const float4 c4 = __ldg(P.g_radiance.col + j); lcol[0] = c4.x; lcol[1] = c4.y; lcol[2] = c4.z; }
						}
						add = close || fg_caustic;
					}
					if(add)
					{
						float e[3];
						if((mat1 & BF_EMIT) && mat_emit(s, wo, e)) for(int c = 0; c < 3; ++c) lcol[c] += e[c];
						film_put(P, film, film64, pixel, si, lcol[0] * thr[0], lcol[1] * thr[1], lcol[2] * thr[2]);
					}
					// next direction: All when close, else specular only (finalGathering :625-628)
					const uint32_t offs = static_cast<uint32_t>(P.path_samples) * sample_ + offset_ + sub;
					float s1 = gbrt::low_discrepancy_f(sc.lds, 4 * depth + 3, offs);
					float s2 = gbrt::low_discrepancy_f(sc.lds, 4 * depth + 4, offs);
					if(division > 1) { s1 += deco1; if(s1 > 1.f) s1 -= 1.f; s2 += deco2; if(s2 > 1.f) s2 -= 1.f; }
					const uint32_t fl = close ? BF_ALL : (BF_SPECULAR | BF_REFLECT | BF_TRANSMIT | BF_FILTER);
					float wi[3], scol[3], w, pdf;
					uint32_t sf;
					mat_sample(s, wo, s1, s2, fl, wi, scol, w, pdf, sf);
					if(pdf > 1.0e-6f)
					{
						float nt[3];
						for(int c = 0; c < 3; ++c) nt[c] = thr[c] * (scol[c] * w);
						pm_cont = true;
						W.p_thr[path] = make_float4(nt[0], nt[1], nt[2], 0.f);
						W.p_state[path] = (k + 1u) | (mat1 << 8) | ((fg_caustic ? 1u : 0u) << 16) | (((sf & (BF_SPECULAR | BF_FILTER)) ? 1u : 0u) << 17);
						W.p_pm[path] = make_float4(length, lcol[0], lcol[1], lcol[2]);
						nray[0] = s.p[0]; nray[1] = s.p[1]; nray[2] = s.p[2]; nray[3] = kRayMinDist;
						nray[4] = wi[0]; nray[5] = wi[1]; nray[6] = wi[2]; nray[7] = -1.f;
					}
				}
				else if(mat1 & (BF_DIFFUSE | BF_GLOSSY))
				{
					// end of the gather path: radiance-map lookup (:650-664); without a
					// radiance photon the last lcol stands
					const int j = gbrt::find_nearest(P.g_radiance, s.p, nf, P.pm_lookup_r2);
					if(j >= 0) { const float4 c4 = __ldg(P.g_radiance.col + j); lcol[0] = c4.x; lcol[1] = c4.y; lcol[2] = c4.z; }
					float e[3];
					if((mat1 & BF_EMIT) && mat_emit(s, wo, e)) for(int c = 0; c < 3; ++c) lcol[c] += e[c];
					film_put(P, film, film64, pixel, si, lcol[0] * thr[0], lcol[1] * thr[1], lcol[2] * thr[2]);
				}
			}
			else
			{
				if(k == 1) mat1 = s.m->flags;
				if(k >= 2 && static_cast<int>(k) - 1 > P.rr_min)   // integrator_path_tracer.cc:267-273
				{
					const float r = rng01(pixel, sample_ * 64u + sub, k, tseed);
					const float prob = fmaxf(thr[0], fmaxf(thr[1], thr[2]));
					if(prob <= 0.f || prob < r) rr_dead = true;
					else { const float ip = __fdiv_rn(1.f, prob); for(int c = 0; c < 3; ++c) thr[c] = xm(thr[c], ip); }
				}
				if(!rr_dead)
				{
					do_nee_one = P.n_lights > 0 && (k == 1 || (mat1 & BF_DIFFUSE));
					if(do_nee_one)
					{
						const float r = rng01(pixel, sample_ * 64u + sub, k, tseed ^ 0x9e3779b9u);
						nee_light = min(static_cast<uint32_t>(r * static_cast<float>(P.n_lights)), P.n_lights - 1u);
						for(int c = 0; c < 3; ++c) nee_weight[c] = xm(thr[c], static_cast<float>(P.n_lights));
						n_shadow = light_shadow_rays(sc.lights[nee_light], division, P.lmult);
					}
					float e[3];
					if((k == 1 && (s.m->flags & BF_EMIT)) || (k >= 2 && (mat1 & BF_EMIT) && caustic))
						if(mat_emit(s, wo, e))
						{
							film_put(P, film, film64, pixel, si, xm(thr[0], e[0]), xm(thr[1], e[1]), xm(thr[2], e[2]));
							if(kGuide && W.p_sum) path_sum_add(W, path, xm(thr[0], e[0]), xm(thr[1], e[1]), xm(thr[2], e[2]));
						}
				}
			}
		}
		// --- reserve shadow-queue slots for the warp (prefix sum of counts) ---
		uint32_t incl = n_shadow;
		for(int off = 1; off < 32; off <<= 1)
		{
			const uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
			if(lane >= static_cast<uint32_t>(off)) incl += v;
		}
		const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
		uint32_t wbase = 0;
		if(lane == 31 && total) wbase = atomicAdd(W.count + 2, total);
		wbase = __shfl_sync(0xffffffffu, wbase, 31);
		ShadowWriter sw{W.s_ray, W.s_col, W.s_pix, W.s_path, path, wbase + incl - n_shadow, wbase + incl};
		if(sw.end > shadow_cap) sw.end = sw.slot > shadow_cap ? sw.slot : shadow_cap;
		if(do_nee_all)
			for(uint32_t l = 0; l < P.n_lights; ++l)
				light_estimation<kLean>(sc, s, wo, l, l, sample_, offset_, nee_weight, pixel, sw, division, P.lmult);
		if(do_nee_one) light_estimation<kLean>(sc, s, wo, nee_light, nee_light, sample_, offset_, nee_weight, pixel, sw, division, P.lmult);
		sw.close();
		// --- spawned integrate() calls of the recursive split ----------------
		if(!kLean && W.sp_out && __any_sync(0xffffffffu, n_spawn != 0u))
		{
			uint32_t sincl = n_spawn;
			for(int off = 1; off < 32; off <<= 1)
			{
				const uint32_t v = __shfl_up_sync(0xffffffffu, sincl, off);
				if(lane >= static_cast<uint32_t>(off)) sincl += v;
			}
			const uint32_t stotal = __shfl_sync(0xffffffffu, sincl, 31);
			uint32_t sbase = 0;
			if(lane == 31) sbase = atomicAdd(W.sp_count, stotal);
			sbase = __shfl_sync(0xffffffffu, sbase, 31);
			SpawnWriter spw{W.sp_out, sbase + sincl - n_spawn, sbase + sincl, W.sp_cap, sid};
			if(n_spawn)
				spawn_children(sc, P, s, wo, thr, pixel, si, sample_, offset_, level + 1u, addl, division, branch, deco1, deco2,
				               do_glossy, do_spec, spw);
			spw.close();
		}
		// --- continuation ray ----------------------------------------------
		// (photonmapping: only the zero'th final-gather bounce comes here)
		if(hit && !rr_dead && !(!kLean && P.pm && k >= 1))
		{
			float s1 = -1.f, s2 = 0.f;
			uint32_t req = BF_ALL;
			if(k == 0)
			{
				// path_flags = Diffuse, or All with no_recursive (integrator_path_tracer.cc:177-200)
				const uint32_t path_flags = (P.no_recursive && !P.pm) ? BF_ALL : BF_DIFFUSE;
				if((s.m->flags & path_flags) && (!P.pm || P.pm_fg))
				{
					const uint32_t offs = static_cast<uint32_t>(P.path_samples) * sample_ + offset_ + sub;
					s1 = gbrt::ri_vdc(offs);
					s2 = gbrt::low_discrepancy_f(sc.lds, 2, offs);
					if(division > 1)   // math::addMod1 with the split's decorrelation
					{
						s1 += deco1; if(s1 > 1.f) s1 -= 1.f;
						s2 += deco2; if(s2 > 1.f) s2 -= 1.f;
					}
					req = path_flags | BF_DIFFUSE | BF_REFLECT | BF_TRANSMIT;
				}
			}
			else if(static_cast<int>(k) < P.bounces)
			{
				const uint32_t offs = static_cast<uint32_t>(P.path_samples) * sample_ + offset_ + sub;
				const int d4 = 4 * static_cast<int>(k);
				if(d4 + 4 < gbrt::kLdsDims)
				{
					s1 = gbrt::low_discrepancy_f(sc.lds, d4 + 3, offs);
					s2 = gbrt::low_discrepancy_f(sc.lds, d4 + 4, offs);
				}
				else
				{
					s1 = rng01(pixel, sample_ * 64u + sub, 1000u + k, tseed);
					s2 = rng01(pixel, sample_ * 64u + sub, 2000u + k, tseed);
				}
			}
			if(s1 >= 0.f)
			{
				float wi[3], scol[3], w, pdf;
				uint32_t sflags;
				float mult[3], mpdf = 0.f, hf = 0.f;
				const bool guidable = (s.m->type == GBRT_MAT_SHINYDIFFUSE && s.m->sd == SD_DIFFUSE) || s.m->type == GBRT_MAT_GLOSSY;
				if(kGuide && P.guiding && guidable)
				{
					// one-sample MIS of the guide mixture q and the BSDF sampler
					// (true density p): weight = h(w) / (alpha q(w) + (1 - alpha) p(w)),
					// h(w) = (sample colour x weight)(w) * p(w), the integrand the
					// plain estimator targets, so guided and plain converge alike.
					const float *lob = W.lobes + static_cast<size_t>(gbrt::kGuideOut) * q;
					const uint32_t key = sample_ * 64u + sub;
					const float u = rng01(pixel, key, k, tseed ^ 0x51ed270bu);
					float fw[3], ptrue;
					if(u < P.alpha)
					{
						gbrt::mixture_sample(lob, rng01(pixel, key, k, tseed ^ 0x2545f491u), rng01(pixel, key, k, tseed ^ 0x6c8e9cf5u),
						                     rng01(pixel, key, k, tseed ^ 0x1b873593u), wi);
						bsdf_eval_at(s, wo, wi, req, fw);
						ptrue = bsdf_true_pdf(s, wo, wi, req);
						sflags = BF_DIFFUSE | BF_REFLECT;
					}
					else
					{
						// the BSDF technique drawn exactly, so its density is ptrue
						mat_sample<true>(s, wo, s1, s2, req, wi, scol, w, pdf, sflags);
						normalize3(wi);
						for(int c = 0; c < 3; ++c) fw[c] = xm(scol[c], w);
						ptrue = bsdf_true_pdf(s, wo, wi, req);
					}
					const float qp = gbrt::mixture_pdf(lob, wi);
					mpdf = P.alpha * qp + (1.f - P.alpha) * ptrue;
					const float f = mpdf > 0.f ? ptrue / mpdf : 0.f;
					for(int c = 0; c < 3; ++c) mult[c] = fw[c] * f;
					hf = (0.2126f * fw[0] + 0.7152f * fw[1] + 0.0722f * fw[2]) * ptrue;
				}
				else
				{
					mat_sample_l<kLean>(s, wo, s1, s2, req, wi, scol, w, pdf, sflags);
					for(int c = 0; c < 3; ++c) mult[c] = xm(scol[c], w);
					if(kGuide && P.record && guidable)
					{
						mpdf = bsdf_true_pdf(s, wo, wi, req);
						hf = (0.2126f * mult[0] + 0.7152f * mult[1] + 0.0722f * mult[2]) * mpdf;
					}
				}
				float nt[3];
				for(int c = 0; c < 3; ++c) nt[c] = xm(thr[c], mult[c]);
				if(k == 0)
				{
					// path_col / n_samples, n_samples = max(1, path_samples / division)
					const int n_samples = max(1, P.path_samples / static_cast<int>(division));
					const float inv_ps = __fdiv_rn(1.f, static_cast<float>(n_samples));
					for(int c = 0; c < 3; ++c) nt[c] = xm(nt[c], inv_ps);
				}
				if(nt[0] != 0.f || nt[1] != 0.f || nt[2] != 0.f)
				{
					cont = true;
					if(kGuide && P.record && mpdf > 0.f && k < P.rec_stride)
					{
						const size_t slot = static_cast<size_t>(path) * P.rec_stride + k;
						W.r_pos[slot] = make_float4(s.p[0], s.p[1], s.p[2], mpdf);
						W.r_dir[slot] = make_float4(wi[0], wi[1], wi[2], hf);
						W.r_thr[slot] = make_float4(nt[0], nt[1], nt[2], 0.f);
						W.r_valid[slot] = 2u;     // waiting for the next vertex
					}
					caustic = (P.pt_caustic_path && (sflags & (BF_SPECULAR | BF_GLOSSY | BF_FILTER))) ? 1u : 0u;
					if(!kLean && P.pm) { caustic = 0u; W.p_pm[path] = make_float4(0.f, 0.f, 0.f, 0.f); }
					W.p_thr[path] = make_float4(nt[0], nt[1], nt[2], 0.f);
					W.p_state[path] = (k + 1u) | (mat1 << 8) | (caustic << 16);
					nray[0] = s.p[0]; nray[1] = s.p[1]; nray[2] = s.p[2]; nray[3] = kRayMinDist;
					nray[4] = wi[0]; nray[5] = wi[1]; nray[6] = wi[2]; nray[7] = -1.f;
				}
			}
		}
		cont = cont || pm_cont;
		const uint32_t ballot = __ballot_sync(0xffffffffu, cont);
		if(ballot)
		{
			uint32_t qbase = 0;
			const uint32_t leader = __ffs(ballot) - 1u;
			if(lane == leader) qbase = atomicAdd(W.count + nxt, static_cast<uint32_t>(__popc(ballot)));
			qbase = __shfl_sync(0xffffffffu, qbase, leader);
			if(cont)
			{
				const uint32_t slot = qbase + __popc(ballot & lt_mask);
				W.q_ray[nxt][2ull * slot] = make_float4(nray[0], nray[1], nray[2], nray[3]);
				W.q_ray[nxt][2ull * slot + 1] = make_float4(nray[4], nray[5], nray[6], nray[7]);
				W.q_path[nxt][slot] = path;
			}
			if(lane == leader) atomicAdd(W.stats, static_cast<unsigned long long>(__popc(ballot)));
		}
	}
}

template <bool kTex, bool kGuide>
__global__ void __launch_bounds__(kThreads, 4) k_shade(SceneDev sc, Params P, Work W, int cur, uint32_t shadow_cap, float *film,
                                                    double *film64)
{
	shade_queue<OneScene, false, kTex, kGuide>(OneScene{sc, P, film, film64}, W, cur, shadow_cap);
}

// The same for plain scenes (shade_queue kLean).
__global__ void __launch_bounds__(kThreads, 6) k_shade_plain(SceneDev sc, Params P, Work W, int cur, uint32_t shadow_cap, float *film,
                                                          double *film64)
{
	shade_queue<OneScene, true>(OneScene{sc, P, film, film64}, W, cur, shadow_cap);
}

// The same for a batch of scenes: every path's scene from the table.
template <bool kTex>
__global__ void __launch_bounds__(kThreads, 4) k_shade_batch(const BatchScene *__restrict__ bs, Work W, int cur, uint32_t shadow_cap)
{
	shade_queue<SceneTable, false, kTex>(SceneTable{bs}, W, cur, shadow_cap);
}

// Material::getTransparency of a shadow-ray hit, wo = the shadow ray's
// direction, n = the shading normal face-forwarded by the geometric one
// (SurfacePoint::normalFaceForward): ShinyDiffuseMaterial (material_shiny_diffuse.cc:541-563:
// accum = 1 - kr x specular_reflect with a mirror layer, then
// accum *= transparency x accum, times the transmit colour) and Glass /
// RoughGlass (material_glass.cc:297-303, material_rough_glass.cc:349-355:
// kt x filter colour).
__device__ __forceinline__ void mat_transparency(const DevMaterial &m, const float ng[3], const float ns[3], const float wo[3], const float *dcol,
                                                 float out[3])
{
	const bool flip = dot3(ng, wo) < 0.f;
	const float n[3] = {flip ? -ns[0] : ns[0], flip ? -ns[1] : ns[1], flip ? -ns[2] : ns[2]};
	if(m.type == GBRT_MAT_SHINYDIFFUSE)
	{
		const float kr = shiny_kr(m, wo, n);
		float accum = 1.f;
		if(m.sd & SD_MIRROR) accum = 1.f - kr * m.sdc[0];
		accum *= m.sdc[1] * accum;
		for(int k = 0; k < 3; ++k) out[k] = accum * (m.dtex < 0 ? m.tcol[k] : m.tf * dcol[k] + (1.f - m.tf));
	}
	else
	{
		float kr, kt;
		vec_fresnel(wo, n, m.ior, kr, kt);
		for(int k = 0; k < 3; ++k) out[k] = kt * m.col[k];
	}
}

// A transparent surface's filter colour with what varies over it: a
// textured diffuse colour, node-tree slot colours, a shading normal (out of
// line: the shadow walk keeps its registers for the traversal).
__device__ __noinline__ void shaded_transparency(const SceneDev &sc, const DevMaterial &m, int32_t prim, const float *from, const float *dir,
                                                 float t, float u, float v, const float ng[3], float tr[3])
{
	// the hit point as Accelerator::primitiveIntersectionTransparentShadow forms it (from + t dir)
	const float p[3] = {xa(from[0], xm(t, dir[0])), xa(from[1], xm(t, dir[1])), xa(from[2], xm(t, dir[2]))};
	float dcol[3] = {0.f, 0.f, 0.f};
	if(m.dtex >= 0)
	{
		float uv[2];
		hit_uv(sc, prim, u, v, uv);
		tex_color(sc, sc.tex[m.dtex], p, ng, uv, dcol);
	}
	float ns[3];
	shading_normal(sc, prim, u, v, ng, ns);
	if(m.has_nodes)
	{
		// the slot colours (diffuse, filter) and the bumped normal of this point
		Surface s;
		for(int k = 0; k < 3; ++k) { s.p[k] = p[k]; s.ng[k] = ng[k]; s.dcol[k] = dcol[k]; s.n[k] = ns[k]; }
		coords_system(s.n, s.u, s.v);
		s.m = &m;
		DevMaterial ml;
		surface_nodes(sc, s, prim, u, v, ml);
		mat_transparency(ml, ng, s.n, dir, s.dcol, tr);
	}
	else mat_transparency(m, ng, ns, dir, dcol, tr);
}

// Accelerator::primitiveIntersectionTransparentShadow (accelerator.h:147-169):
// an opaque material blocks; a transparent one multiplies the shadow colour
// by its transparency, until more than shadowDepth transparent surfaces lie
// on the ray (then it blocks too).
template <bool kTex>
struct TransparentHits {
	static constexpr bool kTransparent = true;
	const SceneDev *sc;          // textures of a textured diffuse colour
	const DevMaterial *mats;
	const float4 *prim_ng;
	int max_depth;
	int depth;
	float col[3];
	__device__ __forceinline__ void reset() { depth = 0; col[0] = col[1] = col[2] = 1.f; }
	__device__ __forceinline__ bool blocks(int32_t prim, const float *from, const float *dir, float t, float u, float v)
	{
		const float4 g = __ldg(prim_ng + prim);
		const DevMaterial &m = mats[__float_as_uint(g.w)];
		if(!m.transparent || depth >= max_depth) return true;
		const float ng[3] = {g.x, g.y, g.z};
		float tr[3];
		if(kTex && (m.dtex >= 0 || m.has_nodes)) shaded_transparency(*sc, m, prim, from, dir, t, u, v, ng, tr);
		else
		{
			const float dcol[3] = {0.f, 0.f, 0.f};
			float ns[3];
			shading_normal(*sc, prim, u, v, ng, ns);
			mat_transparency(m, ng, ns, dir, dcol, tr);
		}
		for(int k = 0; k < 3; ++k) col[k] *= tr[k];
		++depth;
		return false;
	}
};

// kFilm: the film has a filter (film_splat); the plain-sum variant keeps
// the splat's registers out of this kernel.  kTransparent: transparent
// shadows (the unoccluded colour times the filter colour of the transparent
// surfaces passed).
template <bool kFilm, bool kTransparent, bool kTex = false>
__global__ void __launch_bounds__(kThreads) k_shadow(SceneDev sc, Params P, Work W, uint32_t shadow_cap, float *film, double *film64)
{
	const gbrt::BvhView &bv = sc.bv;
	__shared__ uint2 stack[gbrt::kStackShared * kThreads];
	const uint32_t n = min(W.count[2], shadow_cap);
	uint32_t traced = 0;
	using Filter = typename std::conditional<kTransparent, TransparentHits<kTex>, gbrt::OpaqueHits>::type;
	Filter f;
	if constexpr(kTransparent)
	{
		f.sc = &sc;
		f.mats = sc.mats;
		f.prim_ng = sc.prim_ng;
		f.max_depth = P.shadow_depth;
	}
	gbrt::trace_persistent_filtered<true>(
		bv, n, W.count + 5, stack + threadIdx.x, kThreads, f,
		[&](uint32_t i, float r[8]) {
			if(W.s_pix[i] == kDead) return false;
			const float4 a = W.s_ray[2ull * i], b = W.s_ray[2ull * i + 1];
			r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
			++traced;
			return true;
		},
		[&](uint32_t i, const gbrt::Hit &h) {
			if(h.prim < 0)
			{
				float4 c = W.s_col[i];
				if constexpr(kTransparent) { c.x *= f.col[0]; c.y *= f.col[1]; c.z *= f.col[2]; }
				if(kFilm) film_splat(P, film, film64, W.s_pix[i], W.p_si[W.s_path[i]], c.x, c.y, c.z, false);
				else film_add(film, film64, W.s_pix[i], c.x, c.y, c.z);
				if(W.p_sum) path_sum_add(W, W.s_path[i], c.x, c.y, c.z);
			}
		});
	for(int off = 16; off > 0; off >>= 1) traced += __shfl_xor_sync(0xffffffffu, traced, off);
	if((threadIdx.x & 31u) == 0 && traced) atomicAdd(W.stats + 1, static_cast<unsigned long long>(traced));
}

// ---- a batch of scenes in one wavefront --------------------------------------
// The batch kernels run every scene's paths together: a wave is a range of
// the batch's path indices (the scenes' sample-major orders back to back),
// every path carries its scene's index, and each kernel reads the scene
// (hierarchy, materials, lights, parameters, film) from the table.

__global__ void __launch_bounds__(kThreads) k_camera_batch(const BatchScene *__restrict__ bs, uint32_t n_scenes, uint32_t wave_start,
                                                           uint32_t wave_n, Work W)
{
	for(uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < wave_n; s += gridDim.x * blockDim.x)
	{
		const uint32_t g = wave_start + s;
		uint32_t lo = 0, hi = n_scenes;            // the last scene whose range starts at or before g
		while(hi - lo > 1)
		{
			const uint32_t mid = (lo + hi) >> 1;
			if(bs[mid].path_begin <= g) lo = mid;
			else hi = mid;
		}
		W.p_scene[s] = lo;
		camera_path(bs[lo].cam, bs[lo].P, W, s, g - bs[lo].path_begin);
	}
	if(blockIdx.x == 0 && threadIdx.x == 0)
	{
		W.count[0] = wave_n;
		atomicAdd(W.stats, static_cast<unsigned long long>(wave_n));
	}
}

__global__ void __launch_bounds__(kThreads) k_extend_batch(const BatchScene *__restrict__ bs, Work W, int cur)
{
	__shared__ uint2 stack[gbrt::kStackShared * kThreads];
	const float4 *__restrict__ rays = W.q_ray[cur];
	gbrt::OpaqueHits f;
	gbrt::trace_persistent_filtered<false, true>(
		bs[0].sc.bv, W.count[cur], W.count + 4, stack + threadIdx.x, kThreads, f,
		[&](uint32_t i, float r[8], gbrt::BvhView &bv) {
			const float4 a = rays[2ull * i], b = rays[2ull * i + 1];
			r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
			bv = bs[W.p_scene[W.q_path[cur][i]]].sc.bv;
			return true;
		},
		[&](uint32_t i, const gbrt::Hit &h) { W.hits[i] = make_float4(__int_as_float(h.prim), h.t, h.u, h.v); });
}

template <bool kFilm, bool kTransparent, bool kTex = false>
__global__ void __launch_bounds__(kThreads) k_shadow_batch(const BatchScene *__restrict__ bs, Work W, uint32_t shadow_cap)
{
	__shared__ uint2 stack[gbrt::kStackShared * kThreads];
	const uint32_t n = min(W.count[2], shadow_cap);
	uint32_t traced = 0;
	using Filter = typename std::conditional<kTransparent, TransparentHits<kTex>, gbrt::OpaqueHits>::type;
	Filter f;
	gbrt::trace_persistent_filtered<true, true>(
		bs[0].sc.bv, n, W.count + 5, stack + threadIdx.x, kThreads, f,
		[&](uint32_t i, float r[8], gbrt::BvhView &bv) {
			if(W.s_pix[i] == kDead) return false;
			const float4 a = W.s_ray[2ull * i], b = W.s_ray[2ull * i + 1];
			r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
			const BatchScene &B = bs[W.p_scene[W.s_path[i]]];
			bv = B.sc.bv;
			if constexpr(kTransparent)
			{
				f.sc = &B.sc;
				f.mats = B.sc.mats;
				f.prim_ng = B.sc.prim_ng;
				f.max_depth = B.P.shadow_depth;
			}
			++traced;
			return true;
		},
		[&](uint32_t i, const gbrt::Hit &h) {
			if(h.prim < 0)
			{
				const uint32_t path = W.s_path[i];
				const BatchScene &B = bs[W.p_scene[path]];
				float4 c = W.s_col[i];
				if constexpr(kTransparent) { c.x *= f.col[0]; c.y *= f.col[1]; c.z *= f.col[2]; }
				if(kFilm) film_splat(B.P, B.film, nullptr, W.s_pix[i], W.p_si[path], c.x, c.y, c.z, false);
				else film_add(B.film, nullptr, W.s_pix[i], c.x, c.y, c.z);
			}
		});
	for(int off = 16; off > 0; off >>= 1) traced += __shfl_xor_sync(0xffffffffu, traced, off);
	if((threadIdx.x & 31u) == 0 && traced) atomicAdd(W.stats + 1, static_cast<unsigned long long>(traced));
}

// Records of a finished wave -> training records {pos, dir, c, 0} with
// c = luminance(incident radiance) x h / mixture pdf, where h is the BSDF x
// cosine factor of the estimator (the guide learns the product), incident
// radiance = (path total - contributions before the next vertex) /
// throughput after sampling.
__global__ void k_make_records(Work W, uint32_t n_paths, uint32_t stride, int radiance_target)
{
	const uint32_t lane = threadIdx.x & 31u;
	const size_t total = static_cast<size_t>(n_paths) * stride;
	for(size_t base = blockIdx.x * static_cast<size_t>(blockDim.x); base < total; base += static_cast<size_t>(gridDim.x) * blockDim.x)
	{
		const size_t slot = base + threadIdx.x;
		bool ok = false;
		float4 pos = make_float4(0.f, 0.f, 0.f, 0.f), dir = pos;
		float c = 0.f;
		if(slot < total && W.r_valid[slot] == 1u)
		{
			const uint32_t path = static_cast<uint32_t>(slot / stride);
			const float4 sum = W.p_sum[path], pre = W.r_pre[slot], thr = W.r_thr[slot];
			pos = W.r_pos[slot];
			dir = W.r_dir[slot];
			const float L[3] = {thr.x > 0.f ? (sum.x - pre.x) / thr.x : 0.f, thr.y > 0.f ? (sum.y - pre.y) / thr.y : 0.f,
			                    thr.z > 0.f ? (sum.z - pre.z) / thr.z : 0.f};
			// target density ~ incident radiance x (BSDF x cosine): c = L h / m
			const float lum = fmaxf(0.f, 0.2126f * L[0] + 0.7152f * L[1] + 0.0722f * L[2]);
			c = pos.w > 0.f ? lum * (radiance_target ? 1.f : fmaxf(dir.w, 0.f)) / pos.w : 0.f;
			ok = c > 0.f && isfinite(c);
			c = fminf(c, 1e4f);
		}
		const uint32_t ballot = __ballot_sync(0xffffffffu, ok);
		if(!ballot) continue;
		const uint32_t leader = __ffs(ballot) - 1u;
		uint32_t b = 0;
		if(lane == leader) b = atomicAdd(W.count + 3, static_cast<uint32_t>(__popc(ballot)));
		b = __shfl_sync(0xffffffffu, b, leader);
		if(ok)
		{
			const uint32_t i = b + __popc(ballot & ((1u << lane) - 1u));
			if(i < W.train_cap)
			{
				float4 *o = reinterpret_cast<float4 *>(W.train + 8ull * i);
				o[0] = make_float4(pos.x, pos.y, pos.z, dir.x);
				o[1] = make_float4(dir.y, dir.z, c, 0.f);
			}
		}
	}
}

// A training batch of `batch` records drawn uniformly (with replacement)
// from the n records of the wave, so a step sees the whole image.
__global__ void k_gather_batch(const float4 *__restrict__ rec, uint32_t n, uint32_t batch, uint32_t seed, float4 *__restrict__ out)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < batch; i += gridDim.x * blockDim.x)
	{
		const uint32_t j = hash32(i * 0x9e3779b9u ^ hash32(seed)) % n;
		out[2ull * i] = rec[2ull * j];
		out[2ull * i + 1] = rec[2ull * j + 1];
	}
}

// Queue counts of the next vertex level; count[4] / count[5] are the chunk
// counters of k_extend / k_shadow (gbrt::trace_persistent).
__global__ void k_reset(uint32_t *count, int which) { count[which] = 0u; count[2] = 0u; count[4] = 0u; count[5] = 0u; }

// Spawned integrate() calls -> paths of a new wave (dead records skipped,
// live ones compacted into path slots and the first ray queue).
__global__ void __launch_bounds__(kThreads) k_spawn_init(Work W, const float4 *__restrict__ rec, uint32_t n)
{
	const uint32_t lane = threadIdx.x & 31u;
	for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
	{
		const uint32_t i = base + threadIdx.x;
		float4 r3 = make_float4(0.f, 0.f, 0.f, 0.f);
		bool live = false;
		if(i < n)
		{
			r3 = rec[5ull * i + 3];
			live = __float_as_uint(r3.x) != kDead;
		}
		const uint32_t ballot = __ballot_sync(0xffffffffu, live);
		if(!ballot) continue;
		const uint32_t leader = __ffs(ballot) - 1u;
		uint32_t qbase = 0;
		if(lane == leader)
		{
			qbase = atomicAdd(W.count, static_cast<uint32_t>(__popc(ballot)));
			atomicAdd(W.stats, static_cast<unsigned long long>(__popc(ballot)));
		}
		qbase = __shfl_sync(0xffffffffu, qbase, leader);
		if(live)
		{
			const uint32_t slot = qbase + __popc(ballot & ((1u << lane) - 1u));
			const float4 r0 = rec[5ull * i], r1 = rec[5ull * i + 1], r2 = rec[5ull * i + 2], r4 = rec[5ull * i + 4];
			W.p_pixel[slot] = __float_as_uint(r3.x);
			W.p_si[slot] = __float_as_uint(r3.y);
			W.p_thr[slot] = make_float4(r2.x, r2.y, r2.z, 0.f);
			W.p_state[slot] = 0u;
			W.p_task[slot] = make_uint4(__float_as_uint(r3.z), __float_as_uint(r3.w), __float_as_uint(r4.x), __float_as_uint(r4.y));
			if(W.p_scene) W.p_scene[slot] = __float_as_uint(r4.z);
			W.q_ray[0][2ull * slot] = r0;
			W.q_ray[0][2ull * slot + 1] = r1;
			W.q_path[0][slot] = slot;
		}
	}
}

__global__ void k_mean(const float *sum, const double *sum64, float *out, size_t n, float inv)
{
	for(size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
		out[i] = sum64 ? static_cast<float>(sum64[i] * static_cast<double>(inv)) : sum[i] * inv;
}

// ---- adaptive anti-aliasing: ImageFilm::nextPass (imagefilm.cc:365-547) ----
struct AaDev {
	float threshold;
	int color_noise, dark_type;
	float dark_factor;
	int var_half, var_pixels;
};

// Combined colour of a pixel normalised by its weight: Rgba::normalized and
// operator / (color.h:294-298, 538-542) multiply by the reciprocal.  Every
// camera sample here carries alpha 1 (no transparent background), so the
// alpha sum equals the weight sum and alpha = w x (1 / w); 0 without samples.
__device__ __forceinline__ float4 aa_color(const float *film, const float *w, int i)
{
	const float wt = w[i];
	if(wt == 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
	const float r = __fdiv_rn(1.f, wt);
	return make_float4(xm(film[3 * i], r), xm(film[3 * i + 1], r), xm(film[3 * i + 2], r), xm(wt, r));
}
// Rgb::col2Bri (color.h:57), unfused like the reference's host build
__device__ __forceinline__ float aa_bri(float4 c) { return xa(xa(xm(0.2126f, c.x), xm(0.7152f, c.y)), xm(0.0722f, c.z)); }

// Rgba::colorDifference (color.h:434-452)
__device__ __forceinline__ float aa_diff(float4 a, float4 b, int color_noise)
{
	float d = fabsf(xs(aa_bri(b), aa_bri(a)));
	if(color_noise)
	{
		d = fmaxf(d, fabsf(xs(b.x, a.x))); d = fmaxf(d, fabsf(xs(b.y, a.y)));
		d = fmaxf(d, fabsf(xs(b.z, a.z))); d = fmaxf(d, fabsf(xs(b.w, a.w)));
	}
	return d;
}

// ImageFilm::darkThresholdCurveInterpolate (imagefilm.cc:882-899)
__device__ float aa_dark_curve(float b)
{
	// brightness knots and thresholds; between knots linear:
	// t0 + (b - b0) x (t1 - t0) / (b1 - b0), each operation rounded in float
	constexpr float kb[13] = {0.10f, 0.20f, 0.30f, 0.40f, 0.50f, 0.60f, 0.70f, 0.80f, 0.90f, 1.00f, 1.20f, 1.40f, 1.80f};
	constexpr float kt[13] = {0.0001f, 0.0010f, 0.0020f, 0.0035f, 0.0055f, 0.0075f, 0.0100f, 0.0150f, 0.0250f, 0.0400f, 0.0800f, 0.0950f, 0.1000f};
	constexpr float kw[13] = {0.f, 0.10f, 0.10f, 0.10f, 0.10f, 0.10f, 0.10f, 0.10f, 0.10f, 0.10f, 0.20f, 0.20f, 0.40f};
	if(b <= kb[0]) return kt[0];
	for(int k = 1; k < 13; ++k)
		if(b <= kb[k]) return xa(kt[k - 1], __fdiv_rn(xm(xs(b, kb[k - 1]), kt[k] - kt[k - 1]), kw[k]));
	return kt[12];
}

// Pixels without samples are flagged first, the rest cleared.
__global__ void k_aa_init(const float *__restrict__ w, uint32_t n, uint8_t *__restrict__ flags)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) flags[i] = w[i] > 0.f ? 0u : 1u;
}

// One thread per pixel (x < W-1, y < H-1): neighbour differences set both
// pixels' flags; the variance window flags a block around the pixel.
// Every write stores 1, so concurrent writers agree.
__global__ void k_aa_detect(const float *__restrict__ film, const float *__restrict__ w, int W, int H, AaDev a, uint8_t *flags)
{
	const uint32_t n = static_cast<uint32_t>(W - 1) * static_cast<uint32_t>(H - 1);
	for(uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
	{
		const int x = static_cast<int>(t % static_cast<uint32_t>(W - 1)), y = static_cast<int>(t / static_cast<uint32_t>(W - 1));
		const int i = y * W + x;
		const float4 c = aa_color(film, w, i);
		const float bri = aa_bri(make_float4(fabsf(c.x), fabsf(c.y), fabsf(c.z), 0.f));  // Rgb::abscol2Bri (color.h:58)
		float thr = a.threshold;
		if(a.dark_type == 1 && a.dark_factor > 0.f) thr = xm(a.threshold, xa(xs(1.f, a.dark_factor), xm(bri, a.dark_factor)));
		else if(a.dark_type == 2) thr = aa_dark_curve(bri);
		if(aa_diff(c, aa_color(film, w, i + 1), a.color_noise) >= thr) { flags[i] = 1u; flags[i + 1] = 1u; }
		if(aa_diff(c, aa_color(film, w, i + W), a.color_noise) >= thr) { flags[i] = 1u; flags[i + W] = 1u; }
		if(aa_diff(c, aa_color(film, w, i + W + 1), a.color_noise) >= thr) { flags[i] = 1u; flags[i + W + 1] = 1u; }
		if(x > 0 && aa_diff(c, aa_color(film, w, i + W - 1), a.color_noise) >= thr) { flags[i] = 1u; flags[i + W - 1] = 1u; }
		if(a.var_pixels > 0)
		{
			int vx = 0, vy = 0;
			for(int xd = -a.var_half; xd < a.var_half - 1; ++xd)
			{
				const int xi = min(max(x + xd, 0), W - 2);
				if(aa_diff(aa_color(film, w, y * W + xi), aa_color(film, w, y * W + xi + 1), a.color_noise) >= thr) ++vx;
			}
			for(int yd = -a.var_half; yd < a.var_half - 1; ++yd)
			{
				const int yi = min(max(y + yd, 0), H - 2);
				if(aa_diff(aa_color(film, w, yi * W + x), aa_color(film, w, (yi + 1) * W + x), a.color_noise) >= thr) ++vy;
			}
			if(vx + vy >= a.var_pixels)
				for(int xd = -a.var_half; xd < a.var_half; ++xd)
					for(int yd = -a.var_half; yd < a.var_half; ++yd)
					{
						const int xi = min(max(x + xd, 0), W - 1), yi = min(max(y + yd, 0), H - 1);
						flags[yi * W + xi] = 1u;
					}
		}
	}
}

// Flagged pixels -> list (order irrelevant: a pixel's samples depend only on
// the pixel and the sample index); count only without a list.
__global__ void k_aa_compact(const uint8_t *__restrict__ flags, uint32_t n, uint32_t *__restrict__ list, uint32_t *count)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if(flags[i])
		{
			const uint32_t k = atomicAdd(count, 1u);
			if(list) list[k] = i;
		}
}

// ---- SPPM hit points (SppmIntegrator::HitPoint, integrator_sppm.h) ----
__global__ void k_sppm_init(float4 *hp, float *r2, float4 *pass, uint32_t n, float r2_0)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		hp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
		r2[i] = r2_0;
		pass[i] = make_float4(0.f, 0.f, 0.f, 0.f);
	}
}

// Progressive refinement and the indirect estimate of one pass
// (SppmIntegrator::renderTile, integrator_sppm.cc:278-292): with M photons
// gathered, g = min((N + 0.7 M) / (N + M), 1), r^2 *= g, N += 0.7 M,
// flux = (flux + pass flux) g; the pixel's sample adds flux / (r^2 pi
// photons so far).  hp = {flux xyz, N}.
__global__ void k_sppm_update(Params P, float4 *hp, float *r2, float4 *pass, uint32_t n, float total_photons, float *film)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		float4 h = hp[i];
		float r = r2[i];
		const float4 g4 = pass[i];
		if(g4.w > 0.f)
		{
			const float g = fminf(__fdiv_rn(xa(h.w, xm(0.7f, g4.w)), xa(h.w, g4.w)), 1.f);
			r = xm(r, g);
			h.w = xa(h.w, xm(g4.w, 0.7f));
			h.x = xm(xa(h.x, g4.x), g); h.y = xm(xa(h.y, g4.y), g); h.z = xm(xa(h.z, g4.z), g);
			hp[i] = h;
			r2[i] = r;
		}
		pass[i] = make_float4(0.f, 0.f, 0.f, 0.f);
		const float inv = __fdiv_rn(1.f, xm(xm(r, kPi), total_photons));
		film_put(P, film, nullptr, i, 0u, xm(h.x, inv), xm(h.y, inv), xm(h.z, inv));
	}
}

// Rgba::normalized (color.h:294-298, 538-542): sum x (1 / weight), 0 where the weight is 0.
__global__ void k_normalize(const float *sum, const double *sum64, const float *w, float *out, size_t n)
{
	for(size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
	{
		const float wt = w[i / 3];
		const float v = sum64 ? static_cast<float>(sum64[i]) : sum[i];
		out[i] = wt != 0.f ? v * (1.f / wt) : 0.f;
	}
}

// kind: 0 lowDiscrepancySampling(dim, x), 1 riVdC, 2 riLp, 3 riS, 4 fnv32ABuf,
// 5 radical inverse base 2, 6 radical inverse base 3, 7 FAST_TRIG sin and
// cos of the float whose bits are x (sin in the value, cos via dim = 1),
// 8 FAST_MATH pow, 9 / 10 the FP64-free float forms of kinds 0 / 6.
__host__ __device__ inline double sampler_value(const gbrt::LdsTables &t, int kind, int dim, uint32_t x)
{
	switch(kind)
	{
		case 0: return gbrt::low_discrepancy(t, dim, x);
		case 1: return gbrt::ri_vdc(x);
		case 2: return gbrt::ri_lp(x);
		case 3: return gbrt::ri_s(x);
		case 4: return static_cast<double>(gbrt::fnv32(x));
		case 5: return gbrt::radical_inverse(x, 2);
		case 6: return gbrt::radical_inverse(x, 3);
		case 9: return gbrt::low_discrepancy_f(t, dim, x);
		case 10: return gbrt::radical_inverse3_f(t, x);
		case 8:
		{
			// FAST_MATH pow: base = float bits of x, exponent = float bits of dim
			float f, e;
			memcpy(&f, &x, 4);
			memcpy(&e, &dim, 4);
			return gbrt::fast_pow(f, e);
		}
		default:
		{
			float f;
			memcpy(&f, &x, 4);
			return dim == 1 ? gbrt::fast_cos(f) : gbrt::fast_sin(f);
		}
	}
}

__global__ void k_sampler(gbrt::LdsTables t, int kind, int dim, const uint32_t *in, uint32_t n, double *out)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) out[i] = sampler_value(t, kind, dim, in[i]);
}


// ---- photon shooting (PhotonIntegrator::diffuseWorker, integrator_photon_mapping.cc:157-280;
// CausticPhotonIntegrator::causticWorker, integrator_photon_caustic.cc:102-223) ----

struct PhotonJob {
	uint32_t n;               // photon paths: Halton indices 0 .. n - 1
	float inv_n;              // 1 / n (the diffuse worker's light-pick sample is i * (1 / n))
	int caustic;              // 1: caustic map, 0: diffuse map
	int max_bounces;          // bounces / caustic_depth
	int radiance_points;      // diffuse map with final gather: keep 1 in 8 diffuse hits as radiance points
	uint32_t n_lights;
	const float *light_cdf;   // Pdf1D over the lights' totalEnergy().energy() (sample_pdf1d.h:59-94)
	const float *light_pdf;
	uint32_t seed;
	float4 *pos, *dir, *col;  // deposited photons
	uint32_t *count;          // [0] photons, [1] radiance points
	uint32_t cap, rp_cap;
	float4 *rp_pos, *rp_nrm, *rp_refl, *rp_transm;
	// SPPM (SppmIntegrator::photonWorker, integrator_sppm.cc:353-505): photon
	// i of this pass is number base + i of the render; emission samples
	// from Halton bases 2 / 3 / 5 / 7, scattering over every BSDF
	// component, deposits only of indirect photons
	int sppm;
	uint32_t base;
};

// sample::sphere (include/sampler/sample.h:56-74), FAST_TRIG
__device__ __forceinline__ void sample_sphere(float s1, float s2, float d[3])
{
	d[2] = 1.f - 2.f * s1;
	float r = 1.f - d[2] * d[2];
	if(r > 0.f)
	{
		r = sqrtf(r);
		const float a = 6.28318530717958647692f * s2;
		d[0] = gbrt::fast_cos(a) * r;
		d[1] = gbrt::fast_sin(a) * r;
	}
	else d[0] = d[1] = 0.f;
}

// Warp-aggregated append: one atomic per warp and call site.
__device__ __forceinline__ uint32_t append_slot(uint32_t *counter, bool want)
{
	const uint32_t m = __activemask();
	const uint32_t b = __ballot_sync(m, want);
	if(!b) return 0xFFFFFFFFu;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t leader = __ffs(b) - 1u;
	uint32_t base = 0;
	if(lane == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(b)));
	base = __shfl_sync(m, base, leader);
	return want ? base + __popc(b & ((1u << lane) - 1u)) : 0xFFFFFFFFu;
}

// Material::getReflectivity (src/material/material.cc:198-216): mean of
// 16 sample colour x weight over fixed incoming directions.
__device__ void reflectivity(const SceneDev &sc, const Surface &s, uint32_t flags, float out[3])
{
	out[0] = out[1] = out[2] = 0.f;
	if(!(flags & (BF_TRANSMIT | BF_REFLECT) & s.m->flags)) return;
	for(int i = 0; i < 16; ++i)
	{
		const float s1 = 0.03125f + 0.0625f * static_cast<float>(i);
		const float s2 = gbrt::ri_vdc(static_cast<uint32_t>(i));
		const float s3 = gbrt::low_discrepancy_f(sc.lds, 2, static_cast<uint32_t>(i));
		const float s4 = gbrt::low_discrepancy_f(sc.lds, 3, static_cast<uint32_t>(i));
		float wo[3], wi[3], col[3], w, pdf;
		uint32_t sf;
		cos_hemisphere(s.n, s.u, s.v, s1, s2, wo);
		mat_sample(s, wo, s3, s4, flags, wi, col, w, pdf, sf);
		for(int k = 0; k < 3; ++k) out[k] += col[k] * w;
	}
	for(int k = 0; k < 3; ++k) out[k] *= 0.0625f;
}

template <bool kTex>
__global__ void __launch_bounds__(kThreads) k_photon_shoot(SceneDev sc, PhotonJob J)
{
	__shared__ uint2 stack[gbrt::kStackShared * kThreads];
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < J.n; i += gridDim.x * blockDim.x)
	{
		const uint32_t pi = J.base + i;
		float s1, s2, s3, s4;
		if(J.sppm)
		{
			// hal_1_ .. hal_4_ {2, 0}, {3, 0}, {5, 0}, {7, 0}: the n-th getNext is index n
			s1 = gbrt::radical_inverse(pi + 1u, 2); s2 = gbrt::radical_inverse3_f(sc.lds, pi + 1u);
			s3 = gbrt::radical_inverse(pi + 1u, 5); s4 = gbrt::radical_inverse(pi + 1u, 7);
		}
		else
		{
			s1 = gbrt::ri_vdc(i);
			s2 = gbrt::low_discrepancy_f(sc.lds, 2, i);
			s3 = gbrt::low_discrepancy_f(sc.lds, 3, i);
			s4 = gbrt::low_discrepancy_f(sc.lds, 4, i);
		}
		const float s_l = J.caustic ? static_cast<float>(i) / static_cast<float>(J.n) : static_cast<float>(i) * J.inv_n;
		uint32_t ln = 0;
		if(s_l >= 1.f) ln = J.n_lights - 1u;
		else if(s_l > 0.f) { while(ln + 1u < J.n_lights && J.light_cdf[ln] < s_l) ++ln; }   // std::lower_bound
		const DevLight &L = sc.lights[ln];
		float o[3], d[3], pcol[3], ipdf;
		if(L.type == GBRT_LIGHT_POINT)
		{
			// PointLight::emitPhoton (light_point.cc:99-104)
			for(int k = 0; k < 3; ++k) { o[k] = L.c[k]; pcol[k] = L.col[k]; }
			sample_sphere(s1, s2, d);
			ipdf = 4.f * kPi;
		}
		else
		{
			// AreaLight::emitPhoton (light_area.cc:126-133): cosine hemisphere
			// around normal_ = -normal_flipped_ (not normalised), frame duv_
			float nrm[3], u[3], v[3];
			for(int k = 0; k < 3; ++k) { o[k] = L.c[k] + s3 * L.tx[k] + s4 * L.ty[k]; nrm[k] = -L.nflip[k]; u[k] = L.tx[k]; pcol[k] = L.col[k]; }
			normalize3(u);
			v[0] = nrm[1] * u[2] - nrm[2] * u[1]; v[1] = nrm[2] * u[0] - nrm[0] * u[2]; v[2] = nrm[0] * u[1] - nrm[1] * u[0];
			cos_hemisphere(nrm, u, v, s1, s2, d);
			ipdf = 1.f;                                // area_ (light_area.h:79)
		}
		const float f = static_cast<float>(J.n_lights) * ipdf / J.light_pdf[ln];
		for(int k = 0; k < 3; ++k) pcol[k] *= f;
		if(pcol[0] == 0.f && pcol[1] == 0.f && pcol[2] == 0.f) continue;
		bool caustic = false, direct = true;
		float tmin = kRayMinDist;
		for(int nb = 0;; ++nb)
		{
			const gbrt::Hit h = gbrt::trace_ray<false>(sc.bv, o[0], o[1], o[2], tmin, d[0], d[1], d[2], -1.f, stack + threadIdx.x, kThreads);
			if(h.prim < 0) break;
			Surface s;
			for(int k = 0; k < 3; ++k) s.p[k] = xa(o[k], xm(h.t, d[k]));
			const float4 ng = __ldg(sc.prim_ng + h.prim);
			s.ng[0] = ng.x; s.ng[1] = ng.y; s.ng[2] = ng.z;
			shading_normal(sc, h.prim, h.u, h.v, s.ng, s.n);
			s.m = sc.mats + __float_as_uint(ng.w);
			coords_system(s.n, s.u, s.v);
			DevMaterial mloc;
			surface_color<kTex>(sc, s, h.prim, h.u, h.v, mloc);
			const float wi[3] = {-d[0], -d[1], -d[2]};
			const uint32_t mf = s.m->flags;
			const bool dep = (!J.sppm || !direct) && (J.caustic ? ((mf & (BF_DIFFUSE | BF_GLOSSY)) && caustic) : ((mf & BF_DIFFUSE) && !caustic));
			const uint32_t slot = append_slot(J.count, dep);
			if(dep && slot < J.cap)
			{
				J.pos[slot] = make_float4(s.p[0], s.p[1], s.p[2], 0.f);
				J.dir[slot] = make_float4(wi[0], wi[1], wi[2], 0.f);
				J.col[slot] = make_float4(pcol[0], pcol[1], pcol[2], 0.f);
			}
			if(J.radiance_points)
			{
				// 1 in 8 diffuse hits (the reference draws FastRandom < 0.125)
				const bool rp = (mf & BF_DIFFUSE) && !caustic && rng01(i, static_cast<uint32_t>(nb), 0x7adu, J.seed) < 0.125f;
				const uint32_t rs = append_slot(J.count + 1, rp);
				if(rp && rs < J.rp_cap)
				{
					float nf[3], refl[3], tr[3];
					face_forward(s, wi, nf);
					reflectivity(sc, s, BF_DIFFUSE | BF_GLOSSY | BF_REFLECT, refl);
					reflectivity(sc, s, BF_DIFFUSE | BF_GLOSSY | BF_TRANSMIT, tr);
					J.rp_pos[rs] = make_float4(s.p[0], s.p[1], s.p[2], 0.f);
					J.rp_nrm[rs] = make_float4(nf[0], nf[1], nf[2], 0.f);
					J.rp_refl[rs] = make_float4(refl[0], refl[1], refl[2], 0.f);
					J.rp_transm[rs] = make_float4(tr[0], tr[1], tr[2], 0.f);
				}
			}
			if(nb == J.max_bounces) break;
			// Material::scatterPhoton (src/material/material.cc:179-196)
			const int d5 = 3 * nb + 5;
			const float s5 = gbrt::low_discrepancy_f(sc.lds, d5, pi);
			const float s6 = gbrt::low_discrepancy_f(sc.lds, d5 + 1, pi);
			const float s7 = gbrt::low_discrepancy_f(sc.lds, d5 + 2, pi);
			const uint32_t flags = J.caustic && !J.sppm ? (BF_SPECULAR | BF_REFLECT | BF_TRANSMIT | BF_GLOSSY | BF_FILTER | BF_DISPERSIVE) : BF_ALL;
			float wo[3], scol[3], w, pdf;
			uint32_t sf;
			mat_sample(s, wi, s5, s6, flags, wo, scol, w, pdf, sf);
			if(!(pdf > 1.0e-6f)) break;
			float cnew[3];
			for(int k = 0; k < 3; ++k) cnew[k] = pcol[k] * 1.f * scol[k] * w;
			const float new_max = fmaxf(cnew[0], fmaxf(cnew[1], cnew[2]));
			const float old_max = fmaxf(pcol[0], fmaxf(pcol[1], pcol[2]));
			const float prob = fminf(1.f, new_max / old_max);
			if(!(s7 <= prob && prob > 1e-4f)) break;
			for(int k = 0; k < 3; ++k) pcol[k] = cnew[k] / prob;
			caustic = ((sf & (BF_GLOSSY | BF_SPECULAR | BF_DISPERSIVE)) && direct) ||
			          ((sf & (BF_GLOSSY | BF_SPECULAR | BF_FILTER | BF_DISPERSIVE)) && caustic);
			direct = (sf & BF_FILTER) && direct;
			if(J.caustic && !J.sppm && !(caustic || direct)) break;
			for(int k = 0; k < 3; ++k) { o[k] = s.p[k]; d[k] = wo[k]; }
			tmin = kRayMinDist;
		}
	}
}

// Rgb::clampProportionalRgb (include/color/color.h:399-432): the largest
// component down to max_value, the others scaled by the same factor.
__device__ __forceinline__ void clamp_proportional(float c[3], float max_value)
{
	const float m = fmaxf(c[0], fmaxf(c[1], c[2]));
	const float adj = __fdiv_rn(max_value, m);
	if(!(m > max_value)) return;
	if(c[0] >= m) { c[0] = max_value; c[1] = xm(c[1], adj); c[2] = xm(c[2], adj); }
	else if(c[1] >= m) { c[1] = max_value; c[0] = xm(c[0], adj); c[2] = xm(c[2], adj); }
	else { c[2] = max_value; c[0] = xm(c[0], adj); c[1] = xm(c[1], adj); }
}

// Material::eval with explicit BSDF flags, for the photon estimates.
__device__ __forceinline__ void eval_flags(const Surface &s, const float wo[3], const float wl[3], uint32_t flags, float out[3])
{
	out[0] = out[1] = out[2] = 0.f;
	if(s.m->type == GBRT_MAT_GLOSSY) { glossy_eval(s, wo, wl, flags, out); return; }
	if(s.m->type == GBRT_MAT_SHINYDIFFUSE && (flags & BF_DIFFUSE)) mat_eval(s, wo, wl, out);
}

// Photon estimates at the roots of integrate() calls (vertex level 0 of a
// wave), PhotonIntegrator::integrate (integrator_photon_mapping.cc:762-793)
// and CausticPhotonIntegrator::estimateCausticPhotons (integrator_photon_caustic.cc:284-304).
template <bool kTex>
__global__ void __launch_bounds__(kThreads) k_pm_root(SceneDev sc, Params P, Work W, int cur, float *film, double *film64)
{
	const uint32_t n = W.count[cur];
	for(uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
	{
		const uint32_t path = W.q_path[cur][q];
		const float4 h = W.hits[q];
		const int32_t prim = __float_as_int(h.x);
		if(prim < 0) continue;
		if(W.p_si[path] % static_cast<uint32_t>(P.path_samples) != 0u) continue;
		const float4 ng = __ldg(sc.prim_ng + prim);
		Surface s;
		s.m = sc.mats + __float_as_uint(ng.w);
		if(!(s.m->flags & BF_DIFFUSE) && !(P.pm == 3 && P.sppm_ire)) continue;
		const float4 ra = W.q_ray[cur][2ull * q], rb = W.q_ray[cur][2ull * q + 1];
		const float dir[3] = {rb.x, rb.y, rb.z};
		s.p[0] = xa(ra.x, xm(h.y, dir[0])); s.p[1] = xa(ra.y, xm(h.y, dir[1])); s.p[2] = xa(ra.z, xm(h.y, dir[2]));
		s.ng[0] = ng.x; s.ng[1] = ng.y; s.ng[2] = ng.z;
		shading_normal(sc, prim, h.z, h.w, s.ng, s.n);
		coords_system(s.n, s.u, s.v);
		DevMaterial mloc;
		surface_color<kTex>(sc, s, prim, h.z, h.w, mloc);
		const float wo[3] = {-dir[0], -dir[1], -dir[2]};
		if(P.pm == 3)
		{
			// SppmIntegrator::traceGatherRay (integrator_sppm.cc:727-748): every
			// caustic photon within the pixel's radius, f(wo, photon dir) x
			// photon colour; the count weighted 1 / (glossy split product)
			const uint32_t pixel = W.p_pixel[path];
			if(P.sppm_ire && !P.sppm_ire[pixel])
			{
				// pmIRE at any material (:648-667): the smaller of the shrunk radii
				uint32_t idx[gbrt::kMaxGather];
				float d2[gbrt::kMaxGather];
				float r1 = P.sppm_ire_r2, r2b = P.sppm_ire_r2;
				const int n1 = P.g_diffuse.n ? gbrt::knn_gather(P.g_diffuse, s.p, P.sppm_ire_k, r1, idx, d2) : 0;
				const int n2 = P.g_caustic.n ? gbrt::knn_gather(P.g_caustic, s.p, P.sppm_ire_k, r2b, idx, d2) : 0;
				if(n1 > 0 || n2 > 0)
				{
					P.sppm_r2[pixel] = r1 < r2b ? r1 : r2b;
					P.sppm_ire[pixel] = 1u;
				}
			}
			if(!(s.m->flags & BF_DIFFUSE) || !P.g_caustic.n) continue;
			const float r2 = P.sppm_r2[pixel];
			// the reference gathers at most n_max_gather_ = 1000 photons, the
			// nearest (integrator_sppm.h:118, PhotonMap::gather): beyond that
			// many within the radius, the 1000th smallest squared distance
			// (bisection over its float bits) bounds the sum
			float flux[3] = {0.f, 0.f, 0.f};
			uint32_t cnt = 0;
			auto gather = [&](bool capped, float cap) {
				flux[0] = flux[1] = flux[2] = 0.f;
				cnt = 0;
				gbrt::grid_range(P.g_caustic, s.p, r2, [&](uint32_t j) {
					if(capped)
					{
						const float4 q = __ldg(P.g_caustic.pos + j);
						const float vx = q.x - s.p[0], vy = q.y - s.p[1], vz = q.z - s.p[2];
						if(!(vx * vx + vy * vy + vz * vz <= cap)) return;
					}
					const float4 pd = __ldg(P.g_caustic.dir + j), pc = __ldg(P.g_caustic.col + j);
					const float pdir[3] = {pd.x, pd.y, pd.z};
					float sc3[3];
					eval_flags(s, wo, pdir, BF_ALL, sc3);
					flux[0] += sc3[0] * pc.x; flux[1] += sc3[1] * pc.y; flux[2] += sc3[2] * pc.z;
					++cnt;
				});
			};
			gather(false, r2);
			if(cnt > kSppmMaxGather)
			{
				uint32_t lo = 0u, hi = __float_as_uint(r2);        // count(d2 <= lo) < 1000 <= count(d2 <= hi)
				for(int it = 0; it < 32 && hi - lo > 1u; ++it)
				{
					const uint32_t mid = lo + (hi - lo) / 2u;
					const float x = __uint_as_float(mid);
					uint32_t c = 0;
					gbrt::grid_range(P.g_caustic, s.p, r2, [&](uint32_t j) {
						const float4 q = __ldg(P.g_caustic.pos + j);
						const float vx = q.x - s.p[0], vy = q.y - s.p[1], vz = q.z - s.p[2];
						if(vx * vx + vy * vy + vz * vz <= x) ++c;
					});
					if(c >= kSppmMaxGather) hi = mid;
					else lo = mid;
				}
				gather(true, __uint_as_float(hi));
			}
			if(cnt)
			{
				const float4 t4 = W.p_thr[path];
				const uint32_t division = max(1u, W.p_task[path].x >> 16);
				float *acc = reinterpret_cast<float *>(P.sppm_pass + pixel);
				atomicAdd(acc, flux[0] * t4.x); atomicAdd(acc + 1, flux[1] * t4.y); atomicAdd(acc + 2, flux[2] * t4.z);
				atomicAdd(acc + 3, static_cast<float>(cnt) / static_cast<float>(division));
			}
			continue;
		}
		float est[3] = {0.f, 0.f, 0.f};
		uint32_t idx[gbrt::kMaxGather];
		float d2[gbrt::kMaxGather];
		if(P.pm_diffuse && !P.pm_fg && P.g_diffuse.n)
		{
			float r2 = P.pm_diffuse_r2;
			const int f = gbrt::knn_gather(P.g_diffuse, s.p, P.pm_diffuse_k, r2, idx, d2);
			if(f > 0)
			{
				const float scale = 1.f / (P.pm_diffuse_paths * r2 * kPi);
				for(int j = 0; j < f; ++j)
				{
					const float4 pd = __ldg(P.g_diffuse.dir + idx[j]), pc = __ldg(P.g_diffuse.col + idx[j]);
					const float pdir[3] = {pd.x, pd.y, pd.z};
					float sc3[3];
					eval_flags(s, wo, pdir, BF_DIFFUSE, sc3);
					est[0] += sc3[0] * scale * pc.x; est[1] += sc3[1] * scale * pc.y; est[2] += sc3[2] * scale * pc.z;
				}
			}
		}
		if(P.pm_caustics && P.g_caustic.n)
		{
			float r2 = P.pm_caustic_r2;
			const int f = gbrt::knn_gather(P.g_caustic, s.p, P.pm_caustic_k, r2, idx, d2);
			if(f > 0)
			{
				const float ir2 = 1.f / r2;
				float sum[3] = {0.f, 0.f, 0.f};
				for(int j = 0; j < f; ++j)
				{
					const float4 pd = __ldg(P.g_caustic.dir + idx[j]), pc = __ldg(P.g_caustic.col + idx[j]);
					const float pdir[3] = {pd.x, pd.y, pd.z};
					float sc3[3];
					eval_flags(s, wo, pdir, BF_ALL, sc3);
					// sample::kernel (include/sampler/sample.h:29-33)
					const float t = 1.f - d2[j] * ir2;
					const float kk = 3.f * ir2 * 0.318309886183790671538f * t * t;
					sum[0] += sc3[0] * kk * pc.x; sum[1] += sc3[1] * kk * pc.y; sum[2] += sc3[2] * kk * pc.z;
				}
				const float inv = 1.f / P.pm_caustic_paths;
				for(int c = 0; c < 3; ++c) sum[c] *= inv;
				// CausticPhotonIntegrator::causticPhotons (integrator_photon_caustic.cc:91-100)
				if(P.clamp_indirect > 0.f) clamp_proportional(sum, P.clamp_indirect);
				for(int c = 0; c < 3; ++c) est[c] += sum[c];
			}
		}
		if(est[0] != 0.f || est[1] != 0.f || est[2] != 0.f)
		{
			const float4 t4 = W.p_thr[path];
			film_put(P, film, film64, W.p_pixel[path], W.p_si[path], est[0] * t4.x, est[1] * t4.y, est[2] * t4.z);
		}
	}
}

// Radiance points, "remove too close radiance points" (integrator_photon_mapping.cc:527-540):
// the reference keeps each point whose lookup still finds it unused, in its
// (thread-scheduled) order, and drops the points within r^2 = 0.01 x
// diffuse_radius whose normals face the same side.  Here the order is a
// random priority and the result is that greedy's, computed in rounds: a
// point joins when no undecided neighbour precedes it, and leaves when a
// neighbour joined.  States: 0 undecided, 1 kept, 2 dropped.
__device__ __forceinline__ bool rp_before(uint32_t a, uint32_t b, uint32_t seed)
{
	const uint32_t ha = hash32(a ^ seed), hb = hash32(b ^ seed);
	return ha < hb || (ha == hb && a < b);
}

__global__ void k_rp_round(gbrt::PhotonGrid g, float r2, uint32_t seed, const uint8_t *__restrict__ st_in, uint8_t *__restrict__ st_out,
                           uint32_t *__restrict__ undecided)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x)
	{
		uint8_t st = st_in[i];
		if(st == 0)
		{
			const float4 pi = __ldg(g.pos + i), ni = __ldg(g.dir + i);
			const float p[3] = {pi.x, pi.y, pi.z};
			const uint32_t oi = __float_as_uint(pi.w);
			bool drop = false, wait = false;
			gbrt::grid_visit(g, p, [&](uint32_t first, uint32_t end) {
				for(uint32_t j = first; j < end && !drop; ++j)
				{
					if(j == i) continue;
					const uint8_t sj = st_in[j];
					if(sj == 2) continue;
					const float4 pj = __ldg(g.pos + j);
					const float vx = pj.x - p[0], vy = pj.y - p[1], vz = pj.z - p[2];
					if(!(vx * vx + vy * vy + vz * vz < r2)) continue;
					const float4 nj = __ldg(g.dir + j);
					if(!(nj.x * ni.x + nj.y * ni.y + nj.z * ni.z > 0.f)) continue;
					if(sj == 1) drop = true;
					else if(rp_before(__float_as_uint(pj.w), oi, seed)) wait = true;
				}
			});
			st = drop ? 2 : (wait ? 0 : 1);
			if(st == 0) atomicAdd(undecided, 1u);
		}
		st_out[i] = st;
	}
}

// Pre-gathered radiance of the kept points (preGatherWorker, :98-146):
// sum over the k nearest diffuse photons of (reflectance or transmittance by
// the side the photon came from) x col / (paths x pi x r^2).
__global__ void k_pregather(gbrt::PhotonGrid rp, const uint8_t *__restrict__ st, const float4 *__restrict__ refl, const float4 *__restrict__ transm,
                            gbrt::PhotonGrid dm, float r2_0, int k, float inv_scale_paths,
                            float4 *__restrict__ opos, float4 *__restrict__ odir, float4 *__restrict__ ocol, uint32_t *__restrict__ count)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rp.n; i += gridDim.x * blockDim.x)
	{
		if(st[i] != 1) continue;
		const float4 pi = __ldg(rp.pos + i), ni = __ldg(rp.dir + i);
		const uint32_t oi = __float_as_uint(pi.w);
		const float p[3] = {pi.x, pi.y, pi.z};
		uint32_t idx[gbrt::kMaxGather];
		float d2[gbrt::kMaxGather];
		float r2 = r2_0;
		const int f = dm.n ? gbrt::knn_gather(dm, p, k, r2, idx, d2) : 0;
		float sum[3] = {0.f, 0.f, 0.f};
		if(f > 0)
		{
			const float scale = inv_scale_paths / r2;
			const float4 rf = refl[oi], tr = transm[oi];
			for(int j = 0; j < f; ++j)
			{
				const float4 pd = __ldg(dm.dir + idx[j]), pc = __ldg(dm.col + idx[j]);
				const bool front = ni.x * pd.x + ni.y * pd.y + ni.z * pd.z > 0.f;
				const float4 a = front ? rf : tr;
				sum[0] += a.x * scale * pc.x; sum[1] += a.y * scale * pc.y; sum[2] += a.z * scale * pc.z;
			}
		}
		const uint32_t o = atomicAdd(count, 1u);
		opos[o] = make_float4(p[0], p[1], p[2], 0.f);
		odir[o] = make_float4(ni.x, ni.y, ni.z, 0.f);
		ocol[o] = make_float4(sum[0], sum[1], sum[2], 0.f);
	}
}

// ---- photon grid build ------------------------------------------------------

__global__ void k_index_w(float4 *__restrict__ pos, uint32_t n)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pos[i].w = __uint_as_float(i);
}

__global__ void k_grid_count(const float4 *__restrict__ pos, uint32_t n, gbrt::PhotonGrid g, uint32_t *__restrict__ key, uint32_t *__restrict__ cnt)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 q = pos[i];
		const float p[3] = {q.x, q.y, q.z};
		int c[3];
		gbrt::grid_cell(g, p, c);
		const uint32_t b = gbrt::grid_bucket(c[0], c[1], c[2], g.buckets);
		key[i] = b;
		atomicAdd(cnt + b, 1u);
	}
}

__global__ void k_grid_scatter(const float4 *__restrict__ pos, const float4 *__restrict__ dir, const float4 *__restrict__ col, uint32_t n,
                               const uint32_t *__restrict__ key, const uint32_t *__restrict__ start, uint32_t *__restrict__ cursor,
                               float4 *__restrict__ opos, float4 *__restrict__ odir, float4 *__restrict__ ocol)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const uint32_t b = key[i];
		const uint32_t j = start[b] + atomicAdd(cursor + b, 1u);
		opos[j] = pos[i];
		if(dir) odir[j] = dir[i];
		if(col) ocol[j] = col[i];
	}
}

// Exclusive scan in three passes: per-block scan of 4096 words, scan of the
// block totals by one block, add-back.
__global__ void __launch_bounds__(1024) k_scan_local(uint32_t *__restrict__ data, uint32_t n, uint32_t *__restrict__ totals)
{
	__shared__ uint32_t s[1024];
	const uint32_t base = blockIdx.x * 4096u + threadIdx.x * 4u;
	uint32_t v[4], sum = 0;
	for(int k = 0; k < 4; ++k) { v[k] = base + k < n ? data[base + k] : 0u; sum += v[k]; }
	s[threadIdx.x] = sum;
	__syncthreads();
	for(int off = 1; off < 1024; off <<= 1)
	{
		const uint32_t t = threadIdx.x >= static_cast<unsigned>(off) ? s[threadIdx.x - off] : 0u;
		__syncthreads();
		s[threadIdx.x] += t;
		__syncthreads();
	}
	uint32_t run = s[threadIdx.x] - sum;
	for(int k = 0; k < 4; ++k) { if(base + k < n) data[base + k] = run; run += v[k]; }
	if(threadIdx.x == 1023) totals[blockIdx.x] = s[1023];
}

__global__ void __launch_bounds__(1024) k_scan_totals(uint32_t *__restrict__ t, uint32_t m)
{
	__shared__ uint32_t s[1024];
	const uint32_t per = (m + 1023u) / 1024u, lo = threadIdx.x * per, hi = min(lo + per, m);
	uint32_t sum = 0;
	for(uint32_t i = lo; i < hi; ++i) sum += t[i];
	s[threadIdx.x] = sum;
	__syncthreads();
	for(int off = 1; off < 1024; off <<= 1)
	{
		const uint32_t v = threadIdx.x >= static_cast<unsigned>(off) ? s[threadIdx.x - off] : 0u;
		__syncthreads();
		s[threadIdx.x] += v;
		__syncthreads();
	}
	uint32_t run = s[threadIdx.x] - sum;
	for(uint32_t i = lo; i < hi; ++i) { const uint32_t x = t[i]; t[i] = run; run += x; }
}

__global__ void k_scan_add(uint32_t *__restrict__ data, uint32_t n, const uint32_t *__restrict__ totals)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) data[i] += totals[i / 4096u];
}

// HashGrid bucket of each point (test entry for the cell assignment).
__global__ void k_grid_buckets(gbrt::PhotonGrid g, const float *__restrict__ p, uint32_t n, uint32_t *__restrict__ out)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float q[3] = {p[3ull * i], p[3ull * i + 1], p[3ull * i + 2]};
		int c[3];
		gbrt::grid_cell(g, q, c);
		out[i] = gbrt::grid_bucket(c[0], c[1], c[2], g.buckets);
	}
}

// kNN over a grid of bare points (test entry): counts, final r^2, indices
// into the caller's point order (kept in pos.w).
__global__ void k_knn_test(gbrt::PhotonGrid g, const float *__restrict__ q, uint32_t m, int k, float r2,
                           int32_t *__restrict__ cnt, float *__restrict__ r2_out, uint32_t *__restrict__ idx_out)
{
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
	{
		const float p[3] = {q[3ull * i], q[3ull * i + 1], q[3ull * i + 2]};
		uint32_t idx[gbrt::kMaxGather];
		float d2[gbrt::kMaxGather];
		float r = r2;
		const int f = gbrt::knn_gather(g, p, k, r, idx, d2);
		cnt[i] = f;
		r2_out[i] = r;
		for(int j = 0; j < f; ++j) idx_out[static_cast<size_t>(i) * k + j] = __float_as_uint(__ldg(g.pos + idx[j]).w);
	}
}

} // namespace

struct gbrt_scene;
static bool plain_scene(const gbrt_scene *S);
static bool textured_scene(const gbrt_scene *S);

struct gbrt_scene {
	const gbrt_bvh *bvh = nullptr;
	int device = 0;
	int n_sm = 0;
	uint32_t n_prims = 0, n_mats = 0, n_lights = 0;
	float4 *prim_ng = nullptr;
	DevMaterial *mats = nullptr;
	DevLight *lights = nullptr;
	uint16_t *lds_perm = nullptr;
	uint32_t *lds_off = nullptr, *lds_base = nullptr;
	double *lds_inv = nullptr;
	double *lds_sfac = nullptr;
	uint32_t *lds_sfac_off = nullptr, *lds_sfac_nd = nullptr;
	uint4 *lds_fx = nullptr;           // integer tables of the FP64-free sample streams
	uint32_t lds_fx_dims = 0, lds_fx_rad3 = 0;
	// materials that start the recursive split, for its buffer sizing
	bool split_glossy = false, split_glossy_transmit = false, split_specular = false;
	uint32_t max_addl = 0;
	// work buffers (grown on demand)
	size_t cap_paths = 0, cap_shadow = 0, cap_stride = 0;
	void *work = nullptr;
	Work w{};
	std::vector<DevLight> lights_host;
	// spawn buffers: one per ray level of the recursive split
	float4 *spawn = nullptr;
	uint32_t *spawn_count = nullptr;
	size_t spawn_cap = 0;
	int spawn_levels = 0;
	cudaEvent_t ev_last = nullptr;      // recorded after each render: the buffers' last use
	float *filter_dev = nullptr;        // 16 x 16 film filter table of the current render
	float filter_host[256];
	// textures (gbrt_scene_set_textures)
	DevTexture *tex = nullptr;
	float4 *texels = nullptr;
	float2 *uv = nullptr;
	uint4 *face_uv = nullptr;
	std::vector<uint8_t> face_quad;     // per face: a quad (for the implicit uv)
	// shading normals (gbrt_scene_set_normals)
	float4 *vnrm = nullptr;
	uint4 *face_nrm = nullptr;
	// noise tables of the procedural textures (gbrt_scene_set_noise_tables)
	uint8_t *noise_dev = nullptr;
	// shader node trees (gbrt_scene_set_shader_nodes)
	gbrt_shader_node *nodes = nullptr;
	uint32_t *prim_slot = nullptr;      // primitive -> BVH leaf-order record (bump mapping)
	uint32_t n_tex = 0;
	std::vector<DevMaterial> mats_host;
	std::mutex mu;
};

// prim_slot[ids[i] without the quad bit] = i: each primitive's record in
// the BVH's leaf order.
__global__ void k_prim_slot(const uint32_t *__restrict__ ids, uint32_t n, uint32_t *__restrict__ slot)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const uint32_t p = ids[i] & ~GBRT_QUAD_BIT;
	if(p < n) slot[p] = i;
}

// Every material plain (the diffuse layer of shinydiffuse alone, an
// untextured colour, or light_mat) and no shading normals: the scenes
// k_shade_plain serves.
static bool textured_scene(const gbrt_scene *S)
{
	for(const DevMaterial &m : S->mats_host)
		if(m.dtex >= 0 || m.has_nodes) return true;
	return false;
}

static bool plain_scene(const gbrt_scene *S)
{
	if(S->face_nrm) return false;
	for(const DevMaterial &m : S->mats_host)
	{
		if(m.type == GBRT_MAT_LIGHT) continue;
		if(m.type == GBRT_MAT_SHINYDIFFUSE && m.sd == SD_DIFFUSE && m.dtex < 0 && !m.has_nodes) continue;
		return false;
	}
	return true;
}

namespace {

// The render buffers below are stream-ordered allocations from the device's
// default pool, which keeps freed memory for reuse: growing or releasing
// them does not synchronise the device, so scenes rendered concurrently on
// their own streams (gbrt_pt_render_batch) do not stall each other.
void pool_retain(int dev)
{
	static std::atomic<uint64_t> done{0};
	if(dev < 0 || dev >= 64 || ((done.load() >> dev) & 1u)) return;
	cudaMemPool_t pool;
	if(cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
	{
		uint64_t keep = ~0ull;
		cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
	}
	done.fetch_or(1ull << dev);
}

int alloc_work(gbrt_scene *S, size_t paths, size_t shadow, size_t stride, cudaStream_t s)
{
	if(paths <= S->cap_paths && shadow <= S->cap_shadow && stride <= S->cap_stride) return GBRT_OK;
	paths = std::max(paths, S->cap_paths);
	shadow = std::max(shadow, S->cap_shadow);
	stride = std::max(stride, S->cap_stride);
	pool_retain(S->device);
	if(S->ev_last) cudaStreamWaitEvent(s, S->ev_last, 0);
	if(S->work) { cudaFreeAsync(S->work, s); S->work = nullptr; }
	size_t off = 0;
	auto carve = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
	const size_t o_pix = carve(4 * paths), o_si = carve(4 * paths), o_st = carve(4 * paths), o_thr = carve(16 * paths);
	const size_t o_task = carve(16 * paths), o_pm = carve(16 * paths);
	const size_t o_qr0 = carve(32 * paths), o_qr1 = carve(32 * paths), o_qp0 = carve(4 * paths), o_qp1 = carve(4 * paths);
	const size_t o_hit = carve(16 * paths), o_scene = carve(4 * paths);
	const size_t o_sr = carve(32 * shadow), o_sc = carve(16 * shadow), o_sp = carve(4 * shadow), o_spath = carve(4 * shadow);
	const size_t o_cnt = carve(64), o_stats = carve(64);
	size_t o_hp = 0, o_lob = 0, o_psum = 0, o_rpos = 0, o_rdir = 0, o_rthr = 0, o_rpre = 0, o_rval = 0, o_train = 0;
	const size_t recs = paths * stride;
	if(stride)
	{
		o_hp = carve(12 * paths); o_lob = carve(4ull * gbrt::kGuideOut * paths); o_psum = carve(16 * paths);
		o_rpos = carve(16 * recs); o_rdir = carve(16 * recs); o_rthr = carve(16 * recs); o_rpre = carve(16 * recs);
		o_rval = carve(4 * recs); o_train = carve(32 * (recs + kMaxBatch));
	}
	cudaError_t e = cudaMallocAsync(&S->work, off, s);
	if(e != cudaSuccess) { S->work = nullptr; S->cap_paths = S->cap_shadow = S->cap_stride = 0; return gbrt_set_error(GBRT_ERR_OOM, "path tracer work buffers (%zu bytes): %s", off, cudaGetErrorString(e)); }
	char *b = static_cast<char *>(S->work);
	Work &w = S->w;
	w = Work{};
	w.p_pixel = reinterpret_cast<uint32_t *>(b + o_pix);
	w.p_si = reinterpret_cast<uint32_t *>(b + o_si);
	w.p_state = reinterpret_cast<uint32_t *>(b + o_st);
	w.p_thr = reinterpret_cast<float4 *>(b + o_thr);
	w.p_task = reinterpret_cast<uint4 *>(b + o_task);
	w.p_pm = reinterpret_cast<float4 *>(b + o_pm);
	w.q_ray[0] = reinterpret_cast<float4 *>(b + o_qr0);
	w.q_ray[1] = reinterpret_cast<float4 *>(b + o_qr1);
	w.q_path[0] = reinterpret_cast<uint32_t *>(b + o_qp0);
	w.q_path[1] = reinterpret_cast<uint32_t *>(b + o_qp1);
	w.hits = reinterpret_cast<float4 *>(b + o_hit);
	w.p_scene = reinterpret_cast<uint32_t *>(b + o_scene);
	w.s_ray = reinterpret_cast<float4 *>(b + o_sr);
	w.s_col = reinterpret_cast<float4 *>(b + o_sc);
	w.s_pix = reinterpret_cast<uint32_t *>(b + o_sp);
	w.s_path = reinterpret_cast<uint32_t *>(b + o_spath);
	w.count = reinterpret_cast<uint32_t *>(b + o_cnt);
	w.stats = reinterpret_cast<unsigned long long *>(b + o_stats);
	if(stride)
	{
		w.hitpos = reinterpret_cast<float *>(b + o_hp);
		w.lobes = reinterpret_cast<float *>(b + o_lob);
		w.p_sum = reinterpret_cast<float4 *>(b + o_psum);
		w.r_pos = reinterpret_cast<float4 *>(b + o_rpos);
		w.r_dir = reinterpret_cast<float4 *>(b + o_rdir);
		w.r_thr = reinterpret_cast<float4 *>(b + o_rthr);
		w.r_pre = reinterpret_cast<float4 *>(b + o_rpre);
		w.r_valid = reinterpret_cast<uint32_t *>(b + o_rval);
		w.train = reinterpret_cast<float *>(b + o_train);
		w.train_cap = static_cast<uint32_t>(std::min<size_t>(recs + kMaxBatch, 0xFFFFFFFFull));
	}
	S->cap_paths = paths;
	S->cap_shadow = shadow;
	S->cap_stride = stride;
	return GBRT_OK;
}

int alloc_spawn(gbrt_scene *S, size_t cap, int levels, cudaStream_t s)
{
	if(cap <= S->spawn_cap && levels <= S->spawn_levels) return GBRT_OK;
	cap = std::max(cap, S->spawn_cap);
	levels = std::max(levels, S->spawn_levels);
	pool_retain(S->device);
	if(S->ev_last) cudaStreamWaitEvent(s, S->ev_last, 0);
	if(S->spawn) { cudaFreeAsync(S->spawn, s); S->spawn = nullptr; }
	if(S->spawn_count) { cudaFreeAsync(S->spawn_count, s); S->spawn_count = nullptr; }
	S->spawn_cap = 0; S->spawn_levels = 0;
	cudaError_t e = cudaMallocAsync(&S->spawn, cap * levels * 5 * sizeof(float4), s);
	if(e == cudaSuccess) e = cudaMallocAsync(&S->spawn_count, levels * sizeof(uint32_t), s);
	if(e != cudaSuccess)
		return gbrt_set_error(GBRT_ERR_OOM, "recursive split buffers (%zu records x %d levels): %s", cap, levels, cudaGetErrorString(e));
	S->spawn_cap = cap;
	S->spawn_levels = levels;
	return GBRT_OK;
}

// Frees a scene's work and spawn buffers (they are re-made by the next render).
void release_work(gbrt_scene *S, cudaStream_t s)
{
	if(S->ev_last) cudaStreamWaitEvent(s, S->ev_last, 0);
	if(S->work) cudaFreeAsync(S->work, s);
	if(S->spawn) cudaFreeAsync(S->spawn, s);
	if(S->spawn_count) cudaFreeAsync(S->spawn_count, s);
	S->work = nullptr; S->spawn = nullptr; S->spawn_count = nullptr;
	S->w = Work{};
	S->cap_paths = S->cap_shadow = S->cap_stride = 0;
	S->spawn_cap = 0; S->spawn_levels = 0;
}

// Upper bound of the spawn records one hit can write (largest at division 1).
uint32_t split_fanout(const gbrt_scene *S, int path_samples)
{
	const uint32_t ps = static_cast<uint32_t>(std::max(1, path_samples));
	uint32_t f = 0;
	if(S->split_glossy) f += 8u * (S->split_glossy_transmit ? 2u : 1u) * std::max(1u, ps / 8u);
	if(S->split_specular) f += 2u * ps;
	return f;
}

// Camera::Camera axes (camera.cc:96-103) and PerspectiveCamera::setAxis
// (camera_perspective.cc:97-111), in float like the reference.
Camera make_camera(const gbrt_camera_desc &c)
{
	auto sub = [](const float *a, const float *b, float *o) { for(int k = 0; k < 3; ++k) o[k] = a[k] - b[k]; };
	auto cross = [](const float *a, const float *b, float *o) {
		o[0] = a[1] * b[2] - a[2] * b[1]; o[1] = a[2] * b[0] - a[0] * b[2]; o[2] = a[0] * b[1] - a[1] * b[0];
	};
	auto normalize = [](float *v) {
		const float l2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
		if(l2 != 0.f) { const float inv = 1.f / std::sqrt(l2); for(int k = 0; k < 3; ++k) v[k] *= inv; }
	};
	float cy[3], cz[3], cx[3];
	sub(c.up, c.from, cy);
	sub(c.to, c.from, cz);
	cross(cz, cy, cx);
	cross(cz, cx, cy);
	normalize(cx); normalize(cy); normalize(cz);
	const float aspect = 1.f * static_cast<float>(c.resy) / static_cast<float>(c.resx);
	Camera cam{};
	for(int k = 0; k < 3; ++k)
	{
		cam.from[k] = c.from[k];
		cam.vright[k] = cx[k];
		cam.vup[k] = aspect * cy[k];
	}
	for(int k = 0; k < 3; ++k) cam.vto[k] = (cz[k] * c.focal) - 0.5f * (cam.vup[k] + cam.vright[k]);
	for(int k = 0; k < 3; ++k) { cam.vup[k] /= static_cast<float>(c.resy); cam.vright[k] /= static_cast<float>(c.resx); }
	cam.resx = c.resx;
	cam.resy = c.resy;
	return cam;
}

unsigned grid_for(size_t n, int n_sm)
{
	const size_t want = (n + kThreads - 1) / kThreads;
	const size_t cap = static_cast<size_t>(n_sm > 0 ? n_sm : 148) * 16;
	return static_cast<unsigned>(std::max<size_t>(1, std::min(want, cap)));
}

// Grid of a gbrt::trace_persistent kernel: the blocks that fit on the GPU at
// once, no more than n queries need.
template <typename K>
unsigned persistent_grid(K kernel, size_t n, int n_sm)
{
	// resident blocks per SM, queried once per kernel (all devices are GB300s)
	static std::atomic<int> cached{0};
	int bps = cached.load(std::memory_order_relaxed);
	if(bps == 0)
	{
		if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, kThreads, 0) != cudaSuccess || bps < 1) bps = 1;
		cached.store(bps, std::memory_order_relaxed);
	}
	const size_t want = (n + kThreads - 1) / kThreads;
	const size_t cap = static_cast<size_t>(n_sm > 0 ? n_sm : 148) * static_cast<size_t>(bps);
	return static_cast<unsigned>(std::max<size_t>(1, std::min(want, cap)));
}


// ---- photon maps (host side) ------------------------------------------------

struct DevBuf {
	void *p = nullptr;
	DevBuf() = default;
	DevBuf(const DevBuf &) = delete;
	DevBuf &operator=(const DevBuf &) = delete;
	~DevBuf() { if(p) cudaFree(p); }
	template<typename T> T *as() const { return static_cast<T *>(p); }
	int alloc(size_t bytes)
	{
		if(p) cudaFree(p);
		p = nullptr;
		const cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
		if(e != cudaSuccess) { p = nullptr; return gbrt_set_error(GBRT_ERR_OOM, "device buffers (%zu bytes): %s", bytes, cudaGetErrorString(e)); }
		return GBRT_OK;
	}
};

struct GridStore {
	DevBuf pos, dir, col, start, key, cursor, totals;
	gbrt::PhotonGrid g{};
};

// Sorts n points (and their dir / col when given) into a hashed grid of cell
// edge `cell` (>= every query radius made of it).
int build_grid(const float4 *pos, const float4 *dir, const float4 *col, uint32_t n, float cell, const float lo[3], int n_sm,
               GridStore &G, cudaStream_t s)
{
	// buckets: the photon count (HashGrid's grid_size is a free parameter), at least 1024
	const uint32_t T = std::max<uint32_t>(1024u, std::min<uint32_t>(n, 1u << 27));
	const uint32_t words = T + 1, nblk = (words + 4095u) / 4096u;
	if(int rc = G.pos.alloc(16ull * n)) return rc;
	if(dir) if(int rc = G.dir.alloc(16ull * n)) return rc;
	if(col) if(int rc = G.col.alloc(16ull * n)) return rc;
	if(int rc = G.start.alloc(4ull * words)) return rc;
	if(int rc = G.key.alloc(4ull * n)) return rc;
	if(int rc = G.cursor.alloc(4ull * T)) return rc;
	if(int rc = G.totals.alloc(4ull * nblk)) return rc;
	GBRT_CK(cudaMemsetAsync(G.start.p, 0, 4ull * words, s));
	GBRT_CK(cudaMemsetAsync(G.cursor.p, 0, 4ull * T, s));
	gbrt::PhotonGrid &g = G.g;
	g = gbrt::PhotonGrid{};
	g.pos = G.pos.as<float4>();
	g.dir = dir ? G.dir.as<float4>() : nullptr;
	g.col = col ? G.col.as<float4>() : nullptr;
	g.start = G.start.as<uint32_t>();
	g.buckets = T;
	g.n = n;
	for(int a = 0; a < 3; ++a) g.lo[a] = lo[a];
	// a hair wider than the largest query radius, so float rounding of the cell
	// coordinates never puts a photon within the radius two cells away
	g.inv_cell = static_cast<float>(1.0 / (static_cast<double>(cell) * (1.0 + 1.0 / 1024.0)));
	if(n)
		k_grid_count<<<grid_for(n, n_sm), kThreads, 0, s>>>(pos, n, g, G.key.as<uint32_t>(), G.start.as<uint32_t>());
	k_scan_local<<<nblk, 1024, 0, s>>>(G.start.as<uint32_t>(), words, G.totals.as<uint32_t>());
	k_scan_totals<<<1, 1024, 0, s>>>(G.totals.as<uint32_t>(), nblk);
	k_scan_add<<<grid_for(words, n_sm), kThreads, 0, s>>>(G.start.as<uint32_t>(), words, G.totals.as<uint32_t>());
	if(n)
		k_grid_scatter<<<grid_for(n, n_sm), kThreads, 0, s>>>(pos, dir, col, n, G.key.as<uint32_t>(), G.start.as<uint32_t>(),
		                                                      G.cursor.as<uint32_t>(), G.pos.as<float4>(), G.dir.as<float4>(), G.col.as<float4>());
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

// Pdf1D over the lights' totalEnergy().energy() (sample_pdf1d.h:59-80):
// cdf and pdf = function x inv_integral, in the reference's float/double mix.
void light_pdf_tables(const std::vector<DevLight> &ls, std::vector<float> &cdf, std::vector<float> &pdf)
{
	const size_t n = ls.size();
	std::vector<float> fn(n);
	for(size_t i = 0; i < n; ++i)
	{
		const DevLight &L = ls[i];
		float e[3];
		for(int k = 0; k < 3; ++k) e[k] = L.type == GBRT_LIGHT_POINT ? L.col[k] * 4.0f * 3.14159265358979323846f : L.col[k] * 1.f;
		fn[i] = (e[0] + e[1] + e[2]) * 0.333333f;      // Rgb::energy (color.h:55)
	}
	cdf.assign(n, 0.f);
	pdf.assign(n, 0.f);
	const double delta = 1.0 / static_cast<double>(n);
	double c = 0.0;
	for(size_t i = 0; i < n; ++i) { c += static_cast<double>(fn[i]) * delta; cdf[i] = static_cast<float>(c); }
	const float integral = static_cast<float>(c);
	for(auto &x : cdf) x /= integral;
	const float inv = 1.f / integral;
	for(size_t i = 0; i < n; ++i) pdf[i] = fn[i] * inv;
}

struct ShotMap {
	DevBuf pos, dir, col, count, rp_pos, rp_nrm, rp_refl, rp_transm;
	uint32_t n = 0, paths = 0, n_rp = 0;
};

// One photon map: shoots n photon paths, keeps the deposits (and, for the
// diffuse map with final gather, the radiance points).
int shoot_map(gbrt_scene *S, const SceneDev &sc, bool caustic, uint32_t n, int max_bounces, bool radiance_points, uint32_t seed,
              ShotMap &M, cudaStream_t s, bool sppm = false, uint32_t base = 0)
{
	M.paths = n;
	M.n = M.n_rp = 0;
	if(n == 0 || S->n_lights == 0) return GBRT_OK;
	std::vector<float> cdf, pdf;
	light_pdf_tables(S->lights_host, cdf, pdf);
	DevBuf dcdf, dpdf;
	if(int rc = dcdf.alloc(4 * cdf.size())) return rc;
	if(int rc = dpdf.alloc(4 * pdf.size())) return rc;
	GBRT_CK(cudaMemcpyAsync(dcdf.p, cdf.data(), 4 * cdf.size(), cudaMemcpyHostToDevice, s));
	GBRT_CK(cudaMemcpyAsync(dpdf.p, pdf.data(), 4 * pdf.size(), cudaMemcpyHostToDevice, s));
	const uint64_t cap64 = static_cast<uint64_t>(n) * static_cast<uint64_t>(max_bounces + 1);
	if(cap64 >= (1ull << 31)) return gbrt_set_error(GBRT_ERR_CAPACITY, "photon map: %u paths x %d bounces exceed 2^31 photons", n, max_bounces + 1);
	const uint32_t cap = static_cast<uint32_t>(cap64);
	const uint32_t rp_cap = radiance_points ? cap / 4u + 4096u : 0u;
	if(int rc = M.pos.alloc(16ull * cap)) return rc;
	if(int rc = M.dir.alloc(16ull * cap)) return rc;
	if(int rc = M.col.alloc(16ull * cap)) return rc;
	if(int rc = M.count.alloc(8)) return rc;
	if(radiance_points)
	{
		if(int rc = M.rp_pos.alloc(16ull * rp_cap)) return rc;
		if(int rc = M.rp_nrm.alloc(16ull * rp_cap)) return rc;
		if(int rc = M.rp_refl.alloc(16ull * rp_cap)) return rc;
		if(int rc = M.rp_transm.alloc(16ull * rp_cap)) return rc;
	}
	GBRT_CK(cudaMemsetAsync(M.count.p, 0, 8, s));
	PhotonJob J{};
	J.n = n;
	J.inv_n = 1.f / static_cast<float>(n);
	J.caustic = caustic ? 1 : 0;
	J.max_bounces = max_bounces;
	J.radiance_points = radiance_points ? 1 : 0;
	J.n_lights = S->n_lights;
	J.light_cdf = dcdf.as<float>();
	J.light_pdf = dpdf.as<float>();
	J.seed = seed;
	J.sppm = sppm ? 1 : 0;
	J.base = base;
	J.pos = M.pos.as<float4>(); J.dir = M.dir.as<float4>(); J.col = M.col.as<float4>();
	J.count = M.count.as<uint32_t>();
	J.cap = cap; J.rp_cap = rp_cap;
	J.rp_pos = M.rp_pos.as<float4>(); J.rp_nrm = M.rp_nrm.as<float4>(); J.rp_refl = M.rp_refl.as<float4>(); J.rp_transm = M.rp_transm.as<float4>();
	if(textured_scene(S)) k_photon_shoot<true><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, J);
	else k_photon_shoot<false><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, J);
	GBRT_CK(cudaGetLastError());
	uint32_t cnt[2];
	GBRT_CK(cudaMemcpyAsync(cnt, M.count.p, 8, cudaMemcpyDeviceToHost, s));
	GBRT_CK(cudaStreamSynchronize(s));
	if(cnt[0] > cap || cnt[1] > rp_cap) return gbrt_set_error(GBRT_ERR_CAPACITY, "photon map: %u photons / %u radiance points overflow %u / %u", cnt[0], cnt[1], cap, rp_cap);
	M.n = cnt[0];
	M.n_rp = cnt[1];
	return GBRT_OK;
}

// Device views of the scene's noise tables (one allocation: hash 512 B,
// stdp_p 514 B padded to 1,032 B, then the float tables).
constexpr size_t kNoiseHash = 0, kNoiseStdpP = 512, kNoiseFloats = 1040;
constexpr size_t kNoiseBytes = kNoiseFloats + 4 * (768 + 768 + 514 * 3);
gbrt::NoiseTables noise_view(const gbrt_scene *S)
{
	if(!S->noise_dev) return gbrt::NoiseTables{nullptr, nullptr, nullptr, nullptr, nullptr};
	const uint8_t *b = S->noise_dev;
	const float *f = reinterpret_cast<const float *>(b + kNoiseFloats);
	return gbrt::NoiseTables{b + kNoiseHash, f, f + 768, b + kNoiseStdpP, f + 1536};
}

SceneDev scene_dev(const gbrt_scene *S)
{
	return SceneDev{gbrt::view_of(S->bvh), S->prim_ng, S->mats, S->lights, {S->lds_perm, S->lds_off, S->lds_base, S->lds_inv, S->lds_sfac, S->lds_sfac_off, S->lds_sfac_nd,
	                                                                         S->lds_fx, S->lds_fx_dims, S->lds_fx_rad3},
	                S->tex, S->texels, S->uv, S->face_uv, S->vnrm, S->face_nrm, noise_view(S), S->nodes, S->prim_slot};
}

} // namespace

extern "C" {

int gbrt_scene_create(const gbrt_bvh *bvh, const float *vertices, uint32_t n_vertices, const uint32_t *faces, uint32_t n_faces,
                      const int32_t *face_material, const gbrt_material_desc *materials, uint32_t n_materials,
                      const gbrt_light_desc *lights, uint32_t n_lights, gbrt_scene **out)
{
	if(!out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: out is NULL");
	*out = nullptr;
	if(!bvh || (n_faces && (!vertices || !faces || !face_material)) || (n_materials && !materials) || (n_lights && !lights))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: NULL argument");
	gbrt_bvh_info info{};
	if(int rc = gbrt_bvh_get_info(bvh, &info)) return rc;
	if(info.n_prims != n_faces) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: %u faces but the BVH holds %u", n_faces, info.n_prims);
	// materials
	std::vector<DevMaterial> mats(n_materials);
	for(uint32_t i = 0; i < n_materials; ++i)
	{
		const gbrt_material_desc &m = materials[i];
		DevMaterial &d = mats[i];
		std::memset(&d, 0, sizeof(d));
		d.type = m.type;
		d.dtex = -1;
		for(int k = 0; k < GBRT_SLOTS; ++k) d.nroot[k] = d.nfirst[k] = -1;
		if(m.type == GBRT_MAT_SHINYDIFFUSE)
		{
			// ShinyDiffuseMaterial ctor + config (material_shiny_diffuse.cc:133-189);
			// ParamMap defaults: diffuse_reflect 1, mirror_color 1, IOR 1.33
			const float diffuse_reflect = m.params[0] > 0.f ? m.params[0] : 1.f;
			const float specular_reflect = m.params[1], transparency = m.params[2], translucency = m.params[3];
			const float transmit_filter = m.params[4];
			const bool fresnel = m.params[6] > 0.5f;
			const float ior = m.params[7] > 0.f ? m.params[7] : 1.33f;
			const bool mirror_set = m.color2[0] != 0.f || m.color2[1] != 0.f || m.color2[2] != 0.f;
			float acc = 1.f;
			d.flags = 0u;
			d.sd = fresnel ? SD_FRESNEL : 0u;
			if(specular_reflect > 0.00001f)
			{
				d.sd |= SD_MIRROR;
				if(!fresnel) acc = 1.f - specular_reflect;
				d.flags |= BF_SPECULAR | BF_REFLECT;
			}
			if(transparency * acc > 0.00001f)
			{
				d.sd |= SD_TRANSPARENT;
				d.transparent = 1u;
				acc *= 1.f - transparency;
				d.flags |= BF_TRANSMIT | BF_FILTER;
			}
			if(translucency * acc > 0.00001f)
			{
				d.sd |= SD_TRANSLUCENT;
				acc *= 1.f - transparency;      // (sic) the reference's config
				d.flags |= BF_DIFFUSE | BF_TRANSMIT;
			}
			if(diffuse_reflect * acc > 0.00001f)
			{
				d.sd |= SD_DIFFUSE;
				d.flags |= BF_DIFFUSE | BF_REFLECT;
			}
			d.sdc[0] = (d.sd & SD_MIRROR) ? specular_reflect : 0.f;
			d.sdc[1] = (d.sd & SD_TRANSPARENT) ? transparency : 0.f;
			d.sdc[2] = (d.sd & SD_TRANSLUCENT) ? translucency : 0.f;
			d.sdc[3] = (d.sd & SD_DIFFUSE) ? diffuse_reflect : 0.f;
			d.ior = ior * ior;
			const float emit = m.power;
			if(emit > 0.f) d.flags |= BF_EMIT;
			d.tf = transmit_filter;
			d.emit = emit;
			for(int k = 0; k < 3; ++k)
			{
				d.col[k] = m.color[k];
				d.col2[k] = mirror_set ? m.color2[k] : 1.f;
				d.tcol[k] = transmit_filter * m.color[k] + (1.f - transmit_filter);
				d.ecol[k] = emit * m.color[k];
			}
		}
		else if(m.type == GBRT_MAT_LIGHT)
		{
			d.flags = BF_EMIT;
			for(int k = 0; k < 3; ++k) d.col[k] = m.color[k] * m.power;    // light_col_ = color * power
			d.double_sided = m.params[0] > 0.5f ? 1u : 0u;
		}
		else if(m.type == GBRT_MAT_GLOSSY)
		{
			// GlossyMaterial ctor and initBsdf (material_glossy.cc:128-148); params:
			// exponent, glossy_reflect, diffuse_reflect, as_diffuse (1 = default)
			d.exponent = m.params[0] > 0.f ? m.params[0] : 50.f;
			d.m_glossy = m.params[1];
			d.m_diffuse = m.params[2];
			d.as_diffuse = m.params[3] < 0.5f ? 0u : 1u;
			d.with_diffuse = d.m_diffuse > 0.f ? 1u : 0u;
			d.flags = (d.with_diffuse ? (BF_DIFFUSE | BF_REFLECT) : 0u) | (d.as_diffuse ? (BF_DIFFUSE | BF_REFLECT) : (BF_GLOSSY | BF_REFLECT));
			d.p_diffuse = std::min(0.6f, 1.f - (d.m_glossy / (d.m_glossy + (1.f - d.m_glossy) * d.m_diffuse)));
			for(int k = 0; k < 3; ++k) { d.col[k] = m.color[k]; d.col2[k] = m.color2[k]; }
		}
		else if(m.type == GBRT_MAT_GLASS || m.type == GBRT_MAT_ROUGH_GLASS)
		{
			// GlassMaterial / RoughGlassMaterial ctors (material_glass.cc:140-151,
			// material_rough_glass.cc:143-154; material_rough_glass.h:91-94):
			// filter_color_ = transmit_filter x filter_color + (1 - transmit_filter)
			const float tf = m.params[1];
			for(int k = 0; k < 3; ++k) { d.col[k] = tf * m.color[k] + (1.f - tf); d.col2[k] = m.color2[k]; }
			d.ior = m.params[0] > 0.f ? m.params[0] : 1.4f;
			if(m.type == GBRT_MAT_GLASS) d.flags = BF_SPECULAR | BF_REFLECT | BF_TRANSMIT;
			else
			{
				const float alpha = m.params[2] > 0.f ? m.params[2] : 0.5f;
				const float a = std::max(1e-4f, std::min(alpha * 0.5f, 1.f));
				d.a2 = a * a;
				d.flags = BF_GLOSSY | BF_REFLECT | BF_TRANSMIT;
			}
			// fake_shadows: transparent to shadow rays, Filter in the BSDF flags
			// (material_glass.cc:146, material_rough_glass.cc:148)
			if(m.params[3] > 0.5f)
			{
				d.transparent = 1u;
				d.flags |= BF_FILTER;
			}
		}
		else return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: material %u has unsupported type %u", i, m.type);
		d.addl_depth = static_cast<uint32_t>(std::max(0.f, std::min(m.params[5], 32.f)));    // additionaldepth (material.h:177)
	}
	// lights
	std::vector<DevLight> ls(n_lights);
	for(uint32_t i = 0; i < n_lights; ++i)
	{
		const gbrt_light_desc &L = lights[i];
		if(L.type != GBRT_LIGHT_AREA && L.type != GBRT_LIGHT_POINT)
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: light %u has unsupported type %u", i, L.type);
		DevLight &d = ls[i];
		std::memset(&d, 0, sizeof(d));
		d.type = L.type;
		if(L.type == GBRT_LIGHT_POINT)
		{
			// PointLight: color_ = color x power (light_point.h:64)
			for(int k = 0; k < 3; ++k) { d.c[k] = L.corner[k]; d.col[k] = L.color[k] * L.power; }
			d.samples = 1;
			continue;
		}
		if(L.samples < 1) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: light %u has %d samples", i, L.samples);
		float tx[3], ty[3];
		for(int k = 0; k < 3; ++k) { d.c[k] = L.corner[k]; tx[k] = L.point1[k] - L.corner[k]; ty[k] = L.point2[k] - L.corner[k]; }
		for(int k = 0; k < 3; ++k) { d.tx[k] = tx[k]; d.ty[k] = ty[k]; }
		// normal_flipped_ = (point2 - corner) ^ (point1 - corner), not normalised (light_area.h:75)
		d.nflip[0] = ty[1] * tx[2] - ty[2] * tx[1];
		d.nflip[1] = ty[2] * tx[0] - ty[0] * tx[2];
		d.nflip[2] = ty[0] * tx[1] - ty[1] * tx[0];
		for(int k = 0; k < 3; ++k) d.col[k] = L.color[k] * L.power * 3.14159265358979323846f;   // light_area.h:78
		// area_quad_ = {corner, point1, point1 + point2 - corner, point2} (light_area.h:72)
		for(int k = 0; k < 3; ++k)
		{
			const float v2 = (L.point1[k] + L.point2[k]) - L.corner[k];
			d.e1[k] = L.point1[k] - L.corner[k];
			d.e2[k] = v2 - L.corner[k];
			d.e3[k] = L.point2[k] - L.corner[k];
		}
		d.samples = L.samples;
	}
	// per-primitive geometric normal ((v1-v0) ^ (v2-v0)).normalize(), shape_polygon.h:58-62
	std::vector<float4> ng(n_faces ? n_faces : 1);
	for(uint32_t i = 0; i < n_faces; ++i)
	{
		const uint32_t *f = faces + 4ull * i;
		for(int k = 0; k < 3; ++k)
			if(f[k] >= n_vertices) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: face %u references vertex %u >= %u", i, f[k], n_vertices);
		if(face_material[i] < 0 || static_cast<uint32_t>(face_material[i]) >= n_materials)
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_create: face %u has material %d of %u", i, face_material[i], n_materials);
		const float *v0 = vertices + 3ull * f[0], *v1 = vertices + 3ull * f[1], *v2 = vertices + 3ull * f[2];
		const float a[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
		const float b[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
		float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
		const float l2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
		if(l2 != 0.f) { const float inv = 1.f / std::sqrt(l2); for(int k = 0; k < 3; ++k) n[k] *= inv; }
		uint32_t mi = static_cast<uint32_t>(face_material[i]);
		float w;
		std::memcpy(&w, &mi, 4);
		ng[i] = make_float4(n[0], n[1], n[2], w);
	}
	gbrt_scene *S = new gbrt_scene();
	S->bvh = bvh;
	S->lights_host = ls;
	S->mats_host = mats;
	S->face_quad.resize(n_faces);
	for(uint32_t i = 0; i < n_faces; ++i) S->face_quad[i] = faces[4ull * i + 3] != GBRT_TRIANGLE ? 1u : 0u;
	for(const DevMaterial &d : mats)
	{
		if((d.flags & BF_GLOSSY) && (d.flags & BF_REFLECT)) { S->split_glossy = true; if(d.flags & BF_TRANSMIT) S->split_glossy_transmit = true; }
		if(d.flags & (BF_SPECULAR | BF_FILTER)) S->split_specular = true;
		S->max_addl = std::max(S->max_addl, d.addl_depth);
	}
	S->n_prims = n_faces; S->n_mats = n_materials; S->n_lights = n_lights;
	auto fail = [&](int rc) { gbrt_scene_destroy(S); return rc; };
	cudaError_t e;
	if((e = cudaGetDevice(&S->device)) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e)));
	cudaDeviceGetAttribute(&S->n_sm, cudaDevAttrMultiProcessorCount, S->device);
	const auto T = gbrt::make_lds_tables();
	struct Up { void **dst; const void *src; size_t bytes; };
	const Up ups[] = {
		{reinterpret_cast<void **>(&S->prim_ng), ng.data(), ng.size() * sizeof(float4)},
		{reinterpret_cast<void **>(&S->mats), mats.data(), std::max<size_t>(1, mats.size()) * sizeof(DevMaterial)},
		{reinterpret_cast<void **>(&S->lights), ls.data(), std::max<size_t>(1, ls.size()) * sizeof(DevLight)},
		{reinterpret_cast<void **>(&S->lds_perm), T.perm.data(), T.perm.size() * sizeof(uint16_t)},
		{reinterpret_cast<void **>(&S->lds_off), T.offset.data(), T.offset.size() * sizeof(uint32_t)},
		{reinterpret_cast<void **>(&S->lds_base), T.base.data(), T.base.size() * sizeof(uint32_t)},
		{reinterpret_cast<void **>(&S->lds_inv), T.inv.data(), T.inv.size() * sizeof(double)},
		{reinterpret_cast<void **>(&S->lds_sfac), T.sfac.data(), T.sfac.size() * sizeof(double)},
		{reinterpret_cast<void **>(&S->lds_sfac_off), T.sfac_offset.data(), T.sfac_offset.size() * sizeof(uint32_t)},
		{reinterpret_cast<void **>(&S->lds_sfac_nd), T.sfac_digits.data(), T.sfac_digits.size() * sizeof(uint32_t)},
		{reinterpret_cast<void **>(&S->lds_fx), T.fx.data(), T.fx.size() * sizeof(uint4)},
	};
	S->lds_fx_dims = T.fx_dims;
	S->lds_fx_rad3 = T.fx_rad3;
	for(const Up &u : ups)
	{
		if((e = cudaMalloc(u.dst, u.bytes)) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_OOM, "gbrt_scene_create: %s", cudaGetErrorString(e)));
		const size_t src_bytes = u.bytes;
		if(u.src && (e = cudaMemcpy(*u.dst, u.src, src_bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "gbrt_scene_create: %s", cudaGetErrorString(e)));
	}
	*out = S;
	return GBRT_OK;
}

// Texture coordinates, image textures and the materials they drive.
int gbrt_scene_set_textures(gbrt_scene *S, const float *uv, uint32_t n_uv, const uint32_t *face_uv, const gbrt_texture_desc *textures,
                            uint32_t n_textures, const int32_t *material_diffuse_texture, uint32_t n_materials)
{
	if(!S) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: NULL scene");
	if((n_uv && !uv) || (n_textures && !textures) || (n_materials && !material_diffuse_texture) || (face_uv && !n_uv))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: NULL array");
	if(n_materials != S->n_mats)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: %u material entries for %u materials", n_materials, S->n_mats);
	std::vector<DevTexture> tex(std::max<uint32_t>(1, n_textures));
	size_t n_texels = 0;
	for(uint32_t i = 0; i < n_textures; ++i)
	{
		const gbrt_texture_desc &t = textures[i];
		const bool image = t.kind == GBRT_TEX_IMAGE;
		if(t.kind > GBRT_TEX_RGB_CUBE) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: kind %u", i, t.kind);
		if(image && (t.width <= 0 || t.height <= 0 || !t.rgba))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u has no image (%d x %d)", i, t.width, t.height);
		// the lookups index a texture's texels with 32-bit ints (y * w + x)
		if(image && static_cast<uint64_t>(t.width) * static_cast<uint64_t>(t.height) >= (1ull << 31))
			return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_scene_set_textures: texture %u has %d x %d texels (at most 2^31 - 1 per texture)",
			                      i, t.width, t.height);
		if(t.interpolate > GBRT_INTERP_BICUBIC || t.clipping > GBRT_CLIP_CHECKER || t.texco > GBRT_TEXCO_UV || t.mapping > GBRT_MAPPING_SPHERE)
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: unsupported interpolate / clipping / texco / mapping", i);
		DevTexture &d = tex[i];
		d.kind = t.kind;
		if(!image)
		{
			if(!S->noise_dev)
				return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u is procedural: set the noise tables first", i);
			const gbrt_procedural_desc &q = t.proc;
			if(q.noise_type > GBRT_NOISE_VORONOI_CRACKLE || q.noise_type2 > GBRT_NOISE_VORONOI_CRACKLE || q.distance_metric > GBRT_DIST_MINKOVSKY ||
			   q.bias > GBRT_BIAS_NEGATIVE || q.shape > GBRT_SHAPE_TRI || q.wood_type > GBRT_WOOD_RINGS ||
			   q.blend_type > GBRT_PROGRESSION_RADIAL || q.color_mode > GBRT_VORONOI_POSITION_OUTLINE_INTENSITY ||
			   q.musgrave_type > GBRT_MUSGRAVE_RIDGED || q.ramp_mode > GBRT_RAMP_HSL || q.ramp_interpolation > GBRT_RAMP_CONSTANT ||
			   q.ramp_hue_interpolation > GBRT_HUE_COUNTERCLOCKWISE || q.depth < 0 || q.depth > 30)
				return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: procedural parameter out of range", i);
			if(!gbrt::proc_from_desc(t, d.proc))
				return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: %d ramp items (at most %d)", i, q.ramp_n, GBRT_RAMP_MAX);
		}
		d.off = static_cast<uint32_t>(n_texels);
		d.w = image ? t.width : 0; d.h = image ? t.height : 0;
		d.interp = t.interpolate; d.clip = t.clipping; d.texco = t.texco; d.mapping = t.mapping;
		d.xrep = t.xrepeat; d.yrep = t.yrepeat; d.rot90 = t.rot90 ? 1 : 0;
		for(int k = 0; k < 4; ++k) d.crop[k] = t.crop[k];
		d.crop_x = (t.crop[0] != 0.f || t.crop[2] != 1.f) ? 1 : 0;      // texture_image.h:104-105
		d.crop_y = (t.crop[1] != 0.f || t.crop[3] != 1.f) ? 1 : 0;
		d.intensity = t.adj_intensity; d.contrast = t.adj_contrast;
		d.adj_ic = (t.adj_intensity != 1.f || t.adj_contrast != 1.f) ? 1 : 0;
		d.adj_clamp = t.adj_clamp ? 1 : 0;
		for(int k = 0; k < 3; ++k) d.mult[k] = t.adj_mult_factor[k];
		d.saturation = t.adj_saturation;
		d.hue6 = t.adj_hue / 60.f;
		d.adj = (d.adj_ic || d.adj_clamp || t.adj_mult_factor[0] != 1.f || t.adj_mult_factor[1] != 1.f || t.adj_mult_factor[2] != 1.f ||
		         t.adj_saturation != 1.f || t.adj_hue != 0.f) ? 1 : 0;
		d.layer = t.layer ? 1 : 0;
		if(t.blend_mode > GBRT_BLEND_LIGHTEN) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: blend mode %u", i, t.blend_mode);
		d.blend = static_cast<int>(t.blend_mode);
		d.negative = t.negative ? 1 : 0; d.no_rgb = t.no_rgb ? 1 : 0; d.stencil = t.stencil ? 1 : 0;
		d.mirror_x = t.mirror_x ? 1 : 0; d.mirror_y = t.mirror_y ? 1 : 0;
		d.even_tiles = t.even_tiles ? 1 : 0; d.odd_tiles = t.odd_tiles ? 1 : 0;
		d.checker_dist = t.checker_dist;
		d.colfac = t.colfac;
		for(int k = 0; k < 4; ++k) d.upper[k] = t.upper_color[k];
		for(int k = 0; k < 3; ++k) d.def_col[k] = t.def_col[k];
		for(int k = 0; k < 3; ++k)
		{
			if(t.proj[k] < 0 || t.proj[k] > 3) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: texture %u: proj %d", i, t.proj[k]);
			d.proj[k] = t.proj[k];
			d.scale[k] = t.scale[k];
			d.offset2[k] = 2.f * t.offset[k];
		}
		if(image) n_texels += static_cast<size_t>(t.width) * t.height;
		if(n_texels >= (1ull << 32)) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_scene_set_textures: more than 2^32 texels");
	}
	std::vector<float4> texels(std::max<size_t>(1, n_texels));
	for(uint32_t i = 0; i < n_textures; ++i)
		if(textures[i].kind == GBRT_TEX_IMAGE)
			std::memcpy(&texels[tex[i].off], textures[i].rgba, sizeof(float4) * static_cast<size_t>(textures[i].width) * textures[i].height);
	std::vector<uint4> fuv(std::max<uint32_t>(1, S->n_prims));
	for(uint32_t f = 0; f < S->n_prims; ++f)
	{
		const bool quad = S->face_quad[f] != 0;
		if(!face_uv) { fuv[f] = make_uint4(kNoIdx, kNoIdx, kNoIdx, quad ? 0u : kNoIdx); continue; }
		const uint32_t *q = face_uv + 4ull * f;
		for(int k = 0; k < (quad ? 4 : 3); ++k)
			if(q[k] >= n_uv) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: face %u uses uv %u of %u", f, q[k], n_uv);
		fuv[f] = make_uint4(q[0], q[1], q[2], quad ? q[3] : kNoIdx);
	}
	std::vector<DevMaterial> mats = S->mats_host;
	for(uint32_t m = 0; m < n_materials; ++m)
	{
		const int32_t t = material_diffuse_texture[m];
		if(t >= 0 && (static_cast<uint32_t>(t) >= n_textures || mats[m].type != GBRT_MAT_SHINYDIFFUSE))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_textures: material %u: texture %d (shinydiffuse only, %u textures)", m, t, n_textures);
		mats[m].dtex = t >= 0 ? t : -1;
	}
	std::lock_guard<std::mutex> lock(S->mu);
	if(S->ev_last) GBRT_CK(cudaEventSynchronize(S->ev_last));
	for(void *p : {static_cast<void *>(S->tex), static_cast<void *>(S->texels), static_cast<void *>(S->uv), static_cast<void *>(S->face_uv)})
		if(p) cudaFree(p);
	S->tex = nullptr; S->texels = nullptr; S->uv = nullptr; S->face_uv = nullptr;
	struct Up { void **dst; const void *src; size_t bytes; };
	const Up ups[] = {{reinterpret_cast<void **>(&S->tex), tex.data(), tex.size() * sizeof(DevTexture)},
	                  {reinterpret_cast<void **>(&S->texels), texels.data(), texels.size() * sizeof(float4)},
	                  {reinterpret_cast<void **>(&S->uv), n_uv ? static_cast<const void *>(uv) : nullptr, std::max<size_t>(1, n_uv) * sizeof(float2)},
	                  {reinterpret_cast<void **>(&S->face_uv), fuv.data(), fuv.size() * sizeof(uint4)}};
	for(const Up &u : ups)
	{
		GBRT_CK(cudaMalloc(u.dst, u.bytes));
		if(u.src) GBRT_CK(cudaMemcpy(*u.dst, u.src, u.bytes, cudaMemcpyHostToDevice));
	}
	GBRT_CK(cudaMemcpy(S->mats, mats.data(), mats.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice));
	S->mats_host = mats;
	S->n_tex = n_textures;
	return GBRT_OK;
}

int gbrt_scene_set_shader_nodes(gbrt_scene *S, const gbrt_shader_node *nodes, uint32_t n_nodes, const int32_t *slots, uint32_t n_materials)
{
	if(!S || (n_nodes && !nodes) || (n_materials && !slots)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: NULL argument");
	if(n_materials != S->n_mats)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: %u material entries for %u materials", n_materials, S->n_mats);
	for(uint32_t i = 0; i < n_nodes; ++i)
	{
		const gbrt_shader_node &N = nodes[i];
		const int32_t ii = static_cast<int32_t>(i);
		auto bad_input = [&](int32_t j) { return j >= ii || j < -1; };
		if(N.type > GBRT_NODE_LAYER || bad_input(N.input1) || bad_input(N.input2) || bad_input(N.input_factor))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: node %u: type %u or an input not below it", i, N.type);
		if(N.type == GBRT_NODE_TEXTURE && (N.texture < 0 || static_cast<uint32_t>(N.texture) >= S->n_tex))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: node %u: texture %d of %u (set the textures first)", i,
			                      N.texture, S->n_tex);
		if(N.type == GBRT_NODE_MIX && N.mode > GBRT_MIX_OVERLAY)
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: node %u: mix mode %u", i, N.mode);
		if(N.type == GBRT_NODE_LAYER && (N.input1 < 0 || N.mode > GBRT_BLEND_LIGHTEN))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: node %u: a layer needs an input and a blend mode", i);
	}
	std::vector<DevMaterial> mats = S->mats_host;
	for(uint32_t m = 0; m < n_materials; ++m)
	{
		DevMaterial &d = mats[m];
		d.has_nodes = 0u;
		for(int k = 0; k < GBRT_SLOTS; ++k)
		{
			const int32_t root = slots[static_cast<size_t>(m) * GBRT_SLOTS + k];
			d.nroot[k] = d.nfirst[k] = -1;
			d.nmask[k] = 0u;
			if(root < 0) continue;
			if(static_cast<uint32_t>(root) >= n_nodes)
				return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: material %u slot %d: node %d of %u", m, k, root, n_nodes);
			const bool ok = (k == GBRT_SLOT_BUMP && d.type != GBRT_MAT_LIGHT) ||
			                (k == GBRT_SLOT_DIFFUSE && (d.type == GBRT_MAT_SHINYDIFFUSE || d.type == GBRT_MAT_GLOSSY)) ||
			                (k == GBRT_SLOT_GLOSSY && d.type == GBRT_MAT_GLOSSY) ||
			                (k == GBRT_SLOT_MIRROR_COLOR && (d.type == GBRT_MAT_SHINYDIFFUSE || d.type == GBRT_MAT_GLASS || d.type == GBRT_MAT_ROUGH_GLASS)) ||
			                (k == GBRT_SLOT_FILTER_COLOR && (d.type == GBRT_MAT_GLASS || d.type == GBRT_MAT_ROUGH_GLASS));
			if(!ok)
				return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_shader_nodes: material %u (type %u) has no slot %d", m, d.type, k);
			// the nodes the root reads, through its inputs, and the lowest of them
			int32_t first = root;
			std::vector<int32_t> todo{root}, tree;
			while(!todo.empty())
			{
				const int32_t j = todo.back();
				todo.pop_back();
				first = std::min(first, j);
				tree.push_back(j);
				for(int32_t q : {nodes[j].input1, nodes[j].input2, nodes[j].input_factor})
					if(q >= 0) todo.push_back(q);
			}
			if(root - first + 1 > GBRT_TREE_MAX)
				return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_scene_set_shader_nodes: material %u slot %d: a tree spanning %d nodes (at most %d)",
				                      m, k, root - first + 1, GBRT_TREE_MAX);
			d.nroot[k] = root;
			d.nfirst[k] = first;
			for(int32_t j : tree) d.nmask[k] |= 1u << (j - first);
			d.has_nodes = 1u;
		}
	}
	bool bump = false;
	for(const DevMaterial &d : mats) bump = bump || d.nroot[GBRT_SLOT_BUMP] >= 0;
	std::lock_guard<std::mutex> lock(S->mu);
	if(S->ev_last) GBRT_CK(cudaEventSynchronize(S->ev_last));
	if(S->nodes) cudaFree(S->nodes);
	S->nodes = nullptr;
	if(bump && !S->prim_slot && S->n_prims)
	{
		// the inverse of the BVH's leaf order, for the faces' edge vectors
		GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&S->prim_slot), S->n_prims * sizeof(uint32_t)));
		k_prim_slot<<<(S->n_prims + 255) / 256, 256>>>(S->bvh->wids, S->n_prims, S->prim_slot);
		GBRT_CK(cudaGetLastError());
		GBRT_CK(cudaDeviceSynchronize());
	}
	GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&S->nodes), std::max<uint32_t>(1, n_nodes) * sizeof(gbrt_shader_node)));
	if(n_nodes) GBRT_CK(cudaMemcpy(S->nodes, nodes, n_nodes * sizeof(gbrt_shader_node), cudaMemcpyHostToDevice));
	GBRT_CK(cudaMemcpy(S->mats, mats.data(), mats.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice));
	S->mats_host = mats;
	return GBRT_OK;
}

int gbrt_scene_set_noise_tables(gbrt_scene *S, const gbrt_noise_tables *t)
{
	if(!S || !t || !t->hash || !t->hashpntf || !t->hashvectf || !t->stdp_p || !t->stdp_g)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_noise_tables: NULL argument");
	std::vector<uint8_t> b(kNoiseBytes, 0);
	std::memcpy(b.data() + kNoiseHash, t->hash, 512);
	std::memcpy(b.data() + kNoiseStdpP, t->stdp_p, 514);
	float *f = reinterpret_cast<float *>(b.data() + kNoiseFloats);
	std::memcpy(f, t->hashpntf, 4 * 768);
	std::memcpy(f + 768, t->hashvectf, 4 * 768);
	std::memcpy(f + 1536, t->stdp_g, 4 * 514 * 3);
	std::lock_guard<std::mutex> lock(S->mu);
	if(S->ev_last) GBRT_CK(cudaEventSynchronize(S->ev_last));
	if(!S->noise_dev) GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&S->noise_dev), kNoiseBytes));
	GBRT_CK(cudaMemcpy(S->noise_dev, b.data(), kNoiseBytes, cudaMemcpyHostToDevice));
	return GBRT_OK;
}

int gbrt_scene_set_normals(gbrt_scene *S, const float *normals, uint32_t n_normals, const uint32_t *face_normals)
{
	if(!S) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_normals: NULL scene");
	if(n_normals && !normals) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_normals: NULL normals");
	if(n_normals >= kTriFace) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_scene_set_normals: %u normals", n_normals);
	std::vector<float4> vn(std::max<uint32_t>(1, n_normals), make_float4(0.f, 0.f, 0.f, 0.f));
	for(uint32_t i = 0; i < n_normals; ++i) vn[i] = make_float4(normals[3ull * i], normals[3ull * i + 1], normals[3ull * i + 2], 0.f);
	std::vector<uint4> fn;
	if(face_normals)
	{
		fn.resize(std::max<uint32_t>(1, S->n_prims));
		for(uint32_t f = 0; f < S->n_prims; ++f)
		{
			const uint32_t *q = face_normals + 4ull * f;
			const bool quad = S->face_quad[f] != 0;
			if(q[0] == GBRT_FLAT_FACE) { fn[f] = make_uint4(kFlatFace, kFlatFace, kFlatFace, quad ? kFlatFace : kTriFace); continue; }
			for(int k = 0; k < (quad ? 4 : 3); ++k)
				if(q[k] != GBRT_NO_NORMAL && q[k] >= n_normals)
					return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_scene_set_normals: face %u uses normal %u of %u", f, q[k], n_normals);
			fn[f] = make_uint4(q[0], q[1], q[2], quad ? q[3] : kTriFace);
		}
	}
	std::lock_guard<std::mutex> lock(S->mu);
	if(S->ev_last) GBRT_CK(cudaEventSynchronize(S->ev_last));
	for(void *p : {static_cast<void *>(S->vnrm), static_cast<void *>(S->face_nrm)})
		if(p) cudaFree(p);
	S->vnrm = nullptr; S->face_nrm = nullptr;
	if(!face_normals) return GBRT_OK;
	GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&S->vnrm), vn.size() * sizeof(float4)));
	GBRT_CK(cudaMemcpy(S->vnrm, vn.data(), vn.size() * sizeof(float4), cudaMemcpyHostToDevice));
	GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&S->face_nrm), fn.size() * sizeof(uint4)));
	GBRT_CK(cudaMemcpy(S->face_nrm, fn.data(), fn.size() * sizeof(uint4), cudaMemcpyHostToDevice));
	return GBRT_OK;
}

int gbrt_scene_destroy(gbrt_scene *S)
{
	if(!S) return GBRT_OK;
	void *ptrs[] = {S->prim_ng, S->mats, S->lights, S->lds_perm, S->lds_off, S->lds_base, S->lds_inv, S->lds_sfac, S->lds_sfac_off,
	                S->lds_sfac_nd, S->lds_fx, S->work, S->spawn, S->spawn_count};
	for(void *p : ptrs) if(p) cudaFree(p);
	for(void *p : {static_cast<void *>(S->tex), static_cast<void *>(S->texels), static_cast<void *>(S->uv), static_cast<void *>(S->face_uv),
	               static_cast<void *>(S->vnrm), static_cast<void *>(S->face_nrm), static_cast<void *>(S->noise_dev), static_cast<void *>(S->nodes),
	               static_cast<void *>(S->prim_slot)})
		if(p) cudaFree(p);
	if(S->filter_dev) cudaFree(S->filter_dev);
	if(S->ev_last) cudaEventDestroy(S->ev_last);
	delete S;
	return GBRT_OK;
}

// ImageFilm filter table (imagefilm.cc:231-264, math/filter.h): filter
// width from AA_pixelwidth (x 2.6 Mitchell, x 2 Gauss, clamped to
// [0.501, 4]), table[y][x] = f((x + 0.5) / 16, (y + 0.5) / 16), table scale
// 0.9999 x 16 / width.  FAST_MATH exp and FAST_TRIG sin as the reference.
static int film_filter_table(uint32_t type, float pixel_width, float table[256], float &width, float &scale)
{
	using gbrt::fmul; using gbrt::fadd; using gbrt::fsub;
	width = (pixel_width > 0.f ? pixel_width : 1.5f) * 0.5f;
	if(type == GBRT_FILTER_MITCHELL) width *= 2.6f;
	else if(type == GBRT_FILTER_GAUSS) width *= 2.f;
	else if(type != GBRT_FILTER_BOX && type != GBRT_FILTER_LANCZOS)
		return gbrt_set_error(GBRT_ERR_INVALID, "film filter type %u unknown", type);
	width = std::min(std::max(0.501f, width), 0.5f * 8.f);
	for(int y = 0; y < 16; ++y)
		for(int x = 0; x < 16; ++x)
		{
			const float dx = fmul(fadd(static_cast<float>(x), 0.5f), 1.f / 16.f), dy = fmul(fadd(static_cast<float>(y), 0.5f), 1.f / 16.f);
			const float r2 = fadd(fmul(dx, dx), fmul(dy, dy));
			float f = 1.f;
			if(type == GBRT_FILTER_GAUSS)
				f = std::max(0.f, fsub(gbrt::fast_exp2(fmul(1.4426950408889634f, fmul(-6.f, r2))), 0.00247875f));
			else if(type == GBRT_FILTER_MITCHELL)
			{
				const float xx = fmul(2.f, std::sqrt(r2));
				if(xx >= 2.f) f = 0.f;
				else if(xx >= 1.f) f = fadd(fmul(xx, fsub(fmul(xx, fadd(fmul(xx, -0.38888889f), 2.0f)), 3.33333333f)), 1.77777778f);
				else f = fadd(fmul(fmul(xx, xx), fsub(fmul(1.16666666f, xx), 2.0f)), 0.88888889f);
			}
			else if(type == GBRT_FILTER_LANCZOS)
			{
				const float xx = std::sqrt(r2);
				if(xx == 0.f) f = 1.f;
				else if(-2.f < xx && xx < 2.f)
				{
					const float a = fmul(3.14159265358979323846f, xx), b = fmul(1.57079632679489661923f, xx);
					f = fmul(gbrt::fast_sin(a), gbrt::fast_sin(b)) / fmul(a, b);
				}
				else f = 0.f;
			}
			table[y * 16 + x] = f;
		}
	scale = fmul(0.9999f, 16.f) / width;
	return GBRT_OK;
}

// The wavefront render of gbrt_pt_render / gbrt_pm_render (scene lock held).
// pm: photonmapping setup (the PM fields of Params and its photon grids), or
// NULL for pathtracing.
// One pass of an adaptive anti-aliasing render (TiledIntegrator::render /
// renderPass): the pixels to sample (NULL: all), whether the render has
// more than one pass (sample positions), the light sample multiplier.
// The film filter of a render (ImageFilm's table and weights) into P.
static int film_setup(gbrt_scene *S, const gbrt_pt_params &pp, Params &P, cudaStream_t s)
{
	if(pp.filter_type == GBRT_FILTER_PIXEL) return GBRT_OK;
	if(!pp.film_weight_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render: filter type %u needs film_weight_dev", pp.filter_type);
	if(int rc = film_filter_table(pp.filter_type, pp.aa_pixel_width, S->filter_host, P.filter_width, P.filter_scale)) return rc;
	if(!S->filter_dev) GBRT_CK(cudaMalloc(&S->filter_dev, sizeof(S->filter_host)));
	GBRT_CK(cudaMemcpyAsync(S->filter_dev, S->filter_host, sizeof(S->filter_host), cudaMemcpyHostToDevice, s));
	P.film_w = pp.film_weight_dev;
	P.filter_tab = S->filter_dev;
	return GBRT_OK;
}

struct AaPass {
	const uint32_t *list;
	uint32_t n_list;
	int multipass;
	float lmult;
};

static int render_locked(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params &pp_in, const Params *pm, float *film_dev,
                         double *film64_dev, gbrt_pt_stats *stats, cudaStream_t s, const AaPass *aa = nullptr)
{
	gbrt_pt_params pp = pp_in;
	// the scene's buffers and filter table: after its previous render, whatever stream that used
	if(S->ev_last) GBRT_CK(cudaStreamWaitEvent(s, S->ev_last, 0));
	if(pm && pm->pm)
	{
		// camera sample = one integrate(); with final gathering, fg_samples gather
		// paths of fg_bounces + 1 vertices each (path_samples / bounces slots)
		pp.path_samples = pm->pm_fg ? pm->path_samples : 1;
		pp.bounces = pm->pm_fg ? pm->pm_fg_bounces + 1 : 0;
		pp.guide = nullptr;
		pp.guide_alpha = 0.f;
		pp.guide_train_steps = 0;
	}
	if(camera->resx <= 0 || camera->resy <= 0 || pp.spp <= 0 || pp.path_samples <= 0 || pp.bounces < 0 || pp.path_samples > 64)
		return gbrt_set_error(GBRT_ERR_INVALID, "render: bad resolution or sampling parameters");
	const uint64_t n_pixels = (aa && aa->list) ? aa->n_list : static_cast<uint64_t>(camera->resx) * camera->resy;
	const float lmult = aa ? aa->lmult : 1.f;
	const uint64_t total = n_pixels * pp.spp * pp.path_samples;
	if(total >= (1ull << 32)) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pt_render: %llu paths exceed 2^32", static_cast<unsigned long long>(total));
	gbrt_guide *guide = pp.guide;
	if(pp.guide_batch > kMaxBatch) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pt_render: guide_batch %u > %u", pp.guide_batch, kMaxBatch);
	const bool guiding = guide && pp.guide_alpha > 0.f;
	const bool record = guide && pp.guide_train_steps > 0;
	uint64_t wave = std::min<uint64_t>(total, pp.wave_paths ? pp.wave_paths : (record ? (1ull << 20) : (1ull << 22)));
	// recursive split: spawned integrate() calls go to one buffer per ray
	// level; waves are cut so one wave's children always fit a buffer
	const int raydepth = pp.raydepth > 0 ? pp.raydepth : 5;
	const uint32_t fanout = split_fanout(S, pp.path_samples);
	const int split_levels = fanout ? std::min(19, raydepth + static_cast<int>(S->max_addl)) : 0;
	// spawn records per wave: only the first path sample of an integrate()
	// call spawns (at most `fanout` records); a camera wave of W paths holds
	// at most W / path_samples + 2 such roots, a chunk of c spawned records at
	// most c / n_min + 1, n_min = the fewest path samples a spawned call gets
	// (the glossy split divides by up to 8)
	constexpr uint64_t kSpawnCap = 1ull << 24;
	const uint64_t ps = static_cast<uint64_t>(pp.path_samples);
	const uint64_t n_min = std::max<uint64_t>(1, ps / (S->split_glossy ? 8u : 1u));
	size_t spawn_cap = 0;
	uint64_t chunk = wave;
	if(split_levels > 0)
	{
		const uint64_t roots = std::max<uint64_t>(1, kSpawnCap / fanout - 2);
		wave = std::max<uint64_t>(1, std::min<uint64_t>(wave, roots * ps));
		spawn_cap = static_cast<size_t>((wave / ps + 2) * fanout);
		chunk = std::max<uint64_t>(1, std::min<uint64_t>(wave, (spawn_cap / fanout - 1) * n_min));
		if(int rc = alloc_spawn(S, spawn_cap, split_levels, s)) return rc;
	}
	uint32_t max_shadow = 0;
	{
		uint32_t all = 0, one = 0;
		for(const auto &l : S->lights_host)
		{
			const uint32_t n = 2u * static_cast<uint32_t>(std::ceil(static_cast<float>(l.samples) * lmult));
			all += n;
			one = std::max(one, n);
		}
		max_shadow = std::max(all, one);
	}
	const size_t shadow_cap = std::max<size_t>(1, wave * max_shadow);
	const uint32_t stride = static_cast<uint32_t>(std::max(1, pp.bounces));
	if(int rc = alloc_work(S, wave, shadow_cap, guide ? stride : 0, s)) return rc;
	Camera cam = make_camera(*camera);
	const SceneDev sc = scene_dev(S);
	Params P{};
	P.spp = pp.spp; P.path_samples = pp.path_samples; P.bounces = pp.bounces; P.rr_min = pp.russian_roulette_min_bounces;
	P.raydepth = raydepth;
	P.film_resx = camera->resx;
	P.film_resy = camera->resy;
	P.lmult = lmult;
	P.aa_multipass = aa ? aa->multipass : 0;
	P.pix_list = aa ? aa->list : nullptr;
	P.n_list = aa ? aa->n_list : 0u;
	P.tshadow = pp.transparent_shadows ? 1 : 0;
	P.shadow_depth = pp.shadow_depth;
	if(int rc = film_setup(S, pp, P, s)) return rc;
	if(pm)
	{
		P.pm = pm->pm; P.pm_fg = pm->pm_fg; P.pm_fg_bounces = pm->pm_fg_bounces; P.pm_gather_dist = pm->pm_gather_dist;
		P.pm_diffuse = pm->pm_diffuse; P.pm_caustics = pm->pm_caustics; P.pm_diffuse_r2 = pm->pm_diffuse_r2; P.pm_diffuse_k = pm->pm_diffuse_k;
		P.pm_caustic_r2 = pm->pm_caustic_r2; P.pm_caustic_k = pm->pm_caustic_k; P.pm_diffuse_paths = pm->pm_diffuse_paths;
		P.pm_caustic_paths = pm->pm_caustic_paths; P.pm_lookup_r2 = pm->pm_lookup_r2;
		P.g_diffuse = pm->g_diffuse; P.g_caustic = pm->g_caustic; P.g_radiance = pm->g_radiance;
		P.sppm_r2 = pm->sppm_r2; P.sppm_pass = pm->sppm_pass;
		P.sppm_ire = pm->sppm_ire; P.sppm_ire_r2 = pm->sppm_ire_r2; P.sppm_ire_k = pm->sppm_ire_k;
	}
	P.base_offset = pp.base_sampling_offset; P.seed = pp.seed;
	P.pt_caustic_path = (pp.caustic_type == GBRT_CAUSTIC_PATH || pp.caustic_type == GBRT_CAUSTIC_BOTH) ? 1 : 0;
	P.no_recursive = pp.no_recursive ? 1 : 0;
	P.clamp_indirect = pp.clamp_indirect;
	P.d1 = 1.f / static_cast<float>(pp.spp);
	P.n_lights = S->n_lights;
	P.guiding = guiding ? 1 : 0;
	P.alpha = guiding ? std::min(1.f, pp.guide_alpha) : 0.f;
	P.record = record ? 1 : 0;
	P.rec_stride = stride;
	Work W = S->w;
	if(!record) W.p_sum = nullptr;
	float *film = film64_dev ? nullptr : film_dev;
	// the lean shading kernel serves pathtracing over plain scenes; kernels
	// with the texture and node-tree code only serve scenes that use them
	const bool plain = !pm && plain_scene(S);
	const bool tex = textured_scene(S);
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	if(stats)
	{
		GBRT_CK(cudaEventCreate(&e0)); GBRT_CK(cudaEventCreate(&e1));
		GBRT_CK(cudaEventRecord(e0, s));
	}
	GBRT_CK(cudaMemsetAsync(S->w.stats, 0, 2 * sizeof(unsigned long long), s));
	// one wave: the paths in the path slots (count[0] of them, at most n)
	// advance vertex by vertex
	auto vertex_loop = [&](Params &Pw, const Work &Ww, uint32_t n, bool camera_wave) -> int {
		Pw.wave_n = n;
		int cur = 0;
		for(int vtx = 0; vtx <= pp.bounces; ++vtx)
		{
			// guide only the first guide_max_vertex vertex levels (a wavefront
			// level holds the paths' vertex vtx, so the network runs only there)
			const bool level_guided = guiding && (pp.guide_max_vertex == 0 || vtx < static_cast<int>(pp.guide_max_vertex));
			Pw.guiding = level_guided ? 1 : 0;
			Pw.record = (camera_wave && record && (pp.guide_max_vertex == 0 || vtx < static_cast<int>(pp.guide_max_vertex))) ? 1 : 0;
			k_reset<<<1, 1, 0, s>>>(Ww.count, cur ^ 1);
			k_extend<<<persistent_grid(k_extend, n, S->n_sm), kThreads, 0, s>>>(sc.bv, Ww.q_ray[cur], Ww.count + cur, Ww.count + 4, Ww.hits,
			                                                                     level_guided ? Ww.hitpos : nullptr);
			if(vtx == 0 && (Pw.pm_caustics || (Pw.pm && Pw.pm_diffuse && !Pw.pm_fg)))
			{
				if(tex) k_pm_root<true><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, film, film64_dev);
				else k_pm_root<false><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, film, film64_dev);
			}
			if(level_guided)
				if(int rc = gbrt_guide_eval_queue(guide, Ww.hitpos, n, Ww.count + cur, Ww.lobes, s)) return rc;
			if(plain && !Pw.guiding && !Pw.record)
				k_shade_plain<<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, static_cast<uint32_t>(shadow_cap), film, film64_dev);
			else if(guide)
			{
				// the guided instances also serve the vertex levels past guide_max_vertex (no guiding, no records there)
				if(tex) k_shade<true, true><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, static_cast<uint32_t>(shadow_cap), film, film64_dev);
				else k_shade<false, true><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, static_cast<uint32_t>(shadow_cap), film, film64_dev);
			}
			else if(tex)
				k_shade<true, false><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, static_cast<uint32_t>(shadow_cap), film, film64_dev);
			else
				k_shade<false, false><<<grid_for(n, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, cur, static_cast<uint32_t>(shadow_cap), film, film64_dev);
			const uint32_t scap = static_cast<uint32_t>(shadow_cap);
			if(Pw.film_w && Pw.tshadow && tex)
				k_shadow<true, true, true><<<persistent_grid(k_shadow<true, true, true>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film,
				                                                                                                          film64_dev);
			else if(Pw.tshadow && tex)
				k_shadow<false, true, true><<<persistent_grid(k_shadow<false, true, true>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film,
				                                                                                                            film64_dev);
			else if(Pw.film_w && Pw.tshadow)
				k_shadow<true, true><<<persistent_grid(k_shadow<true, true>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film, film64_dev);
			else if(Pw.film_w)
				k_shadow<true, false><<<persistent_grid(k_shadow<true, false>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film, film64_dev);
			else if(Pw.tshadow)
				k_shadow<false, true><<<persistent_grid(k_shadow<false, true>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film, film64_dev);
			else
				k_shadow<false, false><<<persistent_grid(k_shadow<false, false>, shadow_cap, S->n_sm), kThreads, 0, s>>>(sc, Pw, Ww, scap, film, film64_dev);
			cur ^= 1;
		}
		return GBRT_OK;
	};
	// spawn buffer of ray level L (1 .. split_levels)
	auto spawn_buf = [&](int L) { return S->spawn + static_cast<size_t>(L - 1) * spawn_cap * 5; };
	auto spawn_target = [&](Work &Ww, int child_level) -> int {
		if(child_level > split_levels) { Ww.sp_out = nullptr; Ww.sp_count = nullptr; Ww.sp_cap = 0; return GBRT_OK; }
		Ww.sp_out = spawn_buf(child_level);
		Ww.sp_count = S->spawn_count + (child_level - 1);
		Ww.sp_cap = static_cast<uint32_t>(spawn_cap);
		GBRT_CK(cudaMemsetAsync(Ww.sp_count, 0, sizeof(uint32_t), s));
		return GBRT_OK;
	};
	auto spawned = [&](int child_level, uint32_t &n) -> int {
		n = 0;
		if(child_level > split_levels) return GBRT_OK;
		GBRT_CK(cudaMemcpyAsync(&n, S->spawn_count + (child_level - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
		GBRT_CK(cudaStreamSynchronize(s));
		if(n > spawn_cap) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pt_render: %u spawned rays at level %d exceed %zu", n, child_level, spawn_cap);
		return GBRT_OK;
	};
	// integrate() calls of ray level L, depth first: a chunk of them, then
	// everything they spawned, then the next chunk
	std::function<int(int, uint32_t)> process_level = [&](int L, uint32_t n) -> int {
		for(uint32_t c0 = 0; c0 < n; c0 += static_cast<uint32_t>(chunk))
		{
			const uint32_t cn = static_cast<uint32_t>(std::min<uint64_t>(chunk, n - c0));
			Params Pc = P;
			Work Wc = W;
			Wc.p_sum = nullptr;
			if(int rc = spawn_target(Wc, L + 1)) return rc;
			GBRT_CK(cudaMemsetAsync(Wc.count, 0, sizeof(uint32_t), s));
			k_spawn_init<<<grid_for(cn, S->n_sm), kThreads, 0, s>>>(Wc, spawn_buf(L) + 5ull * c0, cn);
			if(int rc = vertex_loop(Pc, Wc, cn, false)) return rc;
			uint32_t nc = 0;
			if(int rc = spawned(L + 1, nc)) return rc;
			if(nc)
				if(int rc = process_level(L + 1, nc)) return rc;
		}
		return GBRT_OK;
	};
	for(uint64_t start = 0; start < total; start += wave)
	{
		P.wave_start = static_cast<uint32_t>(start);
		P.wave_n = static_cast<uint32_t>(std::min<uint64_t>(wave, total - start));
		Work Wv = W;
		if(int rc = spawn_target(Wv, 1)) return rc;
		k_camera<<<grid_for(P.wave_n, S->n_sm), kThreads, 0, s>>>(cam, P, Wv);
		if(int rc = vertex_loop(P, Wv, P.wave_n, true)) return rc;
		if(record)
		{
			GBRT_CK(cudaMemsetAsync(W.count + 3, 0, sizeof(uint32_t), s));
			k_make_records<<<grid_for(static_cast<size_t>(P.wave_n) * stride, S->n_sm), kThreads, 0, s>>>(W, P.wave_n, stride,
			                                                                                             (pp.flags & GBRT_PT_GUIDE_RADIANCE) ? 1 : 0);
			uint32_t n_rec = 0;
			GBRT_CK(cudaMemcpyAsync(&n_rec, W.count + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
			GBRT_CK(cudaStreamSynchronize(s));
			n_rec = std::min(n_rec, W.train_cap);
			const uint32_t batch = pp.guide_batch ? pp.guide_batch : 65536u;
			if(n_rec > 0)
				for(uint32_t st = 0; st < pp.guide_train_steps; ++st)
				{
					float *bbuf = W.train + 8ull * W.train_cap - 8ull * batch;   // batch area at the end of the buffer
					if(static_cast<uint64_t>(n_rec) + batch > W.train_cap)
					{
						n_rec = W.train_cap > batch ? W.train_cap - batch : 0;
						if(n_rec == 0) break;
					}
					k_gather_batch<<<grid_for(batch, S->n_sm), kThreads, 0, s>>>(reinterpret_cast<const float4 *>(W.train), n_rec, batch,
					                                                          pp.seed * 7919u + static_cast<uint32_t>(start) + st * 131u,
					                                                          reinterpret_cast<float4 *>(bbuf));
					if(int rc = gbrt_guide_step(guide, bbuf, batch, nullptr, s)) return rc;
				}
		}
		uint32_t nc = 0;
		if(int rc = spawned(1, nc)) return rc;
		if(nc)
			if(int rc = process_level(1, nc)) return rc;
	}
	GBRT_CK(cudaGetLastError());
	if(!S->ev_last) GBRT_CK(cudaEventCreateWithFlags(&S->ev_last, cudaEventDisableTiming));
	GBRT_CK(cudaEventRecord(S->ev_last, s));
	if(stats)
	{
		GBRT_CK(cudaEventRecord(e1, s));
		unsigned long long st[2];
		GBRT_CK(cudaMemcpyAsync(st, S->w.stats, sizeof(st), cudaMemcpyDeviceToHost, s));
		GBRT_CK(cudaStreamSynchronize(s));
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		cudaEventDestroy(e0); cudaEventDestroy(e1);
		*stats = gbrt_pt_stats{};
		stats->camera_samples = total / pp.path_samples;
		stats->extension_rays = st[0];
		stats->shadow_rays = st[1];
		stats->ms = ms;
	}
	return GBRT_OK;
}

// PathIntegrator::preprocess with caustic_type photon or both
// (integrator_path_tracer.cc:100-103): the caustic photon map of
// CausticPhotonIntegrator::createCausticMap, gridded for the estimate at the
// roots of the camera paths (integrator_path_tracer.cc:164-171).
struct PtCaustics {
	Params M{};
	ShotMap C;
	GridStore G;
	bool on = false;
};

static int pt_caustics(gbrt_scene *S, const gbrt_pt_params &pp, PtCaustics &K, cudaStream_t s)
{
	if(pp.caustic_type > GBRT_CAUSTIC_BOTH) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render: caustic_type %u", pp.caustic_type);
	if(pp.caustic_type != GBRT_CAUSTIC_PHOTON && pp.caustic_type != GBRT_CAUSTIC_BOTH) return GBRT_OK;
	gbrt_pm_params d{};
	gbrt_pm_default_params(&d);
	const gbrt_pm_params &c = pp.caustic ? *pp.caustic : d;
	if(c.caustic_mix < 1 || c.caustic_mix > gbrt::kMaxGather || !(c.caustic_radius > 0.f) || c.caustic_depth < 0 || c.caustic_photons < 0)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render: bad caustic parameters (caustic_mix in [1, %d])", gbrt::kMaxGather);
	float bound[6];
	if(int rc = gbrt_bvh_get_bound(S->bvh, bound)) return rc;
	const float lo[3] = {bound[0], bound[1], bound[2]};
	const uint32_t seed = pp.seed * 0x9e3779b9u + pp.base_sampling_offset;
	if(int rc = shoot_map(S, scene_dev(S), true, static_cast<uint32_t>(c.caustic_photons), c.caustic_depth, false, seed, K.C, s)) return rc;
	if(int rc = build_grid(K.C.pos.as<float4>(), K.C.dir.as<float4>(), K.C.col.as<float4>(), K.C.n, c.caustic_radius, lo, S->n_sm, K.G, s))
		return rc;
	K.M.pm_caustics = 1;
	K.M.pm_caustic_r2 = c.caustic_radius * c.caustic_radius;
	K.M.pm_caustic_k = c.caustic_mix;
	K.M.pm_caustic_paths = static_cast<float>(K.C.paths);
	K.M.g_caustic = K.G.g;
	K.on = true;
	return GBRT_OK;
}

int gbrt_pt_render(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, float *film_dev, double *film64_dev,
                   gbrt_pt_stats *stats, void *stream)
{
	if(!S || !camera || !params) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render: NULL argument");
	if(!film_dev && !film64_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render: no film buffer");
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	std::lock_guard<std::mutex> lock(S->mu);
	PtCaustics K;
	if(int rc = pt_caustics(S, *params, K, s)) return rc;
	const int rc = render_locked(S, camera, *params, K.on ? &K.M : nullptr, film_dev, film64_dev, stats, s);
	if(K.on) cudaStreamSynchronize(s);       // the caustic map is freed on return
	return rc;
}

// Device film around a render call, per-pixel means copied to the host.
static int render_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params_in, const gbrt_pm_params *pm,
                       float *image_out, gbrt_pt_stats *stats, int kind)
{
	const size_t n_pix = static_cast<size_t>(camera->resx) * camera->resy, n = 3 * n_pix;
	gbrt_pt_params params = *params_in;
	const bool fp64 = (params.flags & GBRT_PT_FP64_FILM) != 0;
	const bool filtered = params.filter_type != GBRT_FILTER_PIXEL;
	DevBuf sum, mean, weight;
	if(int rc = sum.alloc(n * (fp64 ? 8 : 4))) return rc;
	if(int rc = mean.alloc(n * 4)) return rc;
	if(filtered)
	{
		if(int rc = weight.alloc(n_pix * 4)) return rc;
		GBRT_CK(cudaMemset(weight.p, 0, n_pix * 4));
		params.film_weight_dev = weight.as<float>();
	}
	GBRT_CK(cudaMemset(sum.p, 0, n * (fp64 ? 8 : 4)));
	float *f32 = fp64 ? nullptr : sum.as<float>();
	double *f64 = fp64 ? sum.as<double>() : nullptr;
	const int rc = kind == 1 ? gbrt_pm_render(S, camera, &params, pm, f32, f64, stats, nullptr)
	             : kind == 2 ? gbrt_dl_render(S, camera, &params, pm, f32, f64, stats, nullptr)
	                         : gbrt_pt_render(S, camera, &params, f32, f64, stats, nullptr);
	if(rc) return rc;
	if(filtered) k_normalize<<<grid_for(n, S->n_sm), kThreads>>>(f32, f64, weight.as<float>(), mean.as<float>(), n);
	else k_mean<<<grid_for(n, S->n_sm), kThreads>>>(f32, f64, mean.as<float>(), n, 1.f / static_cast<float>(params.spp));
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(image_out, mean.p, n * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_pt_render_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, float *image_out, gbrt_pt_stats *stats)
{
	if(!S || !camera || !params || !image_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_host: NULL argument");
	return render_host(S, camera, params, nullptr, image_out, stats, 0);
}

int gbrt_pm_render_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                        float *image_out, gbrt_pt_stats *stats)
{
	if(!S || !camera || !params || !pm || !image_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render_host: NULL argument");
	return render_host(S, camera, params, pm, image_out, stats, 1);
}

int gbrt_dl_render_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                        float *image_out, gbrt_pt_stats *stats)
{
	if(!S || !camera || !params || !image_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_dl_render_host: NULL argument");
	return render_host(S, camera, params, caustic, image_out, stats, 2);
}

// ---- adaptive anti-aliasing passes ----

// ImageFilm::nextPass detection (imagefilm.cc:399-512): flags and the list of
// flagged pixels on stream s; the number flagged on the host.
static int aa_detect(const float *film, const float *w, int W, int H, const gbrt_aa_params &a, float thr, uint8_t *flags, uint32_t *list,
                     uint32_t *d_count, uint32_t &n_flagged, int n_sm, cudaStream_t s)
{
	const uint32_t n = static_cast<uint32_t>(W) * static_cast<uint32_t>(H);
	k_aa_init<<<grid_for(n, n_sm), kThreads, 0, s>>>(w, n, flags);
	if(W > 1 && H > 1)
	{
		const AaDev d{thr, a.detect_color_noise != 0, a.dark_detection_type, a.dark_threshold_factor, a.variance_edge_size / 2, a.variance_pixels};
		k_aa_detect<<<grid_for(static_cast<size_t>(W - 1) * (H - 1), n_sm), kThreads, 0, s>>>(film, w, W, H, d, flags);
	}
	GBRT_CK(cudaMemsetAsync(d_count, 0, 4, s));
	k_aa_compact<<<grid_for(n, n_sm), kThreads, 0, s>>>(flags, n, list, d_count);
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpyAsync(&n_flagged, d_count, 4, cudaMemcpyDeviceToHost, s));
	GBRT_CK(cudaStreamSynchronize(s));
	return GBRT_OK;
}

static int aa_check(const gbrt_aa_params &a, const char *who)
{
	if(a.passes < 1 || a.inc_samples < 0 || a.variance_edge_size < 0 || a.dark_detection_type < 0 || a.dark_detection_type > 2)
		return gbrt_set_error(GBRT_ERR_INVALID, "%s: bad AA parameters (passes %d, inc_samples %d, variance_edge_size %d, dark_detection_type %d)",
		                      who, a.passes, a.inc_samples, a.variance_edge_size, a.dark_detection_type);
	return GBRT_OK;
}

// TiledIntegrator::render's pass loop (integrator_tiled.cc:160-214): pass 0
// renders every pixel with AA_samples; pass i multiplies the sample and
// light-sample multipliers, re-runs the detection (skipped once a pass
// flagged nothing and the threshold stayed), renders ceil(inc_samples x
// sample multiplier) more samples per flagged pixel (every pixel when the
// threshold is <= 0, ImageFilm::doMoreSamples, imagefilm.cc:763-766) at
// sample offset base + samples so far, and lowers the threshold by
// 10 % x min(8, floor / flagged) while fewer than the floor were flagged.
static int aa_render_locked(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params &pp, const gbrt_aa_params &a, float *film,
                            gbrt_pt_stats *stats, uint32_t *resampled, cudaStream_t s, const Params *pm = nullptr)
{
	const int W = camera->resx, H = camera->resy;
	if(W <= 0 || H <= 0) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa: bad resolution");
	const uint32_t n_pix = static_cast<uint32_t>(W) * static_cast<uint32_t>(H);
	DevBuf flags, list, count;
	if(a.passes > 1)
	{
		if(int rc = flags.alloc(n_pix)) return rc;
		if(int rc = list.alloc(4ull * n_pix)) return rc;
		if(int rc = count.alloc(4)) return rc;
	}
	gbrt_pt_stats sum{}, one{};
	auto add = [&]() {
		sum.camera_samples += one.camera_samples; sum.extension_rays += one.extension_rays;
		sum.shadow_rays += one.shadow_rays; sum.ms += one.ms;
	};
	const AaPass first{nullptr, 0, a.passes > 1 ? 1 : 0, 1.f};
	if(int rc = render_locked(S, camera, pp, pm, film, nullptr, stats ? &one : nullptr, s, &first)) return rc;
	add();
	if(resampled) resampled[0] = n_pix;
	float smult = 1.f, lmult = 1.f, thr = a.threshold;
	bool thr_changed = true;
	int64_t n_res = 0;
	uint32_t acum = static_cast<uint32_t>(pp.spp);
	const int floor_pix = static_cast<int>(floorf(a.resampled_floor * static_cast<float>(n_pix) / 100.f));
	for(int i = 1; i < a.passes; ++i)
	{
		smult *= a.sample_multiplier_factor;
		lmult *= a.light_sample_multiplier_factor;
		const bool all = !(thr > 0.f);
		if(n_res > 0 || thr_changed)
		{
			if(all) n_res = n_pix;
			else
			{
				uint32_t nf = 0;
				if(int rc = aa_detect(film, pp.film_weight_dev, W, H, a, thr, flags.as<uint8_t>(), list.as<uint32_t>(), count.as<uint32_t>(), nf, S->n_sm, s)) return rc;
				n_res = nf;
			}
			thr_changed = false;
		}
		const int mult = static_cast<int>(ceilf(static_cast<float>(a.inc_samples) * smult));
		if(n_res > 0 && mult > 0)
		{
			gbrt_pt_params q = pp;
			q.spp = mult;
			q.base_sampling_offset = pp.base_sampling_offset + acum;
			const AaPass pass{all ? nullptr : list.as<uint32_t>(), all ? 0u : static_cast<uint32_t>(n_res), 1, lmult};
			if(int rc = render_locked(S, camera, q, pm, film, nullptr, stats ? &one : nullptr, s, &pass)) return rc;
			add();
		}
		if(resampled) resampled[i] = static_cast<uint32_t>(std::max<int64_t>(0, n_res));
		acum += static_cast<uint32_t>(mult);
		if(n_res < floor_pix)
		{
			const float ratio = std::min(8.f, static_cast<float>(floor_pix) / static_cast<float>(n_res));
			thr = thr * (1.f - 0.1f * ratio);
			if(a.threshold > 0.f) thr_changed = true;
		}
	}
	if(stats) *stats = sum;
	return GBRT_OK;
}

int gbrt_pt_render_aa(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_aa_params *aa, float *film_dev,
                      gbrt_pt_stats *stats, uint32_t *resampled, void *stream)
{
	if(!S || !camera || !params || !aa || !film_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa: NULL argument");
	if(int rc = aa_check(*aa, "gbrt_pt_render_aa")) return rc;
	if(params->filter_type == GBRT_FILTER_PIXEL || !params->film_weight_dev)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa: adaptive AA needs a filtered film (filter_type != PIXEL, film_weight_dev)");
	if(params->guide) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa: no path guide in adaptive AA renders");
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	std::lock_guard<std::mutex> lock(S->mu);
	PtCaustics K;
	if(int rc = pt_caustics(S, *params, K, s)) return rc;
	const int rc = aa_render_locked(S, camera, *params, *aa, film_dev, stats, resampled, s, K.on ? &K.M : nullptr);
	if(K.on) cudaStreamSynchronize(s);
	return rc;
}

int gbrt_pt_render_aa_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params_in, const gbrt_aa_params *aa,
                           float *image_out, gbrt_pt_stats *stats, uint32_t *resampled)
{
	if(!S || !camera || !params_in || !aa || !image_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa_host: NULL argument");
	if(camera->resx <= 0 || camera->resy <= 0) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa_host: bad resolution");
	if(params_in->filter_type == GBRT_FILTER_PIXEL)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_aa_host: adaptive AA needs a filtered film (filter_type != PIXEL)");
	const size_t n_pix = static_cast<size_t>(camera->resx) * camera->resy, n = 3 * n_pix;
	gbrt_pt_params params = *params_in;
	DevBuf sum, mean, weight;
	if(int rc = sum.alloc(n * 4)) return rc;
	if(int rc = mean.alloc(n * 4)) return rc;
	if(int rc = weight.alloc(n_pix * 4)) return rc;
	GBRT_CK(cudaMemset(sum.p, 0, n * 4));
	GBRT_CK(cudaMemset(weight.p, 0, n_pix * 4));
	params.film_weight_dev = weight.as<float>();
	if(int rc = gbrt_pt_render_aa(S, camera, &params, aa, sum.as<float>(), stats, resampled, nullptr)) return rc;
	k_normalize<<<grid_for(n, S->n_sm), kThreads>>>(sum.as<float>(), nullptr, weight.as<float>(), mean.as<float>(), n);
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(image_out, mean.p, n * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_aa_flags(const float *film_dev, const float *weight_dev, int32_t resx, int32_t resy, const gbrt_aa_params *aa, float threshold,
                  uint8_t *flags_dev, uint32_t *n_flagged)
{
	if(!film_dev || !weight_dev || !aa || !flags_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_aa_flags: NULL argument");
	if(resx <= 0 || resy <= 0) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_aa_flags: bad resolution");
	if(int rc = aa_check(*aa, "gbrt_aa_flags")) return rc;
	int dev = 0, n_sm = 0;
	GBRT_CK(cudaGetDevice(&dev));
	GBRT_CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
	DevBuf count;
	if(int rc = count.alloc(4)) return rc;
	uint32_t nf = 0;
	if(int rc = aa_detect(film_dev, weight_dev, resx, resy, *aa, threshold, flags_dev, nullptr, count.as<uint32_t>(), nf, n_sm, nullptr)) return rc;
	if(n_flagged) *n_flagged = nf;
	return GBRT_OK;
}

// Diagnostics: evaluates one sampling primitive on n inputs, on the device
// (on_device != 0) or with the host build of the same code.
int gbrt_sampler_eval(int kind, int dim, const uint32_t *input, uint32_t n, double *out, int on_device)
{
	if(!input || !out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sampler_eval: NULL buffer");
	if(kind < 0 || kind > 10 || ((kind == 0 || kind == 9) && (dim < 1 || dim >= gbrt::kLdsDims)))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sampler_eval: bad kind %d / dim %d", kind, dim);
	const auto T = gbrt::make_lds_tables();
	if(!on_device)
	{
		const gbrt::LdsTables t = T.view();
		for(uint32_t i = 0; i < n; ++i) out[i] = sampler_value(t, kind, dim, input[i]);
		return GBRT_OK;
	}
	if(n == 0) return GBRT_OK;
	void *d_perm = nullptr, *d_off = nullptr, *d_base = nullptr, *d_inv = nullptr, *d_in = nullptr, *d_out = nullptr;
	void *d_sf = nullptr, *d_sfo = nullptr, *d_sfd = nullptr, *d_fx = nullptr;
	int rc = GBRT_OK;
	cudaError_t e = cudaSuccess;
	struct Up { void **dst; const void *src; size_t bytes; };
	const Up ups[] = {{&d_perm, T.perm.data(), T.perm.size() * 2}, {&d_off, T.offset.data(), T.offset.size() * 4},
	                  {&d_base, T.base.data(), T.base.size() * 4}, {&d_inv, T.inv.data(), T.inv.size() * 8},
	                  {&d_sf, T.sfac.data(), T.sfac.size() * 8}, {&d_sfo, T.sfac_offset.data(), T.sfac_offset.size() * 4},
	                  {&d_sfd, T.sfac_digits.data(), T.sfac_digits.size() * 4}, {&d_fx, T.fx.data(), T.fx.size() * sizeof(uint4)},
	                  {&d_in, input, 4ull * n}, {&d_out, nullptr, 8ull * n}};
	for(const Up &u : ups)
	{
		if(e == cudaSuccess) e = cudaMalloc(u.dst, u.bytes);
		if(e == cudaSuccess && u.src) e = cudaMemcpy(*u.dst, u.src, u.bytes, cudaMemcpyHostToDevice);
	}
	if(e == cudaSuccess)
	{
		const gbrt::LdsTables t{static_cast<uint16_t *>(d_perm), static_cast<uint32_t *>(d_off), static_cast<uint32_t *>(d_base),
		                        static_cast<double *>(d_inv), static_cast<double *>(d_sf), static_cast<uint32_t *>(d_sfo), static_cast<uint32_t *>(d_sfd),
		                        static_cast<uint4 *>(d_fx), T.fx_dims, T.fx_rad3};
		k_sampler<<<(n + 127) / 128, 128>>>(t, kind, dim, static_cast<const uint32_t *>(d_in), n, static_cast<double *>(d_out));
		e = cudaGetLastError();
		if(e == cudaSuccess) e = cudaMemcpy(out, d_out, 8ull * n, cudaMemcpyDeviceToHost);
	}
	if(e != cudaSuccess) rc = gbrt_set_error(GBRT_ERR_CUDA, "gbrt_sampler_eval: %s", cudaGetErrorString(e));
	for(void *p : {d_perm, d_off, d_base, d_inv, d_sf, d_sfo, d_sfd, d_fx, d_in, d_out}) if(p) cudaFree(p);
	return rc;
}

int gbrt_pm_default_params(gbrt_pm_params *p)
{
	if(!p) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_default_params: NULL");
	// PhotonIntegrator / CausticPhotonIntegrator parameter defaults
	// (integrator_photon_mapping.h:65-74, integrator_photon_caustic.h:44-49)
	p->diffuse_photons = 100000;
	p->caustic_photons = 500000;
	p->diffuse_radius = 0.1f;
	p->diffuse_search = 50;
	p->caustic_radius = 0.25f;
	p->caustic_mix = 50;
	p->caustic_depth = 10;
	p->bounces = 3;
	p->caustics = 0;
	p->diffuse = 1;
	p->final_gather = 1;
	p->fg_samples = 32;
	p->fg_bounces = 2;
	p->fg_min_pathlen = -1.f;
	return GBRT_OK;
}

int gbrt_pm_photons(gbrt_scene *S, const gbrt_pm_params *pm, int which, float *out, uint32_t cap, uint32_t *n_photons, uint32_t *n_paths)
{
	if(!S || !pm || (which != 0 && which != 1)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_photons: bad argument");
	std::lock_guard<std::mutex> lock(S->mu);
	const SceneDev sc = scene_dev(S);
	ShotMap M;
	const bool caustic = which == 1;
	if(int rc = shoot_map(S, sc, caustic, static_cast<uint32_t>(std::max(0, caustic ? pm->caustic_photons : pm->diffuse_photons)),
	                      caustic ? pm->caustic_depth : pm->bounces, false, 1u, M, nullptr)) return rc;
	if(n_photons) *n_photons = M.n;
	if(n_paths) *n_paths = M.paths;
	if(out && M.n)
	{
		if(cap < M.n) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pm_photons: %u photons, room for %u", M.n, cap);
		std::vector<float4> p(M.n), d(M.n), c(M.n);
		GBRT_CK(cudaMemcpy(p.data(), M.pos.p, 16ull * M.n, cudaMemcpyDeviceToHost));
		GBRT_CK(cudaMemcpy(d.data(), M.dir.p, 16ull * M.n, cudaMemcpyDeviceToHost));
		GBRT_CK(cudaMemcpy(c.data(), M.col.p, 16ull * M.n, cudaMemcpyDeviceToHost));
		for(uint32_t i = 0; i < M.n; ++i)
		{
			float *o = out + 9ull * i;
			o[0] = d[i].x; o[1] = d[i].y; o[2] = d[i].z;
			o[3] = p[i].x; o[4] = p[i].y; o[5] = p[i].z;
			o[6] = c[i].x; o[7] = c[i].y; o[8] = c[i].z;
		}
	}
	return GBRT_OK;
}

int gbrt_knn_gather(const float *points, uint32_t n, const float *queries, uint32_t m, float cell, int k, float r2,
                    int32_t *count_out, float *r2_out, uint32_t *idx_out)
{
	if((n && !points) || (m && (!queries || !count_out || !r2_out || !idx_out)) || !(cell > 0.f) || k < 1 || k > gbrt::kMaxGather)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_knn_gather: bad argument (k in [1, %d], cell > 0)", gbrt::kMaxGather);
	if(!(cell * cell >= r2)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_knn_gather: cell edge %g below the search radius", cell);
	int dev = 0, n_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
	std::vector<float4> p4(n);
	float lo[3] = {0.f, 0.f, 0.f};
	for(uint32_t i = 0; i < n; ++i)
	{
		p4[i] = make_float4(points[3ull * i], points[3ull * i + 1], points[3ull * i + 2], 0.f);
		for(int a = 0; a < 3; ++a) lo[a] = i ? std::min(lo[a], points[3ull * i + a]) : points[3ull * i + a];
	}
	DevBuf raw, q, cnt, rr, idx;
	if(int rc = raw.alloc(16ull * n)) return rc;
	if(int rc = q.alloc(12ull * m)) return rc;
	if(int rc = cnt.alloc(4ull * m)) return rc;
	if(int rc = rr.alloc(4ull * m)) return rc;
	if(int rc = idx.alloc(4ull * m * k)) return rc;
	GBRT_CK(cudaMemcpy(raw.p, p4.data(), 16ull * n, cudaMemcpyHostToDevice));
	GBRT_CK(cudaMemcpy(q.p, queries, 12ull * m, cudaMemcpyHostToDevice));
	GBRT_CK(cudaMemset(idx.p, 0xFF, 4ull * m * k));
	if(n) k_index_w<<<grid_for(n, n_sm), kThreads>>>(raw.as<float4>(), n);
	GridStore G;
	if(int rc = build_grid(raw.as<float4>(), nullptr, nullptr, n, cell, lo, n_sm, G, nullptr)) return rc;
	if(m) k_knn_test<<<grid_for(m, n_sm), kThreads>>>(G.g, q.as<float>(), m, k, r2, cnt.as<int32_t>(), rr.as<float>(), idx.as<uint32_t>());
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(count_out, cnt.p, 4ull * m, cudaMemcpyDeviceToHost));
	GBRT_CK(cudaMemcpy(r2_out, rr.p, 4ull * m, cudaMemcpyDeviceToHost));
	GBRT_CK(cudaMemcpy(idx_out, idx.p, 4ull * m * k, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

// photonmapping: the photon maps once (PhotonIntegrator::preprocess), then
// one render, or the adaptive passes (aa) over them.
static int pm_render_impl(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                          float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream, const gbrt_aa_params *aa,
                          uint32_t *resampled)
{
	if(!S || !camera || !params || !pm) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render: NULL argument");
	if(!film_dev && !film64_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render: no film buffer");
	const gbrt_pm_params &q = *pm;
	if(q.diffuse_search < 1 || q.diffuse_search > gbrt::kMaxGather || q.caustic_mix < 1 || q.caustic_mix > gbrt::kMaxGather ||
	   !(q.diffuse_radius > 0.f) || !(q.caustic_radius > 0.f) || q.fg_samples < 1 || q.fg_samples > 64 || q.fg_bounces < 0 ||
	   q.bounces < 0 || q.caustic_depth < 0 || q.diffuse_photons < 0 || q.caustic_photons < 0)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render: bad photon-mapping parameters (searches in [1, %d], fg_samples in [1, 64])", gbrt::kMaxGather);
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	std::lock_guard<std::mutex> lock(S->mu);
	const SceneDev sc = scene_dev(S);
	float bound[6];
	if(int rc = gbrt_bvh_get_bound(S->bvh, bound)) return rc;
	const float lo[3] = {bound[0], bound[1], bound[2]};
	const bool fg = q.final_gather && q.diffuse;
	const float dr = q.diffuse_radius;
	Params M{};
	M.pm = 1;
	M.pm_fg = fg ? 1 : 0;
	M.path_samples = q.fg_samples;
	M.pm_fg_bounces = q.fg_bounces;
	M.pm_gather_dist = q.fg_min_pathlen < 0.f ? dr : q.fg_min_pathlen;
	M.pm_diffuse = q.diffuse ? 1 : 0;
	M.pm_caustics = q.caustics ? 1 : 0;
	M.pm_diffuse_r2 = dr;
	M.pm_diffuse_k = q.diffuse_search;
	M.pm_caustic_r2 = q.caustic_radius * q.caustic_radius;
	M.pm_caustic_k = q.caustic_mix;
	M.pm_lookup_r2 = 4.f * dr * dr;
	const uint32_t seed = params->seed * 0x9e3779b9u + params->base_sampling_offset;
	cudaEvent_t p0 = nullptr, p1 = nullptr;
	if(stats)
	{
		GBRT_CK(cudaEventCreate(&p0)); GBRT_CK(cudaEventCreate(&p1));
		GBRT_CK(cudaEventRecord(p0, s));
	}
	uint32_t n_radiance = 0;
	ShotMap D, C;
	GridStore GD, GC, GP, GR;
	DevBuf st0, st1, und, rpos, rdir, rcol, rcnt;
	if(q.diffuse)
	{
		if(int rc = shoot_map(S, sc, false, static_cast<uint32_t>(q.diffuse_photons), q.bounces, fg, seed, D, s)) return rc;
		if(D.n < 50) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render: too few diffuse photons (%u)", D.n);
		M.pm_diffuse_paths = static_cast<float>(D.paths);
		if(int rc = build_grid(D.pos.as<float4>(), D.dir.as<float4>(), D.col.as<float4>(), D.n, fg ? dr : std::sqrt(dr), lo, S->n_sm, GD, s)) return rc;
		M.g_diffuse = GD.g;
	}
	if(q.caustics)
	{
		if(int rc = shoot_map(S, sc, true, static_cast<uint32_t>(q.caustic_photons), q.caustic_depth, false, seed, C, s)) return rc;
		M.pm_caustic_paths = static_cast<float>(C.paths);
		if(int rc = build_grid(C.pos.as<float4>(), C.dir.as<float4>(), C.col.as<float4>(), C.n, q.caustic_radius, lo, S->n_sm, GC, s)) return rc;
		M.g_caustic = GC.g;
	}
	if(fg)
	{
		// radiance map: thin the radiance points, pre-gather their radiance,
		// grid them for findNearest within 2 x diffuse_radius
		const uint32_t n = D.n_rp;
		const float r2c = 0.01f * dr;
		if(n) k_index_w<<<grid_for(n, S->n_sm), kThreads, 0, s>>>(D.rp_pos.as<float4>(), n);
		if(int rc = build_grid(D.rp_pos.as<float4>(), D.rp_nrm.as<float4>(), nullptr, n, std::sqrt(r2c), lo, S->n_sm, GP, s)) return rc;
		if(int rc = st0.alloc(n)) return rc;
		if(int rc = st1.alloc(n)) return rc;
		if(int rc = und.alloc(4)) return rc;
		GBRT_CK(cudaMemsetAsync(st0.p, 0, n, s));
		uint8_t *sa = st0.as<uint8_t>(), *sb = st1.as<uint8_t>();
		for(int round = 0; n; ++round)
		{
			if(round == 4096) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render: radiance point thinning did not settle");
			GBRT_CK(cudaMemsetAsync(und.p, 0, 4, s));
			k_rp_round<<<grid_for(n, S->n_sm), kThreads, 0, s>>>(GP.g, r2c, seed, sa, sb, und.as<uint32_t>());
			std::swap(sa, sb);
			uint32_t left = 0;
			GBRT_CK(cudaMemcpyAsync(&left, und.p, 4, cudaMemcpyDeviceToHost, s));
			GBRT_CK(cudaStreamSynchronize(s));
			if(!left) break;
		}
		if(int rc = rpos.alloc(16ull * n)) return rc;
		if(int rc = rdir.alloc(16ull * n)) return rc;
		if(int rc = rcol.alloc(16ull * n)) return rc;
		if(int rc = rcnt.alloc(4)) return rc;
		GBRT_CK(cudaMemsetAsync(rcnt.p, 0, 4, s));
		const float inv_scale = 1.f / (static_cast<float>(D.paths) * 3.14159265358979323846f);
		if(n)
			k_pregather<<<grid_for(n, S->n_sm), kThreads, 0, s>>>(GP.g, sa, D.rp_refl.as<float4>(), D.rp_transm.as<float4>(), GD.g, dr * dr,
			                                                   q.diffuse_search, inv_scale, rpos.as<float4>(), rdir.as<float4>(), rcol.as<float4>(),
			                                                   rcnt.as<uint32_t>());
		uint32_t nr = 0;
		GBRT_CK(cudaMemcpyAsync(&nr, rcnt.p, 4, cudaMemcpyDeviceToHost, s));
		GBRT_CK(cudaStreamSynchronize(s));
		if(int rc = build_grid(rpos.as<float4>(), rdir.as<float4>(), rcol.as<float4>(), nr, 2.f * dr, lo, S->n_sm, GR, s)) return rc;
		M.g_radiance = GR.g;
		n_radiance = nr;
	}
	float photon_ms = 0.f;
	if(stats)
	{
		GBRT_CK(cudaEventRecord(p1, s));
		GBRT_CK(cudaEventSynchronize(p1));
		cudaEventElapsedTime(&photon_ms, p0, p1);
		cudaEventDestroy(p0); cudaEventDestroy(p1);
	}
	if(aa && aa->indirect_sample_multiplier_factor != 1.f && fg)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pm_render_aa: AA_indirect_sample_multiplier_factor != 1 is not built");
	const int rc = aa ? aa_render_locked(S, camera, *params, *aa, film_dev, stats, resampled, s, &M)
	                  : render_locked(S, camera, *params, &M, film_dev, film64_dev, stats, s);
	cudaStreamSynchronize(s);      // the photon buffers are freed on return
	if(stats && !rc)
	{
		stats->photon_paths = static_cast<uint64_t>(D.paths) + C.paths;
		stats->photons_stored = static_cast<uint64_t>(D.n) + C.n;
		stats->radiance_photons = n_radiance;
		stats->photon_ms = photon_ms;
	}
	return rc;
}

// SppmIntegrator::render (integrator_sppm.cc:99-201): initializePpm, then per
// pass the photon pass (prePass: the caustic photons of this pass's photon
// paths, gridded with cells of the initial radius, which bounds every later
// one), one eye sample per pixel and the hit points' refinement.
static int sppm_locked(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params &pp, const gbrt_sppm_params &q, float *film,
                       gbrt_pt_stats *stats, cudaStream_t s)
{
	const uint32_t n_pix = static_cast<uint32_t>(camera->resx) * static_cast<uint32_t>(camera->resy);
	float bound[6];
	if(int rc = gbrt_bvh_get_bound(S->bvh, bound)) return rc;
	const float lo[3] = {bound[0], bound[1], bound[2]};
	// initializePpm (:1054-1073): the scene bound's mean edge over the mean resolution, x 2, at most 1
	float r0 = (((bound[3] - bound[0]) + (bound[4] - bound[1]) + (bound[5] - bound[2])) / 3.f) /
	           (static_cast<float>(camera->resx + camera->resy) / 2.0f) * 2.f;
	r0 = std::min(r0, 1.f);
	DevBuf hp, r2, pass, ire;
	if(int rc = hp.alloc(16ull * n_pix)) return rc;
	if(int rc = r2.alloc(4ull * n_pix)) return rc;
	if(int rc = pass.alloc(16ull * n_pix)) return rc;
	if(q.pm_ire)
	{
		if(int rc = ire.alloc(n_pix)) return rc;
		GBRT_CK(cudaMemsetAsync(ire.p, 0, n_pix, s));
	}
	// grid cells bound every query radius: the initial one, or photonRadius with pmIRE
	const float cell = q.pm_ire ? std::max(r0, q.photon_radius) : r0;
	k_sppm_init<<<grid_for(n_pix, S->n_sm), kThreads, 0, s>>>(hp.as<float4>(), r2.as<float>(), pass.as<float4>(), n_pix, (r0 * 1.f) * (r0 * 1.f));
	GBRT_CK(cudaGetLastError());
	const SceneDev sc = scene_dev(S);
	Params M{};
	M.pm = 3;
	M.pm_diffuse = 1;          // launches the root gather (k_pm_root)
	M.pm_caustics = 1;
	M.sppm_r2 = r2.as<float>();
	M.sppm_pass = pass.as<float4>();
	gbrt_pt_params e = pp;
	e.spp = 1;
	e.guide = nullptr; e.guide_alpha = 0.f; e.guide_train_steps = 0;
	Params F{};                // the film view of the refinement kernel
	F.spp = 1; F.path_samples = 1; F.d1 = 1.f;
	F.film_resx = camera->resx; F.film_resy = camera->resy;
	F.aa_multipass = 1;
	if(int rc = film_setup(S, pp, F, s)) return rc;
	const AaPass multipass{nullptr, 0, 1, 1.f};
	gbrt_pt_stats sum{}, one{};
	uint64_t total = 0, stored = 0;
	const uint32_t n_ph = static_cast<uint32_t>(q.photons);
	for(int i = 0; i < q.passes; ++i)
	{
		ShotMap C, D;
		GridStore GC, GD;
		// photon paths of sample index base_sampling_offset + i: one render's
		// passes use the Halton indices the reference's generators run through,
		// renders at disjoint sample offsets disjoint photon paths
		const uint64_t base = (static_cast<uint64_t>(pp.base_sampling_offset) + static_cast<uint64_t>(i)) * n_ph;
		if(base + n_ph >= (1ull << 32)) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_sppm_render: more than 2^32 photon paths");
		if(int rc = shoot_map(S, sc, true, n_ph, q.bounces, false, pp.seed, C, s, true, static_cast<uint32_t>(base))) return rc;
		total += n_ph;
		stored += C.n;
		if(int rc = build_grid(C.pos.as<float4>(), C.dir.as<float4>(), C.col.as<float4>(), C.n, cell, lo, S->n_sm, GC, s)) return rc;
		M.g_caustic = GC.g;
		M.sppm_ire = nullptr;
		M.g_diffuse = gbrt::PhotonGrid{};
		if(q.pm_ire && i == 0)
		{
			// the first pass's diffuse map (the same photon paths' non-caustic indirect deposits)
			if(int rc = shoot_map(S, sc, false, n_ph, q.bounces, false, pp.seed, D, s, true, static_cast<uint32_t>(base))) return rc;
			if(int rc = build_grid(D.pos.as<float4>(), D.dir.as<float4>(), D.col.as<float4>(), D.n, cell, lo, S->n_sm, GD, s)) return rc;
			M.g_diffuse = GD.g;
			M.sppm_ire = ire.as<uint8_t>();
			M.sppm_ire_r2 = q.photon_radius * q.photon_radius;
			M.sppm_ire_k = q.search_num;
		}
		e.base_sampling_offset = pp.base_sampling_offset + static_cast<uint32_t>(i);
		if(int rc = render_locked(S, camera, e, &M, film, nullptr, stats ? &one : nullptr, s, &multipass)) return rc;
		F.base_offset = e.base_sampling_offset;
		k_sppm_update<<<grid_for(n_pix, S->n_sm), kThreads, 0, s>>>(F, hp.as<float4>(), r2.as<float>(), pass.as<float4>(), n_pix,
		                                                         static_cast<float>(total), film);
		GBRT_CK(cudaGetLastError());
		GBRT_CK(cudaStreamSynchronize(s));     // the pass's photon buffers are freed at the end of the iteration
		if(stats)
		{
			sum.camera_samples += one.camera_samples; sum.extension_rays += one.extension_rays;
			sum.shadow_rays += one.shadow_rays; sum.ms += one.ms;
		}
	}
	if(stats)
	{
		*stats = sum;
		stats->photon_paths = total;
		stats->photons_stored = stored;
	}
	return GBRT_OK;
}

int gbrt_sppm_render(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_sppm_params *sppm,
                     float *film_dev, gbrt_pt_stats *stats, void *stream)
{
	if(!S || !camera || !params || !sppm || !film_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sppm_render: NULL argument");
	if(sppm->photons < 1 || sppm->passes < 1 || sppm->bounces < 0 || camera->resx <= 0 || camera->resy <= 0 ||
	   (sppm->pm_ire && (sppm->search_num < 1 || sppm->search_num > gbrt::kMaxGather || !(sppm->photon_radius > 0.f))))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sppm_render: bad parameters (photons %d, passes %d, bounces %d)", sppm->photons,
		                      sppm->passes, sppm->bounces);
	std::lock_guard<std::mutex> lock(S->mu);
	return sppm_locked(S, camera, *params, *sppm, film_dev, stats, static_cast<cudaStream_t>(stream));
}

int gbrt_sppm_render_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params_in, const gbrt_sppm_params *sppm,
                          float *image_out, gbrt_pt_stats *stats)
{
	if(!S || !camera || !params_in || !sppm || !image_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sppm_render_host: NULL argument");
	if(camera->resx <= 0 || camera->resy <= 0 || sppm->passes < 1) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_sppm_render_host: bad parameters");
	const size_t n_pix = static_cast<size_t>(camera->resx) * camera->resy, n = 3 * n_pix;
	gbrt_pt_params params = *params_in;
	const bool filtered = params.filter_type != GBRT_FILTER_PIXEL;
	DevBuf sum, mean, weight;
	if(int rc = sum.alloc(n * 4)) return rc;
	if(int rc = mean.alloc(n * 4)) return rc;
	GBRT_CK(cudaMemset(sum.p, 0, n * 4));
	if(filtered)
	{
		if(int rc = weight.alloc(n_pix * 4)) return rc;
		GBRT_CK(cudaMemset(weight.p, 0, n_pix * 4));
		params.film_weight_dev = weight.as<float>();
	}
	if(int rc = gbrt_sppm_render(S, camera, &params, sppm, sum.as<float>(), stats, nullptr)) return rc;
	if(filtered) k_normalize<<<grid_for(n, S->n_sm), kThreads>>>(sum.as<float>(), nullptr, weight.as<float>(), mean.as<float>(), n);
	else k_mean<<<grid_for(n, S->n_sm), kThreads>>>(sum.as<float>(), nullptr, mean.as<float>(), n, 1.f / static_cast<float>(sppm->passes));
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(image_out, mean.p, n * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_pm_render(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                   float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream)
{
	return pm_render_impl(S, camera, params, pm, film_dev, film64_dev, stats, stream, nullptr, nullptr);
}

// ---- a batch of scenes in one wavefront --------------------------------------
// Every scene's camera samples form one index range (scene after scene, each
// in its own sample-major order); a wave is a stretch of that range, so the
// kernels of a vertex level serve all scenes at once (k_camera_batch,
// k_extend_batch, k_shade_batch, k_shadow_batch) and the spawned calls of
// the recursive split carry their scene along.  The first scene's work and
// spawn buffers serve the batch.

struct BatchPlan {
	uint32_t wave;              // paths per wave
	uint32_t shade_block;       // threads per block of k_shade_batch
	uint32_t trace_bps;         // resident blocks per SM of the persistent traversal grids
	uint32_t streams;           // waves in flight: one stream (and host thread) each
};

// Resident blocks per SM of a persistent kernel at kThreads threads.
static int max_blocks_per_sm(const void *kernel)
{
	int bps = 1;
	if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, kThreads, 0) != cudaSuccess || bps < 1) bps = 1;
	return bps;
}

// Spawn records a batch wave may leave per ray level (80 bytes each).
constexpr uint64_t kBatchSpawnCap = 1ull << 24;

static int batch_render_locked(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params,
                               float *const *films, uint32_t n, const BatchPlan &plan, int spp_override, gbrt_pt_stats *stats,
                               cudaStream_t s)
{
	gbrt_scene *S0 = scenes[0];
	const bool tshadow = params[0].transparent_shadows != 0;
	const bool filtered = params[0].filter_type != GBRT_FILTER_PIXEL;
	bool tex = false;
	for(uint32_t i = 0; i < n; ++i) tex = tex || textured_scene(scenes[i]);
	std::vector<BatchScene> host(n);
	uint64_t total = 0;
	uint32_t fanout = 0, max_shadow = 0;
	int split_levels = 0, bounces = 0;
	uint64_t n_min = ~0ull;
	for(uint32_t i = 0; i < n; ++i)
	{
		gbrt_scene *S = scenes[i];
		gbrt_pt_params pp = params[i];
		if(spp_override > 0) pp.spp = spp_override;
		const gbrt_camera_desc &c = cameras[i];
		if(S->device != S0->device) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: scene %u is on another device", i);
		if(pp.guide || (pp.caustic_type != GBRT_CAUSTIC_PATH && pp.caustic_type != GBRT_CAUSTIC_NONE))
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: scene %u: no guide or photon caustics in a batch", i);
		if((pp.transparent_shadows != 0) != tshadow || (pp.filter_type != GBRT_FILTER_PIXEL) != filtered)
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: scene %u: film filtering and transparent shadows must agree", i);
		if(c.resx <= 0 || c.resy <= 0 || pp.spp <= 0 || pp.path_samples <= 0 || pp.bounces < 0 || pp.path_samples > 64 || !films[i])
			return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: scene %u: bad resolution, sampling parameters or film", i);
		if(S->ev_last) GBRT_CK(cudaStreamWaitEvent(s, S->ev_last, 0));
		BatchScene &B = host[i];
		B.sc = scene_dev(S);
		Params &P = B.P;
		P = Params{};
		P.spp = pp.spp; P.path_samples = pp.path_samples; P.bounces = pp.bounces; P.rr_min = pp.russian_roulette_min_bounces;
		P.raydepth = pp.raydepth > 0 ? pp.raydepth : 5;
		P.film_resx = c.resx; P.film_resy = c.resy;
		P.lmult = 1.f;
		P.tshadow = pp.transparent_shadows ? 1 : 0;
		P.shadow_depth = pp.shadow_depth;
		if(int rc = film_setup(S, pp, P, s)) return rc;
		P.base_offset = pp.base_sampling_offset; P.seed = pp.seed;
		P.pt_caustic_path = pp.caustic_type == GBRT_CAUSTIC_PATH ? 1 : 0;
		P.no_recursive = pp.no_recursive ? 1 : 0;
		P.clamp_indirect = pp.clamp_indirect;
		P.d1 = 1.f / static_cast<float>(pp.spp);
		P.n_lights = S->n_lights;
		B.cam = make_camera(c);
		B.film = films[i];
		const uint64_t paths = static_cast<uint64_t>(c.resx) * c.resy * pp.spp * pp.path_samples;
		B.path_begin = static_cast<uint32_t>(total);
		B.paths = static_cast<uint32_t>(paths);
		total += paths;
		if(total >= (1ull << 32)) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pt_render_multi: more than 2^32 paths in the batch");
		const uint32_t f = split_fanout(S, pp.path_samples);
		fanout = std::max(fanout, f);
		if(f) split_levels = std::max(split_levels, std::min(19, P.raydepth + static_cast<int>(S->max_addl)));
		n_min = std::min<uint64_t>(n_min, std::max<uint64_t>(1, static_cast<uint64_t>(pp.path_samples) / (S->split_glossy ? 8u : 1u)));
		bounces = std::max(bounces, pp.bounces);
		uint32_t all = 0, one = 0;
		for(const auto &l : S->lights_host)
		{
			const uint32_t ns = 2u * static_cast<uint32_t>(std::ceil(static_cast<float>(l.samples)));
			all += ns;
			one = std::max(one, ns);
		}
		max_shadow = std::max(max_shadow, std::max(all, one));
	}
	// waves are cut so the spawned calls of one wave always fit
	uint64_t wave = std::min<uint64_t>(total, std::max<uint32_t>(plan.wave, 256u));
	size_t spawn_cap = 0;
	uint64_t chunk = wave;
	if(split_levels > 0)
	{
		const uint64_t roots = std::max<uint64_t>(1, kBatchSpawnCap / fanout - 2);
		wave = std::max<uint64_t>(1, std::min<uint64_t>(wave, roots));
		spawn_cap = static_cast<size_t>((wave + 2) * fanout);
		chunk = std::max<uint64_t>(1, std::min<uint64_t>(wave, (spawn_cap / fanout - 1) * n_min));
	}
	const size_t shadow_cap = std::max<size_t>(1, wave * max_shadow);
	const uint64_t n_waves = (total + wave - 1) / wave;
	// every stream works in its own scene's buffers (the scenes are locked)
	const uint32_t n_streams = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>({plan.streams ? plan.streams : 1u, n, n_waves})));
	BatchScene *table = nullptr;
	GBRT_CK(cudaMallocAsync(reinterpret_cast<void **>(&table), sizeof(BatchScene) * n, s));
	GBRT_CK(cudaMemcpyAsync(table, host.data(), sizeof(BatchScene) * n, cudaMemcpyHostToDevice, s));
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	GBRT_CK(cudaEventCreate(&e0));
	GBRT_CK(cudaEventCreate(&e1));
	GBRT_CK(cudaEventRecord(e0, s));
	const int n_sm = S0->n_sm;
	const uint32_t scap = static_cast<uint32_t>(shadow_cap);
	const uint32_t sblock = std::max(32u, std::min<uint32_t>(kThreads, plan.shade_block & ~31u));
	static const int bps_extend = max_blocks_per_sm(reinterpret_cast<const void *>(k_extend_batch));
	static const int bps_shadow[4] = {max_blocks_per_sm(reinterpret_cast<const void *>(k_shadow_batch<false, false>)),
	                                  max_blocks_per_sm(reinterpret_cast<const void *>(k_shadow_batch<false, true>)),
	                                  max_blocks_per_sm(reinterpret_cast<const void *>(k_shadow_batch<true, false>)),
	                                  max_blocks_per_sm(reinterpret_cast<const void *>(k_shadow_batch<true, true>))};
	auto trace_grid = [&](size_t nq, int bps_max) {
		const int bps = std::max(1, std::min<int>(bps_max, plan.trace_bps ? static_cast<int>(plan.trace_bps) : bps_max));
		const size_t want = (nq + kThreads - 1) / kThreads;
		return static_cast<unsigned>(std::max<size_t>(1, std::min(want, static_cast<size_t>(n_sm) * bps)));
	};
	std::atomic<uint64_t> next_wave{0};
	std::atomic<int> first_rc{GBRT_OK};
	std::mutex err_mu;
	std::string err_msg;
	std::vector<unsigned long long> rays(2ull * n_streams, 0ull);
	std::vector<cudaEvent_t> done(n_streams, nullptr);
	auto fail = [&](int rc) {
		int expect = GBRT_OK;
		if(first_rc.compare_exchange_strong(expect, rc))
		{
			std::lock_guard<std::mutex> g(err_mu);
			err_msg = gbrt_last_error();
		}
		return rc;
	};
	// one stream's share of the waves
	auto worker = [&](uint32_t k) -> int {
		if(cudaSetDevice(S0->device) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: cudaSetDevice"));
		gbrt_scene *H = scenes[k];                 // the buffers this stream works in
		cudaStream_t st = s;
		if(k > 0 && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: stream creation"));
		if(k > 0) cudaStreamWaitEvent(st, e0, 0);
		int rc = GBRT_OK;
		if(split_levels > 0) rc = alloc_spawn(H, spawn_cap, split_levels, st);
		if(!rc) rc = alloc_work(H, wave, shadow_cap, 0, st);
		Work W = H->w;
		if(!rc && cudaMemsetAsync(W.stats, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess)
			rc = gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: memset");
		auto vertex_loop = [&](const Work &Ww, uint32_t nq) {
			int cur = 0;
			for(int vtx = 0; vtx <= bounces; ++vtx)
			{
				k_reset<<<1, 1, 0, st>>>(Ww.count, cur ^ 1);
				k_extend_batch<<<trace_grid(nq, bps_extend), kThreads, 0, st>>>(table, Ww, cur);
				const unsigned blocks = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((nq + sblock - 1) / sblock,
				                                                                                   static_cast<size_t>(n_sm) * 16 * (kThreads / sblock))));
				if(tex) k_shade_batch<true><<<blocks, sblock, 0, st>>>(table, Ww, cur, scap);
				else k_shade_batch<false><<<blocks, sblock, 0, st>>>(table, Ww, cur, scap);
				const unsigned sg = trace_grid(shadow_cap, bps_shadow[(filtered ? 2 : 0) + (tshadow ? 1 : 0)]);
				if(filtered && tshadow && tex) k_shadow_batch<true, true, true><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				else if(tshadow && tex) k_shadow_batch<false, true, true><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				else if(filtered && tshadow) k_shadow_batch<true, true><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				else if(filtered) k_shadow_batch<true, false><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				else if(tshadow) k_shadow_batch<false, true><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				else k_shadow_batch<false, false><<<sg, kThreads, 0, st>>>(table, Ww, scap);
				cur ^= 1;
			}
		};
		auto spawn_buf = [&](int L) { return H->spawn + static_cast<size_t>(L - 1) * spawn_cap * 5; };
		auto spawn_target = [&](Work &Ww, int child_level) -> int {
			if(child_level > split_levels) { Ww.sp_out = nullptr; Ww.sp_count = nullptr; Ww.sp_cap = 0; return GBRT_OK; }
			Ww.sp_out = spawn_buf(child_level);
			Ww.sp_count = H->spawn_count + (child_level - 1);
			Ww.sp_cap = static_cast<uint32_t>(spawn_cap);
			GBRT_CK(cudaMemsetAsync(Ww.sp_count, 0, sizeof(uint32_t), st));
			return GBRT_OK;
		};
		auto spawned = [&](int child_level, uint32_t &nc) -> int {
			nc = 0;
			if(child_level > split_levels) return GBRT_OK;
			GBRT_CK(cudaMemcpyAsync(&nc, H->spawn_count + (child_level - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
			GBRT_CK(cudaStreamSynchronize(st));
			if(nc > spawn_cap)
				return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_pt_render_multi: %u spawned rays at level %d exceed %zu", nc, child_level, spawn_cap);
			return GBRT_OK;
		};
		std::function<int(int, uint32_t)> process_level = [&](int L, uint32_t nl) -> int {
			for(uint32_t c0 = 0; c0 < nl; c0 += static_cast<uint32_t>(chunk))
			{
				const uint32_t cn = static_cast<uint32_t>(std::min<uint64_t>(chunk, nl - c0));
				Work Wc = W;
				if(int r = spawn_target(Wc, L + 1)) return r;
				GBRT_CK(cudaMemsetAsync(Wc.count, 0, sizeof(uint32_t), st));
				k_spawn_init<<<grid_for(cn, n_sm), kThreads, 0, st>>>(Wc, spawn_buf(L) + 5ull * c0, cn);
				vertex_loop(Wc, cn);
				uint32_t nc = 0;
				if(int r = spawned(L + 1, nc)) return r;
				if(nc)
					if(int r = process_level(L + 1, nc)) return r;
			}
			return GBRT_OK;
		};
		while(!rc && first_rc.load() == GBRT_OK)
		{
			const uint64_t wv = next_wave.fetch_add(1);
			if(wv >= n_waves) break;
			const uint64_t start = wv * wave;
			const uint32_t wn = static_cast<uint32_t>(std::min<uint64_t>(wave, total - start));
			Work Wv = W;
			if((rc = spawn_target(Wv, 1))) break;
			k_camera_batch<<<grid_for(wn, n_sm), kThreads, 0, st>>>(table, n, static_cast<uint32_t>(start), wn, Wv);
			vertex_loop(Wv, wn);
			uint32_t nc = 0;
			if((rc = spawned(1, nc))) break;
			if(nc) rc = process_level(1, nc);
		}
		if(!rc && cudaGetLastError() != cudaSuccess) rc = gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: launch failed");
		if(!rc) cudaMemcpyAsync(&rays[2 * k], W.stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
		release_work(H, st);                    // back to the pool
		if(k > 0)
		{
			cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
			cudaEventRecord(done[k], st);
			if(cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: stream error");
			cudaStreamDestroy(st);
		}
		return rc ? fail(rc) : GBRT_OK;
	};
	std::vector<std::thread> pool;
	for(uint32_t k = 1; k < n_streams; ++k) pool.emplace_back(worker, k);
	worker(0);
	for(auto &t : pool) t.join();
	for(uint32_t k = 1; k < n_streams; ++k)
		if(done[k]) { cudaStreamWaitEvent(s, done[k], 0); cudaEventDestroy(done[k]); }
	cudaEventRecord(e1, s);
	cudaFreeAsync(table, s);
	for(uint32_t i = 0; i < n; ++i)
	{
		gbrt_scene *S = scenes[i];
		if(!S->ev_last) cudaEventCreateWithFlags(&S->ev_last, cudaEventDisableTiming);
		cudaEventRecord(S->ev_last, s);
	}
	const cudaError_t se = cudaStreamSynchronize(s);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if(first_rc.load() != GBRT_OK) return gbrt_set_error(first_rc.load(), "%s", err_msg.c_str());
	if(se != cudaSuccess) return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_pt_render_multi: %s", cudaGetErrorString(se));
	if(stats)
	{
		*stats = gbrt_pt_stats{};
		for(uint32_t i = 0; i < n; ++i) stats->camera_samples += host[i].paths / static_cast<uint32_t>(host[i].P.path_samples);
		for(uint32_t k = 0; k < n_streams; ++k) { stats->extension_rays += rays[2 * k]; stats->shadow_rays += rays[2 * k + 1]; }
		stats->ms = ms;
	}
	return GBRT_OK;
}

// The autotuner: short trial renders of the whole batch at 1 sample per
// pixel into scratch films, device-timed, coordinate descent over the
// number of waves in flight, then the wave size, then the shading block
// size, then the traversal grids' residency (from the defaults 4 streams,
// 1 Mi paths, 128 threads, what fits; residency tried at what fits and
// half of it).
static int batch_autotune(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params, uint32_t n,
                          gbrt_batch_tuning &t, cudaStream_t s)
{
	size_t film_max = 0, w_max = 0;
	for(uint32_t i = 0; i < n; ++i)
	{
		const size_t px = static_cast<size_t>(cameras[i].resx) * cameras[i].resy;
		film_max = std::max(film_max, 3 * px);
		w_max = std::max(w_max, px);
	}
	float *scratch = nullptr, *wscratch = nullptr;
	GBRT_CK(cudaMallocAsync(reinterpret_cast<void **>(&scratch), 4 * film_max, s));
	GBRT_CK(cudaMallocAsync(reinterpret_cast<void **>(&wscratch), 4 * w_max, s));
	std::vector<float *> films(n, scratch);
	std::vector<gbrt_pt_params> pp(params, params + n);
	for(auto &p : pp) if(p.filter_type != GBRT_FILTER_PIXEL) p.film_weight_dev = wscratch;
	const int bps_max = max_blocks_per_sm(reinterpret_cast<const void *>(k_extend_batch));
	BatchPlan plan{t.wave_paths ? t.wave_paths : (1u << 20), t.shade_block ? t.shade_block : kThreads,
	               t.trace_blocks_per_sm ? t.trace_blocks_per_sm : static_cast<uint32_t>(bps_max), t.streams ? t.streams : 4u};
	float spent = 0.f;
	int rc = GBRT_OK;
	auto trial = [&](const BatchPlan &pl, float &ms) -> int {
		gbrt_pt_stats st{};
		if(int r = batch_render_locked(scenes, cameras, pp.data(), films.data(), n, pl, 1, &st, s)) return r;
		ms = st.ms;
		spent += st.ms;
		return GBRT_OK;
	};
	float ms0 = 0.f;
	rc = trial(plan, ms0);               // warm: buffers grown, code loaded
	if(!rc && !t.streams)
	{
		float best = 3.4e38f;
		uint32_t pick = plan.streams;
		for(uint32_t k : {1u, 2u, 4u, 8u})
		{
			BatchPlan pl = plan;
			pl.streams = k;
			float ms = 0.f;
			if((rc = trial(pl, ms))) break;
			if(ms < best) { best = ms; pick = k; }
		}
		plan.streams = pick;
	}
	if(!rc && !t.wave_paths)
	{
		float best = 3.4e38f;
		uint32_t pick = plan.wave;
		for(uint32_t w : {1u << 19, 1u << 20, 1u << 21, 1u << 22})
		{
			BatchPlan pl = plan;
			pl.wave = w;
			float ms = 0.f;
			if((rc = trial(pl, ms))) break;
			if(ms < best) { best = ms; pick = w; }
		}
		plan.wave = pick;
	}
	if(!rc && !t.shade_block)
	{
		float best = 3.4e38f;
		uint32_t pick = plan.shade_block;
		for(uint32_t b : {64u, 128u})
		{
			BatchPlan pl = plan;
			pl.shade_block = b;
			float ms = 0.f;
			if((rc = trial(pl, ms))) break;
			if(ms < best) { best = ms; pick = b; }
		}
		plan.shade_block = pick;
	}
	if(!rc && !t.trace_blocks_per_sm)
	{
		float best = 3.4e38f;
		uint32_t pick = plan.trace_bps;
		for(uint32_t b : {static_cast<uint32_t>(bps_max), std::max(1u, static_cast<uint32_t>(bps_max) / 2u)})
		{
			BatchPlan pl = plan;
			pl.trace_bps = b;
			float ms = 0.f;
			if((rc = trial(pl, ms))) break;
			if(ms < best) { best = ms; pick = b; }
		}
		plan.trace_bps = pick;
	}
	cudaFreeAsync(scratch, s);
	cudaFreeAsync(wscratch, s);
	if(rc) return rc;
	t.wave_paths = plan.wave;
	t.shade_block = plan.shade_block;
	t.trace_blocks_per_sm = plan.trace_bps;
	t.streams = plan.streams;
	t.tune_ms = spent;
	return GBRT_OK;
}

int gbrt_pt_render_multi(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params, float *const *films,
                         uint32_t n, gbrt_batch_tuning *tuning, gbrt_pt_stats *stats, void *stream)
{
	if(n == 0) return GBRT_OK;
	if(!scenes || !cameras || !params || !films) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: NULL argument");
	for(uint32_t i = 0; i < n; ++i)
		if(!scenes[i] || !films[i]) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_pt_render_multi: scene or film %u is NULL", i);
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	// every scene's lock, in address order (concurrent batches over shared scenes)
	std::vector<gbrt_scene *> order(scenes, scenes + n);
	std::sort(order.begin(), order.end());
	order.erase(std::unique(order.begin(), order.end()), order.end());
	std::vector<std::unique_lock<std::mutex>> locks;
	for(gbrt_scene *S : order) locks.emplace_back(S->mu);
	gbrt_batch_tuning t{};
	if(tuning) t = *tuning;
	if(!t.wave_paths || !t.shade_block || !t.trace_blocks_per_sm || !t.streams)
		if(int rc = batch_autotune(scenes, cameras, params, n, t, s)) return rc;
	if(tuning) *tuning = t;
	const BatchPlan plan{t.wave_paths, t.shade_block, t.trace_blocks_per_sm, t.streams};
	return batch_render_locked(scenes, cameras, params, films, n, plan, 0, stats, s);
}

int gbrt_pt_render_batch(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params, float *const *films,
                         uint32_t n, uint32_t concurrency, gbrt_pt_stats *stats)
{
	(void)concurrency;
	gbrt_pt_stats total{};
	if(int rc = gbrt_pt_render_multi(scenes, cameras, params, films, n, nullptr, stats ? &total : nullptr, nullptr)) return rc;
	if(stats)
	{
		// each scene's camera samples; the batch's rays and device time in entry 0
		for(uint32_t i = 0; i < n; ++i)
		{
			stats[i] = gbrt_pt_stats{};
			stats[i].camera_samples = static_cast<uint64_t>(cameras[i].resx) * cameras[i].resy * params[i].spp;
		}
		stats[0].extension_rays = total.extension_rays;
		stats[0].shadow_rays = total.shadow_rays;
		stats[0].ms = total.ms;
	}
	return GBRT_OK;
}

static int dl_render_impl(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                          float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream, const gbrt_aa_params *aa,
                          uint32_t *resampled)
{
	if(!S || !camera || !params) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_dl_render: NULL argument");
	if(!film_dev && !film64_dev) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_dl_render: no film buffer");
	const bool caustics = caustic && caustic->caustics;
	if(caustics && (caustic->caustic_mix < 1 || caustic->caustic_mix > gbrt::kMaxGather || !(caustic->caustic_radius > 0.f) ||
	                caustic->caustic_depth < 0 || caustic->caustic_photons < 0))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_dl_render: bad caustic parameters (caustic_mix in [1, %d])", gbrt::kMaxGather);
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	std::lock_guard<std::mutex> lock(S->mu);
	Params M{};
	M.pm = 2;
	M.path_samples = 1;
	ShotMap C;
	GridStore GC;
	if(caustics)
	{
		float bound[6];
		if(int rc = gbrt_bvh_get_bound(S->bvh, bound)) return rc;
		const float lo[3] = {bound[0], bound[1], bound[2]};
		const uint32_t seed = params->seed * 0x9e3779b9u + params->base_sampling_offset;
		if(int rc = shoot_map(S, scene_dev(S), true, static_cast<uint32_t>(caustic->caustic_photons), caustic->caustic_depth, false, seed, C, s)) return rc;
		if(int rc = build_grid(C.pos.as<float4>(), C.dir.as<float4>(), C.col.as<float4>(), C.n, caustic->caustic_radius, lo, S->n_sm, GC, s)) return rc;
		M.pm_caustics = 1;
		M.pm_caustic_r2 = caustic->caustic_radius * caustic->caustic_radius;
		M.pm_caustic_k = caustic->caustic_mix;
		M.pm_caustic_paths = static_cast<float>(C.paths);
		M.g_caustic = GC.g;
	}
	const int rc = aa ? aa_render_locked(S, camera, *params, *aa, film_dev, stats, resampled, s, &M)
	                  : render_locked(S, camera, *params, &M, film_dev, film64_dev, stats, s);
	cudaStreamSynchronize(s);
	return rc;
}

int gbrt_dl_render(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                   float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream)
{
	return dl_render_impl(S, camera, params, caustic, film_dev, film64_dev, stats, stream, nullptr, nullptr);
}

// Adaptive passes of the photonmapping (kind 1) or directlighting (kind 2)
// integrator over a device film built here; normalised image to the host.
static int aa_host_other(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params_in, const gbrt_pm_params *pm,
                         const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled, int kind)
{
	if(!S || !camera || !params_in || !aa || !image_out || (kind == 1 && !pm)) return gbrt_set_error(GBRT_ERR_INVALID, "render_aa_host: NULL argument");
	if(int rc = aa_check(*aa, "render_aa_host")) return rc;
	if(camera->resx <= 0 || camera->resy <= 0) return gbrt_set_error(GBRT_ERR_INVALID, "render_aa_host: bad resolution");
	if(params_in->filter_type == GBRT_FILTER_PIXEL)
		return gbrt_set_error(GBRT_ERR_INVALID, "render_aa_host: adaptive AA needs a filtered film (filter_type != PIXEL)");
	const size_t n_pix = static_cast<size_t>(camera->resx) * camera->resy, n = 3 * n_pix;
	gbrt_pt_params params = *params_in;
	params.guide = nullptr;
	DevBuf sum, mean, weight;
	if(int rc = sum.alloc(n * 4)) return rc;
	if(int rc = mean.alloc(n * 4)) return rc;
	if(int rc = weight.alloc(n_pix * 4)) return rc;
	GBRT_CK(cudaMemset(sum.p, 0, n * 4));
	GBRT_CK(cudaMemset(weight.p, 0, n_pix * 4));
	params.film_weight_dev = weight.as<float>();
	const int rc = kind == 1 ? pm_render_impl(S, camera, &params, pm, sum.as<float>(), nullptr, stats, nullptr, aa, resampled)
	                         : dl_render_impl(S, camera, &params, pm, sum.as<float>(), nullptr, stats, nullptr, aa, resampled);
	if(rc) return rc;
	k_normalize<<<grid_for(n, S->n_sm), kThreads>>>(sum.as<float>(), nullptr, weight.as<float>(), mean.as<float>(), n);
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(image_out, mean.p, n * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_pm_render_aa_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                           const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled)
{
	return aa_host_other(S, camera, params, pm, aa, image_out, stats, resampled, 1);
}

int gbrt_dl_render_aa_host(gbrt_scene *S, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                           const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled)
{
	return aa_host_other(S, camera, params, caustic, aa, image_out, stats, resampled, 2);
}

int gbrt_grid_buckets(const float *points, uint32_t n, double cell_size, uint32_t grid_size, const float box_lo[3], uint32_t *bucket_out)
{
	if((n && (!points || !bucket_out)) || !box_lo || !(cell_size > 0.0) || grid_size == 0)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_grid_buckets: bad argument");
	if(n == 0) return GBRT_OK;
	gbrt::PhotonGrid g{};
	g.buckets = grid_size;
	for(int a = 0; a < 3; ++a) g.lo[a] = box_lo[a];
	g.inv_cell = static_cast<float>(1.0 / cell_size);
	DevBuf dp, db;
	if(int rc = dp.alloc(12ull * n)) return rc;
	if(int rc = db.alloc(4ull * n)) return rc;
	GBRT_CK(cudaMemcpy(dp.p, points, 12ull * n, cudaMemcpyHostToDevice));
	k_grid_buckets<<<(n + 127) / 128, 128>>>(g, dp.as<float>(), n, db.as<uint32_t>());
	GBRT_CK(cudaGetLastError());
	GBRT_CK(cudaMemcpy(bucket_out, db.p, 4ull * n, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

} // extern "C"
