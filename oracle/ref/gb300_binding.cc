// The reference-side binding of the GB300 hot path (see gb300_binding.h).
#include "gb300_binding.h"

#include "camera/camera.h"
#include "color/color_layers.h"
#include "common/logger.h"
#include "geometry/object/object_mesh.h"
#include "geometry/primitive/primitive_face.h"
#include "geometry/surface.h"
#include "light/light.h"
#include "material/material.h"
#include "render/imagefilm.h"
#include "render/imagesplitter.h"
#include "render/render_control.h"
#include "scene/scene.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>

namespace gb300 {

namespace {

using yafaray::ParamMap;

template <typename T>
T get_or(const ParamMap &pm, const std::string &name, T dflt)
{
	T v = dflt;
	pm.getParam(name, v);
	return v;
}

void put3(float o[3], const yafaray::Vec3f &v) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }
void put3(float o[3], const yafaray::Rgb &c) { o[0] = c.r_; o[1] = c.g_; o[2] = c.b_; }

// Material::getAsParamMap -> gbrt_material_desc (layout of include/gbrt.h)
bool material_desc(const yafaray::Material &m, gbrt_material_desc &d, std::string &error)
{
	const ParamMap pm = m.getAsParamMap(false);
	std::string type;
	pm.getParam("type", type);
	d = gbrt_material_desc{};
	// shader nodes (textures, procedural inputs) are not translated
	for(const auto &[key, value] : pm)
	{
		std::string node;
		if(key.size() > 7 && key.compare(key.size() - 7, 7, "_shader") == 0 && value.getVal(node) && !node.empty())
		{
			error = type + ": shader node '" + node + "' on " + key + " is not translated to the GPU";
			return false;
		}
	}
	d.params[5] = static_cast<float>(get_or<int>(pm, "additionaldepth", 0));
	if(type == "shinydiffusemat")
	{
		d.type = GBRT_MAT_SHINYDIFFUSE;
		put3(d.color, get_or(pm, "color", yafaray::Rgb{1.f}));
		put3(d.color2, get_or(pm, "mirror_color", yafaray::Rgb{1.f}));
		d.power = get_or(pm, "emit", 0.f);
		d.params[0] = get_or(pm, "diffuse_reflect", 1.f);
		d.params[1] = get_or(pm, "specular_reflect", 0.f);
		d.params[2] = get_or(pm, "transparency", 0.f);
		d.params[3] = get_or(pm, "translucency", 0.f);
		d.params[4] = get_or(pm, "transmit_filter", 1.f);
		d.params[6] = get_or(pm, "fresnel_effect", false) ? 1.f : 0.f;
		d.params[7] = get_or(pm, "IOR", 1.33f);
		if(get_or<std::string>(pm, "diffuse_brdf", "lambertian") != "lambertian") { error = "shinydiffusemat: only the lambertian diffuse BRDF is built on the GPU"; return false; }
	}
	else if(type == "light_mat")
	{
		d.type = GBRT_MAT_LIGHT;
		put3(d.color, get_or(pm, "color", yafaray::Rgb{1.f}));
		d.power = get_or(pm, "power", 1.f);
		d.params[0] = get_or(pm, "double_sided", false) ? 1.f : 0.f;
	}
	else if(type == "glossy")
	{
		d.type = GBRT_MAT_GLOSSY;
		put3(d.color, get_or(pm, "color", yafaray::Rgb{1.f}));
		put3(d.color2, get_or(pm, "diffuse_color", yafaray::Rgb{1.f}));
		d.params[0] = get_or(pm, "exponent", 50.f);
		d.params[1] = get_or(pm, "glossy_reflect", 1.f);
		d.params[2] = get_or(pm, "diffuse_reflect", 0.f);
		d.params[3] = get_or(pm, "as_diffuse", true) ? 1.f : 0.f;
		if(get_or(pm, "anisotropic", false)) { error = "glossy: anisotropic lobes are not built on the GPU"; return false; }
	}
	else if(type == "glass" || type == "rough_glass")
	{
		d.type = type == "glass" ? GBRT_MAT_GLASS : GBRT_MAT_ROUGH_GLASS;
		put3(d.color, get_or(pm, "filter_color", yafaray::Rgb{1.f}));
		put3(d.color2, get_or(pm, "mirror_color", yafaray::Rgb{1.f}));
		d.params[0] = get_or(pm, "IOR", 1.4f);
		d.params[1] = get_or(pm, "transmit_filter", 0.f);
		d.params[2] = type == "glass" ? 0.f : get_or(pm, "alpha", 0.5f);
		d.params[3] = get_or(pm, "fake_shadows", false) ? 1.f : 0.f;
		if(get_or(pm, "dispersion_power", 0.f) != 0.f) { error = type + ": dispersion is not built on the GPU"; return false; }
	}
	else
	{
		error = "material type '" + type + "' is not built on the GPU";
		return false;
	}
	return true;
}

bool light_desc(const yafaray::Light &l, gbrt_light_desc &d, std::string &error)
{
	const ParamMap pm = l.getAsParamMap(false);
	std::string type;
	pm.getParam("type", type);
	d = gbrt_light_desc{};
	if(type == "arealight")
	{
		d.type = GBRT_LIGHT_AREA;
		put3(d.corner, get_or(pm, "corner", yafaray::Vec3f{0.f}));
		put3(d.point1, get_or(pm, "point1", yafaray::Vec3f{0.f}));
		put3(d.point2, get_or(pm, "point2", yafaray::Vec3f{0.f}));
		put3(d.color, get_or(pm, "color", yafaray::Rgb{1.f}));
		d.power = get_or(pm, "power", 1.f);
		d.samples = get_or<int>(pm, "samples", 4);
		return true;
	}
	if(type == "pointlight")
	{
		d.type = GBRT_LIGHT_POINT;
		put3(d.corner, get_or(pm, "from", yafaray::Vec3f{0.f}));
		put3(d.color, get_or(pm, "color", yafaray::Rgb{1.f}));
		d.power = get_or(pm, "power", 1.f);
		d.samples = 1;
		return true;
	}
	error = "light type '" + type + "' is not built on the GPU";
	return false;
}

gbrt_ray to_gbrt(const yafaray::Ray &ray, float t_max)
{
	gbrt_ray r{};
	r.org[0] = ray.from_[0]; r.org[1] = ray.from_[1]; r.org[2] = ray.from_[2];
	r.dir[0] = ray.dir_[0]; r.dir[1] = ray.dir_[1]; r.dir[2] = ray.dir_[2];
	r.tmin = ray.tmin_;
	r.tmax = t_max;
	return r;
}

} // namespace

bool translate(const yafaray::Scene &scene, const yafaray::Camera &camera, SceneDesc &out, std::string &error)
{
	out = SceneDesc{};
	// materials in the scene's registry order
	std::map<const yafaray::Material *, int32_t> mat_index;
	for(const auto &[material, name, enabled] : scene.getMaterials())
	{
		if(!material) continue;
		gbrt_material_desc d;
		if(!material_desc(*material, d, error)) { error = "material '" + name + "': " + error; return false; }
		mat_index[material.get()] = static_cast<int32_t>(out.materials.size());
		out.materials.push_back(d);
	}
	for(const auto &[light, name, enabled] : scene.getLights())
	{
		if(!light || !enabled) continue;
		gbrt_light_desc d;
		if(!light_desc(*light, d, error)) { error = "light '" + name + "': " + error; return false; }
		out.lights.push_back(d);
	}
	// faces in Scene::preprocess's primitive order (scene.cc:320-341)
	for(const auto &[object, object_name, object_enabled] : scene.getObjects())
	{
		if(!object || !object_enabled || object->getVisibility() == yafaray::Visibility::None || object->isBaseObject()) continue;
		const auto *mesh = dynamic_cast<const yafaray::MeshObject *>(object.get());
		if(!mesh) { error = "object '" + object_name + "': only meshes are built on the GPU"; return false; }
		if(mesh->hasMotionBlur()) { error = "object '" + object_name + "': motion blur is not built on the GPU"; return false; }
		const bool smooth = mesh->isSmooth() || mesh->hasVerticesNormals(0);
		for(const yafaray::Primitive *prim : mesh->getPrimitives())
		{
			const auto *face = dynamic_cast<const yafaray::FacePrimitive *>(prim);
			if(!face) { error = "object '" + object_name + "': a primitive that is not a face"; return false; }
			const std::vector<yafaray::Point3f> p = face->getVerticesAsVector(0);
			if(p.size() != 3 && p.size() != 4) { error = "object '" + object_name + "': a face of " + std::to_string(p.size()) + " vertices"; return false; }
			const auto mi = mat_index.find(face->getMaterial());
			if(mi == mat_index.end()) { error = "object '" + object_name + "': a face without a registered material"; return false; }
			const uint32_t base = static_cast<uint32_t>(out.vertices.size() / 3);
			uint32_t q[4] = {base, base + 1, base + 2, GBRT_TRIANGLE};
			if(p.size() == 4) q[3] = base + 3;
			for(const auto &v : p) { out.vertices.push_back(v[0]); out.vertices.push_back(v[1]); out.vertices.push_back(v[2]); }
			out.faces.insert(out.faces.end(), q, q + 4);
			out.face_material.push_back(mi->second);
			// shading normals of a smooth mesh, per face corner: the vertex's
			// normal or, without one, the geometric normal
			// (PrimitivePolygon::getSurfacePolygon / FacePrimitive::getVertexNormal)
			uint32_t fn[4] = {GBRT_FLAT_FACE, GBRT_FLAT_FACE, GBRT_FLAT_FACE, GBRT_FLAT_FACE};
			if(smooth)
			{
				out.has_normals = true;
				const yafaray::Vec3f ng = face->getGeometricNormal({}, 0.f, false);
				for(size_t k = 0; k < p.size(); ++k)
				{
					const yafaray::Vec3f n = face->getVertexNormal(static_cast<int>(k), ng, 0);
					fn[k] = static_cast<uint32_t>(out.normals.size() / 3);
					out.normals.push_back(n[0]); out.normals.push_back(n[1]); out.normals.push_back(n[2]);
				}
				if(p.size() == 3) fn[3] = GBRT_NO_NORMAL;
			}
			out.face_normals.insert(out.face_normals.end(), fn, fn + 4);
		}
	}
	const ParamMap cm = camera.getAsParamMap(false);
	std::string ctype;
	cm.getParam("type", ctype);
	if(ctype != "perspective") { error = "camera type '" + ctype + "' is not built on the GPU"; return false; }
	if(get_or(cm, "aperture", 0.f) != 0.f) { error = "camera: depth of field is not built on the GPU"; return false; }
	put3(out.camera.from, get_or(cm, "from", yafaray::Vec3f{0.f}));
	put3(out.camera.to, get_or(cm, "to", yafaray::Vec3f{0.f}));
	put3(out.camera.up, get_or(cm, "up", yafaray::Vec3f{0.f}));
	out.camera.resx = get_or<int>(cm, "resx", 320);
	out.camera.resy = get_or<int>(cm, "resy", 200);
	out.camera.focal = get_or(cm, "focal", 1.f);
	return true;
}

gbrt_pt_params pt_params(const ParamMap &pm, int spp, unsigned base_sampling_offset, gbrt_pm_params &caustic)
{
	// PathIntegrator / MonteCarloIntegrator parameters (integrator_path_tracer.h:55-59,
	// integrator_montecarlo.h:47-49), their names and defaults
	gbrt_pt_params p{};
	p.spp = spp;
	p.path_samples = get_or<int>(pm, "path_samples", 32);
	p.bounces = get_or<int>(pm, "bounces", 3);
	p.russian_roulette_min_bounces = get_or<int>(pm, "russian_roulette_min_bounces", 0);
	p.raydepth = get_or<int>(pm, "raydepth", 5);
	p.transparent_shadows = get_or(pm, "transpShad", false) ? 1 : 0;
	p.shadow_depth = get_or<int>(pm, "shadowDepth", 4);
	p.no_recursive = get_or(pm, "no_recursive", false) ? 1 : 0;
	const std::string ct = get_or<std::string>(pm, "caustic_type", "path");
	p.caustic_type = ct == "none" ? GBRT_CAUSTIC_NONE : ct == "photon" ? GBRT_CAUSTIC_PHOTON : ct == "both" ? GBRT_CAUSTIC_BOTH : GBRT_CAUSTIC_PATH;
	// the caustic photon map's CausticPhotonIntegrator parameters
	// (integrator_photon_caustic.h:48-51)
	gbrt_pm_default_params(&caustic);
	caustic.caustic_photons = get_or<int>(pm, "caustic_photons", caustic.caustic_photons);
	caustic.caustic_radius = get_or(pm, "caustic_radius", caustic.caustic_radius);
	caustic.caustic_mix = get_or<int>(pm, "caustic_mix", caustic.caustic_mix);
	caustic.caustic_depth = get_or<int>(pm, "caustic_depth", caustic.caustic_depth);
	p.caustic = p.caustic_type == GBRT_CAUSTIC_PHOTON || p.caustic_type == GBRT_CAUSTIC_BOTH ? &caustic : nullptr;
	p.base_sampling_offset = base_sampling_offset;
	p.seed = 1;
	p.filter_type = GBRT_FILTER_PIXEL;
	return p;
}

bool film_params(const ParamMap &fm, gbrt_pt_params &p, gbrt_aa_params &aa, std::string &error)
{
	// ImageFilm parameters (imagefilm.h:190-225), their names and defaults
	const std::string ft = get_or<std::string>(fm, "filter_type", "gauss");
	p.filter_type = ft == "box" ? GBRT_FILTER_BOX : ft == "mitchell" ? GBRT_FILTER_MITCHELL : ft == "lanczos" ? GBRT_FILTER_LANCZOS
	                                                                                                           : GBRT_FILTER_GAUSS;
	p.aa_pixel_width = get_or(fm, "AA_pixelwidth", 1.5f);
	if(p.aa_pixel_width >= 2.f) { error = "AA_pixelwidth " + std::to_string(p.aa_pixel_width) + ": the GPU film takes filters narrower than 2 pixels"; return false; }
	p.clamp_indirect = get_or(fm, "AA_clamp_indirect", 0.f);
	aa.passes = get_or<int>(fm, "AA_passes", 1);
	aa.inc_samples = get_or<int>(fm, "AA_inc_samples", 1);
	aa.threshold = get_or(fm, "AA_threshold", 0.05f);
	aa.resampled_floor = get_or(fm, "AA_resampled_floor", 0.f);
	aa.sample_multiplier_factor = get_or(fm, "AA_sample_multiplier_factor", 1.f);
	aa.light_sample_multiplier_factor = get_or(fm, "AA_light_sample_multiplier_factor", 1.f);
	aa.indirect_sample_multiplier_factor = get_or(fm, "AA_indirect_sample_multiplier_factor", 1.f);
	aa.detect_color_noise = get_or(fm, "AA_detect_color_noise", false) ? 1 : 0;
	const std::string dark = get_or<std::string>(fm, "AA_dark_detection_type", "none");
	aa.dark_detection_type = dark == "linear" ? 1 : dark == "curve" ? 2 : 0;
	aa.dark_threshold_factor = get_or(fm, "AA_dark_threshold_factor", 0.f);
	aa.variance_edge_size = get_or<int>(fm, "AA_variance_edge_size", 10);
	aa.variance_pixels = get_or<int>(fm, "AA_variance_pixels", 0);
	if(get_or(fm, "AA_clamp_samples", 0.f) != 0.f) { error = "AA_clamp_samples is not built on the GPU"; return false; }
	return true;
}

int build_gpu_scene(const SceneDesc &d, gbrt_bvh **bvh, gbrt_scene **scene)
{
	*bvh = nullptr;
	*scene = nullptr;
	const uint32_t nv = static_cast<uint32_t>(d.vertices.size() / 3), nf = static_cast<uint32_t>(d.face_material.size());
	if(int rc = gbrt_bvh_build_host(d.vertices.data(), nv, d.faces.data(), nf, nullptr, bvh)) return rc;
	if(int rc = gbrt_scene_create(*bvh, d.vertices.data(), nv, d.faces.data(), nf, d.face_material.data(), d.materials.data(),
	                              static_cast<uint32_t>(d.materials.size()), d.lights.data(), static_cast<uint32_t>(d.lights.size()), scene))
	{
		gbrt_bvh_destroy(*bvh);
		*bvh = nullptr;
		return rc;
	}
	if(d.has_normals)
		if(int rc = gbrt_scene_set_normals(*scene, d.normals.data(), static_cast<uint32_t>(d.normals.size() / 3), d.face_normals.data()))
			return rc;
	return GBRT_OK;
}

// ---- AcceleratorGb300 ----------------------------------------------------------

AcceleratorGb300::AcceleratorGb300(yafaray::Logger &logger, yafaray::ParamResult &param_result, const yafaray::RenderControl *render_control,
                                   const std::vector<const yafaray::Primitive *> &primitives, const ParamMap &param_map)
	: Accelerator(logger, param_result, render_control, param_map), prims_(primitives)
{
	std::vector<float> v;
	std::vector<uint32_t> f;
	for(const yafaray::Primitive *prim : primitives)
	{
		const auto *face = dynamic_cast<const yafaray::FacePrimitive *>(prim);
		if(!face) { logger.logError("AcceleratorGb300: only face primitives are built on the GPU"); return; }
		const std::vector<yafaray::Point3f> p = face->getVerticesAsVector(0);
		const uint32_t base = static_cast<uint32_t>(v.size() / 3);
		for(const auto &x : p) { v.push_back(x[0]); v.push_back(x[1]); v.push_back(x[2]); }
		f.push_back(base); f.push_back(base + 1); f.push_back(base + 2); f.push_back(p.size() == 4 ? base + 3 : GBRT_TRIANGLE);
	}
	if(int rc = gbrt_bvh_build_host(v.data(), static_cast<uint32_t>(v.size() / 3), f.data(), static_cast<uint32_t>(prims_.size()), nullptr, &bvh_))
	{
		logger.logError("AcceleratorGb300: ", gbrt_last_error(), " (status ", rc, ")");
		bvh_ = nullptr;
		return;
	}
	float b[6];
	gbrt_bvh_get_bound(bvh_, b);
	bound_ = yafaray::Bound<float>{{{b[0], b[1], b[2]}}, {{b[3], b[4], b[5]}}};
}

AcceleratorGb300::~AcceleratorGb300()
{
	if(bvh_) gbrt_bvh_destroy(bvh_);
}

int AcceleratorGb300::intersectBatch(const gbrt_ray *rays, uint32_t n, gbrt_hit *hits) const
{
	return gbrt_trace_closest_host(bvh_, rays, n, hits);
}

// One ray per call: a launch and a host round trip each (correct, slow);
// integrators that batch their rays call intersectBatch.
yafaray::IntersectData AcceleratorGb300::intersect(const yafaray::Ray &ray, float t_max) const
{
	yafaray::IntersectData d;
	if(!bvh_) return d;
	const gbrt_ray r = to_gbrt(ray, t_max);
	gbrt_hit h{};
	if(gbrt_trace_closest_host(bvh_, &r, 1, &h) != GBRT_OK || h.prim < 0) return d;
	d.t_hit_ = h.t;
	d.t_max_ = h.t;
	d.uv_ = {h.u, h.v};
	d.primitive_ = prims_[static_cast<size_t>(h.prim)];
	return d;
}

// The segment as Accelerator::isShadowed hands it over (origin already
// advanced by tmin, t_max already shortened): tmin 0 here, so
// gbrt_trace_shadow's own isShadowed set-up leaves it as it is.
yafaray::IntersectData AcceleratorGb300::intersectShadow(const yafaray::Ray &ray, float t_max) const
{
	yafaray::IntersectData d;
	if(!bvh_) return d;
	gbrt_ray r = to_gbrt(ray, t_max >= std::numeric_limits<float>::max() ? -1.f : t_max);
	r.tmin = 0.f;
	int32_t occ = -1;
	if(gbrt_trace_shadow_host(bvh_, &r, 1, &occ) != GBRT_OK || occ < 0) return d;
	d.t_hit_ = 1.f;                // a hit; the occluder's distance is not needed
	d.primitive_ = prims_[static_cast<size_t>(occ)];
	return d;
}

// Transparent shadows walk the closest hits along the segment, as
// Accelerator::primitiveIntersectionTransparentShadow accumulates them.
yafaray::IntersectData AcceleratorGb300::intersectTransparentShadow(const yafaray::Ray &ray, int max_depth, float dist,
                                                                    const yafaray::Camera *camera) const
{
	yafaray::IntersectData d;
	if(!bvh_) return d;
	yafaray::Ray r{ray, yafaray::Ray::DifferentialsCopy::No};
	int depth = 0;
	d.color_ = yafaray::Rgb{1.f};
	float travelled = 0.f;
	while(true)
	{
		const gbrt_ray q = to_gbrt(r, dist - travelled);
		gbrt_hit h{};
		if(gbrt_trace_closest_host(bvh_, &q, 1, &h) != GBRT_OK || h.prim < 0) return d;
		const yafaray::Primitive *prim = prims_[static_cast<size_t>(h.prim)];
		const yafaray::Material *mat = prim->getMaterial();
		if(!mat->isTransparent() || depth >= max_depth) { d.primitive_ = prim; d.t_hit_ = d.t_max_ = travelled + h.t; return d; }
		const yafaray::Point3f hit{r.from_ + h.t * r.dir_};
		const auto sp = prim->getSurface(nullptr, hit, r.time_, {h.u, h.v}, camera);
		if(sp) d.color_ *= sp->getTransparency(r.dir_, camera);
		++depth;
		travelled += h.t;
		r.from_ = hit;
	}
}

// ---- PathIntegratorGb300 -------------------------------------------------------

PathIntegratorGb300::PathIntegratorGb300(yafaray::Logger &logger, yafaray::ParamResult &param_result, const std::string &name,
                                         const ParamMap &param_map)
	: SurfaceIntegrator(logger, param_result, name, param_map), params_copy_(param_map)
{
}

bool PathIntegratorGb300::preprocess(yafaray::RenderMonitor &render_monitor, const yafaray::RenderControl &render_control,
                                     const yafaray::Scene &scene)
{
	scene_ = &scene;
	return SurfaceIntegrator::preprocess(render_monitor, render_control, scene);
}

std::pair<yafaray::Rgb, float> PathIntegratorGb300::integrate(yafaray::Ray &, yafaray::RandomGenerator &, std::vector<int> &, yafaray::ColorLayers *,
                                                              int, bool, float, int, const yafaray::RayDivision &,
                                                              const yafaray::PixelSamplingData &)
{
	return {yafaray::Rgb{0.f}, 1.f};
}

// The whole film on the GPU with the film's own anti-aliasing (filter,
// AA_* passes and thresholds; gbrt_pt_render_aa_host), then the normalised
// colour of every pixel as one sample at its centre into the reference's
// film, so the film's outputs and callbacks see the image.  A centre sample
// stays in its own pixel for AA_pixelwidth < 2 (ImageFilm::addSample's
// footprint, imagefilm.cc:775-778), where the film shows the GPU's image
// unchanged; a wider filter would blur it a second time and is refused.
bool PathIntegratorGb300::render(yafaray::RenderControl &render_control, yafaray::RenderMonitor &render_monitor)
{
	if(!scene_ || !image_film_) return false;
	SceneDesc d;
	std::string error;
	if(!translate(*scene_, *image_film_->getCamera(), d, error))
	{
		logger_.logError(getClassName(), " '", getName(), "': ", error);
		return false;
	}
	const ParamMap fm = image_film_->getAsParamMap(false);
	gbrt_pm_params caustic{};
	gbrt_pt_params p = pt_params(params_copy_, std::max(1, aa_noise_params_->samples_), image_film_->getBaseSamplingOffset(), caustic);
	gbrt_aa_params aa{};
	if(!film_params(fm, p, aa, error))
	{
		logger_.logError(getClassName(), " '", getName(), "': ", error);
		return false;
	}
	gbrt_bvh *bvh = nullptr;
	gbrt_scene *gs = nullptr;
	if(int rc = build_gpu_scene(d, &bvh, &gs))
	{
		logger_.logError(getClassName(), " '", getName(), "': ", gbrt_last_error(), " (status ", rc, ")");
		if(bvh) gbrt_bvh_destroy(bvh);
		return false;
	}
	std::vector<float> img(3ull * d.camera.resx * d.camera.resy);
	gbrt_pt_stats st{};
	const int rc = gbrt_pt_render_aa_host(gs, &d.camera, &p, &aa, img.data(), &st, nullptr);
	gbrt_scene_destroy(gs);
	gbrt_bvh_destroy(bvh);
	if(rc)
	{
		logger_.logError(getClassName(), " '", getName(), "': ", gbrt_last_error(), " (status ", rc, ")");
		return false;
	}
	image_film_->init(render_control, render_monitor, *this);
	yafaray::RenderArea area{};
	area.x_ = area.sx_0_ = 0;
	area.y_ = area.sy_0_ = 0;
	area.w_ = d.camera.resx;
	area.h_ = d.camera.resy;
	area.sx_1_ = d.camera.resx - 1;
	area.sy_1_ = d.camera.resy - 1;
	yafaray::ColorLayers layers(*image_film_->getLayers());
	for(int y = 0; y < d.camera.resy && !render_control.canceled(); ++y)
		for(int x = 0; x < d.camera.resx; ++x)
		{
			layers.setDefaultColors();
			const float *c = &img[3ull * (static_cast<size_t>(y) * d.camera.resx + x)];
			if(yafaray::Rgba *combined = layers.find(yafaray::LayerDef::Combined)) *combined = yafaray::Rgba{c[0], c[1], c[2], 1.f};
			image_film_->addSample({{x, y}}, 0.5f, 0.5f, &area, 0, 0, 1.f, &layers);
		}
	logger_.logInfo(getClassName(), " '", getName(), "': rendered on the GPU in ", st.ms, " ms (", st.extension_rays + st.shadow_rays, " rays)");
	return true;
}

} // namespace gb300
