// The reference-side binding of the GB300 hot path: the classes a libYafaRay
// build adds so that its scene / render C API reaches libgbrt (include/gbrt.h).
//
//  - AcceleratorGb300: an Accelerator (include/accelerator/accelerator.h:37-87)
//    over a gbrt_bvh, selected by the accelerator type "gb300-lbvh".
//  - translate(): a reference Scene as the GPU library takes it (faces in the
//    reference's primitive order, materials, lights, camera).
//  - PathIntegratorGb300: the "pathtracing" integrator (its parameters, names
//    and defaults) whose render() (integrator_surface.h:88) runs the whole
//    film on the GPU and writes it into the reference's ImageFilm.
//    PathIntegrator is final, so this is a SurfaceIntegrator of its own that
//    the factory picks for "pathtracing" with the flag "gpu".
//
// Compiled against the reference's headers by oracle/ref/Makefile; the
// harness binding_dump (render_dump.cc built with GB300_BINDING) uses it.
#pragma once

#include "gbrt.h"

#include "accelerator/accelerator.h"
#include "integrator/surface/integrator_surface.h"
#include "param/param.h"

#include <string>
#include <vector>

namespace yafaray {
class Scene;
class Camera;
} // namespace yafaray

namespace gb300 {

// A reference scene in the GPU library's terms.  Every face keeps its own
// vertices (3 or 4), so the primitive ID of face i is i, as the reference
// numbers its primitives (Scene::preprocess, scene.cc:320-341).
struct SceneDesc {
	std::vector<float> vertices;            // xyz per vertex
	std::vector<uint32_t> faces;            // 4 per face, the 4th GBRT_TRIANGLE for a triangle
	std::vector<int32_t> face_material;
	std::vector<gbrt_material_desc> materials;
	std::vector<gbrt_light_desc> lights;
	std::vector<float> normals;             // xyz per face corner of faces with shading normals
	std::vector<uint32_t> face_normals;     // 4 per face: normal indices, GBRT_FLAT_FACE first for flat faces
	bool has_normals = false;
	gbrt_camera_desc camera{};
};

// Scene + camera -> SceneDesc.  Returns false (with a message) for what the
// GPU path does not build (instances, motion blur, other material, light or
// camera types).
bool translate(const yafaray::Scene &scene, const yafaray::Camera &camera, SceneDesc &out, std::string &error);

// The pathtracing parameters of an integrator's ParamMap (the reference's
// names and defaults) and the film's sampling; `caustic` receives the caustic
// photon map's parameters, which the result points at for caustic_type
// photon / both.
gbrt_pt_params pt_params(const yafaray::ParamMap &integrator_params, int spp, unsigned base_sampling_offset, gbrt_pm_params &caustic);

// The film's filter and AA_* parameters (the reference's names and defaults)
// into the GPU render's; false for what the GPU film does not take.
bool film_params(const yafaray::ParamMap &film_params, gbrt_pt_params &p, gbrt_aa_params &aa, std::string &error);

// Builds the GPU scene (BVH, materials, lights, normals) of a SceneDesc.
int build_gpu_scene(const SceneDesc &d, gbrt_bvh **bvh, gbrt_scene **scene);

class AcceleratorGb300 final : public yafaray::Accelerator
{
	public:
		AcceleratorGb300(yafaray::Logger &logger, yafaray::ParamResult &param_result, const yafaray::RenderControl *render_control,
		                 const std::vector<const yafaray::Primitive *> &primitives, const yafaray::ParamMap &param_map);
		~AcceleratorGb300() override;
		bool ok() const { return bvh_ != nullptr; }
		[[nodiscard]] Type type() const override { return Type{Type::None}; }
		[[nodiscard]] std::map<std::string, const yafaray::ParamMeta *> getParamMetaMap() const override { return {}; }
		yafaray::IntersectData intersect(const yafaray::Ray &ray, float t_max) const override;
		yafaray::IntersectData intersectShadow(const yafaray::Ray &ray, float t_max) const override;
		yafaray::IntersectData intersectTransparentShadow(const yafaray::Ray &ray, int max_depth, float dist, const yafaray::Camera *camera) const override;
		yafaray::Bound<float> getBound() const override { return bound_; }
		// many rays per call (what the integrators should use on a GPU)
		int intersectBatch(const gbrt_ray *rays, uint32_t n, gbrt_hit *hits) const;

	private:
		gbrt_bvh *bvh_ = nullptr;
		std::vector<const yafaray::Primitive *> prims_;
		yafaray::Bound<float> bound_{};
};

class PathIntegratorGb300 final : public yafaray::SurfaceIntegrator
{
	public:
		PathIntegratorGb300(yafaray::Logger &logger, yafaray::ParamResult &param_result, const std::string &name,
		                    const yafaray::ParamMap &param_map);
		[[nodiscard]] Type type() const override { return Type{Type::Path}; }
		[[nodiscard]] std::map<std::string, const yafaray::ParamMeta *> getParamMetaMap() const override { return {}; }
		bool preprocess(yafaray::RenderMonitor &render_monitor, const yafaray::RenderControl &render_control,
		                const yafaray::Scene &scene) override;
		// the GPU renders whole films; no ray is integrated on the CPU
		std::pair<yafaray::Rgb, float> integrate(yafaray::Ray &, yafaray::RandomGenerator &, std::vector<int> &, yafaray::ColorLayers *, int,
		                                         bool, float, int, const yafaray::RayDivision &,
		                                         const yafaray::PixelSamplingData &) override;

	protected:
		bool render(yafaray::RenderControl &render_control, yafaray::RenderMonitor &render_monitor) override;

	private:
		const yafaray::Scene *scene_ = nullptr;
		yafaray::ParamMap params_copy_;
};

} // namespace gb300
