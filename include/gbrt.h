/*
 * gbrt.h — C ABI of the GB300 (sm_103a) ray-tracing kernels behind
 * libyafaray_gb300.  Plain C, no CUDA or torch types: device buffers are
 * passed as plain pointers, streams as `void *` (a cudaStream_t, NULL for the
 * legacy default stream).
 *
 * Conventions
 *   - Every entry point returns an int status: GBRT_OK (0) or a negative
 *     GBRT_ERR_* code; gbrt_last_error() gives the message of the calling
 *     thread's last failure.  Nothing aborts or traps.
 *   - Create calls allocate device memory and own it until the matching
 *     destroy call; inputs are borrowed; outputs are caller-allocated.
 *   - Calls taking `_dev` buffers are asynchronous on the given stream; calls
 *     taking host buffers (`_host`) copy in, compute and copy out, and return
 *     when the result is in host memory.
 *   - A handle may be used from several host threads at once for queries;
 *     build/destroy of one handle must not overlap other calls on it.
 *
 * Primitive layout (mirrors MeshObject faces, src/geometry/object/object_mesh.cc:96-112):
 *   vertices : float[3 * n_vertices]
 *   faces    : uint32[4 * n_faces]; faces[4*i+3] == GBRT_TRIANGLE marks a
 *              triangle, otherwise the face is a quad and stays ONE primitive
 *              (its two triangles are tested as in shape_polygon.h:126-176).
 *   The primitive ID of face i is i (the order Scene::preprocess collects
 *   primitives in, src/scene/scene.cc:320-341).
 */
#ifndef GBRT_H
#define GBRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBRT_TRIANGLE 0xFFFFFFFFu

enum {
	GBRT_OK = 0,
	GBRT_ERR_INVALID = -1,    /* bad argument (null pointer, bad index, size) */
	GBRT_ERR_CUDA = -2,       /* a CUDA runtime call failed */
	GBRT_ERR_OOM = -3,        /* device allocation failed */
	GBRT_ERR_TIMEOUT = -4,    /* a device-side iteration budget ran out */
	GBRT_ERR_CAPACITY = -5,   /* a size exceeds a fixed capacity */
	GBRT_ERR_NO_DEVICE = -6   /* no CUDA device visible */
};

/* Ray record, 32 bytes: Ray::from_, tmin_, dir_, tmax_ (include/geometry/ray.h:46-49).
 * tmax < 0 means unbounded, as in Accelerator::intersect (accelerator.h:91). */
typedef struct gbrt_ray {
	float org[3];
	float tmin;
	float dir[3];
	float tmax;
} gbrt_ray;

/* Hit record, 16 bytes: the primitive ID (-1 = miss), t and the (u,v) that
 * IntersectData carries (src/accelerator/intersect_data.h:30-39). */
typedef struct gbrt_hit {
	int32_t prim;
	float t;
	float u;
	float v;
} gbrt_hit;

typedef struct gbrt_build_params {
	uint32_t max_leaf_size;   /* 1..16; 0 = default (4) */
	float traversal_cost;     /* SAH cost of a node visit; 0 = default (1.0) */
	float intersect_cost;     /* SAH cost of a primitive test; 0 = default (2.0: leaves of one triangle, mostly) */
	uint32_t flags;           /* GBRT_BUILD_* bits; 0 = default */
} gbrt_build_params;

/* gbrt_build_params.flags: skip the treelet restructuring passes (plain
 * LBVH topology; for comparisons). */
#define GBRT_BUILD_NO_TREELETS 1u
/* Collapse the binary hierarchy into the 8-wide one greedily (open the
 * largest-area child until 8) instead of by the SAH dynamic programme
 * (for comparisons). */
#define GBRT_BUILD_GREEDY_WIDE 2u

typedef struct gbrt_bvh_info {
	uint32_t n_prims;
	uint32_t n_nodes;         /* internal nodes actually referenced */
	uint32_t n_leaves;
	uint32_t max_depth;
	float sah_cost;
	float bound[6];           /* reference tree bound: lo xyz, hi xyz */
	uint64_t device_bytes;    /* device memory held by the handle */
} gbrt_bvh_info;

typedef struct gbrt_bvh gbrt_bvh;

/* Library / device ---------------------------------------------------- */
const char *gbrt_last_error(void);
int gbrt_version(void);
int gbrt_device_count(int *count);

/* BVH build.  Replaces the kd-tree construction that Accelerator::factory
 * runs from Scene::preprocess (src/scene/scene.cc:347,
 * src/accelerator/accelerator.cc:44-55, accelerator_kdtree_original.cc:65-141).
 * LBVH: Morton codes, radix sort, Karras hierarchy, SAH treelet
 * restructuring (optimal 7-leaf treelets, bottom-up, three passes), bottom-up
 * refit with an SAH leaf-collapse, then the 8-wide compressed copy the
 * traversal walks.  Device-resident inputs. */
int gbrt_bvh_build(const float *vertices_dev, uint32_t n_vertices,
                   const uint32_t *faces_dev, uint32_t n_faces,
                   const gbrt_build_params *params, void *stream, gbrt_bvh **out);

/* Same from host arrays (copied to the device inside the call). */
int gbrt_bvh_build_host(const float *vertices, uint32_t n_vertices,
                        const uint32_t *faces, uint32_t n_faces,
                        const gbrt_build_params *params, gbrt_bvh **out);

int gbrt_bvh_destroy(gbrt_bvh *bvh);

/* Largest face count gbrt_bvh_build_static accepts. */
#define GBRT_STATIC_MAX_FACES 65536u

/* BVH build that allocates nothing.  This entry point has no counterpart in
 * the reference: it exists for callers that must not allocate device memory
 * at build time — a render loop that rebuilds small per-object hierarchies
 * every frame cannot afford cudaMalloc/cudaFree (they synchronise the whole
 * device and can fail under memory pressure), and a host application that
 * budgets GPU memory itself (through its own pool) hands out only the
 * output buffers.
 *
 * Same inputs and results as gbrt_bvh_build, written into caller buffers in
 * the layout gbrt_bvh_export produces: nodes 64 bytes x max(n_faces-1, 1),
 * prims 48 bytes x n_faces, ids 4 bytes x n_faces (device memory), and the
 * tree bound into bound_out (host memory, 6 floats).
 *
 * The build's temporary arrays live in one fixed device array inside the
 * library, sized for GBRT_STATIC_MAX_FACES faces (about 7 MB, held on every
 * GPU that loads the library until the process exits).  More faces return
 * GBRT_ERR_CAPACITY.  Every call looks up that array's device address in
 * the current context (cudaGetSymbolAddress; the first call on a device also
 * loads the library's module there), so a device reset or a new context is
 * picked up; make the first call on a device before any stream capture.
 * Every call, on every stream, shares the array: calls that
 * overlap on the GPU race and corrupt each other's result, so serialise
 * them.  Synchronises `stream` before returning. */
int gbrt_bvh_build_static(const float *vertices_dev, uint32_t n_vertices,
                          const uint32_t *faces_dev, uint32_t n_faces,
                          const gbrt_build_params *params,
                          void *nodes_dev, size_t nodes_bytes,
                          void *prims_dev, size_t prims_bytes,
                          uint32_t *ids_dev, size_t ids_bytes,
                          float bound_out[6], void *stream);

/* Accelerator::getBound (accelerator.h:53): the primitive bound grown by
 * 0.1 % per axis (accelerator_kdtree_original.cc:99-103).  Synchronises. */
int gbrt_bvh_get_bound(const gbrt_bvh *bvh, float bound_out[6]);
int gbrt_bvh_get_info(const gbrt_bvh *bvh, gbrt_bvh_info *info);

/* Copies the device hierarchy to host buffers (for validation tools):
 * nodes: 64 bytes per node slot (gbrt_bvh_info.n_nodes counts the reachable
 * ones; the slot count is max(n_prims - 1, 1)), prims: 48 bytes and ids: 4
 * bytes per primitive slot.  Any pointer may be NULL to skip that array.
 * Layout: see libyafaray_gb300/csrc/gbrt_internal.cuh.  Synchronises. */
int gbrt_bvh_export(const gbrt_bvh *bvh, void *nodes, size_t nodes_bytes, void *prims, size_t prims_bytes,
                    uint32_t *ids, size_t ids_bytes);

/* Copies the 8-wide compressed hierarchy the traversal walks (for
 * validation tools): *n_nodes and *depth receive its node count and depth;
 * nodes: 80 bytes per node (room for max(n_prims - 1, 1) nodes is always
 * enough), prims: 48 bytes and ids: 4 bytes per primitive, in wide-leaf
 * order.  Any buffer may be NULL to skip it.  Layout: see
 * libyafaray_gb300/csrc/gbrt_internal.cuh.  Synchronises. */
int gbrt_bvh_export_wide(const gbrt_bvh *bvh, uint32_t *n_nodes, uint32_t *depth, void *nodes, size_t nodes_bytes,
                         void *prims, size_t prims_bytes, uint32_t *ids, size_t ids_bytes);

/* Closest hit for n rays: Accelerator::intersect(ray, camera)
 * (accelerator.h:89-101 -> kdtree::intersect<Nearest>,
 * accelerator_kdtree_common.h:108-255), same acceptance rule and dynamic ray
 * bias.  Device buffers, async on stream. */
int gbrt_trace_closest(const gbrt_bvh *bvh, const gbrt_ray *rays_dev, uint32_t n,
                       gbrt_hit *hits_dev, void *stream);

/* Any hit for n shadow rays: Accelerator::isShadowed (accelerator.h:103-111
 * -> kdtree::intersect<Shadow>).  occluder_dev[i] = ID of an occluding
 * primitive or -1.  Device buffers, async on stream. */
int gbrt_trace_shadow(const gbrt_bvh *bvh, const gbrt_ray *rays_dev, uint32_t n,
                      int32_t *occluder_dev, void *stream);

/* Host-buffer variants: copy rays in, trace, copy results out, synchronise.
 * These are what a host Accelerator::intersect batch path binds. */
int gbrt_trace_closest_host(const gbrt_bvh *bvh, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits);
int gbrt_trace_shadow_host(const gbrt_bvh *bvh, const gbrt_ray *rays, uint32_t n, int32_t *occluder);
/* Which way the two calls above would move these buffers: *direct = 1 when
 * the rays and the results (gbrt_hit records, or occluder IDs if shadow)
 * are aligned and each lies in one page-locked allocation the device maps,
 * so the kernel reads and writes them in place in one launch; 0 when they
 * are staged through device buffers in chunks of 2,097,152 rays. */
int gbrt_host_path(const gbrt_ray *rays, uint32_t n, const void *out, int shadow, int *direct);


/* ---- wavefront path tracer (the `pathtracing` integrator) ---------------
 * Replaces PathIntegrator::integrate and MonteCarloIntegrator's light
 * estimation (src/integrator/surface/integrator_path_tracer.cc:138-314,
 * integrator_montecarlo.cc:92-440) run per pixel sample by
 * TiledIntegrator::renderTile (integrator_tiled.cc:253-395), with the film
 * accumulation of ImageFilm::addSample (imagefilm.cc:771-822): single-pixel
 * sums, or any of the reference's filters (gbrt_pt_params.filter_type). */

enum {
	GBRT_MAT_SHINYDIFFUSE = 0,   /* "shinydiffusemat": color, color2 (mirror_color; all 0 -> 1), power (emit),
	                                params = {diffuse_reflect (0 -> 1), specular_reflect, transparency,
	                                translucency, transmit_filter, -, fresnel_effect (0/1), IOR (0 -> 1.33)} */
	GBRT_MAT_LIGHT = 1,          /* "light_mat": color, power, params[0] = double_sided (0/1) */
	GBRT_MAT_GLOSSY = 2,         /* "glossy": color (glossy colour), color2 (diffuse_color), params =
	                                {exponent, glossy_reflect, diffuse_reflect, as_diffuse (1)} */
	GBRT_MAT_ROUGH_GLASS = 3,    /* "rough_glass": color (filter_color), color2 (mirror_color), params =
	                                {IOR (0 -> 1.4), transmit_filter, alpha (0 -> 0.5), fake_shadows (0/1)} */
	GBRT_MAT_GLASS = 4           /* "glass": color (filter_color), color2 (mirror_color), params =
	                                {IOR (0 -> 1.4), transmit_filter, -, fake_shadows (0/1)} */
};
/* Every material: params[5] = additionaldepth (extra recursive ray levels). */
enum { GBRT_LIGHT_AREA = 0, GBRT_LIGHT_POINT = 1 };   /* "pointlight": corner = from, color, power */
enum {
	GBRT_PT_FP64_FILM = 1,        /* accumulate the film in double */
	GBRT_PT_GUIDE_RADIANCE = 2    /* train the guide on incident radiance alone (default: radiance x BSDF cosine) */
};

typedef struct gbrt_material_desc {
	uint32_t type;
	float color[3];
	float color2[3];
	float power;
	float params[8];
} gbrt_material_desc;

/* "arealight": corner, point1, point2, color, power, samples
 * (include/light/light_area.h:51-58). */
typedef struct gbrt_light_desc {
	uint32_t type;
	float corner[3], point1[3], point2[3];
	float color[3];
	float power;
	int32_t samples;
} gbrt_light_desc;

/* "perspective" camera: from, to, up (a point), resx, resy, focal
 * (include/camera/camera.h, camera_perspective.h); aperture 0. */
typedef struct gbrt_camera_desc {
	float from[3], to[3], up[3];
	int32_t resx, resy;
	float focal;
} gbrt_camera_desc;

/* pathtracing / film parameters with the reference's names:
 * AA_minsamples (spp, one pass), path_samples, bounces,
 * russian_roulette_min_bounces, adv_base_sampling_offset. */
typedef struct gbrt_guide gbrt_guide;

typedef struct gbrt_pt_params {
	int32_t spp;
	int32_t path_samples;
	int32_t bounces;
	int32_t russian_roulette_min_bounces;
	uint32_t base_sampling_offset;
	uint32_t seed;              /* random stream of Russian roulette / light choice */
	uint32_t flags;             /* GBRT_PT_FP64_FILM: accumulate in double */
	uint32_t wave_paths;        /* paths per wavefront wave; 0 = 4 Mi (1 Mi while recording) */
	gbrt_guide *guide;          /* path-guiding network, or NULL for plain path tracing */
	float guide_alpha;          /* probability of sampling the guide (one-sample MIS); 0 = plain */
	uint32_t guide_train_steps; /* Adam steps on this render's own records after each wave; 0 = none */
	uint32_t guide_batch;       /* records per step; 0 = 65536 */
	uint32_t guide_max_vertex;  /* guide (and record) only vertices 0 .. guide_max_vertex - 1; 0 = all */
	int32_t raydepth;           /* "raydepth": last ray level of the recursive glossy / specular split
	                               (MonteCarloIntegrator::recursiveRaytrace); 0 = 5 */
	/* Film filter (ImageFilm "filter_type", "AA_pixelwidth"; imagefilm.cc:231-264, 771-822).
	 * GBRT_FILTER_PIXEL (0): each sample lands in its own pixel only and the
	 * film holds plain sums (mean = sum / spp).  Any other type splats every
	 * sample over the reference's filter footprint and adds the filter weights
	 * to film_weight_dev (device, resx * resy floats, caller-zeroed); the
	 * image is sum / weight per pixel, as ImageFilm::flush normalises. */
	uint32_t filter_type;
	float aa_pixel_width;       /* 0 = 1.5 (the reference's default) */
	float *film_weight_dev;
	/* Transparent shadows (MonteCarloIntegrator "transpShad", "shadowDepth";
	 * Accelerator::isShadowedTransparentShadow, accelerator.h:113-169): shadow
	 * rays pass transparent materials (shinydiffuse with transparency, glass /
	 * rough_glass with fake_shadows) times their filter colour; more than
	 * shadow_depth of them block.  shadow_depth is used as given (the
	 * reference's default is 4). */
	int32_t transparent_shadows;
	int32_t shadow_depth;
	/* PathIntegrator "caustic_type" (integrator_path_tracer.h:40-59): path
	 * caustics (emission reached through specular / glossy / filter samples
	 * after the first bounce), photon caustics (a caustic photon map,
	 * CausticPhotonIntegrator::createCausticMap, estimated at the camera-path
	 * root of diffuse surfaces), both or none.  GBRT_CAUSTIC_PATH (0) is the
	 * reference's default. */
	uint32_t caustic_type;
	/* "no_recursive" [false]: the path loop starts at every first hit and
	 * samples all BSDF components there (integrator_path_tracer.cc:177-200). */
	int32_t no_recursive;
	/* Caustic photon map of caustic_type photon / both: caustic_photons,
	 * caustic_mix, caustic_radius, caustic_depth of a gbrt_pm_params, NULL =
	 * the reference's defaults (500000, 50, 0.25, 10). */
	const struct gbrt_pm_params *caustic;
	/* ImageFilm "AA_clamp_indirect" [0 = off]: photon caustic estimates and
	 * final-gather results brighter than this are scaled down to it
	 * (Rgb::clampProportionalRgb; integrator_photon_caustic.cc:94,
	 * integrator_photon_mapping.cc:727). */
	float clamp_indirect;
} gbrt_pt_params;

#define GBRT_CAUSTIC_PATH 0u
#define GBRT_CAUSTIC_NONE 1u
#define GBRT_CAUSTIC_PHOTON 2u
#define GBRT_CAUSTIC_BOTH 3u

/* Adaptive anti-aliasing (ImageFilm / TiledIntegrator parameters with the
 * reference's names and defaults in brackets). */
typedef struct gbrt_aa_params {
	int32_t passes;                          /* AA_passes [1] */
	int32_t inc_samples;                     /* AA_inc_samples [1] */
	float threshold;                         /* AA_threshold [0.05] */
	float resampled_floor;                   /* AA_resampled_floor, percent of the pixels [0] */
	float sample_multiplier_factor;          /* AA_sample_multiplier_factor [1] */
	float light_sample_multiplier_factor;    /* AA_light_sample_multiplier_factor [1] */
	float indirect_sample_multiplier_factor; /* AA_indirect_sample_multiplier_factor [1] (final gathering only) */
	int32_t detect_color_noise;              /* AA_detect_color_noise [0] */
	int32_t dark_detection_type;             /* AA_dark_detection_type: 0 none [default], 1 linear, 2 curve */
	float dark_threshold_factor;             /* AA_dark_threshold_factor [0] */
	int32_t variance_edge_size;              /* AA_variance_edge_size [10] */
	int32_t variance_pixels;                 /* AA_variance_pixels [0] */
} gbrt_aa_params;

#define GBRT_FILTER_PIXEL 0u
#define GBRT_FILTER_BOX 1u
#define GBRT_FILTER_GAUSS 2u
#define GBRT_FILTER_MITCHELL 3u
#define GBRT_FILTER_LANCZOS 4u

typedef struct gbrt_pt_stats {
	uint64_t camera_samples;
	uint64_t extension_rays;    /* camera + path continuation rays traced */
	uint64_t shadow_rays;       /* shadow rays traced */
	float ms;                   /* device time of the render (CUDA events) */
	/* photonmapping only (gbrt_pm_render) */
	uint64_t photon_paths;      /* diffuse + caustic photon paths shot */
	uint64_t photons_stored;    /* diffuse + caustic photons deposited */
	uint64_t radiance_photons;  /* radiance-map photons after thinning */
	float photon_ms;            /* device time of the photon-map preprocess */
} gbrt_pt_stats;

typedef struct gbrt_scene gbrt_scene;

/* Scene for rendering over a built BVH (borrowed; must outlive the scene).
 * vertices/faces are the host arrays the BVH was built from (geometric
 * normals are taken from them); face_material[i] indexes `materials`. */
int gbrt_scene_create(const gbrt_bvh *bvh, const float *vertices, uint32_t n_vertices,
                      const uint32_t *faces, uint32_t n_faces, const int32_t *face_material,
                      const gbrt_material_desc *materials, uint32_t n_materials,
                      const gbrt_light_desc *lights, uint32_t n_lights, gbrt_scene **out);
int gbrt_scene_destroy(gbrt_scene *scene);

/* ---- per-vertex shading normals ------------------------------------------
 * A face whose vertices carry normals shades with the barycentric (quads:
 * bilinear) interpolation of them, normalised, instead of its geometric
 * normal: the smooth branch of PrimitivePolygon::getSurfacePolygon
 * (src/geometry/primitive/primitive_polygon.cc:49-56); a vertex without a
 * normal (GBRT_NO_NORMAL) contributes the face's geometric normal
 * (FacePrimitive::getVertexNormal, primitive_face.h:106-110). */
#define GBRT_NO_NORMAL 0xFFFFFFFFu
/* First index of a face that shades with its geometric normal (a face of a
 * mesh without vertex normals, PrimitivePolygon's flat branch). */
#define GBRT_FLAT_FACE 0xFFFFFFFEu

/* The reference's yafaray_smoothObjectMesh(angle) on one mesh object
 * (MeshObject::smoothVerticesNormals, src/geometry/object/object_mesh.cc:150-262),
 * on the host: angle >= 180 averages every face at a vertex (weighted by the
 * corner angle, one normal per vertex); 0.1 < angle < 180 smooths across
 * faces whose normals lie within `angle` degrees (new normals appended after
 * n_vertices zero entries); otherwise no normals.  Outputs: normals (3
 * floats each, capacity normals_cap; NULL to query *n_normals only) and
 * face_normals (4 indices per face, GBRT_NO_NORMAL where the face keeps its
 * geometric normal).  At most n_vertices + 4 * n_faces normals. */
int gbrt_mesh_smooth_normals(const float *vertices, uint32_t n_vertices, const uint32_t *faces, uint32_t n_faces,
                             float angle, float *normals, uint32_t normals_cap, uint32_t *n_normals,
                             uint32_t *face_normals);

/* Shading normals of a scene's faces (replacing any set before): normals
 * (n_normals x 3 floats, the vertex normals of yafaray_addNormal or
 * gbrt_mesh_smooth_normals) and face_normals (4 indices per face of
 * gbrt_scene_create, the 4th unused for triangles, GBRT_NO_NORMAL for a
 * vertex without a normal, GBRT_FLAT_FACE first for a face of a mesh
 * without vertex normals).  NULL face_normals returns every face to its
 * geometric normal.  Fewer than 0xFFFFFFFD normals. */
int gbrt_scene_set_normals(gbrt_scene *scene, const float *normals, uint32_t n_normals, const uint32_t *face_normals);

/* ---- textures on shinydiffuse diffuse colour -----------------------------
 * An ImageTexture (src/texture/texture_image.cc) over an in-memory float
 * image, or a procedural texture (blend, clouds, marble, wood, voronoi,
 * musgrave, distorted_noise, rgb_cube: src/texture/texture_*.cc), reached
 * through a TextureMapperNode (src/shader/shader_node_texture.cc) set as a
 * shinydiffuse material's "diffuse_shader": the texture's colour replaces
 * the material's diffuse colour wherever the reference reads
 * getShaderColor(Diffuse) (eval, sample, pdf weights, transmit filter,
 * emission).  Parameter names and defaults [..] are the reference's. */
enum { GBRT_TEXCO_GLOBAL = 0, GBRT_TEXCO_UV = 1 };                 /* "texco" ["global"] */
enum { GBRT_MAPPING_PLAIN = 0, GBRT_MAPPING_CUBE = 1, GBRT_MAPPING_TUBE = 2, GBRT_MAPPING_SPHERE = 3 };   /* "mapping" ["plain"] */
enum { GBRT_CLIP_EXTEND = 0, GBRT_CLIP_CLIP = 1, GBRT_CLIP_CLIPCUBE = 2, GBRT_CLIP_REPEAT = 3, GBRT_CLIP_CHECKER = 4 };   /* "clipping" ["repeat"] */
enum { GBRT_INTERP_NONE = 0, GBRT_INTERP_BILINEAR = 1, GBRT_INTERP_BICUBIC = 2 };   /* "interpolate" ["bilinear"] */

/* Texture "type" (Texture::Type, include/texture/texture.h:70-84). */
enum { GBRT_TEX_IMAGE = 0, GBRT_TEX_BLEND = 1, GBRT_TEX_CLOUDS = 2, GBRT_TEX_MARBLE = 3, GBRT_TEX_WOOD = 4, GBRT_TEX_VORONOI = 5,
       GBRT_TEX_MUSGRAVE = 6, GBRT_TEX_DISTORTED_NOISE = 7, GBRT_TEX_RGB_CUBE = 8 };
/* "noise_type" (NoiseGenerator::NoiseType, include/noise/noise_generator.h:32-45) ["newperlin"] */
enum { GBRT_NOISE_BLENDER = 0, GBRT_NOISE_STDPERLIN = 1, GBRT_NOISE_NEWPERLIN = 2, GBRT_NOISE_CELL = 3, GBRT_NOISE_VORONOI_F1 = 4,
       GBRT_NOISE_VORONOI_F2 = 5, GBRT_NOISE_VORONOI_F3 = 6, GBRT_NOISE_VORONOI_F4 = 7, GBRT_NOISE_VORONOI_F2F1 = 8,
       GBRT_NOISE_VORONOI_CRACKLE = 9 };
/* voronoi "distance_metric" ["real"] */
enum { GBRT_DIST_REAL = 0, GBRT_DIST_SQUARED = 1, GBRT_DIST_MANHATTAN = 2, GBRT_DIST_CHEBYCHEV = 3, GBRT_DIST_MINKOVSKY_HALF = 4,
       GBRT_DIST_MINKOVSKY_FOUR = 5, GBRT_DIST_MINKOVSKY = 6 };
/* blend "blend_type" ["linear"] */
enum { GBRT_PROGRESSION_LINEAR = 0, GBRT_PROGRESSION_QUADRATIC = 1, GBRT_PROGRESSION_EASING = 2, GBRT_PROGRESSION_DIAGONAL = 3,
       GBRT_PROGRESSION_SPHERE = 4, GBRT_PROGRESSION_QUAD_SPHERE = 5, GBRT_PROGRESSION_RADIAL = 6 };
enum { GBRT_BIAS_NONE = 0, GBRT_BIAS_POSITIVE = 1, GBRT_BIAS_NEGATIVE = 2 };          /* clouds "bias" ["none"] */
enum { GBRT_SHAPE_SIN = 0, GBRT_SHAPE_SAW = 1, GBRT_SHAPE_TRI = 2 };                  /* marble / wood "shape" ["sin"] */
enum { GBRT_WOOD_BANDS = 0, GBRT_WOOD_RINGS = 1 };                                    /* wood "wood_type" ["bands"] */
/* voronoi "color_mode" ["intensity-without-color"] */
enum { GBRT_VORONOI_INTENSITY = 0, GBRT_VORONOI_POSITION = 1, GBRT_VORONOI_POSITION_OUTLINE = 2,
       GBRT_VORONOI_POSITION_OUTLINE_INTENSITY = 3 };
/* musgrave "musgrave_type" ["fBm"] */
enum { GBRT_MUSGRAVE_FBM = 0, GBRT_MUSGRAVE_MULTIFRACTAL = 1, GBRT_MUSGRAVE_HETERO = 2, GBRT_MUSGRAVE_HYBRID = 3,
       GBRT_MUSGRAVE_RIDGED = 4 };
/* colour ramp "ramp_color_mode" ["RGB"], "ramp_interpolation" ["LINEAR"],
 * "ramp_hue_interpolation" ["NEAR"] (include/color/color_ramp.h:50-80) */
enum { GBRT_RAMP_RGB = 0, GBRT_RAMP_HSV = 1, GBRT_RAMP_HSL = 2 };
enum { GBRT_RAMP_LINEAR = 0, GBRT_RAMP_CONSTANT = 1 };
enum { GBRT_HUE_NEAR = 0, GBRT_HUE_FAR = 1, GBRT_HUE_CLOCKWISE = 2, GBRT_HUE_COUNTERCLOCKWISE = 3 };
#define GBRT_RAMP_MAX 16

/* The parameters of a procedural texture (reference names and defaults). */
typedef struct gbrt_procedural_desc {
	uint32_t noise_type;        /* "noise_type" (distorted_noise: "noise_type1") [GBRT_NOISE_NEWPERLIN] */
	uint32_t noise_type2;       /* distorted_noise "noise_type2" [GBRT_NOISE_NEWPERLIN] */
	float color1[3], color2[3]; /* "color1" [0, 0, 0], "color2" [1, 1, 1] */
	float size;                 /* "size" [1] */
	int32_t depth;              /* clouds / marble / wood "depth" [2] */
	int32_t hard;               /* "hard" [0] */
	uint32_t bias;              /* clouds GBRT_BIAS_* */
	uint32_t shape;             /* marble / wood GBRT_SHAPE_* */
	uint32_t wood_type;         /* GBRT_WOOD_* */
	uint32_t blend_type;        /* blend GBRT_PROGRESSION_* */
	int32_t use_flip_axis;      /* blend "use_flip_axis" [0] */
	float sharpness;            /* marble "sharpness" [1] */
	float turbulence;           /* marble / wood "turbulence" [1] */
	uint32_t distance_metric;   /* voronoi GBRT_DIST_* */
	uint32_t color_mode;        /* voronoi GBRT_VORONOI_* */
	float weight[4];            /* voronoi "weight1" .. "weight4" [1, 0, 0, 0] */
	float mk_exponent;          /* voronoi "mk_exponent" [2.5] */
	float intensity;            /* voronoi / musgrave "intensity" [1] */
	uint32_t musgrave_type;     /* GBRT_MUSGRAVE_* */
	float h, lacunarity, octaves, offset, gain;   /* musgrave "H" [1], "lacunarity" [2], "octaves" [2], "offset" [1], "gain" [1] */
	float distort;              /* distorted_noise "distort" [1] */
	int32_t ramp_n;             /* "ramp_num_items" [0]: no ramp; at most GBRT_RAMP_MAX */
	uint32_t ramp_mode, ramp_interpolation, ramp_hue_interpolation;
	float ramp[GBRT_RAMP_MAX][5];   /* "ramp_item_<i>_color" RGBA and "_position", any order */
} gbrt_procedural_desc;
/* Zero-initialised descriptor with the reference's defaults. */
void gbrt_procedural_defaults(gbrt_procedural_desc *d);

typedef struct gbrt_texture_desc {
	int32_t width, height;
	const float *rgba;          /* host, height rows of width RGBA floats (image x, y -> rgba[4 (y width + x)]),
	                               linear colour (an Image with image_optimization "none") */
	uint32_t interpolate;       /* GBRT_INTERP_* */
	uint32_t clipping;          /* GBRT_CLIP_* */
	int32_t xrepeat, yrepeat;   /* [1, 1] */
	float crop[4];              /* cropmin_x, cropmin_y, cropmax_x, cropmax_y [0, 0, 1, 1] */
	int32_t rot90;              /* [0] */
	float adj_intensity, adj_contrast;     /* [1, 1] */
	float adj_mult_factor[3];   /* red, green, blue [1, 1, 1] */
	int32_t adj_clamp;          /* [0] */
	/* the texture mapper node */
	uint32_t texco;             /* GBRT_TEXCO_* */
	uint32_t mapping;           /* GBRT_MAPPING_* */
	float scale[3];             /* [1, 1, 1] */
	float offset[3];            /* [0, 0, 0] */
	int32_t proj[3];            /* proj_x, proj_y, proj_z: 0 zero, 1 x, 2 y, 3 z [1, 2, 3] */
	/* optional LayerNode over the mapper (src/shader/shader_node_layer.cc:110-193;
	 * colour part, colour input, no upper layer): the material's diffuse
	 * shader is then the layer */
	int32_t layer;              /* 0: the mapper is the diffuse shader; 1: a layer node over it */
	uint32_t blend_mode;        /* GBRT_BLEND_* ["mix"] */
	float colfac;               /* [1] */
	float upper_color[4];       /* [0, 0, 0, 0] (exporters pass the material colour, alpha 1) */
	float def_col[3];           /* [1, 1, 1] */
	int32_t negative, no_rgb, stencil;   /* "negative", "noRGB", "stencil" [0] */
	int32_t mirror_x, mirror_y; /* "mirror_x", "mirror_y" [0]: every other repeat mirrored (clipping repeat) */
	int32_t even_tiles, odd_tiles;       /* clipping checker: "even_tiles" [0], "odd_tiles" [1] (set it: 0 hides those tiles) */
	float checker_dist;         /* "checker_dist" [0]: tiles shrunk about their centres by 1 / (1 - checker_dist) */
	uint32_t kind;              /* GBRT_TEX_* [GBRT_TEX_IMAGE]; procedural textures ignore the image fields
	                               (width, height, rgba, interpolate, clipping, repeats, crop, rot90, mirror, tiles) */
	float adj_saturation, adj_hue;   /* "adj_saturation" [1], "adj_hue" (degrees) [0]: a zeroed descriptor has
	                                    saturation 0, so set them */
	gbrt_procedural_desc proc;  /* kind != GBRT_TEX_IMAGE */
} gbrt_texture_desc;

/* libYafaRay's noise tables (NoiseGenerator::hash_ / hashpntf_,
 * BlenderNoiseGenerator::hashvectf_, StdPerlinNoiseGenerator::stdp_p_ /
 * stdp_g_): the procedural textures index them, and the library carries
 * no copy, so the host hands them over (512 bytes, 768 floats, 768 floats,
 * 514 bytes, 514 x 3 floats). */
typedef struct gbrt_noise_tables {
	const uint8_t *hash;
	const float *hashpntf;
	const float *hashvectf;
	const uint8_t *stdp_p;
	const float *stdp_g;
} gbrt_noise_tables;
/* The scene's noise tables, required before gbrt_scene_set_textures takes
 * a procedural texture. */
int gbrt_scene_set_noise_tables(gbrt_scene *scene, const gbrt_noise_tables *tables);
/* ---- shader node trees on material colour slots -------------------------
 * The reference's shader nodes (src/shader/: texture_mapper, value, mix
 * with its nine blend modes, layer) as a node array; every material colour
 * slot may name a root node, whose tree (the root and every node it reads,
 * all at lower indices) is evaluated per surface point as the reference's
 * Material::evalNodes does.  A texture_mapper node reads a texture of
 * gbrt_scene_set_textures (its texco / mapping / scale / offset / proj are
 * the mapper's; the texture's own layer fields are not used here).
 * Parameter names and defaults [..] are the reference's. */
enum { GBRT_NODE_TEXTURE = 0, GBRT_NODE_VALUE = 1, GBRT_NODE_MIX = 2, GBRT_NODE_LAYER = 3 };
/* mix "blend_mode" (shader_node_mix.h:51-66) ["mix"]; layer nodes take GBRT_BLEND_* */
enum { GBRT_MIX_MIX = 0, GBRT_MIX_ADD = 1, GBRT_MIX_MULTIPLY = 2, GBRT_MIX_SUBTRACT = 3, GBRT_MIX_SCREEN = 4, GBRT_MIX_DIFFERENCE = 5,
       GBRT_MIX_DARKEN = 6, GBRT_MIX_LIGHTEN = 7, GBRT_MIX_OVERLAY = 8 };
/* material slots: shinydiffuse / glossy "diffuse_shader", glossy
 * "glossy_shader", shinydiffuse / glass / rough_glass "mirror_color_shader",
 * glass / rough_glass "filter_color_shader", "bump_shader" */
enum { GBRT_SLOT_DIFFUSE = 0, GBRT_SLOT_GLOSSY = 1, GBRT_SLOT_MIRROR_COLOR = 2, GBRT_SLOT_FILTER_COLOR = 3, GBRT_SLOT_BUMP = 4,
       GBRT_SLOTS = 5 };
#define GBRT_TREE_MAX 16          /* index span from a root back to the lowest node it reads */
typedef struct gbrt_shader_node {
	uint32_t type;              /* GBRT_NODE_* */
	int32_t texture;            /* texture_mapper: texture index */
	int32_t do_scalar;          /* texture_mapper "do_scalar" [1]; layer "do_scalar" [0] */
	/* mix: "input1", "input2", "input_factor"; layer: input1 = "input", input2 = "upper_layer"
	 * (node indices below this node's, or -1) */
	int32_t input1, input2, input_factor;
	float color1[4], color2[4]; /* mix "color1", "color2" [0]; value: color1 = "color" + "alpha" [1, 1];
	                               layer: color1 = "upper_color" [0] */
	float value1, value2;       /* mix "value1", "value2" [0]; value: value1 = "scalar" [1]; layer: value1 = "upper_value" [0] */
	float factor;               /* mix "cfactor" [0.5] */
	uint32_t mode;              /* mix GBRT_MIX_*; layer "blend_mode" GBRT_BLEND_* */
	float def_col[4];           /* layer "def_col" [1] */
	float def_val, colfac, valfac;   /* layer "def_val" [1], "colfac" [1], "valfac" [1] */
	int32_t do_color, color_input, use_alpha, no_rgb, stencil, negative;   /* layer [1, 1, 0, 0, 0, 0] */
	float bump_strength;        /* texture_mapper "bump_strength" [1] (bump slot) */
} gbrt_shader_node;
/* The scene's node trees (replacing any set before; textures first).
 * material_slots: n_materials x GBRT_SLOTS root node indices, -1 for none. */
int gbrt_scene_set_shader_nodes(gbrt_scene *scene, const gbrt_shader_node *nodes, uint32_t n_nodes, const int32_t *material_slots,
                                uint32_t n_materials);

/* Diagnostics: a texture's getColor (RGBA) and getFloat at n texture-space
 * points (xyz, after the mapper) on the host or, on_device != 0, in a
 * kernel (host buffers either way; synchronises).  Procedural kinds only. */
int gbrt_texture_eval(const gbrt_texture_desc *texture, const gbrt_noise_tables *tables, const float *points, uint32_t n,
                      float *rgba, float *value, int on_device);
enum { GBRT_BLEND_MIX = 0, GBRT_BLEND_ADD = 1, GBRT_BLEND_MULTIPLY = 2, GBRT_BLEND_SUBTRACT = 3, GBRT_BLEND_SCREEN = 4,
       GBRT_BLEND_DIVIDE = 5, GBRT_BLEND_DIFFERENCE = 6, GBRT_BLEND_DARKEN = 7, GBRT_BLEND_LIGHTEN = 8 };

/* Texture coordinates and textures of a scene (replacing any set before).
 * uv: n_uv (u, v) pairs (yafaray_addUv); face_uv: one uint32 quadruple per
 * face of gbrt_scene_create, the uv indices of its vertices (the 4th unused
 * for triangles), or NULL (no uvs: the implicit barycentric uv).
 * material_diffuse_texture[m]: texture index driving material m's diffuse
 * colour, -1 for none (n_materials entries; shinydiffuse materials only).
 * Limits: fewer than 2^31 texels per texture and 2^32 in all (else
 * GBRT_ERR_CAPACITY). */
int gbrt_scene_set_textures(gbrt_scene *scene, const float *uv, uint32_t n_uv, const uint32_t *face_uv,
                            const gbrt_texture_desc *textures, uint32_t n_textures,
                            const int32_t *material_diffuse_texture, uint32_t n_materials);

/* Renders spp samples per pixel and ADDS each pixel's sample sum (RGB,
 * resx*resy*3, row-major from the top-left) to film_dev (float) or
 * film64_dev (double, when not NULL).  Asynchronous on `stream` unless
 * `stats` is given (then it synchronises to read the ray counts). */
int gbrt_pt_render(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params,
                   float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream);

/* Same into a host image of per-pixel means (sum / spp), resx*resy*3 floats. */
int gbrt_pt_render_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params,
                        float *image_out, gbrt_pt_stats *stats);


/* TiledIntegrator::render with adaptive anti-aliasing (integrator_tiled.cc:
 * 160-214, ImageFilm::nextPass imagefilm.cc:365-547): pass 0 renders every
 * pixel with params->spp (AA_minsamples) samples; each later pass flags the
 * pixels whose normalised colour differs from a neighbour's by the
 * threshold (dark detection, variance window, threshold lowered below the
 * resampled floor) and renders AA_inc_samples x multiplier more samples in
 * those only.  With more than one pass, sample positions are riVdC / riS.
 * params->filter_type must not be GBRT_FILTER_PIXEL and
 * film_weight_dev is required (device, caller-zeroed, like film_dev);
 * resampled (optional, aa->passes entries): pixels sampled per pass. */
int gbrt_pt_render_aa(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params,
                      const gbrt_aa_params *aa, float *film_dev, gbrt_pt_stats *stats, uint32_t *resampled, void *stream);
/* Same into a host image of resx * resy * 3 floats (sum / weight); the film
 * and weight buffers are allocated inside the call. */
int gbrt_pt_render_aa_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params,
                           const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled);
/* Diagnostics: the pixels ImageFilm::nextPass would flag for resampling on a
 * device film (sums, weights) at the given threshold; flags_dev = 1 byte per
 * pixel.  Synchronises. */
int gbrt_aa_flags(const float *film_dev, const float *weight_dev, int32_t resx, int32_t resy, const gbrt_aa_params *aa,
                  float threshold, uint8_t *flags_dev, uint32_t *n_flagged);

/* ---- a batch of scenes in one wavefront ------------------------------------
 * n scenes (each with its camera, parameters and device film) rendered
 * together: every scene's camera samples form one index range, each wave of
 * the wavefront takes a stretch of it across scenes, and every kernel of a
 * vertex level serves all of them (the per-scene render loop of
 * TiledIntegrator::render, integrator_tiled.cc:222-251, for many scenes at
 * once).  pathtracing only: no guide and no photon caustics; the scenes must
 * agree on film filtering and transparent shadows.  Several waves may be in
 * flight at once, each on its own stream in the work buffers of one of the
 * batch's scenes (released after the call).  Synchronises `stream`.
 *
 * tuning: NULL, or in/out: a zero field is chosen by the autotuner (short
 * device-timed trial renders of the whole batch at 1 sample per pixel into
 * scratch films: the waves in flight, the wave size, the shading block
 * size, then the residency of the persistent traversal grids), which writes
 * back what it chose and the device time it spent; pass the result back to
 * skip tuning.
 * stats: NULL or one entry with the batch's totals. */
typedef struct gbrt_batch_tuning {
	uint32_t wave_paths;            /* paths per wave (the spawn buffers may cap it) */
	uint32_t shade_block;           /* threads per block of the shading kernel, 32 .. 128 */
	uint32_t trace_blocks_per_sm;   /* resident blocks per SM of the traversal grids */
	uint32_t streams;               /* waves in flight, each on its own stream (and host thread),
	                                   in the buffers of scenes 0 .. streams - 1 */
	float tune_ms;                  /* out: device time of the trial renders */
} gbrt_batch_tuning;
int gbrt_pt_render_multi(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params,
                         float *const *films, uint32_t n, gbrt_batch_tuning *tuning, gbrt_pt_stats *stats, void *stream);

/* gbrt_pt_render_multi with the autotuner on the default stream (concurrency
 * is unused).  stats: NULL or n entries: each scene's camera samples, the
 * batch's ray counts and device time in entry 0. */
int gbrt_pt_render_batch(gbrt_scene *const *scenes, const gbrt_camera_desc *cameras, const gbrt_pt_params *params, float *const *films,
                         uint32_t n, uint32_t concurrency, gbrt_pt_stats *stats);

/* ---- photon mapping (the `photonmapping` integrator) ---------------------
 * Replaces PhotonIntegrator::preprocess / integrate / finalGathering and
 * CausticPhotonIntegrator's caustic map and estimate
 * (src/integrator/surface/integrator_photon_mapping.cc:157-828,
 * integrator_photon_caustic.cc:102-304) with photon maps held as hashed
 * grids on the device instead of PointKdTree (include/photon/pkdtree.h).
 * Parameter names and defaults are the reference's; photon paths use Halton
 * indices 0 .. n - 1, the set the reference shoots when n is a multiple of
 * its photon threads (threads_photons). */
typedef struct gbrt_pm_params {
	int32_t diffuse_photons;    /* "diffuse_photons" (100000) */
	int32_t caustic_photons;    /* "caustic_photons" (500000) */
	float diffuse_radius;       /* "diffuse_radius" (0.1) */
	int32_t diffuse_search;     /* "diffuse_search" (50), at most 64 */
	float caustic_radius;       /* "caustic_radius" (0.25) */
	int32_t caustic_mix;        /* "caustic_mix" (50), at most 64 */
	int32_t caustic_depth;      /* "caustic_depth" (10) */
	int32_t bounces;            /* "bounces" (3): diffuse photon bounces */
	int32_t caustics;           /* "caustics" (0): build and use the caustic map */
	int32_t diffuse;            /* "diffuse" (1): build and use the diffuse map */
	int32_t final_gather;       /* "finalGather" (1) */
	int32_t fg_samples;         /* "fg_samples" (32) */
	int32_t fg_bounces;         /* "fg_bounces" (2) */
	float fg_min_pathlen;       /* "fg_min_pathlen"; < 0 = diffuse_radius */
} gbrt_pm_params;
int gbrt_pm_default_params(gbrt_pm_params *params);
/* Renders like gbrt_pt_render with the photonmapping integrator: builds the
 * photon maps (and, with final gather, the radiance map) on the device, then
 * traces the camera samples.  spp, base_sampling_offset, raydepth, seed,
 * flags and wave_paths of `params` apply; path_samples, bounces and the
 * guide fields are not used. */
int gbrt_pm_render(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                   float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream);
/* gbrt_pm_render into a temporary device film; per-pixel means copied to
 * image_out [resy][resx][3] (host). */
int gbrt_pm_render_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                        float *image_out, gbrt_pt_stats *stats);
/* The `directlighting` integrator (DirectLightIntegrator::integrate,
 * src/integrator/surface/integrator_direct_light.cc:97-152): emission,
 * all-light estimation at diffuse hits, the recursive glossy / specular
 * split, and, when caustic != NULL and caustic->caustics, the caustic photon
 * map of CausticPhotonIntegrator (caustic_photons, caustic_radius,
 * caustic_mix, caustic_depth of `caustic`).  Ambient occlusion is not built. */
int gbrt_dl_render(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                   float *film_dev, double *film64_dev, gbrt_pt_stats *stats, void *stream);
int gbrt_dl_render_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                        float *image_out, gbrt_pt_stats *stats);
/* The same passes for the photonmapping and directlighting integrators over
 * photon maps built once (PhotonIntegrator::preprocess), with the host film
 * of gbrt_pm_render_host / gbrt_dl_render_host.  With final gathering,
 * AA_indirect_sample_multiplier_factor must be 1 (the multiplied gather
 * counts are not built). */
int gbrt_pm_render_aa_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *pm,
                           const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled);
int gbrt_dl_render_aa_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_pm_params *caustic,
                           const gbrt_aa_params *aa, float *image_out, gbrt_pt_stats *stats, uint32_t *resampled);

/* ---- stochastic progressive photon mapping (the `SPPM` integrator) -------
 * Replaces SppmIntegrator::render / prePass / photonWorker / traceGatherRay
 * (src/integrator/surface/integrator_sppm.cc:99-1053).  Each of `passes`
 * passes shoots `photons` photon paths (indirect deposits only, `bounces`
 * deep), traces one eye sample per pixel at the multipass sample position of
 * sample index base_sampling_offset + pass (emission, direct light at
 * diffuse hits, the recursive glossy / specular split of traceGatherRay),
 * gathers the caustic photons within each pixel's radius at diffuse hits,
 * refines the radius (alpha 0.7) and adds acc_flux / (r^2 pi photons so far)
 * + the eye sample's radiance to the film.  As in the reference, only the
 * caustic map enters the estimate (its diffuse-map accumulation runs under
 * debug logging only).  The initial radius comes from the scene bound and
 * resolution (initializePpm).  params: spp is ignored
 * (one sample per pass), path_samples / bounces / russian roulette are not
 * used; raydepth, transparent shadows and the film filter are. */
typedef struct gbrt_sppm_params {
	int32_t photons;            /* "photons" [500000] */
	int32_t passes;             /* "passNums" [1000] */
	int32_t bounces;            /* "bounces" [5] */
	/* initial radius estimate ("pmIRE", first pass only, traceGatherRay
	 * :648-667): the first gather point of a pixel takes the smaller of the
	 * radii of its searchNum nearest diffuse and caustic photons within
	 * photonRadius */
	int32_t pm_ire;             /* "pmIRE" [0] */
	float photon_radius;        /* "photonRadius" [1] */
	int32_t search_num;         /* "searchNum" [10], at most 64 */
} gbrt_sppm_params;

int gbrt_sppm_render(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_sppm_params *sppm,
                     float *film_dev, gbrt_pt_stats *stats, void *stream);
int gbrt_sppm_render_host(gbrt_scene *scene, const gbrt_camera_desc *camera, const gbrt_pt_params *params, const gbrt_sppm_params *sppm,
                          float *image_out, gbrt_pt_stats *stats);
/* Diagnostic: shoots one photon map (which = 0 diffuse, 1 caustic) and copies
 * its photons to host `out` [n][9] = (dir xyz, pos xyz, colour rgb) in
 * deposit order; n_photons and n_paths as PhotonMap::nPhotons / nPaths. */
int gbrt_pm_photons(gbrt_scene *scene, const gbrt_pm_params *pm, int which, float *out, uint32_t capacity, uint32_t *n_photons,
                    uint32_t *n_paths);
/* Diagnostic: the photon grid's bucket of each of n host points (xyz) with
 * the reference HashGrid's cell assignment (src/photon/hashgrid.cc:59-75):
 * cell coordinates |int((p - box_lo) x float(1 / cell_size))|, bucket
 * (ix 73856093 ^ iy 19349663 ^ iz 83492791) mod grid_size.  The photon
 * maps are bucketed this way with grid_size = the photon count (at least
 * 1024) and cell_size a hair above the search radius. */
int gbrt_grid_buckets(const float *points, uint32_t n, double cell_size, uint32_t grid_size, const float box_lo[3], uint32_t *bucket_out);
/* Diagnostic: k-nearest gather of PhotonMap::gather semantics over n host
 * points (xyz) for m host queries through the device grid (cell edge >= the
 * search radius): per query the count, the final squared radius and the
 * indices of the found points ([m][k], unordered). */
int gbrt_knn_gather(const float *points, uint32_t n, const float *queries, uint32_t m, float cell, int k, float r2,
                    int32_t *count_out, float *r2_out, uint32_t *idx_out);

/* ---- path-guiding network (no counterpart in the reference) -------------
 * q(w | x): 8-lobe von Mises-Fisher mixture over incident direction,
 * predicted from the hit position by a 16-level x 2-feature hash-grid
 * encoding (2^log2_table entries per level) and an MLP 32 -> 64 -> 64 -> 40.
 * Trained online on records {position xyz, sampled direction xyz,
 * weight = luminance(incident radiance) / sampling pdf, pad} (8 floats),
 * minimising the Monte-Carlo KL divergence  -sum c log q / sum c  with Adam. */
typedef struct gbrt_guide_params {
	uint32_t log2_table;        /* 0 -> 19 */
	float base_resolution;      /* 0 -> 16 */
	float max_resolution;       /* 0 -> 2048 */
	float learning_rate;        /* 0 -> 5e-3 */
	uint32_t seed;
} gbrt_guide_params;

int gbrt_guide_create(const float bound[6], const gbrt_guide_params *params, gbrt_guide **out);
int gbrt_guide_destroy(gbrt_guide *guide);
int gbrt_guide_info(const gbrt_guide *guide, uint32_t *n_mlp_params, uint64_t *n_table_params);
/* Copy parameters out / in (host buffers; either pointer may be NULL).
 * MLP layout: W1[64][32] b1[64] W2[64][64] b2[64] W3[40][64] b3[40];
 * table: [16 levels][2^log2_table][2 features]. */
int gbrt_guide_get_params(const gbrt_guide *guide, float *mlp, float *table);
int gbrt_guide_set_params(gbrt_guide *guide, const float *mlp, const float *table);
/* Mixture parameters for n positions (device, 3 floats each): 40 floats per
 * position, per lobe {mu xyz, kappa, weight}. */
int gbrt_guide_eval(gbrt_guide *guide, const float *pos_dev, uint32_t n, float *lobes_dev, void *stream);
/* Units that run the network (gbrt_guide_eval, the path tracer's per-vertex
 * evaluation, and the forward/backward pass of gbrt_guide_grad and
 * gbrt_guide_step): tensor cores (tcgen05, BF16 operands and activations,
 * FP32 accumulation; the default) or FP32 CUDA cores. */
enum { GBRT_GUIDE_EVAL_TENSOR = 0, GBRT_GUIDE_EVAL_FP32 = 1 };
int gbrt_guide_set_eval_mode(gbrt_guide *guide, int mode);
/* Reads and clears the guide's device status flags (synchronous):
 * bit 0 = a tensor-core MMA completion wait timed out (that kernel stopped
 * early and its outputs are incomplete). */
int gbrt_guide_status(gbrt_guide *guide, uint32_t *flags);
/* Diagnostic: D[128][N] = A[128][K] * B[N][K]^T (host FP32 arrays) computed
 * by one tcgen05 MMA chain with BF16 operands (rounded to nearest) and FP32
 * accumulation; N and K multiples of 16 in [16, 64]. */
int gbrt_tc_selftest(const float *A, const float *B, uint32_t N, uint32_t K, float *D);
/* Loss gradient of n records (device) into the guide's gradient buffers;
 * loss_out (host, optional) receives the batch loss (synchronises). */
int gbrt_guide_grad(gbrt_guide *guide, const float *records_dev, uint32_t n, float *loss_out, void *stream);
int gbrt_guide_get_grads(const gbrt_guide *guide, float *mlp_grad, float *table_grad);
/* The same forward pass on the host (no CUDA calls), from explicit
 * parameters in the gbrt_guide_get_params layout: lobes for n positions. */
int gbrt_guide_forward_host(const float bound[6], const gbrt_guide_params *params, const float *mlp, const float *table,
                            const float *pos, uint32_t n, float *lobes);
/* gbrt_guide_grad followed by one Adam step (gradients are cleared). */
int gbrt_guide_step(gbrt_guide *guide, const float *records_dev, uint32_t n, float *loss_out, void *stream);

/* Diagnostics: evaluates one of the path tracer's sampling primitives on n
 * inputs, on the device (on_device != 0) or with the host build of the same
 * code.  kind: 0 Halton::lowDiscrepancySampling(dim, x) (halton.cc:419-439),
 * 1 sample::riVdC, 2 riLp, 3 riS, 4 fnv32ABuf (sample.h:100-148), 5/6
 * Halton base 2/3 radical inverse of x (halton.h:59-85), 7 FAST_TRIG
 * math::sin (dim 0) or math::cos (dim 1) of the float with bits x
 * (math.h:228-265), 8 FAST_MATH math::pow(a, b) with a = float bits of x
 * and b = float bits of dim (math.h:116-146), 9 / 10 kinds 0 / 6 rounded to
 * float as the kernels form them (exact integer arithmetic, no FP64 except
 * for inputs within a rounding margin). */
int gbrt_sampler_eval(int kind, int dim, const uint32_t *input, uint32_t n, double *out, int on_device);

#ifdef __cplusplus
}
#endif

#endif /* GBRT_H */
