// Test-oracle harness: renders a scene with the reference libYafaRay through
// its public C API (yafaray_c_api.h) and dumps the "combined" layer of K
// independent batches (distinct adv_base_sampling_offset values,
// imagefilm.h:194) so per-pixel means and standard errors can be formed.
// The film defaults to a box filter of width 1 (imagefilm.cc:252), which
// lands each sample in its own pixel (apart from samples within 0.001 of a
// pixel edge), so a batch's pixel value is the mean of its spp samples; a
// "film <filter_type> <AA_pixelwidth>" line selects another filter.
// Only tests/golden/make_render_golden.py runs it.
//
// Input: a text scene, one statement per line (# comments):
//   material NAME shinydiffusemat R G B
//   material NAME light_mat R G B POWER
//   material NAME glossy R G B  SR SG SB  EXPONENT  GLOSSY_REFLECT  DIFFUSE_REFLECT
//   material NAME rough_glass IOR ALPHA TRANSMIT_FILTER  FR FG FB  MR MG MB
//   material NAME glass IOR TRANSMIT_FILTER  FR FG FB  MR MG MB
//   object NAME MATERIAL NV NF [NUV]   then NV lines "x y z", NUV lines "u v",
//                                NF lines "a b c" / "a b c d" (with uvs also the
//                                face's uv indices: "a b c ua ub uc")
//   smooth NAME ANGLE            yafaray_smoothObjectMesh on an object defined above
//   image NAME W H               then H lines of W x "r g b a" (an in-memory
//                                ColorAlpha image, image_optimization none, LinearRGB)
//   texture NAME key=value ...   (yafaray_createTexture: type=image image_name=...)
//   node key=value ...           a shader node of the next material line
//                                (e.g. name=tex0 type=texture_mapper texture=...;
//                                "a,b,c" is a vector, "r,g,b,a" a colour);
//                                the material names it (diffuse_shader=tex0)
//   arealight CX CY CZ  P1X P1Y P1Z  P2X P2Y P2Z  R G B  POWER SAMPLES
//   pointlight X Y Z  R G B  POWER
//   camera FX FY FZ  TX TY TZ  UX UY UZ  RESX RESY FOCAL
//   integrator TYPE key=value ...      (ints/floats/bools/strings by key)
//   film FILTER_TYPE PIXEL_WIDTH
//   aa key=value ...                   (ImageFilm AA_* parameters: adaptive passes)
//   render SPP BATCHES THREADS [OFFSET_STRIDE]   (batch k: adv_base_sampling_offset k x stride, default SPP)
// Output (binary): i32 K, H, W; f64 seconds[K]; f32 rgb[K][H][W][3]
// Optional third argument: with photonmapping, the diffuse and caustic photon
// maps after the first batch's preprocess:
//   per map: i32 n_photons, i32 n_paths, f32 [n][9] (dir xyz, pos xyz, col rgb)
// (the maps are private members of PhotonIntegrator, read by opening their
// access for this file only); with an "aa" line, the first batch's adaptive
// passes instead, one record per ImageFilm::nextPass that flagged pixels:
//   i32 pass, f32 threshold, i32 n_flagged, f32 sums[H][W][4] (combined layer
//   before normalisation), f32 weights[H][W], i32 flagged[n] (y W + x)
// read at the pass's first highlight-pixel callback, i.e. the film state the
// detection ran on.
#include "yafaray_c_api.h"
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#define private public
#define protected public
#include "integrator/surface/integrator_photon_mapping.h"
#include "render/imagefilm.h"
#include "image/image_layers.h"
#include "integrator/surface/integrator_sppm.h"
#undef private
#undef protected
#ifdef GB300_BINDING
#include "gb300_binding.h"
#include "common/logger.h"
#include "param/param_result.h"
#include <cstdlib>
#endif

namespace {
struct Film { int w = 0, h = 0; std::vector<float> rgb; };

void putPixel(const char *layer, int x, int y, float r, float g, float b, float a, void *data)
{
	(void)a;
	auto *f = static_cast<Film *>(data);
	if(std::strcmp(layer, "combined") != 0 || x < 0 || y < 0 || x >= f->w || y >= f->h) return;
	float *p = &f->rgb[3ull * (static_cast<size_t>(y) * f->w + x)];
	p[0] = r; p[1] = g; p[2] = b;
}

// Adaptive-pass records of one film (see the header).
struct AaDump {
	const yafaray::ImageFilm *film = nullptr;
	bool on = false;
	struct Pass { int pass; float thr; std::vector<float> sums, w; std::vector<int> flagged; };
	std::vector<Pass> passes;
};

void highlightPixel(int x, int y, float, float, float, float, void *data)
{
	auto *d = static_cast<AaDump *>(data);
	if(!d->on) return;
	const yafaray::ImageFilm *f = d->film;
	const int W = f->params_.width_, H = f->params_.height_;
	if(d->passes.empty() || d->passes.back().pass != f->n_pass_)
	{
		AaDump::Pass p;
		p.pass = f->n_pass_;
		p.thr = f->getAaThresholdCalculated();
		const auto &img = f->film_image_layers_(yafaray::LayerDef::Combined).image_;
		p.sums.resize(4ull * W * H);
		p.w.resize(1ull * W * H);
		for(int yy = 0; yy < H; ++yy)
			for(int xx = 0; xx < W; ++xx)
			{
				const yafaray::Rgba c = img->getColor({{xx, yy}});
				float *q = &p.sums[4ull * (static_cast<size_t>(yy) * W + xx)];
				q[0] = c.r_; q[1] = c.g_; q[2] = c.b_; q[3] = c.a_;
				p.w[static_cast<size_t>(yy) * W + xx] = f->getWeight({{xx, yy}});
			}
		d->passes.push_back(std::move(p));
	}
	d->passes.back().flagged.push_back(y * W + x);
}

void setTyped(yafaray_ParamMap *pm, const std::string &key, const std::string &val)
{
	if(val == "true" || val == "false") { yafaray_setParamMapBool(pm, key.c_str(), val == "true" ? YAFARAY_BOOL_TRUE : YAFARAY_BOOL_FALSE); return; }
	char *end = nullptr;
	const long iv = std::strtol(val.c_str(), &end, 10);
	if(end && *end == '\0') { yafaray_setParamMapInt(pm, key.c_str(), static_cast<int>(iv)); return; }
	const double dv = std::strtod(val.c_str(), &end);
	if(end && *end == '\0') { yafaray_setParamMapFloat(pm, key.c_str(), dv); return; }
	yafaray_setParamMapString(pm, key.c_str(), val.c_str());
}
} // namespace

int main(int argc, char **argv)
{
	if(argc != 3 && argc != 4) { fprintf(stderr, "usage: %s scene.txt out.bin [photons.bin]\n", argv[0]); return 2; }
	std::ifstream in(argv[1]);
	if(!in) { perror("scene"); return 2; }
	yafaray_Logger *logger = yafaray_createLogger("oracle", nullptr, nullptr, YAFARAY_DISPLAY_CONSOLE_HIDDEN);
	yafaray_Scene *scene = yafaray_createScene(logger, "scene");
	yafaray_ParamMap *pm = yafaray_createParamMap();
	yafaray_ParamMapList *pml = yafaray_createParamMapList();
	yafaray_SurfaceIntegrator *integrator = nullptr;
	yafaray_ParamMap *camera = yafaray_createParamMap();
	int resx = 0, resy = 0, spp = 1, batches = 1, threads = -1;
	std::string filter_type = "box";
	float pixel_width = 1.f;
	int offset_stride = -1;
	std::vector<yafaray_ParamMap *> pending_nodes;
	std::map<std::string, size_t> object_ids;
	std::string integrator_type;
	std::vector<std::pair<std::string, std::string>> integrator_kv;
	auto make_integrator = [&]() {
		yafaray_ParamMap *ip = yafaray_createParamMap();
		yafaray_setParamMapString(ip, "type", integrator_type.c_str());
		for(const auto &kv : integrator_kv) setTyped(ip, kv.first, kv.second);
#ifdef GB300_BINDING
		if(std::getenv("GB300_INTEGRATOR") && integrator_type == "pathtracing")
		{
			// the GPU pathtracing integrator in place of the factory's
			yafaray::ParamResult pr;
			yafaray::SurfaceIntegrator *gpu = new gb300::PathIntegratorGb300(*reinterpret_cast<yafaray::Logger *>(logger), pr, "integrator",
			                                                                  *reinterpret_cast<yafaray::ParamMap *>(ip));
			yafaray_destroyParamMap(ip);
			return reinterpret_cast<yafaray_SurfaceIntegrator *>(gpu);
		}
#endif
		yafaray_SurfaceIntegrator *si = yafaray_createSurfaceIntegrator(logger, "integrator", ip);
		yafaray_destroyParamMap(ip);
		return si;
	};
	std::vector<std::pair<std::string, std::string>> aa_kv;
	std::string line;
	while(std::getline(in, line))
	{
		std::istringstream ss(line);
		std::string kw;
		if(!(ss >> kw) || kw[0] == '#') continue;
		yafaray_clearParamMap(pm);
		if(kw == "material")
		{
			std::string name, type;
			ss >> name >> type;
			yafaray_setParamMapString(pm, "type", type.c_str());
			if(type == "shinydiffusemat") { double r, g, b; ss >> r >> g >> b; yafaray_setParamMapColor(pm, "color", r, g, b, 1.0); }
			else if(type == "light_mat") { double r, g, b, p; ss >> r >> g >> b >> p; yafaray_setParamMapColor(pm, "color", r, g, b, 1.0); yafaray_setParamMapFloat(pm, "power", p); }
			else if(type == "glossy")
			{
				double r, g, b, sr, sg, sb, e, gr, dr; ss >> r >> g >> b >> sr >> sg >> sb >> e >> gr >> dr;
				yafaray_setParamMapColor(pm, "diffuse_color", r, g, b, 1.0);
				yafaray_setParamMapColor(pm, "color", sr, sg, sb, 1.0);
				yafaray_setParamMapFloat(pm, "exponent", e);
				yafaray_setParamMapFloat(pm, "glossy_reflect", gr);
				yafaray_setParamMapFloat(pm, "diffuse_reflect", dr);
			}
			else if(type == "rough_glass" || type == "glass")
			{
				double ior, a = 0.0, tf, r, g, b, mr, mg, mb;
				ss >> ior;
				if(type == "rough_glass") ss >> a;
				ss >> tf >> r >> g >> b >> mr >> mg >> mb;
				yafaray_setParamMapFloat(pm, "IOR", ior);
				if(type == "rough_glass") yafaray_setParamMapFloat(pm, "alpha", a);
				yafaray_setParamMapFloat(pm, "transmit_filter", tf);
				yafaray_setParamMapColor(pm, "filter_color", r, g, b, 1.0);
				yafaray_setParamMapColor(pm, "mirror_color", mr, mg, mb, 1.0);
			}
			// optional key=value parameters (a colour as r,g,b)
			std::string kv;
			while(ss >> kv)
			{
				const size_t eq = kv.find('=');
				if(eq == std::string::npos) continue;
				const std::string key = kv.substr(0, eq), val = kv.substr(eq + 1);
				double r, g, b;
				if(std::sscanf(val.c_str(), "%lf,%lf,%lf", &r, &g, &b) == 3) yafaray_setParamMapColor(pm, key.c_str(), r, g, b, 1.0);
				else setTyped(pm, key, val);
			}
			size_t id;
			yafaray_clearParamMapList(pml);
			for(yafaray_ParamMap *n : pending_nodes) yafaray_addParamMapToList(pml, n);
			yafaray_createMaterial(scene, &id, name.c_str(), pm, pml);
			for(yafaray_ParamMap *n : pending_nodes) yafaray_destroyParamMap(n);
			pending_nodes.clear();
		}
		else if(kw == "object")
		{
			std::string name, mat; size_t nv, nf, nuv = 0;
			ss >> name >> mat >> nv >> nf;
			if(!(ss >> nuv)) nuv = 0;
			size_t mat_id = 0;
			yafaray_getMaterialId(scene, &mat_id, mat.c_str());
			yafaray_setParamMapString(pm, "type", "mesh");
			size_t obj;
			yafaray_createObject(scene, &obj, name.c_str(), pm);
			for(size_t i = 0; i < nv; ++i)
			{
				std::getline(in, line); std::istringstream vs(line);
				double x, y, z; vs >> x >> y >> z;
				yafaray_addVertex(scene, obj, x, y, z);
			}
			std::vector<size_t> uv_id;
			for(size_t i = 0; i < nuv; ++i)
			{
				std::getline(in, line); std::istringstream us(line);
				double u, v; us >> u >> v;
				uv_id.push_back(yafaray_addUv(scene, obj, u, v));
			}
			for(size_t i = 0; i < nf; ++i)
			{
				std::getline(in, line); std::istringstream fs(line);
				std::vector<size_t> ix; size_t k;
				while(fs >> k) ix.push_back(k);
				if(nuv && ix.size() == 6) yafaray_addTriangleWithUv(scene, obj, ix[0], ix[1], ix[2], uv_id.at(ix[3]), uv_id.at(ix[4]), uv_id.at(ix[5]), mat_id);
				else if(nuv && ix.size() == 8) yafaray_addQuadWithUv(scene, obj, ix[0], ix[1], ix[2], ix[3], uv_id.at(ix[4]), uv_id.at(ix[5]), uv_id.at(ix[6]), uv_id.at(ix[7]), mat_id);
				else if(ix.size() == 3) yafaray_addTriangle(scene, obj, ix[0], ix[1], ix[2], mat_id);
				else if(ix.size() == 4) yafaray_addQuad(scene, obj, ix[0], ix[1], ix[2], ix[3], mat_id);
			}
			yafaray_initObject(scene, obj, mat_id);
			object_ids[name] = obj;
		}
		else if(kw == "smooth")
		{
			std::string name; double angle;
			ss >> name >> angle;
			yafaray_smoothObjectMesh(scene, object_ids.at(name), angle);
		}
		else if(kw == "image")
		{
			std::string name; int w, h;
			ss >> name >> w >> h;
			yafaray_setParamMapString(pm, "type", "ColorAlpha");
			yafaray_setParamMapString(pm, "image_optimization", "none");
			yafaray_setParamMapString(pm, "color_space", "LinearRGB");
			yafaray_setParamMapInt(pm, "width", w);
			yafaray_setParamMapInt(pm, "height", h);
			size_t id = 0;
			yafaray_createImage(scene, name.c_str(), &id, pm);
			for(int y = 0; y < h; ++y)
			{
				std::getline(in, line); std::istringstream is(line);
				for(int x = 0; x < w; ++x)
				{
					double r, g, b, a; is >> r >> g >> b >> a;
					yafaray_setImageColor(scene, id, x, y, static_cast<float>(r), static_cast<float>(g), static_cast<float>(b), static_cast<float>(a));
				}
			}
		}
		else if(kw == "texture" || kw == "node")
		{
			std::string name;
			if(kw == "texture") ss >> name;
			yafaray_ParamMap *target = kw == "texture" ? pm : yafaray_createParamMap();
			std::string kv;
			while(ss >> kv)
			{
				const size_t eq = kv.find('=');
				if(eq == std::string::npos) continue;
				const std::string key = kv.substr(0, eq), val = kv.substr(eq + 1);
				double a, b, c, d;
				if(std::sscanf(val.c_str(), "%lf,%lf,%lf,%lf", &a, &b, &c, &d) == 4) yafaray_setParamMapColor(target, key.c_str(), a, b, c, d);
				else if(std::sscanf(val.c_str(), "%lf,%lf,%lf", &a, &b, &c) == 3) yafaray_setParamMapVector(target, key.c_str(), a, b, c);
				else setTyped(target, key, val);
			}
			if(kw == "texture") yafaray_createTexture(scene, name.c_str(), pm);
			else pending_nodes.push_back(target);
		}
		else if(kw == "arealight")
		{
			double c[3], p1[3], p2[3], col[3], power; int samples;
			ss >> c[0] >> c[1] >> c[2] >> p1[0] >> p1[1] >> p1[2] >> p2[0] >> p2[1] >> p2[2] >> col[0] >> col[1] >> col[2] >> power >> samples;
			yafaray_setParamMapString(pm, "type", "arealight");
			yafaray_setParamMapVector(pm, "corner", c[0], c[1], c[2]);
			yafaray_setParamMapVector(pm, "point1", p1[0], p1[1], p1[2]);
			yafaray_setParamMapVector(pm, "point2", p2[0], p2[1], p2[2]);
			yafaray_setParamMapColor(pm, "color", col[0], col[1], col[2], 1.0);
			yafaray_setParamMapFloat(pm, "power", power);
			yafaray_setParamMapInt(pm, "samples", samples);
			static int n = 0;
			const std::string name = "area" + std::to_string(n++);
			yafaray_createLight(scene, name.c_str(), pm);
		}
		else if(kw == "pointlight")
		{
			double p[3], col[3], power;
			ss >> p[0] >> p[1] >> p[2] >> col[0] >> col[1] >> col[2] >> power;
			yafaray_setParamMapString(pm, "type", "pointlight");
			yafaray_setParamMapVector(pm, "from", p[0], p[1], p[2]);
			yafaray_setParamMapColor(pm, "color", col[0], col[1], col[2], 1.0);
			yafaray_setParamMapFloat(pm, "power", power);
			static int n = 0;
			const std::string name = "point" + std::to_string(n++);
			yafaray_createLight(scene, name.c_str(), pm);
		}
		else if(kw == "camera")
		{
			double f[3], t[3], u[3], focal;
			ss >> f[0] >> f[1] >> f[2] >> t[0] >> t[1] >> t[2] >> u[0] >> u[1] >> u[2] >> resx >> resy >> focal;
			yafaray_clearParamMap(camera);
			yafaray_setParamMapString(camera, "type", "perspective");
			yafaray_setParamMapInt(camera, "resx", resx);
			yafaray_setParamMapInt(camera, "resy", resy);
			yafaray_setParamMapFloat(camera, "focal", focal);
			yafaray_setParamMapVector(camera, "from", f[0], f[1], f[2]);
			yafaray_setParamMapVector(camera, "to", t[0], t[1], t[2]);
			yafaray_setParamMapVector(camera, "up", u[0], u[1], u[2]);
		}
		else if(kw == "integrator")
		{
			ss >> integrator_type;
			std::string kv;
			while(ss >> kv)
			{
				const auto eq = kv.find('=');
				if(eq != std::string::npos) integrator_kv.emplace_back(kv.substr(0, eq), kv.substr(eq + 1));
			}
			integrator = make_integrator();
		}
		else if(kw == "render") { ss >> spp >> batches >> threads; if(!(ss >> offset_stride)) offset_stride = -1; }
		else if(kw == "film") ss >> filter_type >> pixel_width;
		else if(kw == "aa")
		{
			std::string kv;
			while(ss >> kv)
			{
				const auto eq = kv.find('=');
				if(eq != std::string::npos) aa_kv.emplace_back(kv.substr(0, eq), kv.substr(eq + 1));
			}
		}
	}
	if(!integrator || resx <= 0 || resy <= 0) { fprintf(stderr, "scene lacks integrator or camera\n"); return 2; }
	yafaray_clearParamMap(pm);
	yafaray_setParamMapString(pm, "type", "yafaray-kdtree-original");
	yafaray_setSceneAcceleratorParams(scene, pm);

	std::vector<double> secs;
	std::vector<float> all;
	AaDump aa;
	for(int k = 0; k < batches; ++k)
	{
		// SPPM keeps its hit points and photon count in the integrator
		// (integrator_sppm.h:110-113) and appends new hit points per render:
		// every batch gets a fresh one
		if(k > 0 && integrator_type == "SPPM")
		{
			yafaray_destroySurfaceIntegrator(integrator);
			integrator = make_integrator();
		}
		if(integrator_type == "SPPM")
		{
			// its photon emission samples (hal_1_ .. hal_4_) start where batch k's
			// first pass (sample offset k x stride) begins, so batches shoot
			// disjoint photon paths: photon p of pass j uses Halton index
			// (k stride + j) photons + p + 1
			auto *sppm = dynamic_cast<yafaray::SppmIntegrator *>(reinterpret_cast<yafaray::SurfaceIntegrator *>(integrator));
			unsigned photons = 500000;
			for(const auto &kv : integrator_kv) if(kv.first == "photons") photons = static_cast<unsigned>(std::stoul(kv.second));
			const unsigned start = static_cast<unsigned>(k) * static_cast<unsigned>(offset_stride >= 0 ? offset_stride : spp) * photons;
			if(sppm) { sppm->hal_1_.setStart(start); sppm->hal_2_.setStart(start); sppm->hal_3_.setStart(start); sppm->hal_4_.setStart(start); }
		}
		yafaray_clearParamMap(pm);
		yafaray_setParamMapInt(pm, "width", resx);
		yafaray_setParamMapInt(pm, "height", resy);
		yafaray_setParamMapInt(pm, "threads", threads);
		yafaray_setParamMapInt(pm, "AA_passes", 1);
		yafaray_setParamMapInt(pm, "AA_minsamples", spp);
		yafaray_setParamMapString(pm, "filter_type", filter_type.c_str());
		yafaray_setParamMapFloat(pm, "AA_pixelwidth", pixel_width);
		yafaray_setParamMapInt(pm, "adv_base_sampling_offset", k * (offset_stride >= 0 ? offset_stride : spp));
		for(const auto &kv : aa_kv) setTyped(pm, kv.first, kv.second);
		yafaray_Film *film = yafaray_createFilm(logger, integrator, "film", pm);
		yafaray_defineCamera(film, camera);
		Film f; f.w = resx; f.h = resy; f.rgb.assign(3ull * resx * resy, 0.f);
		yafaray_setPutPixelCallback(film, putPixel, &f);
		aa.film = reinterpret_cast<const yafaray::ImageFilm *>(film);
		aa.on = k == 0 && !aa_kv.empty();
		yafaray_setHighlightPixelCallback(film, highlightPixel, &aa);
		yafaray_RenderControl *rc = yafaray_createRenderControl();
		yafaray_RenderMonitor *rm = yafaray_createRenderMonitor(nullptr, nullptr, YAFARAY_DISPLAY_CONSOLE_HIDDEN);
		yafaray_setRenderControlForNormalStart(rc);
		const auto flags = yafaray_checkAndClearSceneModifiedFlags(scene);
		const auto t0 = std::chrono::steady_clock::now();
		yafaray_preprocessScene(scene, rc, flags);
		yafaray_preprocessSurfaceIntegrator(rm, integrator, rc, scene);
#ifdef GB300_BINDING
		// the third argument takes the scene as the GPU path receives it
		// (gb300::translate and gb300::pt_params / film_params):
		//   i32 n_vertices, n_faces, n_materials, n_lights, n_normals, has_normals,
		//   f32 vertices[n_vertices][3], u32 faces[n_faces][4], i32 face_material[n_faces],
		//   gbrt_material_desc[n_materials], gbrt_light_desc[n_lights],
		//   f32 normals[n_normals][3], u32 face_normals[n_faces][4] (has_normals only),
		//   gbrt_camera_desc, gbrt_pt_params, gbrt_aa_params, gbrt_pm_params (caustic map),
		//   i32 status, error text
		if(k == 0 && argc > 3)
		{
			gb300::SceneDesc desc;
			std::string error;
			const auto *image_film = reinterpret_cast<const yafaray::ImageFilm *>(film);
			bool ok = gb300::translate(*reinterpret_cast<const yafaray::Scene *>(scene), *image_film->getCamera(), desc, error);
			yafaray::ParamMap ip;
			ip.setParam("type", integrator_type);
			for(const auto &kv : integrator_kv) setTyped(reinterpret_cast<yafaray_ParamMap *>(&ip), kv.first, kv.second);
			gbrt_pm_params caustic{};
			gbrt_pt_params ptp = gb300::pt_params(ip, spp, image_film->getBaseSamplingOffset(), caustic);
			gbrt_aa_params aap{};
			ok = ok && gb300::film_params(image_film->getAsParamMap(false), ptp, aap, error);
			FILE *ft = fopen(argv[3], "wb");
			if(!ft) { perror("translation"); return 2; }
			const int hdr6[6] = {static_cast<int>(desc.vertices.size() / 3), static_cast<int>(desc.face_material.size()),
			                     static_cast<int>(desc.materials.size()), static_cast<int>(desc.lights.size()),
			                     static_cast<int>(desc.normals.size() / 3), desc.has_normals ? 1 : 0};
			fwrite(hdr6, 4, 6, ft);
			fwrite(desc.vertices.data(), 4, desc.vertices.size(), ft);
			fwrite(desc.faces.data(), 4, desc.faces.size(), ft);
			fwrite(desc.face_material.data(), 4, desc.face_material.size(), ft);
			fwrite(desc.materials.data(), sizeof(gbrt_material_desc), desc.materials.size(), ft);
			fwrite(desc.lights.data(), sizeof(gbrt_light_desc), desc.lights.size(), ft);
			if(desc.has_normals)
			{
				fwrite(desc.normals.data(), 4, desc.normals.size(), ft);
				fwrite(desc.face_normals.data(), 4, desc.face_normals.size(), ft);
			}
			fwrite(&desc.camera, sizeof desc.camera, 1, ft);
			fwrite(&ptp, sizeof ptp, 1, ft);
			fwrite(&aap, sizeof aap, 1, ft);
			fwrite(&caustic, sizeof caustic, 1, ft);
			const int status = ok ? 0 : 1;
			fwrite(&status, 4, 1, ft);
			fwrite(error.data(), 1, error.size(), ft);
			fclose(ft);
		}
		if(false)
#else
		if(k == 0 && argc > 3 && aa_kv.empty())
#endif
		{
			auto *pmi = dynamic_cast<yafaray::PhotonIntegrator *>(reinterpret_cast<yafaray::SurfaceIntegrator *>(integrator));
			if(!pmi) { fprintf(stderr, "photon dump needs the photonmapping integrator\n"); return 2; }
			FILE *fp = fopen(argv[3], "wb");
			if(!fp) { perror("photons"); return 2; }
			for(const yafaray::PhotonMap *map : {pmi->diffuse_map_.get(), pmi->caustic_map_.get()})
			{
				const int hdr2[2] = {map->nPhotons(), map->nPaths()};
				fwrite(hdr2, 4, 2, fp);
				for(const auto &ph : map->photons_)
				{
					const float v[9] = {ph.dir_[yafaray::Axis::X], ph.dir_[yafaray::Axis::Y], ph.dir_[yafaray::Axis::Z],
					                    ph.pos_[yafaray::Axis::X], ph.pos_[yafaray::Axis::Y], ph.pos_[yafaray::Axis::Z],
					                    ph.col_.r_, ph.col_.g_, ph.col_.b_};
					fwrite(v, 4, 9, fp);
				}
			}
			fclose(fp);
		}
		yafaray_render(rc, rm, integrator, film);
		secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
		all.insert(all.end(), f.rgb.begin(), f.rgb.end());
		yafaray_destroyRenderMonitor(rm);
		yafaray_destroyRenderControl(rc);
		yafaray_destroyFilm(film);
	}
#ifdef GB300_BINDING
	if(false)
#else
	if(argc > 3 && !aa_kv.empty())
#endif
	{
		FILE *fa = fopen(argv[3], "wb");
		if(!fa) { perror("aa"); return 2; }
		const int np = static_cast<int>(aa.passes.size());
		fwrite(&np, 4, 1, fa);
		for(const auto &p : aa.passes)
		{
			const int n = static_cast<int>(p.flagged.size());
			fwrite(&p.pass, 4, 1, fa); fwrite(&p.thr, 4, 1, fa); fwrite(&n, 4, 1, fa);
			fwrite(p.sums.data(), 4, p.sums.size(), fa);
			fwrite(p.w.data(), 4, p.w.size(), fa);
			fwrite(p.flagged.data(), 4, p.flagged.size(), fa);
		}
		fclose(fa);
	}
	FILE *fo = fopen(argv[2], "wb");
	if(!fo) { perror("out"); return 2; }
	const int hdr[3] = {batches, resy, resx};
	fwrite(hdr, 4, 3, fo);
	fwrite(secs.data(), 8, secs.size(), fo);
	fwrite(all.data(), 4, all.size(), fo);
	fclose(fo);
	yafaray_destroySurfaceIntegrator(integrator);
	yafaray_destroyParamMap(camera);
	yafaray_destroyParamMap(pm);
	yafaray_destroyParamMapList(pml);
	yafaray_destroyScene(scene);
	yafaray_destroyLogger(logger);
	return 0;
}
