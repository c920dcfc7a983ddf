// Test-oracle harness: builds one mesh object through the reference C API,
// lets the reference build its kd-tree (Scene::preprocess, scene.cc:314-403)
// and dumps, ray by ray, what Accelerator::intersect / intersectShadow return
// (accelerator.h:50-51, 89-111).  Links the reference's static library built
// by oracle/ref/Makefile; only tests/golden/make_golden.py runs it.
//
// Input (little endian):
//   char[8]  "GBRTKD01"
//   u32 nv;  f32 v[nv][3]
//   u32 nf;  u32 f[nf][4]        (f[3] == 0xFFFFFFFF marks a triangle)
//   u32 nr;  f32 r[nr][8]        (ox oy oz tmin dx dy dz tmax)
//   u32 mode                     0 closest (Accelerator::intersect(ray, camera) t_max rule)
//                                1 shadow  (Accelerator::isShadowed wrapper)
//   u32 len; char accel_type[len]
// Output:
//   f32 tree_bound[6]             (reference getBound(): a_xyz, g_xyz)
//   f64 build_seconds, f64 trace_seconds
//   per ray: i32 prim (-1 miss), f32 t, f32 u, f32 v
#include "yafaray_c_api.h"
#include "scene/scene.h"
#include "accelerator/accelerator.h"
#include "geometry/object/object.h"
#include "geometry/primitive/primitive.h"
#include <chrono>
#include <cstdio>
#include <cstring>
#include <cfloat>
#include <unordered_map>
#include <vector>
#include <string>

static void rd(FILE *f, void *p, size_t n)
{
	if(fread(p, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

int main(int argc, char **argv)
{
	if(argc != 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
	FILE *fi = fopen(argv[1], "rb");
	if(!fi) { perror("in"); return 2; }
	char magic[8]; rd(fi, magic, 8);
	if(memcmp(magic, "GBRTKD01", 8) != 0) { fprintf(stderr, "bad magic\n"); return 2; }
	uint32_t nv; rd(fi, &nv, 4);
	std::vector<float> v(3ull * nv); rd(fi, v.data(), 12ull * nv);
	uint32_t nf; rd(fi, &nf, 4);
	std::vector<uint32_t> fc(4ull * nf); rd(fi, fc.data(), 16ull * nf);
	uint32_t nr; rd(fi, &nr, 4);
	std::vector<float> rays(8ull * nr); rd(fi, rays.data(), 32ull * nr);
	uint32_t mode; rd(fi, &mode, 4);
	uint32_t len; rd(fi, &len, 4);
	std::string accel(len, '\0'); rd(fi, accel.data(), len);
	fclose(fi);

	yafaray_Logger *logger = yafaray_createLogger("oracle", nullptr, nullptr, YAFARAY_DISPLAY_CONSOLE_HIDDEN);
	yafaray_Scene *scene = yafaray_createScene(logger, "scene");
	yafaray_ParamMap *pm = yafaray_createParamMap();
	yafaray_setParamMapString(pm, "type", "shinydiffusemat");
	yafaray_ParamMapList *pml = yafaray_createParamMapList();
	size_t mat_id = 0;
	yafaray_createMaterial(scene, &mat_id, "mat", pm, pml);
	yafaray_clearParamMap(pm);
	yafaray_setParamMapString(pm, "type", "mesh");
	size_t obj_id = 0;
	yafaray_createObject(scene, &obj_id, "mesh", pm);
	for(uint32_t i = 0; i < nv; ++i) yafaray_addVertex(scene, obj_id, v[3 * i], v[3 * i + 1], v[3 * i + 2]);
	for(uint32_t i = 0; i < nf; ++i)
	{
		const uint32_t *q = &fc[4ull * i];
		if(q[3] == 0xFFFFFFFFu) yafaray_addTriangle(scene, obj_id, q[0], q[1], q[2], mat_id);
		else yafaray_addQuad(scene, obj_id, q[0], q[1], q[2], q[3], mat_id);
	}
	yafaray_initObject(scene, obj_id, mat_id);
	yafaray_clearParamMap(pm);
	yafaray_setParamMapString(pm, "type", accel.c_str());
	yafaray_setSceneAcceleratorParams(scene, pm);
	yafaray_RenderControl *rc = yafaray_createRenderControl();
	yafaray_setRenderControlForNormalStart(rc);
	const auto flags = yafaray_checkAndClearSceneModifiedFlags(scene);
	const auto t0 = std::chrono::steady_clock::now();
	yafaray_preprocessScene(scene, rc, flags);
	const auto t1 = std::chrono::steady_clock::now();

	auto *sc = reinterpret_cast<yafaray::Scene *>(scene);
	const yafaray::Accelerator *acc = sc->getAccelerator();
	const auto [object, res] = sc->getObject(obj_id);
	const auto prims = object->getPrimitives();
	std::unordered_map<const yafaray::Primitive *, int32_t> prim_id;
	for(size_t i = 0; i < prims.size(); ++i) prim_id[prims[i]] = static_cast<int32_t>(i);

	struct Rec { int32_t id; float t, u, v; };
	std::vector<Rec> out(nr);
	const auto t2 = std::chrono::steady_clock::now();
	for(uint32_t i = 0; i < nr; ++i)
	{
		const float *r = &rays[8ull * i];
		yafaray::Ray ray{{{r[0], r[1], r[2]}}, {{r[4], r[5], r[6]}}, 0.f, r[3], r[7]};
		yafaray::IntersectData d;
		if(mode == 0)
		{
			const float t_max = (ray.tmax_ >= 0.f) ? ray.tmax_ : std::numeric_limits<float>::max();
			d = acc->intersect(ray, t_max);
		}
		else
		{
			// Accelerator::isShadowed (accelerator.h:103-111)
			yafaray::Ray sray{ray, yafaray::Ray::DifferentialsCopy::No};
			sray.from_ += sray.dir_ * sray.tmin_;
			const float t_max = (ray.tmax_ >= 0.f) ? sray.tmax_ - 2 * sray.tmin_ : std::numeric_limits<float>::max();
			d = acc->intersectShadow(sray, t_max);
		}
		if(d.isHit() && d.primitive_) out[i] = {prim_id.at(d.primitive_), d.t_hit_, d.uv_.u_, d.uv_.v_};
		else out[i] = {-1, 0.f, 0.f, 0.f};
	}
	const auto t3 = std::chrono::steady_clock::now();
	const auto bound = acc->getBound();
	FILE *fo = fopen(argv[2], "wb");
	if(!fo) { perror("out"); return 2; }
	const float b[6] = {bound.a_[yafaray::Axis::X], bound.a_[yafaray::Axis::Y], bound.a_[yafaray::Axis::Z],
	                    bound.g_[yafaray::Axis::X], bound.g_[yafaray::Axis::Y], bound.g_[yafaray::Axis::Z]};
	fwrite(b, 4, 6, fo);
	const double secs[2] = {std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t3 - t2).count()};
	fwrite(secs, 8, 2, fo);
	fwrite(out.data(), sizeof(Rec), nr, fo);
	fclose(fo);
	yafaray_destroyRenderControl(rc);
	yafaray_destroyParamMap(pm);
	yafaray_destroyParamMapList(pml);
	yafaray_destroyScene(scene);
	yafaray_destroyLogger(logger);
	return 0;
}
