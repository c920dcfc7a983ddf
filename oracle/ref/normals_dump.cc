// Test-oracle harness: the per-face-corner shading normals the reference's
// yafaray_smoothObjectMesh (MeshObject::smoothVerticesNormals,
// src/geometry/object/object_mesh.cc:150-262) gives a mesh object.
// Only tests/golden/make_golden.py runs it.
//
// Input (binary): "GBRTNM01", u32 nv, f32 v[nv][3], u32 nf, u32 faces[nf][4]
// (4th = 0xFFFFFFFF for a triangle), f32 angle.
// Output (binary): u32 nf, then per face and corner (4 per face, the 4th
// unused for triangles): i32 normal index (-1 = none) and f32 normal xyz
// (zero where none).
#include "yafaray_c_api.h"
#include <algorithm>
#include <array>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <vector>
#define private public
#define protected public
#include "geometry/object/object_mesh.h"
#include "geometry/primitive/primitive_face.h"
#include "scene/scene.h"
#undef private
#undef protected

static void rd(FILE *f, void *p, size_t n)
{
	if(fread(p, 1, n, f) != n) { fprintf(stderr, "short read\n"); std::exit(2); }
}

int main(int argc, char **argv)
{
	if(argc != 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
	FILE *fi = fopen(argv[1], "rb");
	if(!fi) { perror("in"); return 2; }
	char magic[8]; rd(fi, magic, 8);
	if(memcmp(magic, "GBRTNM01", 8) != 0) { fprintf(stderr, "bad magic\n"); return 2; }
	uint32_t nv; rd(fi, &nv, 4);
	std::vector<float> v(3ull * nv); rd(fi, v.data(), 12ull * nv);
	uint32_t nf; rd(fi, &nf, 4);
	std::vector<uint32_t> fc(4ull * nf); rd(fi, fc.data(), 16ull * nf);
	float angle; rd(fi, &angle, 4);
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
	yafaray_smoothObjectMesh(scene, obj_id, angle);

	auto *sc = reinterpret_cast<yafaray::Scene *>(scene);
	const auto [object, res] = sc->getObject(obj_id);
	const auto *mesh = static_cast<const yafaray::MeshObject *>(object);
	FILE *fo = fopen(argv[2], "wb");
	if(!fo) { perror("out"); return 2; }
	fwrite(&nf, 4, 1, fo);
	for(uint32_t i = 0; i < nf; ++i)
	{
		const yafaray::FacePrimitive &face = *mesh->faces_[i];
		const auto &ix = face.getFaceIndices();
		for(int k = 0; k < 4; ++k)
		{
			int32_t idx = -1;
			float n[3] = {0.f, 0.f, 0.f};
			if(k < ix.numVertices() && ix[k].normal_ != yafaray::math::invalid<int>)
			{
				idx = ix[k].normal_;
				const yafaray::Vec3f vn = mesh->getVertexNormal(idx, 0);
				n[0] = vn[0]; n[1] = vn[1]; n[2] = vn[2];
			}
			fwrite(&idx, 4, 1, fo);
			fwrite(n, 4, 3, fo);
		}
	}
	fclose(fo);
	yafaray_destroyParamMapList(pml);
	yafaray_destroyParamMap(pm);
	yafaray_destroyScene(scene);
	yafaray_destroyLogger(logger);
	return 0;
}
