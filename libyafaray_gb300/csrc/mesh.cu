// Host-side mesh preparation done once when a scene is built: the smoothed
// per-vertex shading normals of MeshObject::smoothVerticesNormals
// (src/geometry/object/object_mesh.cc:150-262, reached through
// yafaray_smoothObjectMesh / Scene::smoothVerticesNormals, scene.cc:175-189).
// The float operations follow the reference's order (Vec operators of
// include/geometry/vector.h, FAST_TRIG cos, math::asin) so the normals the
// GPU interpolates are the reference's bit for bit.
#include "gbrt.h"
#include "gbrt_internal.cuh"
#include "sampling.cuh"

#include <cmath>
#include <vector>

namespace {

struct V3 {
	float x, y, z;
};

inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(V3 a, float s) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// operator ^ (vector.h:239-245)
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
// Vec::normalize (vector.h:306-315)
inline V3 normalized(V3 a)
{
	const float l2 = dot(a, a);
	if(l2 != 0.f)
	{
		const float inv = 1.f / std::sqrt(l2);
		a.x *= inv; a.y *= inv; a.z *= inv;
	}
	return a;
}

// Vec::sinFromVectors (vector.h:342-349) with math::asin (math.h:280-286):
// despite the name, the angle between the two edges.
float corner_angle(V3 e1, V3 e2)
{
	const float div = (length(e1) * length(e2)) * 0.99999f + 0.00001f;
	float a = (length(cross(e1, e2)) / div) * 0.99999f;
	if(a > 1.f) a = 1.f;
	if(a <= -1.f) return -1.57079632679489661923f;
	if(a >= 1.f) return 1.57079632679489661923f;
	return std::asin(a);
}

} // namespace

extern "C" int gbrt_mesh_smooth_normals(const float *vertices, uint32_t n_vertices, const uint32_t *faces, uint32_t n_faces,
                                        float angle, float *normals, uint32_t normals_cap, uint32_t *n_normals,
                                        uint32_t *face_normals)
{
	if((n_vertices && !vertices) || (n_faces && (!faces || !face_normals)) || !n_normals)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_mesh_smooth_normals: NULL argument");
	const V3 *P = reinterpret_cast<const V3 *>(vertices);
	std::vector<uint32_t> nv_face(n_faces);
	std::vector<V3> fn(n_faces);
	for(uint32_t f = 0; f < n_faces; ++f)
	{
		const uint32_t *q = faces + 4ull * f;
		nv_face[f] = q[3] == GBRT_TRIANGLE ? 3u : 4u;
		for(uint32_t k = 0; k < nv_face[f]; ++k)
			if(q[k] >= n_vertices) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_mesh_smooth_normals: face %u uses vertex %u of %u", f, q[k], n_vertices);
		// PrimitivePolygon's face_normal_geometric_ (primitive_polygon.h:68-71): the first triangle's normal
		fn[f] = normalized(cross(sub(P[q[1]], P[q[0]]), sub(P[q[2]], P[q[0]])));
	}
	// MeshObject::getAngleSine (object_mesh.cc:143-148) at the face's vertex k
	auto angle_at = [&](uint32_t f, uint32_t k) {
		const uint32_t *q = faces + 4ull * f;
		const uint32_t n = nv_face[f];
		const V3 p0 = P[q[k]];
		return corner_angle(sub(P[q[(k + 1) % n]], p0), sub(P[q[(k + 2) % n]], p0));
	};
	// every vertex starts with a zero normal (vertices_normals_.resize(points_size))
	std::vector<V3> out(n_vertices, V3{0.f, 0.f, 0.f});
	for(uint32_t f = 0; f < n_faces; ++f)
		for(uint32_t k = 0; k < 4; ++k) face_normals[4ull * f + k] = GBRT_NO_NORMAL;
	if(angle >= 180.f)
	{
		// every face's vertices take their vertex's normal (generateInitialVerticesNormalsIndices)
		for(uint32_t f = 0; f < n_faces; ++f)
		{
			const uint32_t *q = faces + 4ull * f;
			for(uint32_t k = 0; k < nv_face[f]; ++k)
			{
				out[q[k]] = add(out[q[k]], scale(fn[f], angle_at(f, k)));
				face_normals[4ull * f + k] = q[k];
			}
		}
		for(V3 &n : out) n = normalized(n);
	}
	else if(angle > 0.1f)
	{
		// angle-dependent smoothing: per vertex, each incident face's normal
		// summed with the incident faces within the angle, merged with an
		// earlier normal of the vertex when their cosine exceeds 0.999
		const float threshold = gbrt::fast_cos(angle * 0.01745329251994329576923690768489f);
		std::vector<uint32_t> start(n_vertices + 1, 0);
		for(uint32_t f = 0; f < n_faces; ++f)
			for(uint32_t k = 0; k < nv_face[f]; ++k) ++start[faces[4ull * f + k] + 1];
		for(uint32_t i = 0; i < n_vertices; ++i) start[i + 1] += start[i];
		std::vector<uint32_t> inc_face(start[n_vertices]);
		std::vector<float> inc_angle(start[n_vertices]);
		std::vector<uint32_t> fill(start.begin(), start.end() - 1);
		for(uint32_t f = 0; f < n_faces; ++f)          // faces in order, so each list is in face order
			for(uint32_t k = 0; k < nv_face[f]; ++k)
			{
				const uint32_t v = faces[4ull * f + k];
				inc_face[fill[v]] = f;
				inc_angle[fill[v]++] = angle_at(f, k);
			}
		std::vector<V3> local;
		std::vector<uint32_t> local_idx;
		for(uint32_t v = 0; v < n_vertices; ++v)
		{
			local.clear();
			local_idx.clear();
			for(uint32_t a = start[v]; a < start[v + 1]; ++a)
			{
				const uint32_t f = inc_face[a];
				bool smooth = false;
				V3 n = scale(fn[f], inc_angle[a]);
				for(uint32_t b = start[v]; b < start[v + 1]; ++b)
				{
					const uint32_t g = inc_face[b];
					if(g == f) continue;
					if(dot(fn[f], fn[g]) > threshold)
					{
						smooth = true;
						n = add(n, scale(fn[g], inc_angle[b]));
					}
				}
				uint32_t idx = GBRT_NO_NORMAL;
				if(smooth)
				{
					n = normalized(n);
					for(size_t j = 0; j < local.size(); ++j)
						if(dot(n, local[j]) > 0.999f) { idx = local_idx[j]; break; }
					if(idx == GBRT_NO_NORMAL)
					{
						idx = static_cast<uint32_t>(out.size());
						local.push_back(n);
						local_idx.push_back(idx);
						out.push_back(n);
					}
				}
				// the face's first corner at this vertex takes the index
				for(uint32_t k = 0; k < nv_face[f]; ++k)
					if(faces[4ull * f + k] == v) { face_normals[4ull * f + k] = idx; break; }
			}
		}
	}
	*n_normals = static_cast<uint32_t>(out.size());
	if(!normals) return GBRT_OK;                       // size query
	if(out.size() > normals_cap)
		return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_mesh_smooth_normals: %zu normals exceed the capacity of %u", out.size(), normals_cap);
	for(size_t i = 0; i < out.size(); ++i)
	{
		normals[3 * i] = out[i].x; normals[3 * i + 1] = out[i].y; normals[3 * i + 2] = out[i].z;
	}
	return GBRT_OK;
}
