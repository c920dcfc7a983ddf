// Closest-hit and any-hit traversal of the LBVH.  Replaces
// kdtree::intersect<Nearest / Shadow> (accelerator_kdtree_common.h:108-255)
// and Accelerator::primitiveIntersection{,Shadow} (accelerator.h:122-145).
//
// This file is compiled with --fmad=false: no multiply-add is fused, so the
// Möller–Trumbore test, the tree-bound crossing and the ray set-up round
// exactly like the reference's scalar SSE code, and hit IDs, t and (u,v) are
// bit-identical to it.  The node boxes only decide which primitives get
// tested; they are tested conservatively (grown boxes, widened t interval),
// so a primitive the reference would accept is never culled.
#include "gbrt_internal.cuh"

#include <cfloat>

namespace {

constexpr int kTraceThreads = 128;
constexpr int kStack = 64;

struct RayIn {
	float ox, oy, oz, tmin, dx, dy, dz, tmax;
};

__device__ __forceinline__ RayIn load_ray(const gbrt_ray *__restrict__ rays, uint32_t i)
{
	const float4 a = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i);
	const float4 b = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i + 1);
	return {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

// Bound<float>::cross, Smits method (include/geometry/bound.h:156-198).
__device__ __forceinline__ bool bound_cross(const float *__restrict__ bnd, const float from[3], const float dir[3], float t_max,
                                            float &enter, float &leave)
{
	float lmin = -FLT_MAX, lmax = FLT_MAX;
#pragma unroll
	for(int axis = 0; axis < 3; ++axis)
	{
		const float a = bnd[axis], g = bnd[3 + axis];
		const float p = from[axis] - a;
		if(dir[axis] != 0.f)
		{
			const float inv_dir = 1.f / dir[axis];
			float ltmin, ltmax;
			if(inv_dir > 0.f) { ltmin = -p * inv_dir; ltmax = ((g - a) - p) * inv_dir; }
			else { ltmin = ((g - a) - p) * inv_dir; ltmax = -p * inv_dir; }
			if(axis == 0) { lmin = ltmin; lmax = ltmax; }
			else { lmin = ltmin > lmin ? ltmin : lmin; lmax = ltmax < lmax ? ltmax : lmax; }
			if((lmax < 0.f) || (lmin > t_max)) return false;
		}
	}
	if((lmin <= lmax) && (lmax >= 0.f) && (lmin <= t_max)) { enter = lmin; leave = lmax; return true; }
	return false;
}

// ShapePolygon<float,N>::intersect (shape_polygon.h:126-176), operation for
// operation.  Returns t (0 = no hit).
__device__ __forceinline__ float mt_intersect(const float4 A, const float4 B, const float4 C, bool quad,
                                              const float f[3], const float d[3], float &uo, float &vo)
{
	const float e1x = B.x, e1y = B.y, e1z = B.z;
	const float e2x = C.x, e2y = C.y, e2z = C.z;
	// pvec_2 = dir ^ edge_2
	const float px = d[1] * e2z - d[2] * e2y;
	const float py = d[2] * e2x - d[0] * e2z;
	const float pz = d[0] * e2y - d[1] * e2x;
	const float det = e1x * px + e1y * py + e1z * pz;
	if(det == 0.f) return 0.f;
	const float inv_det = 1.f / det;
	const float tx = f[0] - A.x, ty = f[1] - A.y, tz = f[2] - A.z;
	float u = (tx * px + ty * py + tz * pz) * inv_det;
	if(u >= 0.f && u <= 1.f)
	{
		// qvec_1 = tvec ^ edge_1
		const float qx = ty * e1z - tz * e1y;
		const float qy = tz * e1x - tx * e1z;
		const float qz = tx * e1y - ty * e1x;
		const float v = (d[0] * qx + d[1] * qy + d[2] * qz) * inv_det;
		if(v >= 0.f && (u + v) <= 1.f)
		{
			const float t = (e2x * qx + e2y * qy + e2z * qz) * inv_det;
			if(t > 0.f)
			{
				if(quad) { uo = u + v; vo = v; }
				else { uo = u; vo = v; }
				return t;
			}
		}
		return 0.f;
	}
	if(!quad) return 0.f;
	const float e3x = A.w, e3y = B.w, e3z = C.w;
	// pvec_3 = dir ^ edge_3
	const float sx = d[1] * e3z - d[2] * e3y;
	const float sy = d[2] * e3x - d[0] * e3z;
	const float sz = d[0] * e3y - d[1] * e3x;
	const float det2 = e2x * sx + e2y * sy + e2z * sz;
	if(det2 == 0.f) return 0.f;
	const float inv_det2 = 1.f / det2;
	u = (tx * sx + ty * sy + tz * sz) * inv_det2;
	if(u >= 0.f && u <= 1.f)
	{
		// qvec_2 = tvec ^ edge_2
		const float qx = ty * e2z - tz * e2y;
		const float qy = tz * e2x - tx * e2z;
		const float qz = tx * e2y - ty * e2x;
		const float v = (d[0] * qx + d[1] * qy + d[2] * qz) * inv_det2;
		if(v >= 0.f && (u + v) <= 1.f)
		{
			const float t = (e3x * qx + e3y * qy + e3z * qz) * inv_det2;
			if(t > 0.f) { uo = u; vo = u + v; return t; }
		}
	}
	return 0.f;
}

// Conservative slab test of the two children of a node against [0, t_hi].
__device__ __forceinline__ void child_tests(const float4 n0, const float4 n1, const float4 n2, const float o[3], const float inv[3],
                                            float t_hi, bool &hit0, bool &hit1, float &tn0, float &tn1)
{
	const float ax0 = (n0.x - o[0]) * inv[0], ax1 = (n0.y - o[0]) * inv[0];
	const float ay0 = (n0.z - o[1]) * inv[1], ay1 = (n0.w - o[1]) * inv[1];
	const float az0 = (n2.x - o[2]) * inv[2], az1 = (n2.y - o[2]) * inv[2];
	const float bx0 = (n1.x - o[0]) * inv[0], bx1 = (n1.y - o[0]) * inv[0];
	const float by0 = (n1.z - o[1]) * inv[1], by1 = (n1.w - o[1]) * inv[1];
	const float bz0 = (n2.z - o[2]) * inv[2], bz1 = (n2.w - o[2]) * inv[2];
	const float an = fmaxf(fmaxf(fminf(ax0, ax1), fminf(ay0, ay1)), fmaxf(fminf(az0, az1), 0.f));
	const float af = fminf(fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1)), fminf(fmaxf(az0, az1), t_hi)) * 1.0000004f;
	const float bn = fmaxf(fmaxf(fminf(bx0, bx1), fminf(by0, by1)), fmaxf(fminf(bz0, bz1), 0.f));
	const float bf = fminf(fminf(fmaxf(bx0, bx1), fmaxf(by0, by1)), fminf(fmaxf(bz0, bz1), t_hi)) * 1.0000004f;
	hit0 = an <= af;
	hit1 = bn <= bf;
	tn0 = an;
	tn1 = bn;
}

template <bool kShadow>
__global__ void __launch_bounds__(kTraceThreads)
k_trace(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, const uint32_t *__restrict__ ids,
        const float *__restrict__ meta, uint32_t n_prims, const gbrt_ray *__restrict__ rays, uint32_t n,
        gbrt_hit *__restrict__ hits, int32_t *__restrict__ occ)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const RayIn r = load_ray(rays, i);
	float from[3] = {r.ox, r.oy, r.oz};
	const float dir[3] = {r.dx, r.dy, r.dz};
	float t_max;
	if(!kShadow) t_max = (r.tmax >= 0.f) ? r.tmax : FLT_MAX;            // accelerator.h:91
	else
	{
		from[0] += dir[0] * r.tmin; from[1] += dir[1] * r.tmin; from[2] += dir[2] * r.tmin;  // accelerator.h:106
		t_max = (r.tmax >= 0.f) ? r.tmax - 2 * r.tmin : FLT_MAX;       // accelerator.h:108
	}
	float bnd[6];
#pragma unroll
	for(int k = 0; k < 6; ++k) bnd[k] = __ldg(meta + GBRT_META_BOUND + k);
	float enter, leave;
	int32_t best_id = -1;
	float best_t = t_max, best_u = 0.f, best_v = 0.f;
	if(n_prims > 0 && bound_cross(bnd, from, dir, t_max, enter, leave))
	{
		// accelerator_kdtree_common.h:139, accelerator.h:64
		const float bias = 0.1f * 0.00005f * fabsf(leave - enter);
		const float t_min = kShadow ? bias : fmaxf(r.tmin, bias);
		const float inv[3] = {1.f / dir[0], 1.f / dir[1], 1.f / dir[2]};
		uint32_t stack[kStack];
		int sp = 0;
		uint32_t ref = 0;  // root
		bool done = false;
		while(!done)
		{
			// descend through internal nodes
			while(!(ref & GBRT_LEAF_BIT))
			{
				const float4 *nd = nodes + 4ull * ref;
				const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
				bool h0, h1; float tn0, tn1;
				child_tests(n0, n1, n2, from, inv, best_t, h0, h1, tn0, tn1);
				const uint32_t r0 = __float_as_uint(n3.x), r1 = __float_as_uint(n3.y);
				if(h0 && h1)
				{
					const bool first0 = tn0 <= tn1;
					ref = first0 ? r0 : r1;
					if(sp < kStack) stack[sp++] = first0 ? r1 : r0;
				}
				else if(h0) ref = r0;
				else if(h1) ref = r1;
				else
				{
					if(sp == 0) { done = true; break; }
					ref = stack[--sp];
				}
			}
			if(done) break;
			// leaf
			const uint32_t first = ref & (GBRT_LEAF_MAX_SLOTS - 1u);
			const uint32_t cnt = ((ref >> 27) & 15u) + 1u;
			for(uint32_t k = 0; k < cnt; ++k)
			{
				const uint32_t slot = first + k;
				const float4 A = __ldg(tris + 3ull * slot), B = __ldg(tris + 3ull * slot + 1), C = __ldg(tris + 3ull * slot + 2);
				const uint32_t id = __ldg(ids + slot);
				float u, v;
				const float t = mt_intersect(A, B, C, (id & GBRT_QUAD_BIT) != 0u, from, dir, u, v);
				// accelerator.h:125 / 137
				if(t <= 0.f || t < t_min || t >= t_max) continue;
				const int32_t pid = static_cast<int32_t>(id & ~GBRT_QUAD_BIT);
				if(kShadow) { best_id = pid; done = true; break; }
				if(t < best_t || (t == best_t && best_id >= 0 && pid < best_id)) { best_t = t; best_id = pid; best_u = u; best_v = v; }
			}
			if(done) break;
			if(sp == 0) break;
			ref = stack[--sp];
		}
	}
	if(kShadow) occ[i] = best_id;
	else
	{
		float4 o;
		o.x = __int_as_float(best_id);
		o.y = best_id >= 0 ? best_t : 0.f;
		o.z = best_id >= 0 ? best_u : 0.f;
		o.w = best_id >= 0 ? best_v : 0.f;
		reinterpret_cast<float4 *>(hits)[i] = o;
	}
}

} // namespace

int gbrt_launch_closest(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	const unsigned grid = (n + kTraceThreads - 1) / kTraceThreads;
	k_trace<false><<<grid, kTraceThreads, 0, s>>>(b->nodes, b->tris, b->ids, b->meta, b->n_prims, rays, n, hits, nullptr);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

int gbrt_launch_shadow(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, int32_t *occ, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	const unsigned grid = (n + kTraceThreads - 1) / kTraceThreads;
	k_trace<true><<<grid, kTraceThreads, 0, s>>>(b->nodes, b->tris, b->ids, b->meta, b->n_prims, rays, n, nullptr, occ);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}
