// Device traversal core shared by the trace kernels and the path tracer.
// Replaces kdtree::intersect<Nearest / Shadow> (accelerator_kdtree_common.h:108-255)
// and Accelerator::primitiveIntersection{,Shadow} (accelerator.h:122-145).
//
// Every float operation that decides a result (ray set-up, tree-bound
// crossing, Möller–Trumbore) uses explicit round-to-nearest intrinsics, so
// it rounds like the reference's scalar code whatever the translation unit's
// contraction flags are; hit IDs, t and (u,v) are bit-identical to it.  The
// node box test only decides which primitives get tested and is
// conservative (grown boxes, widened far distance).
#pragma once

#include "gbrt_internal.cuh"

#include <cfloat>

namespace gbrt {

constexpr int kTraceStack = 64;   // > maximum LBVH depth (30 Morton + 32 index bits)

struct BvhView {
	const float4 *nodes;
	const float4 *tris;
	const uint32_t *ids;
	const float *meta;
	uint32_t n_prims;
};

inline BvhView view_of(const gbrt_bvh *b) { return {b->nodes, b->tris, b->ids, b->meta, b->n_prims}; }

__device__ __forceinline__ float xm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xdot(float ax, float ay, float az, float bx, float by, float bz)
{
	return xa(xa(xm(ax, bx), xm(ay, by)), xm(az, bz));
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
		const float p = xs(from[axis], a);
		if(dir[axis] != 0.f)
		{
			const float inv_dir = __fdiv_rn(1.f, dir[axis]);
			float ltmin, ltmax;
			if(inv_dir > 0.f) { ltmin = xm(-p, inv_dir); ltmax = xm(xs(xs(g, a), p), inv_dir); }
			else { ltmin = xm(xs(xs(g, a), p), inv_dir); ltmax = xm(-p, inv_dir); }
			if(axis == 0) { lmin = ltmin; lmax = ltmax; }
			else { lmin = ltmin > lmin ? ltmin : lmin; lmax = ltmax < lmax ? ltmax : lmax; }
			if((lmax < 0.f) || (lmin > t_max)) return false;
		}
	}
	if((lmin <= lmax) && (lmax >= 0.f) && (lmin <= t_max)) { enter = lmin; leave = lmax; return true; }
	return false;
}

// ShapePolygon<float,N>::intersect (shape_polygon.h:126-176), operation for
// operation, on the precomputed edges (v1-v0, v2-v0, v3-v0).  Returns t (0 = no hit).
__device__ __forceinline__ float mt_intersect(const float4 A, const float4 B, const float4 C, bool quad,
                                              const float f[3], const float d[3], float &uo, float &vo)
{
	const float e1x = B.x, e1y = B.y, e1z = B.z;
	const float e2x = C.x, e2y = C.y, e2z = C.z;
	const float px = xs(xm(d[1], e2z), xm(d[2], e2y));
	const float py = xs(xm(d[2], e2x), xm(d[0], e2z));
	const float pz = xs(xm(d[0], e2y), xm(d[1], e2x));
	const float det = xdot(e1x, e1y, e1z, px, py, pz);
	if(det == 0.f) return 0.f;
	const float inv_det = __fdiv_rn(1.f, det);
	const float tx = xs(f[0], A.x), ty = xs(f[1], A.y), tz = xs(f[2], A.z);
	float u = xm(xdot(tx, ty, tz, px, py, pz), inv_det);
	if(u >= 0.f && u <= 1.f)
	{
		const float qx = xs(xm(ty, e1z), xm(tz, e1y));
		const float qy = xs(xm(tz, e1x), xm(tx, e1z));
		const float qz = xs(xm(tx, e1y), xm(ty, e1x));
		const float v = xm(xdot(d[0], d[1], d[2], qx, qy, qz), inv_det);
		if(v >= 0.f && xa(u, v) <= 1.f)
		{
			const float t = xm(xdot(e2x, e2y, e2z, qx, qy, qz), inv_det);
			if(t > 0.f)
			{
				if(quad) { uo = xa(u, v); vo = v; }
				else { uo = u; vo = v; }
				return t;
			}
		}
		return 0.f;
	}
	if(!quad) return 0.f;
	const float e3x = A.w, e3y = B.w, e3z = C.w;
	const float sx = xs(xm(d[1], e3z), xm(d[2], e3y));
	const float sy = xs(xm(d[2], e3x), xm(d[0], e3z));
	const float sz = xs(xm(d[0], e3y), xm(d[1], e3x));
	const float det2 = xdot(e2x, e2y, e2z, sx, sy, sz);
	if(det2 == 0.f) return 0.f;
	const float inv_det2 = __fdiv_rn(1.f, det2);
	u = xm(xdot(tx, ty, tz, sx, sy, sz), inv_det2);
	if(u >= 0.f && u <= 1.f)
	{
		const float qx = xs(xm(ty, e2z), xm(tz, e2y));
		const float qy = xs(xm(tz, e2x), xm(tx, e2z));
		const float qz = xs(xm(tx, e2y), xm(ty, e2x));
		const float v = xm(xdot(d[0], d[1], d[2], qx, qy, qz), inv_det2);
		if(v >= 0.f && xa(u, v) <= 1.f)
		{
			const float t = xm(xdot(e3x, e3y, e3z, qx, qy, qz), inv_det2);
			if(t > 0.f) { uo = u; vo = xa(u, v); return t; }
		}
	}
	return 0.f;
}

// Conservative slab test of a node's two children against [0, t_hi].
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

struct Hit {
	int32_t prim;
	float t, u, v;
};

// One query.  Closest hit follows Accelerator::intersect(ray, camera)
// (accelerator.h:89-101); shadow follows Accelerator::isShadowed
// (accelerator.h:103-111): origin advanced by tmin, t_max = tmax - 2 tmin,
// bias-only t_min, first accepted primitive returns.
template <bool kShadow>
__device__ __forceinline__ Hit trace_ray(const BvhView &bv, float ox, float oy, float oz, float tmin, float dx, float dy, float dz, float tmax)
{
	float from[3] = {ox, oy, oz};
	const float dir[3] = {dx, dy, dz};
	float t_max;
	if(!kShadow) t_max = (tmax >= 0.f) ? tmax : FLT_MAX;
	else
	{
		from[0] = xa(from[0], xm(dir[0], tmin));
		from[1] = xa(from[1], xm(dir[1], tmin));
		from[2] = xa(from[2], xm(dir[2], tmin));
		t_max = (tmax >= 0.f) ? xs(tmax, xm(2.f, tmin)) : FLT_MAX;
	}
	float bnd[6];
#pragma unroll
	for(int k = 0; k < 6; ++k) bnd[k] = __ldg(bv.meta + GBRT_META_BOUND + k);
	float enter, leave;
	Hit h{-1, t_max, 0.f, 0.f};
	if(bv.n_prims == 0 || !bound_cross(bnd, from, dir, t_max, enter, leave)) { h.t = 0.f; return h; }
	// accelerator_kdtree_common.h:139, accelerator.h:64
	const float bias = xm(0.1f * 0.00005f, fabsf(xs(leave, enter)));
	const float t_min = kShadow ? bias : fmaxf(tmin, bias);
	const float inv[3] = {1.f / dir[0], 1.f / dir[1], 1.f / dir[2]};
	uint32_t stack[kTraceStack];
	int sp = 0;
	uint32_t ref = 0;
	bool done = false;
	while(!done)
	{
		while(!(ref & GBRT_LEAF_BIT))
		{
			const float4 *nd = bv.nodes + 4ull * ref;
			const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
			bool h0, h1; float tn0, tn1;
			child_tests(n0, n1, n2, from, inv, h.t, h0, h1, tn0, tn1);
			const uint32_t r0 = __float_as_uint(n3.x), r1 = __float_as_uint(n3.y);
			if(h0 && h1)
			{
				const bool first0 = tn0 <= tn1;
				ref = first0 ? r0 : r1;
				if(sp < kTraceStack) stack[sp++] = first0 ? r1 : r0;
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
		const uint32_t first = ref & (GBRT_LEAF_MAX_SLOTS - 1u);
		const uint32_t cnt = ((ref >> 27) & 15u) + 1u;
		for(uint32_t k = 0; k < cnt; ++k)
		{
			const uint32_t slot = first + k;
			const float4 A = __ldg(bv.tris + 3ull * slot), B = __ldg(bv.tris + 3ull * slot + 1), C = __ldg(bv.tris + 3ull * slot + 2);
			const uint32_t id = __ldg(bv.ids + slot);
			float u, v;
			const float t = mt_intersect(A, B, C, (id & GBRT_QUAD_BIT) != 0u, from, dir, u, v);
			if(t <= 0.f || t < t_min || t >= t_max) continue;   // accelerator.h:125 / 137
			const int32_t pid = static_cast<int32_t>(id & ~GBRT_QUAD_BIT);
			if(kShadow) { h.prim = pid; h.t = t; h.u = u; h.v = v; done = true; break; }
			if(t < h.t || (t == h.t && h.prim >= 0 && pid < h.prim)) { h.t = t; h.prim = pid; h.u = u; h.v = v; }
		}
		if(done) break;
		if(sp == 0) break;
		ref = stack[--sp];
	}
	if(h.prim < 0) { h.t = 0.f; h.u = 0.f; h.v = 0.f; }
	return h;
}

} // namespace gbrt
