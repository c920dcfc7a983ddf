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

// Traversal stack: kStackShared entries per thread in the calling block's
// shared memory, the rest in local memory.  A traversal pushes at most one
// entry per level of the wide hierarchy.
constexpr int kStackShared = 8;
constexpr int kTraceStack = GBRT_WIDE_MAX_LEVELS;

struct BvhView {
	const uint4 *wnodes;        // 8-wide compressed nodes (gbrt_internal.cuh)
	const float4 *tris;         // primitive records in wide-leaf order
	const uint32_t *ids;
	const float *meta;
	uint32_t n_prims;
};

inline BvhView view_of(const gbrt_bvh *b) { return {b->wnodes, b->wtris, b->wids, b->meta, b->n_prims}; }

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

// Byte k of w as a float (exact): 2^23 + b - 2^23.
template <int k>
__device__ __forceinline__ float byte_f(uint32_t w)
{
	return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440 + k)) - 8388608.f;
}

// Conservative test of a wide node's 8 child boxes against [0, t_hi]:
// node-hit bits ((slot ^ oct) for internal children) and primitive-hit bits
// (prim_base-relative) of the children that pass.  Planes are
// origin + q 2^e, rounded outward at build time; t = q (2^e / d) +
// (origin - o) / d with one FMA, the far distance widened by 3 ulp (Ize,
// "Robust BVH ray traversal", JCGT 2013) and the boxes grown at build time
// by more than the rounding of these expressions.  Per axis the near plane
// is the low one when the direction's sign bit is clear (octant bit 0),
// else the high one; a zero direction component gives infinities or NaNs
// that the min/max chains treat conservatively.
__device__ __forceinline__ void wide_node_test(const uint4 w0, const uint4 w1, const uint4 w2, const uint4 w3, const uint4 w4,
                                               const float o[3], const float inv[3], uint32_t oct, float t_hi,
                                               uint32_t &node_hits, uint32_t &prim_hits)
{
	const float ax = __uint_as_float((w0.w & 0xFFu) << 23) * inv[0];
	const float ay = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23) * inv[1];
	const float az = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23) * inv[2];
	const float bx = (__uint_as_float(w0.x) - o[0]) * inv[0];
	const float by = (__uint_as_float(w0.y) - o[1]) * inv[1];
	const float bz = (__uint_as_float(w0.z) - o[2]) * inv[2];
	// near / far plane words of slots 0-3 (index 0) and 4-7 (index 1)
	const bool sx = oct & 1u, sy = oct & 2u, sz = oct & 4u;
	const uint32_t nx0 = sx ? w3.z : w2.x, nx1 = sx ? w3.w : w2.y, fx0 = sx ? w2.x : w3.z, fx1 = sx ? w2.y : w3.w;
	const uint32_t ny0 = sy ? w4.x : w2.z, ny1 = sy ? w4.y : w2.w, fy0 = sy ? w2.z : w4.x, fy1 = sy ? w2.w : w4.y;
	const uint32_t nz0 = sz ? w4.z : w3.x, nz1 = sz ? w4.w : w3.y, fz0 = sz ? w3.x : w4.z, fz1 = sz ? w3.y : w4.w;
	uint32_t hit = 0;
#define GBRT_WIDE_CHILD(K, NX, NY, NZ, FX, FY, FZ, SLOT)                                                   \
	{                                                                                                      \
		const float tn = fmaxf(fmaxf(fmaf(byte_f<(K)>(NX), ax, bx), fmaf(byte_f<(K)>(NY), ay, by)),         \
		                       fmaxf(fmaf(byte_f<(K)>(NZ), az, bz), 0.f));                                 \
		const float tf = fminf(fminf(fmaf(byte_f<(K)>(FX), ax, bx), fmaf(byte_f<(K)>(FY), ay, by)),         \
		                       fminf(fmaf(byte_f<(K)>(FZ), az, bz), t_hi)) * 1.0000004f;                   \
		if(tn <= tf) hit |= 1u << (SLOT);                                                                  \
	}
	GBRT_WIDE_CHILD(0, nx0, ny0, nz0, fx0, fy0, fz0, 0)
	GBRT_WIDE_CHILD(1, nx0, ny0, nz0, fx0, fy0, fz0, 1)
	GBRT_WIDE_CHILD(2, nx0, ny0, nz0, fx0, fy0, fz0, 2)
	GBRT_WIDE_CHILD(3, nx0, ny0, nz0, fx0, fy0, fz0, 3)
	if(w1.w)   // nodes of up to 4 children leave slots 4-7 empty
	{
		GBRT_WIDE_CHILD(0, nx1, ny1, nz1, fx1, fy1, fz1, 4)
		GBRT_WIDE_CHILD(1, nx1, ny1, nz1, fx1, fy1, fz1, 5)
		GBRT_WIDE_CHILD(2, nx1, ny1, nz1, fx1, fy1, fz1, 6)
		GBRT_WIDE_CHILD(3, nx1, ny1, nz1, fx1, fy1, fz1, 7)
	}
#undef GBRT_WIDE_CHILD
	// Empty slots hold inverted boxes (missed except on a degenerate axis)
	// and meta 0, so a stray hit on one adds no bits below.
	const uint32_t m0 = w1.z, m1 = w1.w;
	const uint32_t imask = w0.w >> 24;
	// internal children: bit slot -> bit slot ^ oct (a permutation of 8 bits)
	uint32_t nh = hit & imask;
	if(oct & 1u) nh = ((nh & 0x55u) << 1) | ((nh >> 1) & 0x55u);
	if(oct & 2u) nh = ((nh & 0x33u) << 2) | ((nh >> 2) & 0x33u);
	if(oct & 4u) nh = ((nh & 0x0Fu) << 4) | ((nh >> 4) & 0x0Fu);
	// leaf children: unary count << offset from the meta byte
	uint32_t lh = hit & ~imask, ph = 0;
	while(lh)
	{
		const uint32_t sl = __ffs(lh) - 1u;
		lh &= lh - 1u;
		const uint32_t mb = ((sl < 4u ? m0 : m1) >> (8u * (sl & 3u))) & 0xFFu;
		ph |= (mb >> 5) << (mb & 0x1Fu);
	}
	node_hits = nh;
	prim_hits = ph;
}

struct Hit {
	int32_t prim;
	float t, u, v;
};

// Per-ray traversal state: the ray in the reference's set-up, the best hit
// so far, the current node group (child_base; hit bits 0-7, imask 8-15),
// the current primitive group and the stack depth.
struct TraceState {
	float from[3], dir[3], inv[3];
	float t_min, t_max;
	uint32_t oct;
	Hit h;
	uint32_t nbase, nhits, pbase, phits;
	int sp;
};

// Hit filters of the shadow walk.  OpaqueHits: every hit in range blocks
// (Accelerator::isShadowed).  A transparent-shadow filter
// (isShadowedTransparentShadow, accelerator.h:113-120, 147-169) decides per
// hit: blocks(prim, from, dir, t, u, v) true ends the walk as occluded, false lets the
// ray pass (the filter keeps what it needs, e.g. the filter colour).  Its
// kTransparent = true also selects the transparent walk's t_min,
// max(tmin, bias) (accelerator_kdtree_common.h:139).  The hierarchy holds
// every primitive once, so each is offered to the filter at most once.
struct OpaqueHits {
	static constexpr bool kTransparent = false;
	__device__ __forceinline__ void reset() {}
	__device__ __forceinline__ bool blocks(int32_t, const float *, const float *, float, float, float) { return true; }
};

// Ray set-up.  Closest hit follows Accelerator::intersect(ray, camera)
// (accelerator.h:89-101); shadow follows Accelerator::isShadowed
// (accelerator.h:103-111): origin advanced by tmin, t_max = tmax - 2 tmin,
// bias-only t_min (max(tmin, bias) for transparent shadows).  Returns false
// when the ray misses the tree bound (no traversal).
template <bool kShadow, bool kTransparent = false>
__device__ __forceinline__ bool trace_init(TraceState &S, const BvhView &bv, float ox, float oy, float oz, float tmin, float dx, float dy,
                                           float dz, float tmax)
{
	S.from[0] = ox; S.from[1] = oy; S.from[2] = oz;
	S.dir[0] = dx; S.dir[1] = dy; S.dir[2] = dz;
	if(!kShadow) S.t_max = (tmax >= 0.f) ? tmax : FLT_MAX;
	else
	{
		S.from[0] = xa(S.from[0], xm(dx, tmin));
		S.from[1] = xa(S.from[1], xm(dy, tmin));
		S.from[2] = xa(S.from[2], xm(dz, tmin));
		S.t_max = (tmax >= 0.f) ? xs(tmax, xm(2.f, tmin)) : FLT_MAX;
	}
	float bnd[6];
#pragma unroll
	for(int k = 0; k < 6; ++k) bnd[k] = __ldg(bv.meta + GBRT_META_BOUND + k);
	float enter, leave;
	S.h = Hit{-1, S.t_max, 0.f, 0.f};
	if(bv.n_prims == 0 || !bound_cross(bnd, S.from, S.dir, S.t_max, enter, leave)) return false;
	// accelerator_kdtree_common.h:139, accelerator.h:64
	const float bias = xm(0.1f * 0.00005f, fabsf(xs(leave, enter)));
	S.t_min = (kShadow && !kTransparent) ? bias : fmaxf(tmin, bias);
	// A zero (or denormal) direction component would make 1/d infinite and
	// the node planes' t values infinite or NaN, which the min / max chains
	// ignore: that axis would stop culling and the ray would walk most of
	// the tree.  +-2^64 instead keeps every slab sign exact (power-of-two
	// scaling) and puts planes outside the ray's slab far beyond any hit.
	S.inv[0] = 1.f / dx; S.inv[1] = 1.f / dy; S.inv[2] = 1.f / dz;
	for(int k = 0; k < 3; ++k)
		if(isinf(S.inv[k])) S.inv[k] = copysignf(18446744073709551616.f, S.inv[k]);
	S.oct = (dx < 0.f ? 1u : 0u) | (dy < 0.f ? 2u : 0u) | (dz < 0.f ? 4u : 0u);
	// a virtual group whose only (internal) child, in slot 0, is the root
	S.nbase = 0;
	S.nhits = (1u << S.oct) | (1u << 8);
	S.pbase = 0;
	S.phits = 0;
	S.sp = 0;
	return true;
}

// One step of the walk of the 8-wide hierarchy: open the nearest remaining
// child of the current group by octant order (pushing the rest of the
// group), test the opened node's primitive hits, pop when the group is
// spent.  `sh` is this thread's column of a shared [kStackShared][stride]
// uint2 array, `spill` a local array of kTraceStack - kStackShared entries,
// `f` the shadow walk's hit filter.  Returns true when the query is answered.
template <bool kShadow, typename F = OpaqueHits>
__device__ __forceinline__ bool trace_step(TraceState &S, const BvhView &bv, uint2 *sh, int stride, uint2 *spill, F &f)
{
	if(S.nhits & 0xFFu)
	{
		const uint32_t b = __ffs(S.nhits & 0xFFu) - 1u;
		S.nhits &= ~(1u << b);
		const uint32_t slot = b ^ S.oct;
		const uint32_t idx = S.nbase + __popc((S.nhits >> 8) & ((1u << slot) - 1u));
		if(S.nhits & 0xFFu)
		{
			const uint2 e = make_uint2(S.nbase, S.nhits);
			if(S.sp < kStackShared) sh[S.sp * stride] = e;
			else if(S.sp < kTraceStack) spill[S.sp - kStackShared] = e;
			++S.sp;
		}
		const uint4 *nd = bv.wnodes + 5ull * idx;
		const uint4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3), w4 = __ldg(nd + 4);
		uint32_t nh, ph;
		wide_node_test(w0, w1, w2, w3, w4, S.from, S.inv, S.oct, S.h.t, nh, ph);
		S.nbase = w1.x;
		S.nhits = nh | ((w0.w >> 24) << 8);
		S.pbase = w1.y;
		S.phits = ph;
	}
	while(S.phits)
	{
		const uint32_t slot = S.pbase + __ffs(S.phits) - 1u;
		S.phits &= S.phits - 1u;
		const float4 A = __ldg(bv.tris + 3ull * slot), B = __ldg(bv.tris + 3ull * slot + 1), C = __ldg(bv.tris + 3ull * slot + 2);
		const uint32_t id = __ldg(bv.ids + slot);
		float u, v;
		const float t = mt_intersect(A, B, C, (id & GBRT_QUAD_BIT) != 0u, S.from, S.dir, u, v);
		if(t <= 0.f || t < S.t_min || t >= S.t_max) continue;   // accelerator.h:125 / 137
		const int32_t pid = static_cast<int32_t>(id & ~GBRT_QUAD_BIT);
		if(kShadow)
		{
			if(f.blocks(pid, S.from, S.dir, t, u, v)) { S.h = Hit{pid, t, u, v}; return true; }
			continue;
		}
		if(t < S.h.t || (t == S.h.t && S.h.prim >= 0 && pid < S.h.prim)) S.h = Hit{pid, t, u, v};
	}
	if(!(S.nhits & 0xFFu))
	{
		if(S.sp == 0) return true;
		--S.sp;
		const uint2 e = S.sp < kStackShared ? sh[S.sp * stride] : (S.sp < kTraceStack ? spill[S.sp - kStackShared] : make_uint2(0u, 0u));
		S.nbase = e.x;
		S.nhits = e.y;
	}
	return false;
}

// The answer in the reference's form: a miss has t = u = v = 0.
__device__ __forceinline__ Hit trace_result(const TraceState &S)
{
	if(S.h.prim < 0) return Hit{-1, 0.f, 0.f, 0.f};
	return S.h;
}

// One complete query (see trace_init / trace_step).
template <bool kShadow>
__device__ __forceinline__ Hit trace_ray(const BvhView &bv, float ox, float oy, float oz, float tmin, float dx, float dy, float dz, float tmax,
                                         uint2 *sh, int stride)
{
	TraceState S;
	if(!trace_init<kShadow>(S, bv, ox, oy, oz, tmin, dx, dy, dz, tmax)) return Hit{-1, 0.f, 0.f, 0.f};
	uint2 spill[kTraceStack - kStackShared];
	OpaqueHits f;
	while(!trace_step<kShadow>(S, bv, sh, stride, spill, f)) { }
	return trace_result(S);
}

// Persistent-warp driver for a batch of n queries (Aila & Laine,
// "Understanding the efficiency of ray traversal on GPUs", HPG 2009, with
// dynamic fetch): each warp takes chunks of kTraceChunk query indices from
// *counter (zero before the launch); a lane whose query is answered takes
// the warp's next index at the top of the following step, so lanes do not
// idle while the slowest ray of their warp finishes, and warps that draw
// expensive rays do not hold up the launch.  Launch with every thread of
// every warp (the loop uses full-warp ballots) and a grid that fits on the
// GPU at once.
//   load(i, ray[8]) -> bool   false: entry i holds no query (skipped)
//   store(i, const Hit &)     the answer of query i (f still holds the
//                             query's filter state)
// f: the shadow walk's hit filter, reset before each query.
constexpr uint32_t kTraceChunk = 32;

// kLaneView: every query carries its own hierarchy (a batch of scenes):
// load(i, ray[8], BvhView &view) sets it, and the lane keeps it while it
// walks; otherwise every query walks `bv0`.
template <bool kShadow, bool kLaneView = false, typename F, typename Load, typename Store>
__device__ __forceinline__ void trace_persistent_filtered(const BvhView &bv0, uint32_t n, uint32_t *counter, uint2 *sh, int stride, F &f,
                                                          Load &&load, Store &&store)
{
	BvhView lbv = bv0;
	const BvhView &bv = kLaneView ? lbv : bv0;
	uint2 spill[kTraceStack - kStackShared];
	const uint32_t lane = threadIdx.x & 31u;
	uint32_t next = 0, end = 0;      // the warp's current chunk (warp-uniform)
	bool exhausted = false;
	TraceState S;
	bool active = false;
	uint32_t idx = 0;
	while(true)
	{
		const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
		if(idle && next >= end && !exhausted)
		{
			uint32_t b = 0;
			if(lane == 0) b = atomicAdd(counter, kTraceChunk);
			b = __shfl_sync(0xFFFFFFFFu, b, 0);
			if(b >= n) exhausted = true;
			else { next = b; end = min(b + kTraceChunk, n); }
		}
		if(idle == 0xFFFFFFFFu && exhausted) break;
		if(idle && next < end)
		{
			const uint32_t mine = next + __popc(idle & ((1u << lane) - 1u));
			next = min(next + static_cast<uint32_t>(__popc(idle)), end);
			float r[8];
			bool ok;
			if constexpr(kLaneView) ok = !active && mine < end && load(mine, r, lbv);
			else ok = !active && mine < end && load(mine, r);
			if(ok)
			{
				idx = mine;
				f.reset();
				active = trace_init<kShadow, F::kTransparent>(S, bv, r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7]);
				if(!active) store(idx, Hit{-1, 0.f, 0.f, 0.f});
			}
		}
		if(active && trace_step<kShadow>(S, bv, sh, stride, spill, f))
		{
			store(idx, trace_result(S));
			active = false;
		}
	}
}

template <bool kShadow, typename Load, typename Store>
__device__ __forceinline__ void trace_persistent(const BvhView &bv, uint32_t n, uint32_t *counter, uint2 *sh, int stride, Load &&load,
                                                 Store &&store)
{
	OpaqueHits f;
	trace_persistent_filtered<kShadow>(bv, n, counter, sh, stride, f, load, store);
}

} // namespace gbrt
