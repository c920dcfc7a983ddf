// LBVH construction on the GPU: replaces the SAH kd-tree that
// AcceleratorKdTree builds on one CPU thread
// (src/accelerator/accelerator_kdtree_original.cc:65-141, 437-645).
//
// Stages (all on one stream, no host synchronisation):
//   1. k_setup       primitive bounds, centroids, leaf-order-independent
//                    reductions of the primitive bound and centroid bound
//   2. k_finalize    reference tree bound (grown 0.1 % per axis, offset in
//                    double, accelerator_kdtree_original.cc:99-103)
//   3. k_morton      30-bit Morton code of each centroid
//   4. radix sort    stable LSD, 8-bit digits (histogram / scan / scatter)
//   5. k_karras      binary radix tree over the sorted codes (Karras 2012)
//   6. k_refit       bottom-up boxes, primitive counts and SAH costs; a node
//                    becomes a leaf when that is cheaper and it holds <= max
//                    leaf size primitives
//   7. k_emit_nodes  64-byte nodes holding both children's boxes
//   8. k_emit_prims  48-byte primitive records in leaf order
#include "gbrt_internal.cuh"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kNoParent = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t f2ord(float f)
{
	const uint32_t b = __float_as_uint(f);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t o)
{
	return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__global__ void k_init_meta(float *meta)
{
	uint32_t *m = reinterpret_cast<uint32_t *>(meta);
	const int i = threadIdx.x;
	if(i < 3) { m[GBRT_META_ORD + i] = 0xFFFFFFFFu; m[GBRT_META_ORD + 3 + i] = 0u; }
	else if(i < 6) { m[GBRT_META_ORD + 3 + i] = 0xFFFFFFFFu; m[GBRT_META_ORD + 6 + i] = 0u; }
	if(i == 0) m[GBRT_META_ERR] = 0u;
}

// One thread per face: exact min/max box (primitive_face.h:139-153) and centroid.
__global__ void k_setup(const float *__restrict__ verts, uint32_t nv, const uint32_t *__restrict__ faces, uint32_t nf,
                        float4 *__restrict__ box_lo, float4 *__restrict__ box_hi, float *meta)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
	float c[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
	bool valid = false;
	if(i < nf)
	{
		const uint4 f = reinterpret_cast<const uint4 *>(faces)[i];
		const uint32_t idx[4] = {f.x, f.y, f.z, f.w};
		const int n = (f.w == GBRT_TRIANGLE) ? 3 : 4;
		bool ok = true;
		for(int k = 0; k < n; ++k) ok = ok && idx[k] < nv;
		if(!ok)
		{
			atomicOr(reinterpret_cast<uint32_t *>(meta) + GBRT_META_ERR, 1u);
			box_lo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
			box_hi[i] = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		else
		{
			for(int a = 0; a < 3; ++a) { lo[a] = verts[3ull * idx[0] + a]; hi[a] = lo[a]; }
			for(int k = 1; k < n; ++k)
				for(int a = 0; a < 3; ++a)
				{
					const float x = verts[3ull * idx[k] + a];
					if(x < lo[a]) lo[a] = x;
					if(x > hi[a]) hi[a] = x;
				}
			for(int a = 0; a < 3; ++a) c[a] = 0.5f * (lo[a] + hi[a]);
			box_lo[i] = make_float4(lo[0], lo[1], lo[2], 0.f);
			box_hi[i] = make_float4(hi[0], hi[1], hi[2], 0.f);
			valid = true;
		}
	}
	// block reduction of 12 ordered words (min lo, max hi, min c, max c)
	uint32_t w[12];
	for(int a = 0; a < 3; ++a)
	{
		w[a] = valid ? f2ord(lo[a]) : 0xFFFFFFFFu;
		w[3 + a] = valid ? f2ord(hi[a]) : 0u;
		w[6 + a] = valid ? f2ord(c[a]) : 0xFFFFFFFFu;
		w[9 + a] = valid ? f2ord(c[a]) : 0u;
	}
	for(int off = 16; off > 0; off >>= 1)
		for(int k = 0; k < 12; ++k)
		{
			const uint32_t o = __shfl_xor_sync(0xFFFFFFFFu, w[k], off);
			const bool is_min = (k < 3) || (k >= 6 && k < 9);
			w[k] = is_min ? min(w[k], o) : max(w[k], o);
		}
	__shared__ uint32_t s[32][12];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	if(lane == 0)
		for(int k = 0; k < 12; ++k) s[warp][k] = w[k];
	__syncthreads();
	if(threadIdx.x < 12)
	{
		const int k = threadIdx.x;
		const bool is_min = (k < 3) || (k >= 6 && k < 9);
		uint32_t r = s[0][k];
		for(int j = 1; j < nw; ++j) r = is_min ? min(r, s[j][k]) : max(r, s[j][k]);
		uint32_t *m = reinterpret_cast<uint32_t *>(meta) + GBRT_META_ORD;
		if(is_min) atomicMin(m + k, r); else atomicMax(m + k, r);
	}
}

// Reference tree bound and Morton normalisation constants.
__global__ void k_finalize(float *meta, uint32_t nf)
{
	if(threadIdx.x != 0) return;
	const uint32_t *m = reinterpret_cast<const uint32_t *>(meta) + GBRT_META_ORD;
	float lo[3], hi[3], clo[3], chi[3];
	for(int a = 0; a < 3; ++a)
	{
		lo[a] = ord2f(m[a]); hi[a] = ord2f(m[3 + a]);
		clo[a] = ord2f(m[6 + a]); chi[a] = ord2f(m[9 + a]);
	}
	if(nf == 0)
		for(int a = 0; a < 3; ++a) { lo[a] = hi[a] = clo[a] = chi[a] = 0.f; }
	for(int a = 0; a < 3; ++a)
	{
		const float ext = hi[a] - lo[a];
		const double offset = static_cast<double>(ext) * 0.001;
		meta[GBRT_META_BOUND + a] = lo[a] - static_cast<float>(offset);
		meta[GBRT_META_BOUND + 3 + a] = hi[a] + static_cast<float>(offset);
		meta[GBRT_META_CLO + a] = clo[a];
		const float cext = chi[a] - clo[a];
		meta[GBRT_META_CINV + a] = cext > 0.f ? 1.f / cext : 0.f;
	}
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v)
{
	v = (v * 0x00010001u) & 0xFF0000FFu;
	v = (v * 0x00000101u) & 0x0F00F00Fu;
	v = (v * 0x00000011u) & 0xC30C30C3u;
	v = (v * 0x00000005u) & 0x49249249u;
	return v;
}

__global__ void k_morton(const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi, uint32_t nf,
                         const float *__restrict__ meta, uint32_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nf) return;
	const float4 l = box_lo[i], h = box_hi[i];
	const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
	uint32_t q[3];
	for(int a = 0; a < 3; ++a)
	{
		float x = (c[a] - meta[GBRT_META_CLO + a]) * meta[GBRT_META_CINV + a];
		x = fminf(fmaxf(x * 1024.f, 0.f), 1023.f);
		q[a] = static_cast<uint32_t>(x);
	}
	keys[i] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
	vals[i] = i;
}

// ---- stable LSD radix sort, 8-bit digits --------------------------------
__global__ void k_hist(const uint32_t *__restrict__ keys, uint32_t n, int shift, uint32_t *__restrict__ hist, uint32_t nblk)
{
	__shared__ uint32_t h[256];
	h[threadIdx.x] = 0;
	__syncthreads();
	const uint32_t base = blockIdx.x * kSortTile;
	for(int r = 0; r < kSortItems; ++r)
	{
		const uint32_t idx = base + r * kSortThreads + threadIdx.x;
		if(idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
	}
	__syncthreads();
	hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m words by one block of 1024 threads (m <= a few million).
__global__ void k_scan(uint32_t *__restrict__ data, uint32_t m)
{
	__shared__ uint32_t s[1024];
	const uint32_t per = (m + 1023u) / 1024u;
	const uint32_t lo = threadIdx.x * per;
	const uint32_t hi = min(lo + per, m);
	uint32_t sum = 0;
	for(uint32_t i = lo; i < hi; ++i) sum += data[i];
	s[threadIdx.x] = sum;
	__syncthreads();
	for(int off = 1; off < 1024; off <<= 1)
	{
		const uint32_t v = threadIdx.x >= static_cast<unsigned>(off) ? s[threadIdx.x - off] : 0u;
		__syncthreads();
		s[threadIdx.x] += v;
		__syncthreads();
	}
	uint32_t run = s[threadIdx.x] - sum;
	for(uint32_t i = lo; i < hi; ++i) { const uint32_t x = data[i]; data[i] = run; run += x; }
}

__global__ void k_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t n, int shift,
                          const uint32_t *__restrict__ scan, uint32_t nblk,
                          uint32_t *__restrict__ kout, uint32_t *__restrict__ vout)
{
	__shared__ uint32_t s_base[256];
	__shared__ uint32_t s_cnt[kSortWarps][256];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	s_base[tid] = scan[tid * nblk + blockIdx.x];
	const uint32_t base = blockIdx.x * kSortTile;
	const uint32_t lt_mask = (1u << lane) - 1u;
	for(int r = 0; r < kSortItems; ++r)
	{
		for(int w = 0; w < kSortWarps; ++w) s_cnt[w][tid] = 0;
		__syncthreads();
		const uint32_t idx = base + r * kSortThreads + tid;
		const bool valid = idx < n;
		const uint32_t key = valid ? kin[idx] : 0u;
		const uint32_t d = valid ? ((key >> shift) & 255u) : (256u + static_cast<uint32_t>(lane));
		const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
		const uint32_t rank = __popc(peers & lt_mask);
		if(valid && lane == __ffs(peers) - 1) s_cnt[warp][d] = __popc(peers);
		__syncthreads();
		if(valid)
		{
			uint32_t pos = s_base[d] + rank;
			for(int w = 0; w < warp; ++w) pos += s_cnt[w][d];
			kout[pos] = key;
			vout[pos] = vin[idx];
		}
		__syncthreads();
		uint32_t add = 0;
		for(int w = 0; w < kSortWarps; ++w) add += s_cnt[w][tid];
		s_base[tid] += add;
		__syncthreads();
	}
}

// ---- Karras binary radix tree ---------------------------------------------
__device__ __forceinline__ int delta(const uint32_t *__restrict__ k, int n, int i, int j)
{
	if(j < 0 || j >= n) return -1;
	const uint32_t a = k[i], b = k[j];
	if(a == b) return 32 + __clz(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
	return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t *__restrict__ keys, int n, uint2 *__restrict__ child, uint2 *__restrict__ range,
                         uint32_t *__restrict__ parent_int, uint32_t *__restrict__ parent_leaf)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n - 1) return;
	const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
	const int dmin = delta(keys, n, i, i - d);
	int lmax = 2;
	while(delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
	int l = 0;
	for(int t = lmax >> 1; t >= 1; t >>= 1)
		if(delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
	const int j = i + l * d;
	const int dnode = delta(keys, n, i, j);
	int s = 0;
	int t = l;
	do
	{
		t = (t + 1) >> 1;
		if(delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
	} while(t > 1);
	const int gamma = i + s * d + min(d, 0);
	const int first = min(i, j), last = max(i, j);
	uint32_t left, right;
	if(first == gamma) { left = GBRT_LEAF_BIT | static_cast<uint32_t>(gamma); parent_leaf[gamma] = i; }
	else { left = static_cast<uint32_t>(gamma); parent_int[gamma] = i; }
	if(last == gamma + 1) { right = GBRT_LEAF_BIT | static_cast<uint32_t>(gamma + 1); parent_leaf[gamma + 1] = i; }
	else { right = static_cast<uint32_t>(gamma + 1); parent_int[gamma + 1] = i; }
	child[i] = make_uint2(left, right);
	range[i] = make_uint2(static_cast<uint32_t>(first), static_cast<uint32_t>(last));
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi)
{
	const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
	return dx * dy + dy * dz + dz * dx;
}

// Bottom-up: the second thread to reach a node finishes it.  node_lo.w holds
// the SAH cost, node_hi.w the primitive count (as float bits of an uint).
__global__ void k_refit(const uint32_t *__restrict__ vals, int n, const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi,
                        const uint2 *__restrict__ child, const uint32_t *__restrict__ parent_int, const uint32_t *__restrict__ parent_leaf,
                        float4 *node_lo, float4 *node_hi, uint32_t *flags, uint8_t *collapse,
                        uint32_t max_leaf, float ct, float ci)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= n) return;
	uint32_t p = parent_leaf[j];
	while(p != kNoParent)
	{
		__threadfence();
		if(atomicAdd(&flags[p], 1u) == 0u) return;
		__threadfence();
		const uint2 c = child[p];
		float4 lo[2], hi[2];
		float cost[2];
		uint32_t cnt[2];
		const uint32_t cc[2] = {c.x, c.y};
		for(int k = 0; k < 2; ++k)
		{
			if(cc[k] & GBRT_LEAF_BIT)
			{
				const uint32_t leaf = cc[k] & ~GBRT_LEAF_BIT;
				const uint32_t prim = vals[leaf];
				lo[k] = box_lo[prim]; hi[k] = box_hi[prim];
				cost[k] = ci * half_area(lo[k], hi[k]);
				cnt[k] = 1u;
			}
			else
			{
				lo[k] = __ldcg(&node_lo[cc[k]]); hi[k] = __ldcg(&node_hi[cc[k]]);
				cost[k] = lo[k].w;
				cnt[k] = __float_as_uint(hi[k].w);
			}
		}
		float4 L = make_float4(fminf(lo[0].x, lo[1].x), fminf(lo[0].y, lo[1].y), fminf(lo[0].z, lo[1].z), 0.f);
		float4 H = make_float4(fmaxf(hi[0].x, hi[1].x), fmaxf(hi[0].y, hi[1].y), fmaxf(hi[0].z, hi[1].z), 0.f);
		const float area = half_area(L, H);
		const uint32_t count = cnt[0] + cnt[1];
		const float c_int = ct * area + cost[0] + cost[1];
		const float c_leaf = ci * area * static_cast<float>(count);
		const bool leaf = count <= max_leaf && c_leaf <= c_int;
		L.w = leaf ? c_leaf : c_int;
		H.w = __uint_as_float(count);
		__stcg(&node_lo[p], L);
		__stcg(&node_hi[p], H);
		collapse[p] = leaf ? 1 : 0;
		p = parent_int[p];
	}
}

// Node boxes are grown by 2^-18 of the coordinate plus 2^-18 of the scene
// extent, so float rounding in the traversal's box test never culls a
// primitive that the Möller–Trumbore test would accept (rays grazing an edge).
constexpr float kGrowRel = 3.81469727e-6f;
__device__ __forceinline__ float scene_pad(const float *meta)
{
	float e = 0.f;
	for(int a = 0; a < 3; ++a) e = fmaxf(e, meta[GBRT_META_BOUND + 3 + a] - meta[GBRT_META_BOUND + a]);
	return e * kGrowRel + 1e-30f;
}
__device__ __forceinline__ float grow_down(float x, float pad) { return x - (fabsf(x) * kGrowRel + pad); }
__device__ __forceinline__ float grow_up(float x, float pad) { return x + (fabsf(x) * kGrowRel + pad); }

__global__ void k_emit_nodes(int n_int, const uint32_t *__restrict__ vals, const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi,
                             const uint2 *__restrict__ child, const uint2 *__restrict__ range, const float4 *__restrict__ node_lo,
                             const float4 *__restrict__ node_hi, const uint8_t *__restrict__ collapse, const float *__restrict__ meta,
                             float4 *__restrict__ nodes)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n_int) return;
	const float pad = scene_pad(meta);
	const uint2 c = child[i];
	const uint32_t cc[2] = {c.x, c.y};
	float4 lo[2], hi[2];
	uint32_t ref[2];
	for(int k = 0; k < 2; ++k)
	{
		if(cc[k] & GBRT_LEAF_BIT)
		{
			const uint32_t leaf = cc[k] & ~GBRT_LEAF_BIT;
			const uint32_t prim = vals[leaf];
			lo[k] = box_lo[prim]; hi[k] = box_hi[prim];
			ref[k] = gbrt_leaf_ref(leaf, 1u);
		}
		else
		{
			lo[k] = node_lo[cc[k]]; hi[k] = node_hi[cc[k]];
			if(collapse[cc[k]]) ref[k] = gbrt_leaf_ref(range[cc[k]].x, __float_as_uint(hi[k].w));
			else ref[k] = cc[k];
		}
	}
	float4 *o = nodes + 4ull * i;
	o[0] = make_float4(grow_down(lo[0].x, pad), grow_up(hi[0].x, pad), grow_down(lo[0].y, pad), grow_up(hi[0].y, pad));
	o[1] = make_float4(grow_down(lo[1].x, pad), grow_up(hi[1].x, pad), grow_down(lo[1].y, pad), grow_up(hi[1].y, pad));
	o[2] = make_float4(grow_down(lo[0].z, pad), grow_up(hi[0].z, pad), grow_down(lo[1].z, pad), grow_up(hi[1].z, pad));
	o[3] = make_float4(__uint_as_float(ref[0]), __uint_as_float(ref[1]), 0.f, 0.f);
}

// Single-primitive hierarchy: a root whose second child is an empty box.
__global__ void k_emit_single(const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi, const float *__restrict__ meta,
                              float4 *__restrict__ nodes)
{
	const float4 l = box_lo[0], h = box_hi[0];
	const float pad = scene_pad(meta);
	nodes[0] = make_float4(grow_down(l.x, pad), grow_up(h.x, pad), grow_down(l.y, pad), grow_up(h.y, pad));
	nodes[1] = make_float4(FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX);
	nodes[2] = make_float4(grow_down(l.z, pad), grow_up(h.z, pad), FLT_MAX, -FLT_MAX);
	nodes[3] = make_float4(__uint_as_float(gbrt_leaf_ref(0u, 1u)), __uint_as_float(gbrt_leaf_ref(0u, 1u)), 0.f, 0.f);
}

__global__ void k_emit_prims(const float *__restrict__ verts, const uint32_t *__restrict__ faces, const uint32_t *__restrict__ vals,
                             uint32_t nf, const float *__restrict__ meta, float4 *__restrict__ tris, uint32_t *__restrict__ ids)
{
	const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= nf) return;
	const uint32_t prim = vals ? vals[j] : j;
	const uint4 f = reinterpret_cast<const uint4 *>(faces)[prim];
	const bool quad = f.w != GBRT_TRIANGLE;
	if(reinterpret_cast<const uint32_t *>(meta)[GBRT_META_ERR])
	{
		tris[3ull * j] = tris[3ull * j + 1] = tris[3ull * j + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
		ids[j] = prim;
		return;
	}
	const float3 v0 = make_float3(verts[3ull * f.x], verts[3ull * f.x + 1], verts[3ull * f.x + 2]);
	const float3 v1 = make_float3(verts[3ull * f.y], verts[3ull * f.y + 1], verts[3ull * f.y + 2]);
	const float3 v2 = make_float3(verts[3ull * f.z], verts[3ull * f.z + 1], verts[3ull * f.z + 2]);
	float3 e3 = make_float3(0.f, 0.f, 0.f);
	if(quad)
	{
		const float3 v3 = make_float3(verts[3ull * f.w], verts[3ull * f.w + 1], verts[3ull * f.w + 2]);
		e3 = make_float3(__fsub_rn(v3.x, v0.x), __fsub_rn(v3.y, v0.y), __fsub_rn(v3.z, v0.z));
	}
	tris[3ull * j + 0] = make_float4(v0.x, v0.y, v0.z, e3.x);
	tris[3ull * j + 1] = make_float4(__fsub_rn(v1.x, v0.x), __fsub_rn(v1.y, v0.y), __fsub_rn(v1.z, v0.z), e3.y);
	tris[3ull * j + 2] = make_float4(__fsub_rn(v2.x, v0.x), __fsub_rn(v2.y, v0.y), __fsub_rn(v2.z, v0.z), e3.z);
	ids[j] = prim | (quad ? GBRT_QUAD_BIT : 0u);
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

struct Scratch {
	cudaStream_t s;
	void *p = nullptr;
	explicit Scratch(cudaStream_t st) : s(st) { }
	~Scratch() { if(p) cudaFreeAsync(p, s); }
};

} // namespace

int gbrt_build_impl(const float *verts, uint32_t nv, const uint32_t *faces, uint32_t nf,
                    const gbrt_build_params *params, cudaStream_t s, gbrt_bvh **out)
{
	if(!out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build: out is NULL");
	*out = nullptr;
	if(nf > 0 && (!verts || !faces)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build: NULL vertex or face buffer");
	if(nf >= GBRT_LEAF_MAX_SLOTS) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_build: %u faces exceed the limit of %u", nf, GBRT_LEAF_MAX_SLOTS - 1);
	gbrt_build_params p{};
	if(params) p = *params;
	if(p.max_leaf_size == 0) p.max_leaf_size = 4;
	if(p.max_leaf_size > GBRT_LEAF_MAX_COUNT) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build: max_leaf_size %u > %u", p.max_leaf_size, GBRT_LEAF_MAX_COUNT);
	if(!(p.traversal_cost > 0.f)) p.traversal_cost = 1.f;
	if(!(p.intersect_cost > 0.f)) p.intersect_cost = 1.f;

	gbrt_bvh *b = new gbrt_bvh();
	b->params = p;
	b->n_prims = nf;
	GBRT_CK(cudaGetDevice(&b->device));
	const uint32_t n_int = nf > 1 ? nf - 1 : 1;
	b->n_node_slots = n_int;
	auto fail = [&](int code) { gbrt_bvh_destroy(b); return code; };
	cudaError_t e;
	const size_t node_bytes = 64ull * n_int, tri_bytes = 48ull * (nf ? nf : 1), id_bytes = 4ull * (nf ? nf : 1);
	if((e = cudaMalloc(&b->nodes, node_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->tris, tri_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->ids, id_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->meta, GBRT_META_WORDS * sizeof(float))) != cudaSuccess)
		return fail(gbrt_set_error(GBRT_ERR_OOM, "gbrt_bvh_build: device allocation failed: %s", cudaGetErrorString(e)));
	b->bytes = node_bytes + tri_bytes + id_bytes + GBRT_META_WORDS * sizeof(float);

	k_init_meta<<<1, 32, 0, s>>>(b->meta);
	if(nf == 0)
	{
		k_finalize<<<1, 32, 0, s>>>(b->meta, 0);
		if((e = cudaMemsetAsync(b->nodes, 0, node_bytes, s)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "memset: %s", cudaGetErrorString(e)));
		if((e = cudaGetLastError()) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_CUDA, "build launch: %s", cudaGetErrorString(e)));
		*out = b;
		return GBRT_OK;
	}

	// scratch carve-up (one stream-ordered allocation)
	const uint32_t nblk = blocks_for(nf, kSortTile);
	const size_t hist_words = 256ull * nblk;
	size_t off = 0;
	auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
	const size_t o_blo = carve(16ull * nf), o_bhi = carve(16ull * nf);
	const size_t o_k0 = carve(4ull * nf), o_k1 = carve(4ull * nf), o_v0 = carve(4ull * nf), o_v1 = carve(4ull * nf);
	const size_t o_hist = carve(4 * hist_words);
	const size_t o_child = carve(8ull * n_int), o_range = carve(8ull * n_int);
	const size_t o_pint = carve(4ull * n_int), o_pleaf = carve(4ull * nf);
	const size_t o_nlo = carve(16ull * n_int), o_nhi = carve(16ull * n_int);
	const size_t o_flags = carve(4ull * n_int), o_coll = carve(n_int);
	Scratch sc(s);
	if((e = cudaMallocAsync(&sc.p, off, s)) != cudaSuccess)
		return fail(gbrt_set_error(GBRT_ERR_OOM, "gbrt_bvh_build: scratch allocation of %zu bytes failed: %s", off, cudaGetErrorString(e)));
	char *base = static_cast<char *>(sc.p);
	float4 *blo = reinterpret_cast<float4 *>(base + o_blo), *bhi = reinterpret_cast<float4 *>(base + o_bhi);
	uint32_t *k0 = reinterpret_cast<uint32_t *>(base + o_k0), *k1 = reinterpret_cast<uint32_t *>(base + o_k1);
	uint32_t *v0 = reinterpret_cast<uint32_t *>(base + o_v0), *v1 = reinterpret_cast<uint32_t *>(base + o_v1);
	uint32_t *hist = reinterpret_cast<uint32_t *>(base + o_hist);
	uint2 *child = reinterpret_cast<uint2 *>(base + o_child), *range = reinterpret_cast<uint2 *>(base + o_range);
	uint32_t *pint = reinterpret_cast<uint32_t *>(base + o_pint), *pleaf = reinterpret_cast<uint32_t *>(base + o_pleaf);
	float4 *nlo = reinterpret_cast<float4 *>(base + o_nlo), *nhi = reinterpret_cast<float4 *>(base + o_nhi);
	uint32_t *flags = reinterpret_cast<uint32_t *>(base + o_flags);
	uint8_t *coll = reinterpret_cast<uint8_t *>(base + o_coll);

	k_setup<<<blocks_for(nf, 256), 256, 0, s>>>(verts, nv, faces, nf, blo, bhi, b->meta);
	k_finalize<<<1, 32, 0, s>>>(b->meta, nf);
	if(nf == 1)
	{
		k_emit_single<<<1, 1, 0, s>>>(blo, bhi, b->meta, b->nodes);
		k_emit_prims<<<1, 32, 0, s>>>(verts, faces, nullptr, 1, b->meta, b->tris, b->ids);
	}
	else
	{
		k_morton<<<blocks_for(nf, 256), 256, 0, s>>>(blo, bhi, nf, b->meta, k0, v0);
		uint32_t *kin = k0, *kout = k1, *vin = v0, *vout = v1;
		for(int shift = 0; shift < 30; shift += 8)
		{
			k_hist<<<nblk, kSortThreads, 0, s>>>(kin, nf, shift, hist, nblk);
			k_scan<<<1, 1024, 0, s>>>(hist, static_cast<uint32_t>(hist_words));
			k_scatter<<<nblk, kSortThreads, 0, s>>>(kin, vin, nf, shift, hist, nblk, kout, vout);
			std::swap(kin, kout); std::swap(vin, vout);
		}
		if((e = cudaMemsetAsync(pint, 0xFF, 4ull * n_int, s)) != cudaSuccess ||
		   (e = cudaMemsetAsync(flags, 0, 4ull * n_int, s)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "memset: %s", cudaGetErrorString(e)));
		k_karras<<<blocks_for(n_int, 256), 256, 0, s>>>(kin, static_cast<int>(nf), child, range, pint, pleaf);
		k_refit<<<blocks_for(nf, 256), 256, 0, s>>>(vin, static_cast<int>(nf), blo, bhi, child, pint, pleaf, nlo, nhi, flags, coll,
		                                            p.max_leaf_size, p.traversal_cost, p.intersect_cost);
		k_emit_nodes<<<blocks_for(n_int, 256), 256, 0, s>>>(static_cast<int>(n_int), vin, blo, bhi, child, range, nlo, nhi, coll, b->meta, b->nodes);
		k_emit_prims<<<blocks_for(nf, 256), 256, 0, s>>>(verts, faces, vin, nf, b->meta, b->tris, b->ids);
	}
	if((e = cudaGetLastError()) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_CUDA, "build launch: %s", cudaGetErrorString(e)));
	*out = b;
	return GBRT_OK;
}

// ---- build without device allocation -------------------------------------
// gbrt_bvh_build_static runs the same kernels as gbrt_build_impl, with its
// temporaries carved from one file-scope device array instead of a
// stream-ordered allocation.
namespace {

constexpr size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

struct StaticLayout {
	size_t blo, bhi, k0, k1, v0, v1, hist, child, range, pint, pleaf, nlo, nhi, flags, coll, meta, total;
};

constexpr StaticLayout static_layout(uint64_t nf)
{
	const uint64_t n_int = nf > 1 ? nf - 1 : 1;
	const uint64_t nblk = (nf + kSortTile - 1) / kSortTile;
	StaticLayout L{};
	size_t o = 0;
	L.blo = o; o += round256(16 * nf);
	L.bhi = o; o += round256(16 * nf);
	L.k0 = o; o += round256(4 * nf);
	L.k1 = o; o += round256(4 * nf);
	L.v0 = o; o += round256(4 * nf);
	L.v1 = o; o += round256(4 * nf);
	L.hist = o; o += round256(4 * 256 * nblk);
	L.child = o; o += round256(8 * n_int);
	L.range = o; o += round256(8 * n_int);
	L.pint = o; o += round256(4 * n_int);
	L.pleaf = o; o += round256(4 * nf);
	L.nlo = o; o += round256(16 * n_int);
	L.nhi = o; o += round256(16 * n_int);
	L.flags = o; o += round256(4 * n_int);
	L.coll = o; o += round256(n_int);
	L.meta = o; o += round256(4 * GBRT_META_WORDS);
	L.total = o;
	return L;
}

constexpr size_t kStaticScratchBytes = static_layout(GBRT_STATIC_MAX_FACES).total;

// Shared by every call on a device; see gbrt_bvh_build_static in gbrt.h.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char *g_static_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device, looked up once
// per device (host code must not use the symbol itself as a pointer).
int static_scratch_address(int dev, unsigned char **out)
{
	if(dev < 0 || dev >= kMaxDevices) return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_build_static: device %d out of range", dev);
	std::lock_guard<std::mutex> g(g_static_mu);
	if(!g_static_addr[dev])
	{
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
		if(e != cudaSuccess || !p)
			return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
		g_static_addr[dev] = static_cast<unsigned char *>(p);
	}
	*out = g_static_addr[dev];
	return GBRT_OK;
}

} // namespace

extern "C" int gbrt_bvh_build_static(const float *verts, uint32_t nv, const uint32_t *faces, uint32_t nf,
                                     const gbrt_build_params *params, void *nodes_dev, size_t nodes_bytes,
                                     void *prims_dev, size_t prims_bytes, uint32_t *ids_dev, size_t ids_bytes,
                                     float bound_out[6], void *stream)
{
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	if(nf > GBRT_STATIC_MAX_FACES)
		return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_build_static: %u faces exceed the fixed scratch capacity of %u faces",
		                      nf, GBRT_STATIC_MAX_FACES);
	if(nf > 0 && (!verts || !faces)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: NULL vertex or face buffer");
	if(!bound_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: bound_out is NULL");
	const uint32_t n_int = nf > 1 ? nf - 1 : 1;
	if(!nodes_dev || nodes_bytes < 64ull * n_int || (nf && (!prims_dev || prims_bytes < 48ull * nf || !ids_dev || ids_bytes < 4ull * nf)))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: output buffers missing or too small (need %llu/%llu/%llu bytes)",
		                      64ull * n_int, 48ull * nf, 4ull * nf);
	gbrt_build_params p{};
	if(params) p = *params;
	if(p.max_leaf_size == 0) p.max_leaf_size = 4;
	if(p.max_leaf_size > GBRT_LEAF_MAX_COUNT) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: max_leaf_size %u > %u", p.max_leaf_size, GBRT_LEAF_MAX_COUNT);
	if(!(p.traversal_cost > 0.f)) p.traversal_cost = 1.f;
	if(!(p.intersect_cost > 0.f)) p.intersect_cost = 1.f;
	int dev = 0;
	GBRT_CK(cudaGetDevice(&dev));
	unsigned char *base = nullptr;
	if(int rc = static_scratch_address(dev, &base)) return rc;

	const StaticLayout L = static_layout(nf);
	float *meta = reinterpret_cast<float *>(base + L.meta);
	float4 *nodes = static_cast<float4 *>(nodes_dev);
	k_init_meta<<<1, 32, 0, s>>>(meta);
	if(nf == 0)
	{
		k_finalize<<<1, 32, 0, s>>>(meta, 0);
		GBRT_CK(cudaMemsetAsync(nodes_dev, 0, 64ull * n_int, s));
	}
	else
	{
		float4 *blo = reinterpret_cast<float4 *>(base + L.blo), *bhi = reinterpret_cast<float4 *>(base + L.bhi);
		uint32_t *k0 = reinterpret_cast<uint32_t *>(base + L.k0), *k1 = reinterpret_cast<uint32_t *>(base + L.k1);
		uint32_t *v0 = reinterpret_cast<uint32_t *>(base + L.v0), *v1 = reinterpret_cast<uint32_t *>(base + L.v1);
		uint32_t *hist = reinterpret_cast<uint32_t *>(base + L.hist);
		uint2 *child = reinterpret_cast<uint2 *>(base + L.child), *range = reinterpret_cast<uint2 *>(base + L.range);
		uint32_t *pint = reinterpret_cast<uint32_t *>(base + L.pint), *pleaf = reinterpret_cast<uint32_t *>(base + L.pleaf);
		float4 *nlo = reinterpret_cast<float4 *>(base + L.nlo), *nhi = reinterpret_cast<float4 *>(base + L.nhi);
		uint32_t *flags = reinterpret_cast<uint32_t *>(base + L.flags);
		uint8_t *coll = reinterpret_cast<uint8_t *>(base + L.coll);
		float4 *tris = static_cast<float4 *>(prims_dev);
		k_setup<<<blocks_for(nf, 256), 256, 0, s>>>(verts, nv, faces, nf, blo, bhi, meta);
		k_finalize<<<1, 32, 0, s>>>(meta, nf);
		if(nf == 1)
		{
			k_emit_single<<<1, 1, 0, s>>>(blo, bhi, meta, nodes);
			k_emit_prims<<<1, 32, 0, s>>>(verts, faces, nullptr, 1, meta, tris, ids_dev);
		}
		else
		{
			const uint32_t nblk = blocks_for(nf, kSortTile);
			k_morton<<<blocks_for(nf, 256), 256, 0, s>>>(blo, bhi, nf, meta, k0, v0);
			uint32_t *kin = k0, *kout = k1, *vin = v0, *vout = v1;
			for(int shift = 0; shift < 30; shift += 8)
			{
				k_hist<<<nblk, kSortThreads, 0, s>>>(kin, nf, shift, hist, nblk);
				k_scan<<<1, 1024, 0, s>>>(hist, 256u * nblk);
				k_scatter<<<nblk, kSortThreads, 0, s>>>(kin, vin, nf, shift, hist, nblk, kout, vout);
				std::swap(kin, kout); std::swap(vin, vout);
			}
			// the array keeps the previous call's contents: reset parents and arrival counters
			GBRT_CK(cudaMemsetAsync(pint, 0xFF, 4ull * n_int, s));
			GBRT_CK(cudaMemsetAsync(flags, 0, 4ull * n_int, s));
			k_karras<<<blocks_for(n_int, 256), 256, 0, s>>>(kin, static_cast<int>(nf), child, range, pint, pleaf);
			k_refit<<<blocks_for(nf, 256), 256, 0, s>>>(vin, static_cast<int>(nf), blo, bhi, child, pint, pleaf, nlo, nhi, flags, coll,
			                                            p.max_leaf_size, p.traversal_cost, p.intersect_cost);
			k_emit_nodes<<<blocks_for(n_int, 256), 256, 0, s>>>(static_cast<int>(n_int), vin, blo, bhi, child, range, nlo, nhi, coll, meta, nodes);
			k_emit_prims<<<blocks_for(nf, 256), 256, 0, s>>>(verts, faces, vin, nf, meta, tris, ids_dev);
		}
	}
	GBRT_CK(cudaGetLastError());
	float m[GBRT_META_WORDS];
	GBRT_CK(cudaMemcpyAsync(m, meta, sizeof(m), cudaMemcpyDeviceToHost, s));
	GBRT_CK(cudaStreamSynchronize(s));
	uint32_t err;
	std::memcpy(&err, &m[GBRT_META_ERR], 4);
	if(err) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: a face references a vertex index >= %u", nv);
	std::memcpy(bound_out, &m[GBRT_META_BOUND], 6 * sizeof(float));
	return GBRT_OK;
}
