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
//   7. k_treelet     SAH treelet restructuring (Karras & Aila, "Fast
//                    parallel construction of high-quality bounding volume
//                    hierarchies", HPG 2013): bottom-up, every node over
//                    gamma primitives rebuilds the optimal binary tree over
//                    its 7-leaf treelet by dynamic programming over leaf
//                    subsets; two passes, then k_refit again
//   8. k_order_*     leaf slots in depth-first order (every subtree's
//                    primitives contiguous after restructuring)
//   9. k_emit_nodes  64-byte binary nodes holding both children's boxes
//  10. k_emit_prims  48-byte primitive records in leaf order
//  11. k_wide_cost   SAH dynamic programme over the binary tree choosing
//                    which subtrees become the children of each 8-wide node
//  12. k_wide_level  8-wide compressed hierarchy for the traversal, one
//                    launch per level (layout in gbrt_internal.cuh), after
//                    Ylitie, Karras & Laine, "Efficient incoherent ray
//                    traversal on GPUs through compressed wide BVHs", HPG
//                    2017: the children k_wide_cost chose (or, with
//                    GBRT_BUILD_GREEDY_WIDE, the largest-area child opened
//                    until 8), 8-bit child planes on a per-node
//                    power-of-two grid, slots by ray octant
#include "gbrt_internal.cuh"

#include <cfloat>
#include <cmath>
#include <cstring>

// SAH cost of a primitive test relative to a node visit when the caller
// gives none.  The 8-wide node test is cheaper than the reference's exact
// Moller-Trumbore test, so at 2 nearly every leaf holds one triangle;
// measured on a GB300 (1,048,576-triangle soup, 16.8M incoherent rays),
// cost 1 / 2 / 3: closest hit 2,322 / 2,467 / 2,472 Mrays/s, any hit
// 3,377 / 3,555 / 3,556 (leaf sizes 2-16 at cost 2: within 0.1 %).
constexpr float kDefaultIntersectCost = 2.f;

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kNoParent = 0xFFFFFFFFu;
// Upper bound on any leaf-to-root walk; a longer walk means a broken
// hierarchy: the walk stops and raises GBRT_META_ERR bit 4.
constexpr int kMaxWalk = 1 << 14;
constexpr uint32_t kErrWalk = 4u, kErrWide = 8u;

__device__ __forceinline__ void raise_err(float *meta, uint32_t bit)
{
	atomicOr(reinterpret_cast<uint32_t *>(meta) + GBRT_META_ERR, bit);
}

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

// Exclusive scan of m words in three launches: tiles of kScanTile words
// scanned in place (tile sums to `totals`), the tile sums scanned by one
// block, then added back.
constexpr uint32_t kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__host__ __device__ constexpr uint32_t scan_tiles(uint32_t m) { return (m + kScanTile - 1) / kScanTile; }

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &total)
{
	__shared__ uint32_t warp_sums[kScanThreads / 32];
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint32_t x = v;
	for(int off = 1; off < 32; off <<= 1)
	{
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
		if(lane >= static_cast<uint32_t>(off)) x += y;
	}
	if(lane == 31) warp_sums[warp] = x;
	__syncthreads();
	if(warp == 0)
	{
		uint32_t w = warp_sums[lane];
		for(int off = 1; off < 32; off <<= 1)
		{
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, off);
			if(lane >= static_cast<uint32_t>(off)) w += y;
		}
		warp_sums[lane] = w;
	}
	__syncthreads();
	total = warp_sums[31];
	const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
	__syncthreads();
	return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(uint32_t *__restrict__ data, uint32_t m, uint32_t *__restrict__ totals)
{
	const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
	uint32_t v[kScanItems], sum = 0;
	for(uint32_t k = 0; k < kScanItems; ++k) { v[k] = base + k < m ? data[base + k] : 0u; sum += v[k]; }
	uint32_t total;
	uint32_t run = block_exclusive_scan(sum, total);
	for(uint32_t k = 0; k < kScanItems; ++k)
	{
		if(base + k < m) data[base + k] = run;
		run += v[k];
	}
	if(threadIdx.x == 0) totals[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums (any count, in rounds of kScanThreads)
__global__ void __launch_bounds__(kScanThreads) k_scan_totals(uint32_t *__restrict__ totals, uint32_t tiles)
{
	uint32_t carry = 0;
	for(uint32_t b = 0; b < tiles; b += kScanThreads)
	{
		const uint32_t i = b + threadIdx.x;
		const uint32_t v = i < tiles ? totals[i] : 0u;
		uint32_t total;
		const uint32_t ex = block_exclusive_scan(v, total);
		if(i < tiles) totals[i] = carry + ex;
		carry += total;
	}
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(uint32_t *__restrict__ data, uint32_t m, const uint32_t *__restrict__ totals)
{
	const uint32_t add = totals[blockIdx.x];
	const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
	for(uint32_t k = 0; k < kScanItems; ++k)
		if(base + k < m) data[base + k] += add;
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
                        uint32_t max_leaf, float ct, float ci, float *meta)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= n) return;
	uint32_t p = __ldcg(parent_leaf + j);
	for(int walk = 0; p != kNoParent; ++walk)
	{
		if(walk == kMaxWalk) { raise_err(meta, kErrWalk); return; }
		__threadfence();
		if(atomicAdd(&flags[p], 1u) == 0u) return;
		__threadfence();
		const uint2 c = __ldcg(child + p);
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
		p = __ldcg(parent_int + p);
	}
}

// ---- treelet restructuring -------------------------------------------------
constexpr int kTreeletLeaves = 7;
constexpr uint32_t kTreeletSubsets = 1u << kTreeletLeaves;

// Box, SAH cost and primitive count of a child reference.  Internal nodes are
// rewritten by other threads of the same launch: read them through L2.
__device__ __forceinline__ void ref_info(uint32_t ref, const uint32_t *__restrict__ vals, const float4 *__restrict__ box_lo,
                                         const float4 *__restrict__ box_hi, const float4 *node_lo, const float4 *node_hi, float ci,
                                         float4 &lo, float4 &hi, float &cost, uint32_t &cnt)
{
	if(ref & GBRT_LEAF_BIT)
	{
		const uint32_t prim = __ldg(vals + (ref & ~GBRT_LEAF_BIT));
		lo = __ldg(box_lo + prim); hi = __ldg(box_hi + prim);
		cost = ci * half_area(lo, hi);
		cnt = 1u;
	}
	else
	{
		lo = __ldcg(node_lo + ref); hi = __ldcg(node_hi + ref);
		cost = lo.w;
		cnt = __float_as_uint(hi.w);
	}
}

// Per-warp shared arrays of the treelet dynamic programme.
struct TreeletSmem {
	float C[kTreeletSubsets];          // optimal cost of each leaf subset
	float A[kTreeletSubsets];          // half area of its union box
	uint32_t N[kTreeletSubsets];       // primitives under it
	uint8_t split[kTreeletSubsets];    // best first part (contains the lowest leaf)
};

// Rebuilds the treelet under `root` as the SAH-optimal binary tree over the
// same leaves, reusing its internal node indices; called by all 32 lanes of
// a warp with the same root.  The treelet (at most 7 leaves, grown by
// opening the leaf of largest area) is formed redundantly by every lane;
// subset areas and the costs of the subsets of each size are computed
// across the lanes; lane 0 writes the result.
__device__ __noinline__ void restructure_warp(uint32_t root, TreeletSmem &sm, const uint32_t *__restrict__ vals,
                                              const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi, uint2 *child,
                                              uint32_t *parent_int, uint32_t *parent_leaf, float4 *node_lo, float4 *node_hi,
                                              uint32_t max_leaf, float ct, float ci)
{
	const uint32_t lane = threadIdx.x & 31u;
	uint32_t T[kTreeletLeaves], I[kTreeletLeaves - 1], cnt[kTreeletLeaves];
	float4 lo[kTreeletLeaves], hi[kTreeletLeaves];
	float cost[kTreeletLeaves];
	int m = 2, ni = 1;
	I[0] = root;
	{
		const uint2 c = __ldcg(child + root);
		T[0] = c.x; T[1] = c.y;
		ref_info(c.x, vals, box_lo, box_hi, node_lo, node_hi, ci, lo[0], hi[0], cost[0], cnt[0]);
		ref_info(c.y, vals, box_lo, box_hi, node_lo, node_hi, ci, lo[1], hi[1], cost[1], cnt[1]);
	}
	while(m < kTreeletLeaves)
	{
		int best = -1;
		float ba = -1.f;
		for(int k = 0; k < m; ++k)
			if(!(T[k] & GBRT_LEAF_BIT))
			{
				const float a = half_area(lo[k], hi[k]);
				if(a > ba) { ba = a; best = k; }
			}
		if(best < 0) break;
		const uint32_t r = T[best];
		I[ni++] = r;
		const uint2 c = __ldcg(child + r);
		T[best] = c.x;
		ref_info(c.x, vals, box_lo, box_hi, node_lo, node_hi, ci, lo[best], hi[best], cost[best], cnt[best]);
		T[m] = c.y;
		ref_info(c.y, vals, box_lo, box_hi, node_lo, node_hi, ci, lo[m], hi[m], cost[m], cnt[m]);
		++m;
	}
	if(m < 3) return;   // warp-uniform: every lane formed the same treelet
	const uint32_t full = (1u << m) - 1u;
	// union areas and counts of every subset, 32 subsets at a time
	for(uint32_t S = lane + 1u; S <= full; S += 32u)
	{
		float4 L = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), H = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
		uint32_t N = 0;
		for(int k = 0; k < m; ++k)
			if((S >> k) & 1u)
			{
				L.x = fminf(L.x, lo[k].x); L.y = fminf(L.y, lo[k].y); L.z = fminf(L.z, lo[k].z);
				H.x = fmaxf(H.x, hi[k].x); H.y = fmaxf(H.y, hi[k].y); H.z = fmaxf(H.z, hi[k].z);
				N += cnt[k];
			}
		sm.A[S] = half_area(L, H);
		sm.N[S] = N;
		if(!(S & (S - 1u))) { sm.C[S] = cost[__ffs(S) - 1]; sm.split[S] = 0; }
	}
	__syncwarp();
	// c(S) = min(Ci A(S) N(S) [N <= max leaf], Ct A(S) + min over splits P of c(P) + c(S \ P)),
	// the subsets of one size at a time
	for(int size = 2; size <= m; ++size)
	{
		for(uint32_t S = lane + 1u; S <= full; S += 32u)
		{
			if(__popc(S) != size) continue;
			const uint32_t low = S & (0u - S);
			float best = FLT_MAX;
			uint32_t bp = low;
			for(uint32_t P = (S - 1u) & S; P; P = (P - 1u) & S)
				if(P & low)
				{
					const float c = sm.C[P] + sm.C[S ^ P];
					if(c < best) { best = c; bp = P; }
				}
			const float A = sm.A[S];
			const float c_int = ct * A + best;
			const float c_leaf = sm.N[S] <= max_leaf ? ci * A * static_cast<float>(sm.N[S]) : FLT_MAX;
			sm.C[S] = c_leaf <= c_int ? c_leaf : c_int;
			sm.split[S] = static_cast<uint8_t>(bp);
		}
		__syncwarp();
	}
	if(lane == 0)
	{
		// rewrite: the root keeps its index, the other internal nodes are reused
		uint32_t stS[kTreeletLeaves], stN[kTreeletLeaves];
		int sp = 1, next = 1;
		stS[0] = full; stN[0] = root;
		while(sp > 0)
		{
			--sp;
			const uint32_t S = stS[sp], nd = stN[sp];
			const uint32_t sub[2] = {sm.split[S], S ^ sm.split[S]};
			uint32_t ref[2];
			for(int k = 0; k < 2; ++k)
			{
				if(!(sub[k] & (sub[k] - 1u))) ref[k] = T[__ffs(sub[k]) - 1];
				else { ref[k] = I[next++]; stS[sp] = sub[k]; stN[sp] = ref[k]; ++sp; }
				if(ref[k] & GBRT_LEAF_BIT) parent_leaf[ref[k] & ~GBRT_LEAF_BIT] = nd;
				else parent_int[ref[k]] = nd;
			}
			child[nd] = make_uint2(ref[0], ref[1]);
			float4 L = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), H = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
			for(int k = 0; k < m; ++k)
				if((S >> k) & 1u)
				{
					L.x = fminf(L.x, lo[k].x); L.y = fminf(L.y, lo[k].y); L.z = fminf(L.z, lo[k].z);
					H.x = fmaxf(H.x, hi[k].x); H.y = fmaxf(H.y, hi[k].y); H.z = fmaxf(H.z, hi[k].z);
				}
			L.w = sm.C[S];
			H.w = __uint_as_float(sm.N[S]);
			node_lo[nd] = L;
			node_hi[nd] = H;
		}
		__threadfence();
	}
	__syncwarp();
}

constexpr int kTreeletThreads = 128;

// Bottom-up like k_refit: the second thread to reach a node owns it, and its
// whole subtree is final.  Owned nodes holding at least gamma primitives are
// restructured, one at a time per warp with the whole warp; every lane stays
// in the loop (full-warp ballots) until all lanes of the warp are done.
__global__ void __launch_bounds__(kTreeletThreads)
k_treelet(int n, const uint32_t *__restrict__ vals, const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi,
          uint2 *child, uint32_t *parent_int, uint32_t *parent_leaf, float4 *node_lo, float4 *node_hi,
          uint32_t *flags, uint32_t gamma, uint32_t max_leaf, float ct, float ci, float *meta)
{
	__shared__ TreeletSmem smem[kTreeletThreads / 32];
	TreeletSmem &sm = smem[threadIdx.x >> 5];
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	bool active = j < n;
	uint32_t p = active ? __ldcg(parent_leaf + j) : kNoParent;
	active = active && p != kNoParent;
	for(int walk = 0; __any_sync(0xFFFFFFFFu, active); ++walk)
	{
		bool own = false;
		if(active)
		{
			if(walk == kMaxWalk) { raise_err(meta, kErrWalk); active = false; }
			else
			{
				__threadfence();
				if(atomicAdd(&flags[p], 1u) == 0u) active = false;
				else { __threadfence(); own = __float_as_uint(__ldcg(node_hi + p).w) >= gamma; }
			}
		}
		uint32_t todo = __ballot_sync(0xFFFFFFFFu, own);
		while(todo)
		{
			const int l = __ffs(todo) - 1;
			todo &= todo - 1u;
			const uint32_t root = __shfl_sync(0xFFFFFFFFu, p, l);
			restructure_warp(root, sm, vals, box_lo, box_hi, child, parent_int, parent_leaf, node_lo, node_hi, max_leaf, ct, ci);
		}
		if(active)
		{
			p = __ldcg(parent_int + p);
			active = p != kNoParent;
		}
	}
}

// ---- depth-first leaf order -------------------------------------------------
__device__ __forceinline__ uint32_t ref_count(uint32_t ref, const float4 *__restrict__ node_hi)
{
	return (ref & GBRT_LEAF_BIT) ? 1u : __float_as_uint(node_hi[ref].w);
}

// Primitives before `ref` in depth-first order: the left siblings' counts
// along the path to the root.
__device__ __forceinline__ uint32_t dfs_offset(uint32_t ref, uint32_t p, const uint2 *__restrict__ child, const uint32_t *__restrict__ parent_int,
                                               const float4 *__restrict__ node_hi, float *meta)
{
	uint32_t off = 0;
	for(int walk = 0; p != kNoParent; ++walk)
	{
		if(walk == kMaxWalk) { raise_err(meta, kErrWalk); return 0u; }
		const uint2 c = child[p];
		if(c.y == ref) off += ref_count(c.x, node_hi);
		ref = p;
		p = parent_int[p];
	}
	return off;
}

__global__ void k_order_leaves(int n, const uint32_t *__restrict__ vals, const uint2 *__restrict__ child, const uint32_t *__restrict__ parent_int,
                               const uint32_t *__restrict__ parent_leaf, const float4 *__restrict__ node_hi,
                               uint32_t *__restrict__ pos_leaf, uint32_t *__restrict__ vals_out, float *meta)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= n) return;
	const uint32_t off = dfs_offset(GBRT_LEAF_BIT | static_cast<uint32_t>(j), parent_leaf[j], child, parent_int, node_hi, meta);
	if(off >= static_cast<uint32_t>(n)) { raise_err(meta, kErrWalk); return; }
	pos_leaf[j] = off;
	vals_out[off] = vals[j];
}

__global__ void k_order_nodes(int n_int, const uint2 *__restrict__ child, const uint32_t *__restrict__ parent_int,
                              const float4 *__restrict__ node_hi, uint32_t *__restrict__ first_int, float *meta)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n_int) return;
	first_int[i] = dfs_offset(static_cast<uint32_t>(i), parent_int[i], child, parent_int, node_hi, meta);
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
                             const uint2 *__restrict__ child, const uint32_t *__restrict__ pos_leaf, const uint32_t *__restrict__ first_int,
                             const float4 *__restrict__ node_lo, const float4 *__restrict__ node_hi, const uint8_t *__restrict__ collapse,
                             const float *__restrict__ meta, float4 *__restrict__ nodes)
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
			ref[k] = gbrt_leaf_ref(pos_leaf[leaf], 1u);
		}
		else
		{
			lo[k] = node_lo[cc[k]]; hi[k] = node_hi[cc[k]];
			if(collapse[cc[k]]) ref[k] = gbrt_leaf_ref(first_int[cc[k]], __float_as_uint(hi[k].w));
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

// ---- 8-wide compressed hierarchy -------------------------------------------
constexpr uint32_t kWideLeafMax = 3;      // primitives per wide leaf child (unary count in 3 bits)
constexpr int kWideLevels = GBRT_WIDE_MAX_LEVELS;

struct WideSrc {
	const uint2 *child;
	const uint32_t *vals;          // primitive of each binary leaf (sorted order)
	const float4 *box_lo, *box_hi;
	const float4 *node_lo, *node_hi;
	const uint8_t *collapse;
	const uint32_t *pos_leaf, *first_int;
	const float4 *tris;
	const uint32_t *ids;
	uint32_t n_node_cap;           // wide node slots (= task buffer entries)
	uint32_t n_prims;
	const uint8_t *choice;         // SAH collapse decisions (k_wide_cost), or null for the greedy collapse
};

__device__ __forceinline__ bool wide_leaf(uint32_t ref, const WideSrc &W)
{
	if(ref & GBRT_LEAF_BIT) return true;
	if(W.choice) return W.choice[8ull * ref + 7] != 0u;
	return W.collapse[ref] && __float_as_uint(W.node_hi[ref].w) <= kWideLeafMax;
}

// SAH-optimal collapse of the binary hierarchy into 8-wide nodes, after
// Ylitie, Karras & Laine (HPG 2017, section 3.1), bottom up as k_refit.
// For a binary node n with children L, R, area A and p primitives:
//   D(n, 1)   = min(leaf: ci A p if p <= 3, wide node: ct A + min_k D(L, k) + D(R, 8 - k))
//   D(n, j)   = min(D(n, j - 1), min_k D(L, k) + D(R, j - k))      j = 2..7
// D(n, j) is the cheapest way to hand subtree n to its parent wide node as at
// most j children; a primitive (binary leaf) costs ci A for every j.
// cost[7 n + j - 1] = D(n, j); choice[8 n]: the k of the wide node (R gets
// 8 - k); choice[8 n + j - 1], j = 2..7: 0 = D(n, j - 1), else its k;
// choice[8 n + 7]: 1 = n is a leaf child.
__global__ void k_wide_cost(const uint32_t *__restrict__ vals, int n, const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi,
                            const uint2 *__restrict__ child, const uint32_t *__restrict__ parent_int, const uint32_t *__restrict__ parent_leaf,
                            const float4 *__restrict__ node_lo, const float4 *__restrict__ node_hi, uint32_t *flags, float *cost,
                            uint8_t *choice, float ct, float ci, float *meta)
{
	const int j0 = blockIdx.x * blockDim.x + threadIdx.x;
	if(j0 >= n) return;
	uint32_t p = __ldcg(parent_leaf + j0);
	for(int walk = 0; p != kNoParent; ++walk)
	{
		if(walk == kMaxWalk) { raise_err(meta, kErrWalk); return; }
		__threadfence();
		if(atomicAdd(&flags[p], 1u) == 0u) return;
		__threadfence();
		const uint2 c = __ldcg(child + p);
		const uint32_t cc[2] = {c.x, c.y};
		float d[2][8];
		for(int k = 0; k < 2; ++k)
		{
			if(cc[k] & GBRT_LEAF_BIT)
			{
				const uint32_t prim = vals[cc[k] & ~GBRT_LEAF_BIT];
				const float v = ci * half_area(box_lo[prim], box_hi[prim]);
				for(int jj = 1; jj <= 7; ++jj) d[k][jj] = v;
			}
			else
				for(int jj = 1; jj <= 7; ++jj) d[k][jj] = __ldcg(cost + 7ull * cc[k] + jj - 1);
		}
		const float area = half_area(node_lo[p], node_hi[p]);
		const uint32_t cnt = __float_as_uint(node_hi[p].w);
		uint8_t ch[8];
		float best = FLT_MAX;
		ch[0] = 1;
		for(int k = 1; k <= 7; ++k)
		{
			const float v = d[0][k] + d[1][8 - k];
			if(v < best) { best = v; ch[0] = static_cast<uint8_t>(k); }
		}
		const float c_wide = ct * area + best;
		const float c_leaf = cnt <= kWideLeafMax ? ci * area * static_cast<float>(cnt) : FLT_MAX;
		float dn[8];
		dn[1] = fminf(c_leaf, c_wide);
		ch[7] = c_leaf <= c_wide ? 1 : 0;
		for(int jj = 2; jj <= 7; ++jj)
		{
			float b = dn[jj - 1];
			uint8_t kk = 0;
			for(int k = 1; k < jj; ++k)
			{
				const float v = d[0][k] + d[1][jj - k];
				if(v < b) { b = v; kk = static_cast<uint8_t>(k); }
			}
			dn[jj] = b;
			ch[jj - 1] = kk;
		}
		for(int jj = 1; jj <= 7; ++jj) __stcg(cost + 7ull * p + jj - 1, dn[jj]);
		for(int k = 0; k < 8; ++k) choice[8ull * p + k] = ch[k];
		p = __ldcg(parent_int + p);
	}
}

__device__ __forceinline__ void ref_box(uint32_t ref, const WideSrc &W, float4 &lo, float4 &hi)
{
	if(ref & GBRT_LEAF_BIT)
	{
		const uint32_t prim = W.vals[ref & ~GBRT_LEAF_BIT];
		lo = W.box_lo[prim]; hi = W.box_hi[prim];
	}
	else { lo = W.node_lo[ref]; hi = W.node_hi[ref]; }
}

__device__ __forceinline__ float axis_of(const float4 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

__global__ void k_wide_init(float *meta, uint2 *tasks, uint32_t *counts)
{
	uint32_t *m = reinterpret_cast<uint32_t *>(meta);
	m[GBRT_META_WNODES] = 1u;
	m[GBRT_META_WPRIMS] = 0u;
	m[GBRT_META_WDEPTH] = 0u;
	tasks[0] = make_uint2(0u, 0u);    // binary root -> wide node 0
	counts[0] = 1u;
}

// One thread per wide node of this level: task = (binary node, wide index).
__global__ void __launch_bounds__(128) k_wide_level(int level, const uint2 *__restrict__ tin, uint32_t *counts, uint2 *__restrict__ tout,
                                                    WideSrc W, float *meta, uint4 *__restrict__ wnodes, float4 *__restrict__ wtris,
                                                    uint32_t *__restrict__ wids)
{
	const uint32_t n_in = counts[level];
	if(n_in == 0) return;
	uint32_t *m = reinterpret_cast<uint32_t *>(meta);
	if(blockIdx.x == 0 && threadIdx.x == 0) atomicMax(m + GBRT_META_WDEPTH, static_cast<uint32_t>(level + 1));
	const float pad = scene_pad(meta);
	for(uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_in; t += gridDim.x * blockDim.x)
	{
		const uint2 task = tin[t];
		uint32_t c[8];
		float4 lo[8], hi[8];
		int n = 2;
		{
			const uint2 cc = W.child[task.x];
			c[0] = cc.x; c[1] = cc.y;
			ref_box(c[0], W, lo[0], hi[0]);
			ref_box(c[1], W, lo[1], hi[1]);
		}
		if(W.choice)
		{
			// the children the SAH collapse chose: forests of (node, at most j roots)
			uint32_t st_ref[16], st_j[16];
			int sp = 0;
			const uint32_t k8 = W.choice[8ull * task.x];
			st_ref[sp] = c[1]; st_j[sp++] = 8u - k8;
			st_ref[sp] = c[0]; st_j[sp++] = k8;
			n = 0;
			bool bad = false;
			// at most 8 children and 7 splits, each entry stepping down j at most 6 times
			for(int it = 0; sp > 0 && it < 256; ++it)
			{
				const uint32_t r = st_ref[--sp], jj = st_j[sp];
				uint32_t k = 0;
				if(!(r & GBRT_LEAF_BIT) && jj >= 2u && jj <= 7u) k = W.choice[8ull * r + jj - 1];
				if((r & GBRT_LEAF_BIT) || jj <= 1u || jj > 7u) k = 0xFFu;    // one child
				if(k == 0xFFu)
				{
					if(n >= 8) { bad = true; break; }
					c[n] = r;
					ref_box(r, W, lo[n], hi[n]);
					++n;
				}
				else if(k == 0u)
				{
					st_ref[sp] = r; st_j[sp++] = jj - 1u;
				}
				else
				{
					if(sp + 2 > 16 || k >= jj) { bad = true; break; }
					const uint2 rc = W.child[r];
					st_ref[sp] = rc.y; st_j[sp++] = jj - k;
					st_ref[sp] = rc.x; st_j[sp++] = k;
				}
			}
			if(bad || sp > 0 || n < 2)
			{
				raise_err(meta, kErrWide);
				continue;
			}
		}
		while(!W.choice && n < 8)
		{
			int best = -1;
			float ba = -1.f;
			for(int k = 0; k < n; ++k)
				if(!wide_leaf(c[k], W))
				{
					const float a = half_area(lo[k], hi[k]);
					if(a > ba) { ba = a; best = k; }
				}
			if(best < 0) break;
			const uint2 rc = W.child[c[best]];
			c[best] = rc.x; ref_box(rc.x, W, lo[best], hi[best]);
			c[n] = rc.y; ref_box(rc.y, W, lo[n], hi[n]);
			++n;
		}
		// grown child boxes (as the binary nodes) and the node's grid
		float org[3], top[3];
		for(int a = 0; a < 3; ++a) { org[a] = FLT_MAX; top[a] = -FLT_MAX; }
		for(int k = 0; k < n; ++k)
		{
			lo[k] = make_float4(grow_down(lo[k].x, pad), grow_down(lo[k].y, pad), grow_down(lo[k].z, pad), 0.f);
			hi[k] = make_float4(grow_up(hi[k].x, pad), grow_up(hi[k].y, pad), grow_up(hi[k].z, pad), 0.f);
			for(int a = 0; a < 3; ++a) { org[a] = fminf(org[a], axis_of(lo[k], a)); top[a] = fmaxf(top[a], axis_of(hi[k], a)); }
		}
		int eb[3];
		double scale[3];
		for(int a = 0; a < 3; ++a)
		{
			const double ext = static_cast<double>(top[a]) - static_cast<double>(org[a]);
			int e = -126;
			if(ext > 0.0) { int x; frexp(ext / 255.0, &x); e = x; }
			e = max(-126, min(127, e));
			while(e < 127 && 255.0 * ldexp(1.0, e) < ext) ++e;
			eb[a] = e + 127;
			scale[a] = ldexp(1.0, e);
		}
		// slots by octant: child nearest along octant s's diagonal goes to slot
		// s; up to 4 children use slots 0-3 only (ordered by the x / y signs),
		// so the traversal can skip the empty upper half of the node
		const int n_slots = n <= 4 ? 4 : 8;
		float cost[8][8];
		for(int k = 0; k < n; ++k)
		{
			float d[3];
			for(int a = 0; a < 3; ++a)
				d[a] = 0.5f * (axis_of(lo[k], a) + axis_of(hi[k], a)) - 0.5f * (org[a] + top[a]);
			for(int sl = 0; sl < 8; ++sl)
				cost[k][sl] = ((sl & 1) ? -d[0] : d[0]) + ((sl & 2) ? -d[1] : d[1]) + ((sl & 4) ? -d[2] : d[2]);
		}
		int in_slot[8];
		for(int sl = 0; sl < 8; ++sl) in_slot[sl] = -1;
		uint32_t placed = 0;
		for(int it = 0; it < n; ++it)
		{
			float bc = FLT_MAX;
			int bk = -1, bs = -1;
			for(int k = 0; k < n; ++k)
			{
				if((placed >> k) & 1u) continue;
				for(int sl = 0; sl < n_slots; ++sl)
					if(in_slot[sl] < 0 && (bk < 0 || cost[k][sl] < bc)) { bc = cost[k][sl]; bk = k; bs = sl; }
			}
			in_slot[bs] = bk;
			placed |= 1u << bk;
		}
		uint32_t imask = 0, n_internal = 0, n_leaf_prims = 0;
		for(int sl = 0; sl < 8; ++sl)
		{
			const int k = in_slot[sl];
			if(k < 0) continue;
			if(wide_leaf(c[k], W)) n_leaf_prims += ref_count(c[k], W.node_hi);
			else { imask |= 1u << sl; ++n_internal; }
		}
		const uint32_t child_base = n_internal ? atomicAdd(m + GBRT_META_WNODES, n_internal) : 0u;
		const uint32_t prim_base = n_leaf_prims ? atomicAdd(m + GBRT_META_WPRIMS, n_leaf_prims) : 0u;
		if(child_base + n_internal > W.n_node_cap || prim_base + n_leaf_prims > W.n_prims || task.y >= W.n_node_cap)
		{
			raise_err(meta, kErrWide);
			continue;
		}
		// empty slots: inverted boxes (lo 255, hi 0), which no ray enters
		uint32_t meta_w[2] = {0u, 0u}, q[6][2] = {};
		uint32_t off = 0;
		for(int sl = 0; sl < 8; ++sl)
		{
			const int k = in_slot[sl];
			if(k < 0)
			{
				for(int a = 0; a < 3; ++a) q[a][sl >> 2] |= 0xFFu << (8 * (sl & 3));
				continue;
			}
			uint32_t mb;
			if((imask >> sl) & 1u)
			{
				mb = 0x20u | (24u + static_cast<uint32_t>(sl));
				const uint32_t idx = child_base + __popc(imask & ((1u << sl) - 1u));
				const uint32_t at = atomicAdd(counts + level + 1, 1u);
				if(at < W.n_node_cap) tout[at] = make_uint2(c[k], idx);
				else raise_err(meta, kErrWide);
			}
			else
			{
				uint32_t cnt = ref_count(c[k], W.node_hi);
				if(cnt > kWideLeafMax) { raise_err(meta, kErrWide); cnt = 0; }
				uint32_t first = (c[k] & GBRT_LEAF_BIT) ? W.pos_leaf[c[k] & ~GBRT_LEAF_BIT] : W.first_int[c[k]];
				if(first + cnt > W.n_prims) { raise_err(meta, kErrWide); first = 0; cnt = 0; }
				mb = (((1u << cnt) - 1u) << 5) | off;
				for(uint32_t i = 0; i < cnt; ++i)
				{
					const uint64_t dst = prim_base + off + i, src = first + i;
					wtris[3 * dst] = W.tris[3 * src];
					wtris[3 * dst + 1] = W.tris[3 * src + 1];
					wtris[3 * dst + 2] = W.tris[3 * src + 2];
					wids[dst] = W.ids[src];
				}
				off += cnt;
			}
			meta_w[sl >> 2] |= mb << (8 * (sl & 3));
			// outward-rounded 8-bit planes: org + q 2^e <= lo and >= hi, exactly (double)
			for(int a = 0; a < 3; ++a)
			{
				const double o = org[a], sc = scale[a];
				const double l = axis_of(lo[k], a), h = axis_of(hi[k], a);
				double ql = floor((l - o) / sc);
				while(ql > 0.0 && o + ql * sc > l) ql -= 1.0;
				ql = fmax(ql, 0.0);
				double qh = ceil((h - o) / sc);
				while(qh < 255.0 && o + qh * sc < h) qh += 1.0;
				qh = fmin(qh, 255.0);
				q[a][sl >> 2] |= static_cast<uint32_t>(ql) << (8 * (sl & 3));
				q[3 + a][sl >> 2] |= static_cast<uint32_t>(qh) << (8 * (sl & 3));
			}
		}
		uint4 *o = wnodes + 5ull * task.y;
		o[0] = make_uint4(__float_as_uint(org[0]), __float_as_uint(org[1]), __float_as_uint(org[2]),
		                  static_cast<uint32_t>(eb[0]) | (static_cast<uint32_t>(eb[1]) << 8) | (static_cast<uint32_t>(eb[2]) << 16) | (imask << 24));
		o[1] = make_uint4(child_base, prim_base, meta_w[0], meta_w[1]);
		o[2] = make_uint4(q[0][0], q[0][1], q[1][0], q[1][1]);
		o[3] = make_uint4(q[2][0], q[2][1], q[3][0], q[3][1]);
		o[4] = make_uint4(q[4][0], q[4][1], q[5][0], q[5][1]);
	}
}

// One primitive: a root whose slot 0 is a one-primitive leaf.
__global__ void k_wide_single(const float4 *__restrict__ box_lo, const float4 *__restrict__ box_hi, float *meta, const float4 *__restrict__ tris,
                              const uint32_t *__restrict__ ids, uint4 *wnodes, float4 *wtris, uint32_t *wids)
{
	const float pad = scene_pad(meta);
	const float4 l = box_lo[0], h = box_hi[0];
	const float lo[3] = {grow_down(l.x, pad), grow_down(l.y, pad), grow_down(l.z, pad)};
	const float hi[3] = {grow_up(h.x, pad), grow_up(h.y, pad), grow_up(h.z, pad)};
	uint32_t ebits = 0, qh[3];
	for(int a = 0; a < 3; ++a)
	{
		const double ext = static_cast<double>(hi[a]) - static_cast<double>(lo[a]);
		int e = -126;
		if(ext > 0.0) { int x; frexp(ext / 255.0, &x); e = x; }
		e = max(-126, min(127, e));
		while(e < 127 && 255.0 * ldexp(1.0, e) < ext) ++e;
		const double sc = ldexp(1.0, e);
		double q = ceil(ext / sc);
		while(q < 255.0 && lo[a] + q * sc < hi[a]) q += 1.0;
		qh[a] = static_cast<uint32_t>(fmin(q, 255.0));
		ebits |= static_cast<uint32_t>(e + 127) << (8 * a);
	}
	wnodes[0] = make_uint4(__float_as_uint(lo[0]), __float_as_uint(lo[1]), __float_as_uint(lo[2]), ebits);
	wnodes[1] = make_uint4(0u, 0u, (1u << 5) | 0u, 0u);
	wnodes[2] = make_uint4(0xFFFFFF00u, 0xFFFFFFFFu, 0xFFFFFF00u, 0xFFFFFFFFu);
	wnodes[3] = make_uint4(0xFFFFFF00u, 0xFFFFFFFFu, qh[0], 0u);
	wnodes[4] = make_uint4(qh[1], 0u, qh[2], 0u);
	wtris[0] = tris[0]; wtris[1] = tris[1]; wtris[2] = tris[2];
	wids[0] = ids[0];
	uint32_t *m = reinterpret_cast<uint32_t *>(meta);
	m[GBRT_META_WNODES] = 1u; m[GBRT_META_WPRIMS] = 1u; m[GBRT_META_WDEPTH] = 1u;
}

// Wide levels left unprocessed (deeper than GBRT_WIDE_MAX_LEVELS): flag.
__global__ void k_wide_check(const uint32_t *counts, float *meta)
{
	if(counts[kWideLevels] != 0u) atomicOr(reinterpret_cast<uint32_t *>(meta) + GBRT_META_ERR, 2u);
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

struct Scratch {
	cudaStream_t s;
	void *p = nullptr;
	explicit Scratch(cudaStream_t st) : s(st) { }
	~Scratch() { if(p) cudaFreeAsync(p, s); }
};

// Temporaries of the binary build.  After the sort the key buffers and the
// unused value buffer are free again: the leaf order reuses them.
struct BinaryBufs {
	float4 *blo, *bhi;
	uint32_t *k0, *k1, *v0, *v1, *hist;
	uint2 *child, *range;
	uint32_t *pint, *pleaf;
	float4 *nlo, *nhi;
	uint32_t *flags;
	uint8_t *coll;
	// set by build_binary
	uint32_t *vals = nullptr;        // primitive of each binary leaf (Morton order)
	uint32_t *pos_leaf = nullptr;    // slot of each binary leaf
	uint32_t *first_int = nullptr;   // first slot under each internal node
	uint32_t *vals_dfs = nullptr;    // primitive of each slot
};

// Treelet passes (gamma thresholds).  Measured on a GB300 with one-triangle
// leaves and the SAH wide collapse (1M soup / 2M coherent sphere): passes
// {7, 28} build in 9.3 / 16.1 ms, {7, 14, 28} in 11.8 / 20.8 ms, four or five
// passes in 13-14 / 23-25 ms, every schedule tracing within 0.1 % of the
// others with identical hits.
constexpr uint32_t kTreeletGamma[] = {7u, 28u};

// Morton codes through the emitted binary nodes and primitive records
// (nf >= 2; k_setup and k_finalize have run).
cudaError_t build_binary(BinaryBufs &B, const float *verts, const uint32_t *faces, uint32_t nf, const gbrt_build_params &p,
                         float *meta, float4 *nodes, float4 *tris, uint32_t *ids, cudaStream_t s)
{
	cudaError_t e;
	const uint32_t n_int = nf - 1;
	const uint32_t nblk = blocks_for(nf, kSortTile);
	k_morton<<<blocks_for(nf, 256), 256, 0, s>>>(B.blo, B.bhi, nf, meta, B.k0, B.v0);
	uint32_t *kin = B.k0, *kout = B.k1, *vin = B.v0, *vout = B.v1;
	for(int shift = 0; shift < 30; shift += 8)
	{
		k_hist<<<nblk, kSortThreads, 0, s>>>(kin, nf, shift, B.hist, nblk);
		const uint32_t hw = 256u * nblk, tiles = scan_tiles(hw);
		k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(B.hist, hw, B.hist + hw);
		k_scan_totals<<<1, kScanThreads, 0, s>>>(B.hist + hw, tiles);
		k_scan_add<<<tiles, kScanThreads, 0, s>>>(B.hist, hw, B.hist + hw);
		k_scatter<<<nblk, kSortThreads, 0, s>>>(kin, vin, nf, shift, B.hist, nblk, kout, vout);
		std::swap(kin, kout); std::swap(vin, vout);
	}
	if((e = cudaMemsetAsync(B.pint, 0xFF, 4ull * n_int, s)) != cudaSuccess) return e;
	if((e = cudaMemsetAsync(B.flags, 0, 4ull * n_int, s)) != cudaSuccess) return e;
	k_karras<<<blocks_for(n_int, 256), 256, 0, s>>>(kin, static_cast<int>(nf), B.child, B.range, B.pint, B.pleaf);
	k_refit<<<blocks_for(nf, 256), 256, 0, s>>>(vin, static_cast<int>(nf), B.blo, B.bhi, B.child, B.pint, B.pleaf, B.nlo, B.nhi, B.flags,
	                                            B.coll, p.max_leaf_size, p.traversal_cost, p.intersect_cost, meta);
	if(!(p.flags & GBRT_BUILD_NO_TREELETS))
	{
		for(uint32_t gamma : kTreeletGamma)
		{
			if((e = cudaMemsetAsync(B.flags, 0, 4ull * n_int, s)) != cudaSuccess) return e;
			k_treelet<<<blocks_for(nf, kTreeletThreads), kTreeletThreads, 0, s>>>(static_cast<int>(nf), vin, B.blo, B.bhi, B.child, B.pint, B.pleaf, B.nlo, B.nhi,
			                                              B.flags, gamma, p.max_leaf_size, p.traversal_cost, p.intersect_cost, meta);
		}
		if((e = cudaMemsetAsync(B.flags, 0, 4ull * n_int, s)) != cudaSuccess) return e;
		k_refit<<<blocks_for(nf, 256), 256, 0, s>>>(vin, static_cast<int>(nf), B.blo, B.bhi, B.child, B.pint, B.pleaf, B.nlo, B.nhi, B.flags,
		                                            B.coll, p.max_leaf_size, p.traversal_cost, p.intersect_cost, meta);
	}
	B.vals = vin;
	B.pos_leaf = kin;
	B.first_int = kout;
	B.vals_dfs = vout;
	k_order_leaves<<<blocks_for(nf, 256), 256, 0, s>>>(static_cast<int>(nf), vin, B.child, B.pint, B.pleaf, B.nhi, B.pos_leaf, B.vals_dfs, meta);
	k_order_nodes<<<blocks_for(n_int, 256), 256, 0, s>>>(static_cast<int>(n_int), B.child, B.pint, B.nhi, B.first_int, meta);
	k_emit_nodes<<<blocks_for(n_int, 256), 256, 0, s>>>(static_cast<int>(n_int), vin, B.blo, B.bhi, B.child, B.pos_leaf, B.first_int,
	                                                     B.nlo, B.nhi, B.coll, meta, nodes);
	k_emit_prims<<<blocks_for(nf, 256), 256, 0, s>>>(verts, faces, B.vals_dfs, nf, meta, tris, ids);
	return cudaGetLastError();
}

constexpr int kWideLevelsPerCheck = 12;

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
	if(!(p.intersect_cost > 0.f)) p.intersect_cost = kDefaultIntersectCost;

	gbrt_bvh *b = new gbrt_bvh();
	b->params = p;
	b->n_prims = nf;
	GBRT_CK(cudaGetDevice(&b->device));
	const uint32_t n_int = nf > 1 ? nf - 1 : 1;
	b->n_node_slots = n_int;
	auto fail = [&](int code) { gbrt_bvh_destroy(b); return code; };
	cudaError_t e;
	const size_t node_bytes = 64ull * n_int, tri_bytes = 48ull * (nf ? nf : 1), id_bytes = 4ull * (nf ? nf : 1);
	const size_t wnode_bytes = 80ull * n_int;
	if((e = cudaMalloc(&b->nodes, node_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->tris, tri_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->ids, id_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->meta, GBRT_META_WORDS * sizeof(float))) != cudaSuccess ||
	   (e = cudaMalloc(&b->wnodes, wnode_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->wtris, tri_bytes)) != cudaSuccess ||
	   (e = cudaMalloc(&b->wids, id_bytes)) != cudaSuccess)
		return fail(gbrt_set_error(GBRT_ERR_OOM, "gbrt_bvh_build: device allocation failed: %s", cudaGetErrorString(e)));
	b->bytes = node_bytes + 2 * (tri_bytes + id_bytes) + wnode_bytes + GBRT_META_WORDS * sizeof(float);

	k_init_meta<<<1, 32, 0, s>>>(b->meta);
	if(nf == 0)
	{
		k_finalize<<<1, 32, 0, s>>>(b->meta, 0);
		if((e = cudaMemsetAsync(b->nodes, 0, node_bytes, s)) != cudaSuccess || (e = cudaMemsetAsync(b->wnodes, 0, wnode_bytes, s)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "memset: %s", cudaGetErrorString(e)));
		if((e = cudaGetLastError()) != cudaSuccess) return fail(gbrt_set_error(GBRT_ERR_CUDA, "build launch: %s", cudaGetErrorString(e)));
		*out = b;
		return GBRT_OK;
	}

	// scratch carve-up (one stream-ordered allocation)
	const uint32_t nblk = blocks_for(nf, kSortTile);
	const size_t hist_words = 256ull * nblk + scan_tiles(256u * nblk);   // digit counts + scan tile sums
	size_t off = 0;
	auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
	const size_t o_blo = carve(16ull * nf), o_bhi = carve(16ull * nf);
	const size_t o_k0 = carve(4ull * nf), o_k1 = carve(4ull * nf), o_v0 = carve(4ull * nf), o_v1 = carve(4ull * nf);
	const size_t o_hist = carve(4 * hist_words);
	const size_t o_child = carve(8ull * n_int), o_range = carve(8ull * n_int);
	const size_t o_pint = carve(4ull * n_int), o_pleaf = carve(4ull * nf);
	const size_t o_nlo = carve(16ull * n_int), o_nhi = carve(16ull * n_int);
	const size_t o_flags = carve(4ull * n_int), o_coll = carve(n_int);
	const size_t o_task0 = carve(8ull * n_int), o_task1 = carve(8ull * n_int), o_counts = carve(4ull * (GBRT_WIDE_MAX_LEVELS + 1));
	const bool sah_wide = !(p.flags & GBRT_BUILD_GREEDY_WIDE);
	const size_t o_wcost = sah_wide ? carve(28ull * n_int) : 0, o_wchoice = sah_wide ? carve(8ull * n_int) : 0;
	Scratch sc(s);
	if((e = cudaMallocAsync(&sc.p, off, s)) != cudaSuccess)
		return fail(gbrt_set_error(GBRT_ERR_OOM, "gbrt_bvh_build: scratch allocation of %zu bytes failed: %s", off, cudaGetErrorString(e)));
	char *base = static_cast<char *>(sc.p);
	BinaryBufs B;
	B.blo = reinterpret_cast<float4 *>(base + o_blo); B.bhi = reinterpret_cast<float4 *>(base + o_bhi);
	B.k0 = reinterpret_cast<uint32_t *>(base + o_k0); B.k1 = reinterpret_cast<uint32_t *>(base + o_k1);
	B.v0 = reinterpret_cast<uint32_t *>(base + o_v0); B.v1 = reinterpret_cast<uint32_t *>(base + o_v1);
	B.hist = reinterpret_cast<uint32_t *>(base + o_hist);
	B.child = reinterpret_cast<uint2 *>(base + o_child); B.range = reinterpret_cast<uint2 *>(base + o_range);
	B.pint = reinterpret_cast<uint32_t *>(base + o_pint); B.pleaf = reinterpret_cast<uint32_t *>(base + o_pleaf);
	B.nlo = reinterpret_cast<float4 *>(base + o_nlo); B.nhi = reinterpret_cast<float4 *>(base + o_nhi);
	B.flags = reinterpret_cast<uint32_t *>(base + o_flags);
	B.coll = reinterpret_cast<uint8_t *>(base + o_coll);
	uint2 *task[2] = {reinterpret_cast<uint2 *>(base + o_task0), reinterpret_cast<uint2 *>(base + o_task1)};
	uint32_t *counts = reinterpret_cast<uint32_t *>(base + o_counts);

	k_setup<<<blocks_for(nf, 256), 256, 0, s>>>(verts, nv, faces, nf, B.blo, B.bhi, b->meta);
	k_finalize<<<1, 32, 0, s>>>(b->meta, nf);
	if(nf == 1)
	{
		k_emit_single<<<1, 1, 0, s>>>(B.blo, B.bhi, b->meta, b->nodes);
		k_emit_prims<<<1, 32, 0, s>>>(verts, faces, nullptr, 1, b->meta, b->tris, b->ids);
		k_wide_single<<<1, 1, 0, s>>>(B.blo, B.bhi, b->meta, b->tris, b->ids, b->wnodes, b->wtris, b->wids);
	}
	else
	{
		if((e = build_binary(B, verts, faces, nf, p, b->meta, b->nodes, b->tris, b->ids, s)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "build launch: %s", cudaGetErrorString(e)));
		// wide levels, checked every few levels for remaining work
		if((e = cudaMemsetAsync(counts, 0, 4ull * (GBRT_WIDE_MAX_LEVELS + 1), s)) != cudaSuccess)
			return fail(gbrt_set_error(GBRT_ERR_CUDA, "memset: %s", cudaGetErrorString(e)));
		k_wide_init<<<1, 1, 0, s>>>(b->meta, task[0], counts);
		uint8_t *wchoice = nullptr;
		if(sah_wide)
		{
			float *wcost = reinterpret_cast<float *>(base + o_wcost);
			wchoice = reinterpret_cast<uint8_t *>(base + o_wchoice);
			if((e = cudaMemsetAsync(B.flags, 0, 4ull * n_int, s)) != cudaSuccess)
				return fail(gbrt_set_error(GBRT_ERR_CUDA, "memset: %s", cudaGetErrorString(e)));
			k_wide_cost<<<blocks_for(nf, 256), 256, 0, s>>>(B.vals, static_cast<int>(nf), B.blo, B.bhi, B.child, B.pint, B.pleaf, B.nlo, B.nhi,
			                                               B.flags, wcost, wchoice, p.traversal_cost, p.intersect_cost, b->meta);
		}
		WideSrc W{B.child, B.vals, B.blo, B.bhi, B.nlo, B.nhi, B.coll, B.pos_leaf, B.first_int, b->tris, b->ids, n_int, nf, wchoice};
		int n_sm = 0;
		GBRT_CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device));
		const unsigned wgrid = std::max(1u, std::min(blocks_for(n_int, 128), static_cast<unsigned>(n_sm) * 8u));
		for(int L = 0; L < GBRT_WIDE_MAX_LEVELS; ++L)
		{
			k_wide_level<<<wgrid, 128, 0, s>>>(L, task[L & 1], counts, task[(L + 1) & 1], W, b->meta, b->wnodes, b->wtris, b->wids);
			if((L + 1) % kWideLevelsPerCheck == 0 && L + 1 < GBRT_WIDE_MAX_LEVELS)
			{
				uint32_t left = 0;
				if((e = cudaMemcpyAsync(&left, counts + L + 1, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
				   (e = cudaStreamSynchronize(s)) != cudaSuccess)
					return fail(gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build: %s", cudaGetErrorString(e)));
				if(left == 0) break;
			}
		}
		k_wide_check<<<1, 1, 0, s>>>(counts, b->meta);
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
	L.hist = o; o += round256(4 * (256 * nblk + scan_tiles(static_cast<uint32_t>(256 * nblk))));
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

// Device address of g_static_scratch in the current device's context (host
// code must not use the symbol itself as a pointer).  Looked up on every call,
// not cached: after cudaDeviceReset, or in another context on the same
// device, the module is loaded again at a new address.  Once the module is
// loaded the lookup allocates nothing.
int static_scratch_address(unsigned char **out)
{
	void *p = nullptr;
	const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
	if(e != cudaSuccess || !p)
		return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
	*out = static_cast<unsigned char *>(p);
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
	if(!(p.intersect_cost > 0.f)) p.intersect_cost = kDefaultIntersectCost;
	unsigned char *base = nullptr;
	if(int rc = static_scratch_address(&base)) return rc;

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
		BinaryBufs B;
		B.blo = reinterpret_cast<float4 *>(base + L.blo); B.bhi = reinterpret_cast<float4 *>(base + L.bhi);
		B.k0 = reinterpret_cast<uint32_t *>(base + L.k0); B.k1 = reinterpret_cast<uint32_t *>(base + L.k1);
		B.v0 = reinterpret_cast<uint32_t *>(base + L.v0); B.v1 = reinterpret_cast<uint32_t *>(base + L.v1);
		B.hist = reinterpret_cast<uint32_t *>(base + L.hist);
		B.child = reinterpret_cast<uint2 *>(base + L.child); B.range = reinterpret_cast<uint2 *>(base + L.range);
		B.pint = reinterpret_cast<uint32_t *>(base + L.pint); B.pleaf = reinterpret_cast<uint32_t *>(base + L.pleaf);
		B.nlo = reinterpret_cast<float4 *>(base + L.nlo); B.nhi = reinterpret_cast<float4 *>(base + L.nhi);
		B.flags = reinterpret_cast<uint32_t *>(base + L.flags);
		B.coll = reinterpret_cast<uint8_t *>(base + L.coll);
		float4 *tris = static_cast<float4 *>(prims_dev);
		k_setup<<<blocks_for(nf, 256), 256, 0, s>>>(verts, nv, faces, nf, B.blo, B.bhi, meta);
		k_finalize<<<1, 32, 0, s>>>(meta, nf);
		if(nf == 1)
		{
			k_emit_single<<<1, 1, 0, s>>>(B.blo, B.bhi, meta, nodes);
			k_emit_prims<<<1, 32, 0, s>>>(verts, faces, nullptr, 1, meta, tris, ids_dev);
		}
		else
		{
			// the array keeps the previous call's contents: build_binary resets
			// parents and arrival counters before use
			GBRT_CK(build_binary(B, verts, faces, nf, p, meta, nodes, tris, ids_dev, s));
		}
	}
	GBRT_CK(cudaGetLastError());
	float m[GBRT_META_WORDS];
	GBRT_CK(cudaMemcpyAsync(m, meta, sizeof(m), cudaMemcpyDeviceToHost, s));
	GBRT_CK(cudaStreamSynchronize(s));
	uint32_t err;
	std::memcpy(&err, &m[GBRT_META_ERR], 4);
	if(err & 1u) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_static: a face references a vertex index >= %u", nv);
	if(err) return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build_static: internal error: inconsistent hierarchy (flags 0x%x)", err);
	std::memcpy(bound_out, &m[GBRT_META_BOUND], 6 * sizeof(float));
	return GBRT_OK;
}
