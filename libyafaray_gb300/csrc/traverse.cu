// Closest-hit and any-hit batch kernels over the wide BVH; the per-ray
// query is gbrt::trace_init / trace_step in traverse_core.cuh.
//
// Persistent warps: the grid holds as many warps as fit on the GPU at once,
// each warp owns a contiguous share of the rays, and a lane whose query is
// answered takes the warp's next ray at the top of the following step (Aila
// & Laine, "Understanding the efficiency of ray traversal on GPUs", HPG
// 2009).  Lanes whose rays end early no longer idle until the slowest ray of
// their warp is done.
#include "traverse_core.cuh"

namespace {

constexpr int kTraceThreads = 128;

template <bool kShadow>
__device__ __forceinline__ void store_result(uint32_t i, const gbrt::Hit &h, gbrt_hit *hits, int32_t *occ)
{
	if(kShadow) occ[i] = h.prim;
	else reinterpret_cast<float4 *>(hits)[i] = make_float4(__int_as_float(h.prim), h.t, h.u, h.v);
}

template <bool kShadow>
__global__ void __launch_bounds__(kTraceThreads)
k_trace(gbrt::BvhView bv, const gbrt_ray *__restrict__ rays, uint32_t n, uint32_t per_warp, gbrt_hit *__restrict__ hits,
        int32_t *__restrict__ occ)
{
	__shared__ uint2 stack[gbrt::kStackShared * kTraceThreads];
	uint2 spill[gbrt::kTraceStack - gbrt::kStackShared];
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint64_t first = static_cast<uint64_t>(warp) * per_warp;
	uint32_t next = static_cast<uint32_t>(first < n ? first : n);
	const uint32_t end = static_cast<uint32_t>(first + per_warp < n ? first + per_warp : n);
	gbrt::TraceState S;
	bool active = false;
	uint32_t ray = 0;
	while(true)
	{
		// refill the idle lanes from the warp's share (next is warp-uniform)
		const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
		if(idle == 0xFFFFFFFFu && next >= end) break;
		if(idle && next < end)
		{
			const uint32_t mine = next + __popc(idle & ((1u << lane) - 1u));
			next = min(next + static_cast<uint32_t>(__popc(idle)), end);
			if(!active && mine < end)
			{
				ray = mine;
				const float4 a = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * ray);
				const float4 b = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * ray + 1);
				active = gbrt::trace_init<kShadow>(S, bv, a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w);
				if(!active) store_result<kShadow>(ray, gbrt::Hit{-1, 0.f, 0.f, 0.f}, hits, occ);
			}
		}
		if(active && gbrt::trace_step<kShadow>(S, bv, stack + threadIdx.x, kTraceThreads, spill))
		{
			store_result<kShadow>(ray, gbrt::trace_result(S), hits, occ);
			active = false;
		}
	}
}

template <bool kShadow>
int launch(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, int32_t *occ, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	static int blocks_per_sm[2] = {0, 0}, n_sm = 0;
	int &bps = blocks_per_sm[kShadow ? 1 : 0];
	if(!bps)
	{
		int dev = 0;
		GBRT_CK(cudaGetDevice(&dev));
		GBRT_CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
		GBRT_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<kShadow>, kTraceThreads, 0));
		if(bps < 1) bps = 1;
	}
	const uint64_t warps_needed = (n + 31u) / 32u;
	const uint64_t warps_resident = static_cast<uint64_t>(n_sm) * bps * (kTraceThreads / 32);
	const uint64_t warps = warps_needed < warps_resident ? warps_needed : warps_resident;
	const uint32_t per_warp = static_cast<uint32_t>((n + warps - 1) / warps);
	const unsigned grid = static_cast<unsigned>((warps * 32 + kTraceThreads - 1) / kTraceThreads);
	k_trace<kShadow><<<grid, kTraceThreads, 0, s>>>(gbrt::view_of(b), rays, n, per_warp, hits, occ);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

} // namespace

int gbrt_launch_closest(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, cudaStream_t s)
{
	return launch<false>(b, rays, n, hits, nullptr, s);
}

int gbrt_launch_shadow(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, int32_t *occ, cudaStream_t s)
{
	return launch<true>(b, rays, n, nullptr, occ, s);
}
