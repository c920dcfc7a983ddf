// Closest-hit and any-hit batch kernels over the wide BVH; the per-ray
// query is gbrt::trace_init / trace_step in traverse_core.cuh.
//
// Each launch runs gbrt::trace_persistent: persistent warps fetching 32-ray
// chunks from a per-launch counter.
#include "traverse_core.cuh"

#include <atomic>

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
k_trace(gbrt::BvhView bv, const gbrt_ray *__restrict__ rays, uint32_t n, uint32_t *counter, gbrt_hit *__restrict__ hits,
        int32_t *__restrict__ occ)
{
	__shared__ uint2 stack[gbrt::kStackShared * kTraceThreads];
	gbrt::trace_persistent<kShadow>(
		bv, n, counter, stack + threadIdx.x, kTraceThreads,
		[&](uint32_t i, float r[8]) {
			const float4 a = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i);
			const float4 b = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i + 1);
			r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
			return true;
		},
		[&](uint32_t i, const gbrt::Hit &h) { store_result<kShadow>(i, h, hits, occ); });
}

template <bool kShadow>
int launch(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, int32_t *occ, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	// SM count and resident blocks per SM, queried once per kernel
	static std::atomic<int> cached_sm{0}, cached_bps{0};
	int n_sm = cached_sm.load(std::memory_order_relaxed), bps = cached_bps.load(std::memory_order_relaxed);
	if(n_sm == 0 || bps == 0)
	{
		int dev = 0;
		GBRT_CK(cudaGetDevice(&dev));
		GBRT_CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
		GBRT_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<kShadow>, kTraceThreads, 0));
		if(bps < 1) bps = 1;
		cached_sm.store(n_sm, std::memory_order_relaxed);
		cached_bps.store(bps, std::memory_order_relaxed);
	}
	const uint64_t warps_needed = (n + gbrt::kTraceChunk - 1) / gbrt::kTraceChunk;
	const uint64_t warps_resident = static_cast<uint64_t>(n_sm) * bps * (kTraceThreads / 32);
	const uint64_t warps = warps_needed < warps_resident ? warps_needed : warps_resident;
	const unsigned grid = static_cast<unsigned>((warps * 32 + kTraceThreads - 1) / kTraceThreads);
	// the chunk counter: one stream-ordered word per launch
	void *counter = nullptr;
	GBRT_CK(cudaMallocAsync(&counter, sizeof(uint32_t), s));
	cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
	if(e == cudaSuccess)
	{
		k_trace<kShadow><<<grid, kTraceThreads, 0, s>>>(gbrt::view_of(b), rays, n, static_cast<uint32_t *>(counter), hits, occ);
		e = cudaGetLastError();
	}
	const cudaError_t ef = cudaFreeAsync(counter, s);
	GBRT_CK(e);
	GBRT_CK(ef);
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
