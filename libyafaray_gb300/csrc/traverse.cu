// Closest-hit and any-hit batch kernels over the LBVH (one thread per ray);
// the per-ray query is gbrt::trace_ray in traverse_core.cuh.
#include "traverse_core.cuh"

namespace {

constexpr int kTraceThreads = 128;

template <bool kShadow>
__global__ void __launch_bounds__(kTraceThreads)
k_trace(gbrt::BvhView bv, const gbrt_ray *__restrict__ rays, uint32_t n, gbrt_hit *__restrict__ hits, int32_t *__restrict__ occ)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float4 a = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i);
	const float4 b = __ldg(reinterpret_cast<const float4 *>(rays) + 2ull * i + 1);
	const gbrt::Hit h = gbrt::trace_ray<kShadow>(bv, a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w);
	if(kShadow) occ[i] = h.prim;
	else reinterpret_cast<float4 *>(hits)[i] = make_float4(__int_as_float(h.prim), h.t, h.u, h.v);
}

} // namespace

int gbrt_launch_closest(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	const unsigned grid = (n + kTraceThreads - 1) / kTraceThreads;
	k_trace<false><<<grid, kTraceThreads, 0, s>>>(gbrt::view_of(b), rays, n, hits, nullptr);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

int gbrt_launch_shadow(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, int32_t *occ, cudaStream_t s)
{
	if(n == 0) return GBRT_OK;
	const unsigned grid = (n + kTraceThreads - 1) / kTraceThreads;
	k_trace<true><<<grid, kTraceThreads, 0, s>>>(gbrt::view_of(b), rays, n, nullptr, occ);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}
