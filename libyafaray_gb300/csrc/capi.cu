// extern "C" entry points of libgbrt (declared in include/gbrt.h).
#include "gbrt_internal.cuh"

#include <cuda.h>

#include <cstring>
#include <mutex>
#include <vector>

namespace {
thread_local char g_err[512] = "";

struct DevBuf {
	void *p = nullptr;
	~DevBuf() { if(p) cudaFree(p); }
};
} // namespace

#include <algorithm>

int gbrt_set_error(int code, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
	return code;
}

namespace {
std::mutex g_stage_init_mu;
constexpr uint32_t kStageRays = 1u << 21;  // 2 Mi rays = 64 MiB per slot

// Whether [p, p + bytes) lies inside one page-locked host allocation the
// device can address (pinned memory under unified addressing): the pointer's
// attributes say host memory with a device mapping, and the driver's range
// of the allocation (cuPointerGetAttribute RANGE_START_ADDR / RANGE_SIZE)
// covers the whole span.  Anything else - pageable memory, a failed query -
// answers false.
bool mapped_host_range(const void *p, size_t bytes, void **dev)
{
	cudaPointerAttributes a{};
	if(cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
	if(a.type != cudaMemoryTypeHost || !a.devicePointer || a.devicePointer != p) return false;
	using GetAttr = CUresult (*)(void *, CUpointer_attribute, CUdeviceptr);
	static GetAttr get_attr = [] {
		void *fn = nullptr;
		cudaDriverEntryPointQueryResult q{};
		if(cudaGetDriverEntryPoint("cuPointerGetAttribute", &fn, cudaEnableDefault, &q) != cudaSuccess || q != cudaDriverEntryPointSuccess)
		{
			cudaGetLastError();
			return static_cast<GetAttr>(nullptr);
		}
		return reinterpret_cast<GetAttr>(fn);
	}();
	if(!get_attr) return false;
	CUdeviceptr start = 0;
	size_t size = 0;
	if(get_attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, reinterpret_cast<CUdeviceptr>(p)) != CUDA_SUCCESS ||
	   get_attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, reinterpret_cast<CUdeviceptr>(p)) != CUDA_SUCCESS)
		return false;
	const uintptr_t lo = static_cast<uintptr_t>(start), q = reinterpret_cast<uintptr_t>(p);
	if(q < lo || q - lo > size || bytes > size - (q - lo)) return false;
	*dev = a.devicePointer;
	return true;
}

// Whether host buffers take the direct path: rays 16-byte aligned, results
// 16-byte aligned (4 for occluder IDs), each inside one page-locked
// allocation the device maps.
bool direct_host_path(const void *rays, uint32_t n, const void *out, size_t out_rec, bool shadow, void **rays_dev, void **out_dev)
{
	const bool aligned = (reinterpret_cast<uintptr_t>(rays) & 15u) == 0 && (reinterpret_cast<uintptr_t>(out) & (shadow ? 3u : 15u)) == 0;
	return aligned && mapped_host_range(rays, sizeof(gbrt_ray) * static_cast<size_t>(n), rays_dev) &&
	       mapped_host_range(out, out_rec * static_cast<size_t>(n), out_dev);
}

// Host path.  Rays and results in page-locked host memory that the device
// maps are read and written by the traversal kernel itself, over the
// host-device link, in one launch (no staging copies).  Otherwise the
// pipelined path: chunk k's upload, trace and download run on stream k % 2,
// so the copies of one chunk overlap the traversal of the other (pageable
// buffers still work: the runtime stages them).
int stage_and_trace(gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, void *out, size_t out_rec, bool shadow)
{
	{
		std::lock_guard<std::mutex> g(g_stage_init_mu);
		if(!b->stage_mu) b->stage_mu = new std::mutex();
	}
	std::lock_guard<std::mutex> lock(*static_cast<std::mutex *>(b->stage_mu));
	int dev = -1;
	GBRT_CK(cudaGetDevice(&dev));
	if(dev != b->device) GBRT_CK(cudaSetDevice(b->device));
	for(int k = 0; k < 2; ++k)
	{
		if(!b->stage_stream[k]) GBRT_CK(cudaStreamCreateWithFlags(&b->stage_stream[k], cudaStreamNonBlocking));
		if(!b->stage_rays[k]) GBRT_CK(cudaMalloc(&b->stage_rays[k], sizeof(gbrt_ray) * kStageRays));
		if(!b->stage_out[k]) GBRT_CK(cudaMalloc(&b->stage_out[k], sizeof(gbrt_hit) * kStageRays));
	}
	// gbrt_bvh_build synchronised its stream, so the hierarchy is complete.
	int rc = GBRT_OK;
	void *rays_dev = nullptr, *out_dev = nullptr;
	// the kernel loads rays and stores hits as 16-byte vectors (4-byte occluder IDs)
	if(direct_host_path(rays, n, out, out_rec, shadow, &rays_dev, &out_dev))
	{
		cudaStream_t st = b->stage_stream[0];
		rc = shadow ? gbrt_launch_shadow(b, static_cast<const gbrt_ray *>(rays_dev), n, static_cast<int32_t *>(out_dev), st)
		            : gbrt_launch_closest(b, static_cast<const gbrt_ray *>(rays_dev), n, static_cast<gbrt_hit *>(out_dev), st);
		GBRT_CK(cudaStreamSynchronize(st));
		if(dev != b->device) cudaSetDevice(dev);
		return rc;
	}
	uint32_t chunk = 0;
	for(uint64_t off = 0; off < n; off += kStageRays, ++chunk)
	{
		const uint32_t m = static_cast<uint32_t>(std::min<uint64_t>(kStageRays, n - off));
		const int k = chunk & 1;
		cudaStream_t st = b->stage_stream[k];
		GBRT_CK(cudaMemcpyAsync(b->stage_rays[k], rays + off, sizeof(gbrt_ray) * m, cudaMemcpyHostToDevice, st));
		rc = shadow ? gbrt_launch_shadow(b, static_cast<gbrt_ray *>(b->stage_rays[k]), m, static_cast<int32_t *>(b->stage_out[k]), st)
		            : gbrt_launch_closest(b, static_cast<gbrt_ray *>(b->stage_rays[k]), m, static_cast<gbrt_hit *>(b->stage_out[k]), st);
		if(rc) break;
		GBRT_CK(cudaMemcpyAsync(static_cast<char *>(out) + off * out_rec, b->stage_out[k], out_rec * m, cudaMemcpyDeviceToHost, st));
	}
	for(int k = 0; k < 2; ++k) GBRT_CK(cudaStreamSynchronize(b->stage_stream[k]));
	if(dev != b->device) cudaSetDevice(dev);
	return rc;
}
} // namespace

extern "C" {

const char *gbrt_last_error(void) { return g_err; }

int gbrt_version(void) { return 1; }

int gbrt_device_count(int *count)
{
	if(!count) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_device_count: NULL");
	const cudaError_t e = cudaGetDeviceCount(count);
	if(e != cudaSuccess) { *count = 0; return gbrt_set_error(GBRT_ERR_NO_DEVICE, "cudaGetDeviceCount: %s", cudaGetErrorString(e)); }
	return GBRT_OK;
}

int gbrt_bvh_destroy(gbrt_bvh *b)
{
	if(!b) return GBRT_OK;
	int dev = -1;
	cudaGetDevice(&dev);
	if(dev != b->device) cudaSetDevice(b->device);
	for(int k = 0; k < 2; ++k)
	{
		if(b->stage_stream[k]) cudaStreamSynchronize(b->stage_stream[k]);
		if(b->stage_rays[k]) cudaFree(b->stage_rays[k]);
		if(b->stage_out[k]) cudaFree(b->stage_out[k]);
		if(b->stage_stream[k]) cudaStreamDestroy(b->stage_stream[k]);
	}
	delete static_cast<std::mutex *>(b->stage_mu);
	if(b->nodes) cudaFree(b->nodes);
	if(b->tris) cudaFree(b->tris);
	if(b->ids) cudaFree(b->ids);
	if(b->meta) cudaFree(b->meta);
	if(b->wnodes) cudaFree(b->wnodes);
	if(b->wtris) cudaFree(b->wtris);
	if(b->wids) cudaFree(b->wids);
	if(dev >= 0 && dev != b->device) cudaSetDevice(dev);
	delete b;
	return GBRT_OK;
}

int gbrt_bvh_build(const float *vertices_dev, uint32_t n_vertices, const uint32_t *faces_dev, uint32_t n_faces,
                   const gbrt_build_params *params, void *stream, gbrt_bvh **out)
{
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	int rc = gbrt_build_impl(vertices_dev, n_vertices, faces_dev, n_faces, params, s, out);
	if(rc != GBRT_OK) return rc;
	// One small read-back: the reference tree bound and the bad-index flag.
	float meta[GBRT_META_WORDS];
	cudaError_t e = cudaMemcpyAsync(meta, (*out)->meta, sizeof(meta), cudaMemcpyDeviceToHost, s);
	if(e == cudaSuccess) e = cudaStreamSynchronize(s);
	if(e != cudaSuccess)
	{
		gbrt_bvh_destroy(*out); *out = nullptr;
		return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build: %s", cudaGetErrorString(e));
	}
	uint32_t err;
	std::memcpy(&err, &meta[GBRT_META_ERR], 4);
	if(err & 1u)
	{
		gbrt_bvh_destroy(*out); *out = nullptr;
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build: a face references a vertex index >= %u", n_vertices);
	}
	if(err & 12u)
	{
		gbrt_bvh_destroy(*out); *out = nullptr;
		return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_bvh_build: internal error: inconsistent hierarchy (flags 0x%x)", err);
	}
	if(err & 2u)
	{
		gbrt_bvh_destroy(*out); *out = nullptr;
		return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_build: the wide hierarchy is deeper than %d levels", GBRT_WIDE_MAX_LEVELS);
	}
	uint32_t wn, wd;
	std::memcpy(&wn, &meta[GBRT_META_WNODES], 4);
	std::memcpy(&wd, &meta[GBRT_META_WDEPTH], 4);
	(*out)->n_wide_nodes = n_faces ? wn : 0u;
	(*out)->wide_depth = n_faces ? wd : 0u;
	std::memcpy((*out)->host_bound, &meta[GBRT_META_BOUND], 6 * sizeof(float));
	(*out)->host_bound_valid = true;
	return GBRT_OK;
}

int gbrt_bvh_build_host(const float *vertices, uint32_t n_vertices, const uint32_t *faces, uint32_t n_faces,
                        const gbrt_build_params *params, gbrt_bvh **out)
{
	if(!out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_host: out is NULL");
	*out = nullptr;
	if(n_faces > 0 && (!vertices || !faces)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_build_host: NULL input");
	DevBuf dv, df;
	const size_t vb = 12ull * (n_vertices ? n_vertices : 1), fb = 16ull * (n_faces ? n_faces : 1);
	GBRT_CK(cudaMalloc(&dv.p, vb));
	GBRT_CK(cudaMalloc(&df.p, fb));
	if(n_vertices) GBRT_CK(cudaMemcpy(dv.p, vertices, 12ull * n_vertices, cudaMemcpyHostToDevice));
	if(n_faces) GBRT_CK(cudaMemcpy(df.p, faces, 16ull * n_faces, cudaMemcpyHostToDevice));
	return gbrt_bvh_build(static_cast<const float *>(dv.p), n_vertices, static_cast<const uint32_t *>(df.p), n_faces, params, nullptr, out);
}

int gbrt_bvh_get_bound(const gbrt_bvh *b, float bound_out[6])
{
	if(!b || !bound_out) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_get_bound: NULL");
	std::memcpy(bound_out, b->host_bound, 6 * sizeof(float));
	return GBRT_OK;
}

int gbrt_bvh_get_info(const gbrt_bvh *b, gbrt_bvh_info *info)
{
	if(!b || !info) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_get_info: NULL");
	std::memset(info, 0, sizeof(*info));
	info->n_prims = b->n_prims;
	info->device_bytes = b->bytes;
	std::memcpy(info->bound, b->host_bound, sizeof(info->bound));
	if(b->n_prims == 0) return GBRT_OK;
	// Walk the node array on the host (diagnostics only).
	std::vector<float4> nodes(4ull * b->n_node_slots);
	GBRT_CK(cudaMemcpy(nodes.data(), b->nodes, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost));
	struct Item { uint32_t ref; uint32_t depth; };
	std::vector<Item> st;
	st.push_back({0u, 1u});
	double sah = 0.0;
	float4 rb = nodes[0];
	(void)rb;
	while(!st.empty())
	{
		const Item it = st.back(); st.pop_back();
		if(it.ref & GBRT_LEAF_BIT) { info->n_leaves++; if(it.depth > info->max_depth) info->max_depth = it.depth; continue; }
		info->n_nodes++;
		const float4 *nd = &nodes[4ull * it.ref];
		uint32_t r0, r1;
		std::memcpy(&r0, &nd[3].x, 4); std::memcpy(&r1, &nd[3].y, 4);
		for(int k = 0; k < 2; ++k)
		{
			const float lx = k ? nd[1].x : nd[0].x, hx = k ? nd[1].y : nd[0].y;
			const float ly = k ? nd[1].z : nd[0].z, hy = k ? nd[1].w : nd[0].w;
			const float lz = k ? nd[2].z : nd[2].x, hz = k ? nd[2].w : nd[2].y;
			const uint32_t r = k ? r1 : r0;
			if(hx < lx) continue;
			const double a = double(hx - lx) * (hy - ly) + double(hy - ly) * (hz - lz) + double(hz - lz) * (hx - lx);
			sah += (r & GBRT_LEAF_BIT) ? a * (((r >> 27) & 15u) + 1u) : a;
		}
		st.push_back({r0, it.depth + 1});
		if(b->n_prims > 1) st.push_back({r1, it.depth + 1});
	}
	const float *bd = b->host_bound;
	const double ra = double(bd[3] - bd[0]) * (bd[4] - bd[1]) + double(bd[4] - bd[1]) * (bd[5] - bd[2]) + double(bd[5] - bd[2]) * (bd[3] - bd[0]);
	info->sah_cost = ra > 0 ? static_cast<float>(sah / ra) : 0.f;
	return GBRT_OK;
}

int gbrt_bvh_export(const gbrt_bvh *b, void *nodes, size_t nodes_bytes, void *prims, size_t prims_bytes,
                    uint32_t *ids, size_t ids_bytes)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_export: NULL handle");
	const size_t nb = 64ull * b->n_node_slots, pb = 48ull * b->n_prims, ib = 4ull * b->n_prims;
	if((nodes && nodes_bytes < nb) || (prims && prims_bytes < pb) || (ids && ids_bytes < ib))
		return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_export: buffers too small (need %zu/%zu/%zu bytes)", nb, pb, ib);
	if(nodes) GBRT_CK(cudaMemcpy(nodes, b->nodes, nb, cudaMemcpyDeviceToHost));
	if(prims && pb) GBRT_CK(cudaMemcpy(prims, b->tris, pb, cudaMemcpyDeviceToHost));
	if(ids && ib) GBRT_CK(cudaMemcpy(ids, b->ids, ib, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_bvh_export_wide(const gbrt_bvh *b, uint32_t *n_nodes, uint32_t *depth, void *nodes, size_t nodes_bytes,
                         void *prims, size_t prims_bytes, uint32_t *ids, size_t ids_bytes)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_bvh_export_wide: NULL handle");
	const size_t nb = 80ull * b->n_wide_nodes, pb = 48ull * b->n_prims, ib = 4ull * b->n_prims;
	if((nodes && nodes_bytes < nb) || (prims && prims_bytes < pb) || (ids && ids_bytes < ib))
		return gbrt_set_error(GBRT_ERR_CAPACITY, "gbrt_bvh_export_wide: buffers too small (need %zu/%zu/%zu bytes)", nb, pb, ib);
	if(n_nodes) *n_nodes = b->n_wide_nodes;
	if(depth) *depth = b->wide_depth;
	if(nodes && nb) GBRT_CK(cudaMemcpy(nodes, b->wnodes, nb, cudaMemcpyDeviceToHost));
	if(prims && pb) GBRT_CK(cudaMemcpy(prims, b->wtris, pb, cudaMemcpyDeviceToHost));
	if(ids && ib) GBRT_CK(cudaMemcpy(ids, b->wids, ib, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_trace_closest(const gbrt_bvh *b, const gbrt_ray *rays_dev, uint32_t n, gbrt_hit *hits_dev, void *stream)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_closest: NULL handle");
	if(n && (!rays_dev || !hits_dev)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_closest: NULL buffer");
	return gbrt_launch_closest(b, rays_dev, n, hits_dev, static_cast<cudaStream_t>(stream));
}

int gbrt_trace_shadow(const gbrt_bvh *b, const gbrt_ray *rays_dev, uint32_t n, int32_t *occ_dev, void *stream)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_shadow: NULL handle");
	if(n && (!rays_dev || !occ_dev)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_shadow: NULL buffer");
	return gbrt_launch_shadow(b, rays_dev, n, occ_dev, static_cast<cudaStream_t>(stream));
}

int gbrt_trace_closest_host(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_closest_host: NULL handle");
	if(n == 0) return GBRT_OK;
	if(!rays || !hits) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_closest_host: NULL buffer");
	return stage_and_trace(const_cast<gbrt_bvh *>(b), rays, n, hits, sizeof(gbrt_hit), false);
}

int gbrt_host_path(const gbrt_ray *rays, uint32_t n, const void *out, int shadow, int *direct)
{
	if(!direct) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_host_path: NULL result");
	*direct = 0;
	if(n == 0 || !rays || !out) return GBRT_OK;
	void *rd = nullptr, *od = nullptr;
	*direct = direct_host_path(rays, n, out, shadow ? sizeof(int32_t) : sizeof(gbrt_hit), shadow != 0, &rd, &od) ? 1 : 0;
	return GBRT_OK;
}

int gbrt_trace_shadow_host(const gbrt_bvh *b, const gbrt_ray *rays, uint32_t n, int32_t *occ)
{
	if(!b) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_shadow_host: NULL handle");
	if(n == 0) return GBRT_OK;
	if(!rays || !occ) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_trace_shadow_host: NULL buffer");
	return stage_and_trace(const_cast<gbrt_bvh *>(b), rays, n, occ, sizeof(int32_t), true);
}

} // extern "C"
