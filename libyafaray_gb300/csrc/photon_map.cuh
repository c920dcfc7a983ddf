// Photon maps on the GPU: a hashed uniform grid over the stored photons and
// the two queries the photon integrators make of the reference's
// PointKdTree (include/photon/pkdtree.h:224-291):
//
//   knn_gather    PhotonMap::gather + PhotonGather (src/photon/photon.cc:25-64):
//                 the (at most) k photons nearest to p with d^2 < r^2; once k
//                 are held, r^2 shrinks to the k-th distance, and the final
//                 r^2 is returned like the reference's by-reference radius
//   find_nearest  PhotonMap::findNearest + NearestPhoton (photon.h:93-102):
//                 the nearest photon with dir . n > 0 within r^2
//
// Both return the same photon sets as the kd-tree walk (ties at exactly equal
// distances aside); only the order of the found photons differs, which the
// estimators sum over.  Grid: cells of edge >= the query radius, so a query
// visits the 27 cells around its own.  Cell coordinates and the bucket of a
// cell are the reference's HashGrid (src/photon/hashgrid.cc:59-75,
// include/photon/hashgrid.h:48-51): |int((p - box.a) x float(1 / cell))| per
// axis and (ix 73856093 ^ iy 19349663 ^ iz 83492791) mod the bucket count.
// Photons are sorted by bucket (counting sort); a bucket shared by two of
// the 27 cells is visited once.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbrt {

struct PhotonGrid {
	const float4 *pos;          // xyz; w unused
	const float4 *dir;          // stored direction (photon: towards where it came from; radiance point: normal)
	const float4 *col;          // rgb
	const uint32_t *start;      // [buckets + 1] bucket offsets into the sorted photons
	uint32_t buckets;           // HashGrid grid_size
	uint32_t n;
	float lo[3];                // HashGrid bounding_box.a
	float inv_cell;             // float(1 / cell_size), cell_size in double
};

// HashGrid::hash: int products wrap like the reference's, then mod grid_size.
__host__ __device__ __forceinline__ uint32_t grid_bucket(int ix, int iy, int iz, uint32_t buckets)
{
	const uint32_t h = (static_cast<uint32_t>(ix) * 73856093u) ^ (static_cast<uint32_t>(iy) * 19349663u) ^ (static_cast<uint32_t>(iz) * 83492791u);
	return h % buckets;
}

__host__ __device__ __forceinline__ void grid_cell(const PhotonGrid &g, const float p[3], int c[3])
{
	for(int a = 0; a < 3; ++a)
	{
		const int i = static_cast<int>((p[a] - g.lo[a]) * g.inv_cell);
		c[a] = i < 0 ? -i : i;
	}
}

// Visits every distinct bucket of the 27 cells around p: f(first, end).
template<typename F>
__device__ __forceinline__ void grid_visit(const PhotonGrid &g, const float p[3], F &&f)
{
	int c[3];
	grid_cell(g, p, c);
	uint32_t seen[27];
	int ns = 0;
	for(int dz = -1; dz <= 1; ++dz)
		for(int dy = -1; dy <= 1; ++dy)
			for(int dx = -1; dx <= 1; ++dx)
			{
				// photons lie inside the box, so their cells are >= 0 on every axis
				if(c[0] + dx < 0 || c[1] + dy < 0 || c[2] + dz < 0) continue;
				const uint32_t b = grid_bucket(c[0] + dx, c[1] + dy, c[2] + dz, g.buckets);
				bool dup = false;
				for(int i = 0; i < ns; ++i) dup |= seen[i] == b;
				if(dup) continue;
				seen[ns++] = b;
				f(__ldg(g.start + b), __ldg(g.start + b + 1));
			}
}

constexpr int kMaxGather = 64;

// Max-heap on d2 over the first m entries (std::make_heap / pop_heap /
// push_heap order is irrelevant to the result set).
__device__ __forceinline__ void heap_sift_down(uint32_t *idx, float *d2, int m, int i)
{
	while(true)
	{
		const int l = 2 * i + 1, r = l + 1;
		int big = i;
		if(l < m && d2[l] > d2[big]) big = l;
		if(r < m && d2[r] > d2[big]) big = r;
		if(big == i) return;
		const float td = d2[i]; d2[i] = d2[big]; d2[big] = td;
		const uint32_t ti = idx[i]; idx[i] = idx[big]; idx[big] = ti;
		i = big;
	}
}

__device__ __forceinline__ int knn_gather(const PhotonGrid &g, const float p[3], int k, float &r2, uint32_t *idx, float *d2)
{
	int found = 0;
	float max_d2 = r2;
	grid_visit(g, p, [&](uint32_t first, uint32_t end) {
		for(uint32_t j = first; j < end; ++j)
		{
			const float4 q = __ldg(g.pos + j);
			const float vx = q.x - p[0], vy = q.y - p[1], vz = q.z - p[2];
			const float d = vx * vx + vy * vy + vz * vz;
			if(!(d < max_d2)) continue;
			if(found < k)
			{
				idx[found] = j; d2[found] = d; ++found;
				if(found == k)
				{
					for(int i = k / 2 - 1; i >= 0; --i) heap_sift_down(idx, d2, k, i);
					max_d2 = d2[0];
				}
			}
			else
			{
				idx[0] = j; d2[0] = d;
				heap_sift_down(idx, d2, k, 0);
				max_d2 = d2[0];
			}
		}
	});
	r2 = max_d2;
	return found;
}

// Every photon with d^2 < r2: f(index).
template<typename F>
__device__ __forceinline__ void grid_range(const PhotonGrid &g, const float p[3], float r2, F &&f)
{
	grid_visit(g, p, [&](uint32_t first, uint32_t end) {
		for(uint32_t j = first; j < end; ++j)
		{
			const float4 q = __ldg(g.pos + j);
			const float vx = q.x - p[0], vy = q.y - p[1], vz = q.z - p[2];
			if(vx * vx + vy * vy + vz * vz < r2) f(j);
		}
	});
}

// Nearest photon with dir . n > 0 and d^2 < r2; -1 if none.
__device__ __forceinline__ int find_nearest(const PhotonGrid &g, const float p[3], const float n[3], float r2)
{
	int best = -1;
	float max_d2 = r2;
	grid_visit(g, p, [&](uint32_t first, uint32_t end) {
		for(uint32_t j = first; j < end; ++j)
		{
			const float4 q = __ldg(g.pos + j);
			const float vx = q.x - p[0], vy = q.y - p[1], vz = q.z - p[2];
			const float d = vx * vx + vy * vy + vz * vz;
			if(!(d < max_d2)) continue;
			const float4 w = __ldg(g.dir + j);
			if(w.x * n[0] + w.y * n[1] + w.z * n[2] > 0.f)
			{
				best = static_cast<int>(j);
				max_d2 = d;
			}
		}
	});
	return best;
}

}  // namespace gbrt
