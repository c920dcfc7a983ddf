// Internal definitions shared by the gbrt translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "gbrt.h"

// Leaf child reference: bit 31 set, bits 27..30 = count-1, bits 0..26 = first
// primitive slot.  Internal child reference: node index (bit 31 clear).
#define GBRT_LEAF_BIT 0x80000000u
#define GBRT_LEAF_MAX_SLOTS (1u << 27)
#define GBRT_LEAF_MAX_COUNT 16u
#define GBRT_QUAD_BIT 0x80000000u
// Levels of the 8-wide hierarchy the build accepts; also the traversal
// stack depth (a traversal pushes at most one entry per level).
#define GBRT_WIDE_MAX_LEVELS 96

__host__ __device__ inline uint32_t gbrt_leaf_ref(uint32_t first, uint32_t count)
{
	return GBRT_LEAF_BIT | ((count - 1u) << 27) | first;
}

// Device memory of a built hierarchy.
//   nodes : 4 float4 per internal node (both children's boxes + refs):
//           [0] c0.lo.x c0.hi.x c0.lo.y c0.hi.y
//           [1] c1.lo.x c1.hi.x c1.lo.y c1.hi.y
//           [2] c0.lo.z c0.hi.z c1.lo.z c1.hi.z
//           [3] ref0 ref1 (uint bits) 0 0
//   tris  : 3 float4 per primitive slot, leaf order:
//           [0] v0.xyz e3.x   [1] e1.xyz e3.y   [2] e2.xyz e3.z
//           (e_k = v_k - v0 in float, exactly as shape_polygon.h:130-131,155)
//   ids   : primitive ID per slot, GBRT_QUAD_BIT set for quads
//   meta  : float bound[6] (reference tree bound) + build scratch words
//
// The traversal kernels walk a second, 8-wide copy of the hierarchy built
// from the binary one (the binary layout stays as the export / no-allocation
// build format):
//   wnodes: 5 uint4 (80 bytes) per wide node
//           [0] origin xyz (float bits), exponent bytes ex | ey<<8 | ez<<16 | imask<<24
//           [1] child_base, prim_base, meta bytes of slots 0-3, slots 4-7
//           [2] qlo.x slots 0-7 (2 words), qlo.y slots 0-7
//           [3] qlo.z, qhi.x   [4] qhi.y, qhi.z   (8-bit quantised child boxes)
//       Child box plane = origin + q * 2^(e - 127); planes round outward.
//       meta byte: 0 empty; internal child 0x20 | (24 + slot), its node index
//       child_base + popc(imask below slot); leaf child (unary count << 5) |
//       offset, primitives prim_base + offset .. + count - 1 (count 1..3).
//       Children sit in slots by octant: the child nearest for rays whose
//       direction signs are octant o is in slot o; nodes of up to 4
//       children use slots 0-3 only (x / y signs), leaving slots 4-7 empty.
//   wtris, wids: primitive records and IDs in wide-leaf order.
struct gbrt_bvh {
	int device = 0;
	uint32_t n_prims = 0;
	uint32_t n_node_slots = 0;
	float4 *nodes = nullptr;
	float4 *tris = nullptr;
	uint32_t *ids = nullptr;
	float *meta = nullptr;
	uint4 *wnodes = nullptr;
	float4 *wtris = nullptr;
	uint32_t *wids = nullptr;
	uint32_t n_wide_nodes = 0;
	uint32_t wide_depth = 0;
	uint64_t bytes = 0;
	gbrt_build_params params{};
	float host_bound[6]{};
	bool host_bound_valid = false;
	// Staging for the host-buffer entry points: two device slots of
	// kStageRays rays each, two streams, grown on first use, guarded by mu.
	void *stage_mu = nullptr;          // std::mutex*, kept opaque here
	cudaStream_t stage_stream[2]{};
	void *stage_rays[2]{};
	void *stage_out[2]{};
};

// meta word offsets
enum : int {
	GBRT_META_BOUND = 0,        // 6 floats: reference tree bound
	GBRT_META_CLO = 6,          // 3 floats: centroid bound lo
	GBRT_META_CINV = 9,         // 3 floats: 1 / centroid extent (0 if flat)
	GBRT_META_ORD = 12,         // 12 uints: ordered-int reduction scratch
	GBRT_META_ERR = 24,         // 1 uint: build error flag (bad vertex index)
	GBRT_META_WNODES = 25,      // 1 uint: wide nodes written
	GBRT_META_WDEPTH = 26,      // 1 uint: wide tree depth (levels)
	GBRT_META_WPRIMS = 27,      // 1 uint: primitives placed in wide leaves
	GBRT_META_WORDS = 32
};

int gbrt_set_error(int code, const char *fmt, ...);

#define GBRT_CK(call)                                                                             \
	do {                                                                                          \
		cudaError_t gbrt_e_ = (call);                                                             \
		if(gbrt_e_ != cudaSuccess)                                                                \
			return gbrt_set_error(gbrt_e_ == cudaErrorMemoryAllocation ? GBRT_ERR_OOM : GBRT_ERR_CUDA, \
			                      "%s: %s", #call, cudaGetErrorString(gbrt_e_));                  \
	} while(0)

// Launchers implemented in traverse.cu
int gbrt_launch_closest(const gbrt_bvh *bvh, const gbrt_ray *rays, uint32_t n, gbrt_hit *hits, cudaStream_t s);
int gbrt_launch_shadow(const gbrt_bvh *bvh, const gbrt_ray *rays, uint32_t n, int32_t *occ, cudaStream_t s);
// Implemented in guiding.cu
int gbrt_guide_eval_queue(gbrt_guide *G, const float *pos_dev, uint32_t cap, const uint32_t *count_dev, float *lobes_dev, cudaStream_t s);
// Implemented in bvh_build.cu
int gbrt_build_impl(const float *verts, uint32_t nv, const uint32_t *faces, uint32_t nf,
                    const gbrt_build_params *params, cudaStream_t s, gbrt_bvh **out);
