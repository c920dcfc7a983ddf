// Path-guiding network: shared definitions (no counterpart in the reference).
//
// q(w | x) = sum_k softmax(a)_k vMF(w; mu_k, kappa_k), 8 lobes, predicted from
// the hit position x by a multiresolution hash-grid encoding (16 levels x 2
// features, 2^19 entries per level) and an MLP 32 -> 64 -> 64 -> 40 (ReLU).
// Output k*5 + {0,1,2}: unnormalised mean direction, +3: kappa
// pre-activation (kappa = softplus + kKappaMin), +4: mixture logit.
#pragma once

#include <cstdint>

namespace gbrt {

constexpr int kGuideLevels = 16;
constexpr int kGuideFeatures = 2;
constexpr int kGuideIn = kGuideLevels * kGuideFeatures;   // 32
constexpr int kGuideHidden = 64;
constexpr int kGuideLobes = 8;
constexpr int kGuideOut = kGuideLobes * 5;                 // 40
constexpr int kGuideOutPad = 48;                           // padded for the tensor-core tile
constexpr float kKappaMin = 0.05f;
constexpr float kKappaMax = 2000.f;
constexpr float kTwoPiF = 6.28318530717958647692f;

// Parameter block layout (floats), MLP part:
//   W1 [64][32], b1[64], W2 [64][64], b2[64], W3 [40][64], b3[40]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kGuideHidden * kGuideIn;
constexpr int kOffW2 = kOffB1 + kGuideHidden;
constexpr int kOffB2 = kOffW2 + kGuideHidden * kGuideHidden;
constexpr int kOffW3 = kOffB2 + kGuideHidden;
constexpr int kOffB3 = kOffW3 + kGuideOut * kGuideHidden;
constexpr int kMlpParams = kOffB3 + kGuideOut;              // 8872

struct GuideGrid {
	float lo[3], inv_ext[3];     // scene bound -> [0,1]^3
	uint32_t log2_table;
	float res[kGuideLevels];     // grid resolution per level
	uint32_t dense[kGuideLevels];// 1 = level indexed densely (fits the table)
};

#if defined(__CUDACC__)
#define GBRT_GHD __host__ __device__ __forceinline__
#else
#define GBRT_GHD inline
#endif

// Instant-NGP style spatial hash (primes 1, 2654435761, 805459861).
GBRT_GHD uint32_t grid_index(const GuideGrid &g, int level, uint32_t ix, uint32_t iy, uint32_t iz)
{
	const uint32_t T = 1u << g.log2_table;
	if(g.dense[level])
	{
		const uint32_t r = static_cast<uint32_t>(g.res[level]) + 1u;
		return (ix + r * (iy + r * iz)) & (T - 1u);
	}
	return (ix ^ (iy * 2654435761u) ^ (iz * 805459861u)) & (T - 1u);
}

} // namespace gbrt
