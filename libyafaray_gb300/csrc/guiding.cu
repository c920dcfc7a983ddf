// Path-guiding network (no counterpart in the reference): hash-grid
// encoding + MLP + 8-lobe vMF mixture head, trained online on the tracer's
// own radiance samples.
//
//   k_guide_eval   position -> mixture parameters (mu, kappa, weight per lobe)
//   k_guide_grad   forward + KL-divergence gradient + backward for a batch of
//                  (position, sampled direction, weight L/pdf) records;
//                  weight gradients per block, hash-grid gradients by atomics
//   k_reduce       per-block weight gradients -> one gradient
//   k_adam         Adam step on the MLP and the touched hash-grid entries
//
// The training objective is the Monte-Carlo estimate of the KL divergence
// from the incident-radiance distribution to q:  -sum_j c_j log q(w_j | x_j)
// with c_j = luminance(L_j) / p_j (p_j the pdf w_j was sampled with),
// normalised by sum_j c_j.
#include "gbrt_internal.cuh"
#include "guide_common.cuh"
#include "guide_device.cuh"
#include "tc_sm100.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace {

using namespace gbrt;

constexpr int kEvalThreads = 128;
constexpr int kGradThreads = 64;       // one record per thread, 64 records per chunk
constexpr int kGradChunks = 16;        // chunks per block -> 1024 records per block

GBRT_GHD float2 load_feat(const float *table, size_t off)
{
#if defined(__CUDA_ARCH__)
	return __ldg(reinterpret_cast<const float2 *>(table) + off);
#else
	return make_float2(table[2 * off], table[2 * off + 1]);
#endif
}

GBRT_GHD void encode(const GuideGrid &g, const float *__restrict__ table, const float p[3], float e[kGuideIn],
                                       uint32_t *corner_idx, float *corner_w)
{
	float x[3];
	for(int a = 0; a < 3; ++a) x[a] = fminf(fmaxf((p[a] - g.lo[a]) * g.inv_ext[a], 0.f), 1.f);
	// 4 levels per round: 32 independent L2 gathers in flight per thread
#pragma unroll 4
	for(int l = 0; l < kGuideLevels; ++l)
	{
		const float r = g.res[l];
		float fx[3];
		uint32_t ix[3];
		for(int a = 0; a < 3; ++a)
		{
			const float s = x[a] * r;
			const float fl = fminf(floorf(s), r - 1.f);
			ix[a] = static_cast<uint32_t>(fl);
			fx[a] = s - fl;
		}
		float f0 = 0.f, f1 = 0.f;
		for(int c = 0; c < 8; ++c)
		{
			const uint32_t dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
			const float w = (dx ? fx[0] : 1.f - fx[0]) * (dy ? fx[1] : 1.f - fx[1]) * (dz ? fx[2] : 1.f - fx[2]);
			const uint32_t idx = grid_index(g, l, ix[0] + dx, ix[1] + dy, ix[2] + dz);
			const size_t off = (static_cast<size_t>(l) << g.log2_table) + idx;
			const float2 v = load_feat(table, off);
			f0 += w * v.x;
			f1 += w * v.y;
			if(corner_idx) { corner_idx[l * 8 + c] = static_cast<uint32_t>(off); corner_w[l * 8 + c] = w; }
		}
		e[2 * l] = f0;
		e[2 * l + 1] = f1;
	}
}

// MLP forward from smem weights; returns raw outputs.
GBRT_GHD void mlp_forward(const float *__restrict__ W, const float e[kGuideIn], float h1[kGuideHidden],
                                            float h2[kGuideHidden], float o[kGuideOut])
{
	for(int j = 0; j < kGuideHidden; ++j)
	{
		float acc = W[kOffB1 + j];
		const float *w = W + kOffW1 + j * kGuideIn;
#pragma unroll
		for(int i = 0; i < kGuideIn; ++i) acc += w[i] * e[i];
		h1[j] = fmaxf(acc, 0.f);
	}
	for(int j = 0; j < kGuideHidden; ++j)
	{
		float acc = W[kOffB2 + j];
		const float *w = W + kOffW2 + j * kGuideHidden;
#pragma unroll 16
		for(int i = 0; i < kGuideHidden; ++i) acc += w[i] * h1[i];
		h2[j] = fmaxf(acc, 0.f);
	}
	for(int j = 0; j < kGuideOut; ++j)
	{
		float acc = W[kOffB3 + j];
		const float *w = W + kOffW3 + j * kGuideHidden;
#pragma unroll 16
		for(int i = 0; i < kGuideHidden; ++i) acc += w[i] * h2[i];
		o[j] = acc;
	}
}

__global__ void __launch_bounds__(kEvalThreads) k_guide_eval(GuideGrid g, const float *__restrict__ table, const float *__restrict__ mlp,
                                                             const float *__restrict__ pos, uint32_t n, const uint32_t *__restrict__ n_dev,
                                                             float *__restrict__ lobes)
{
	__shared__ float W[kMlpParams];
	for(int i = threadIdx.x; i < kMlpParams; i += blockDim.x) W[i] = mlp[i];
	__syncthreads();
	const uint32_t count = n_dev ? min(*n_dev, n) : n;
	for(uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x)
	{
		const float p[3] = {pos[3ull * s], pos[3ull * s + 1], pos[3ull * s + 2]};
		float e[kGuideIn], h1[kGuideHidden], h2[kGuideHidden], o[kGuideOut];
		encode(g, table, p, e, nullptr, nullptr);
		mlp_forward(W, e, h1, h2, o);
		float lo[kGuideOut];
		raw_to_lobes(o, lo);
		float4 *out = reinterpret_cast<float4 *>(lobes + static_cast<size_t>(kGuideOut) * s);
		for(int k = 0; k < kGuideOut / 4; ++k) out[k] = make_float4(lo[4 * k], lo[4 * k + 1], lo[4 * k + 2], lo[4 * k + 3]);
	}
}

// d(-log q(w))/d(raw outputs), scaled by c.
__device__ __forceinline__ float head_grad(const float o[kGuideOut], const float w[3], float c, float d[kGuideOut])
{
	float lob[kGuideOut];
	raw_to_lobes(o, lob);
	float logf_k[kGuideLobes], lmax = -1e30f;
	for(int k = 0; k < kGuideLobes; ++k)
	{
		logf_k[k] = logf(lob[5 * k + 4]) + vmf_log_pdf(&lob[5 * k], lob[5 * k + 3], w);
		lmax = fmaxf(lmax, logf_k[k]);
	}
	float sum = 0.f;
	for(int k = 0; k < kGuideLobes; ++k) sum += expf(logf_k[k] - lmax);
	const float logq = lmax + logf(sum);
	for(int k = 0; k < kGuideLobes; ++k)
	{
		const float r = expf(logf_k[k] - logq);          // responsibility
		const float wk = lob[5 * k + 4];
		const float kap = lob[5 * k + 3];
		const float *mu = &lob[5 * k];
		const float mw = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
		d[5 * k + 4] = c * (wk - r);
		const float e2 = expf(-2.f * kap);
		const float dlogf_dk = 1.f / kap - 2.f * e2 / (1.f - e2) + (mw - 1.f);
		const float a = o[5 * k + 3];
		const float sp = softplus(a) + kKappaMin;
		const float dk_da = sp < kKappaMax ? 1.f / (1.f + expf(-a)) : 0.f;
		d[5 * k + 3] = -c * r * dlogf_dk * dk_da;
		const float m0 = o[5 * k], m1 = o[5 * k + 1], m2 = o[5 * k + 2];
		const float len = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
		if(len > 1e-20f)
		{
			const float s = -c * r * kap / len;
			d[5 * k + 0] = s * (w[0] - mw * mu[0]);
			d[5 * k + 1] = s * (w[1] - mw * mu[1]);
			d[5 * k + 2] = s * (w[2] - mw * mu[2]);
		}
		else d[5 * k + 0] = d[5 * k + 1] = d[5 * k + 2] = 0.f;
	}
	return -c * logq;
}

// One block: kGradChunks chunks of 64 records.  Weight gradients accumulate
// in shared memory (each entry owned by one thread) and are written once per
// block; hash-grid gradients are scattered with atomics.
__global__ void __launch_bounds__(kGradThreads) k_guide_grad(GuideGrid g, const float *__restrict__ table, const float *__restrict__ mlp,
                                                             const float *__restrict__ rec, uint32_t n, const float *__restrict__ wsum,
                                                             float *__restrict__ partial, float *__restrict__ grid_grad,
                                                             float *__restrict__ loss_out)
{
	extern __shared__ float sm[];
	float *W = sm;                                        // kMlpParams
	float *G = W + kMlpParams;                            // kMlpParams, block gradient
	float *E = G + kMlpParams;                            // [64][32]
	float *H1 = E + kGradThreads * kGuideIn;              // [64][64]
	float *H2 = H1 + kGradThreads * kGuideHidden;         // [64][64]
	float *D1 = H2 + kGradThreads * kGuideHidden;         // [64][64] dL/d(pre-act 1)
	float *D2 = D1 + kGradThreads * kGuideHidden;         // [64][64]
	float *D3 = D2 + kGradThreads * kGuideHidden;         // [64][40]
	const int t = threadIdx.x;
	const float inv_norm = *wsum > 0.f ? 1.f / *wsum : 0.f;
	for(int i = t; i < kMlpParams; i += blockDim.x) { W[i] = mlp[i]; G[i] = 0.f; }
	__syncthreads();
	float loss = 0.f;
	for(int chunk = 0; chunk < kGradChunks; ++chunk)
	{
		const uint32_t r = (blockIdx.x * kGradChunks + chunk) * kGradThreads + t;
		const bool live = r < n;
		float e[kGuideIn], h1[kGuideHidden], h2[kGuideHidden], o[kGuideOut], d3[kGuideOut];
		uint32_t cidx[kGuideLevels * 8];
		float cw[kGuideLevels * 8];
		if(live)
		{
			const float *q = rec + 8ull * r;   // pos xyz, dir xyz, weight, pad
			const float p[3] = {q[0], q[1], q[2]};
			const float w[3] = {q[3], q[4], q[5]};
			encode(g, table, p, e, cidx, cw);
			mlp_forward(W, e, h1, h2, o);
			loss += head_grad(o, w, q[6] * inv_norm, d3);
		}
		else
		{
			for(int i = 0; i < kGuideIn; ++i) e[i] = 0.f;
			for(int i = 0; i < kGuideHidden; ++i) h1[i] = h2[i] = 0.f;
			for(int i = 0; i < kGuideOut; ++i) d3[i] = 0.f;
		}
		// backward through the MLP
		float d2[kGuideHidden], d1[kGuideHidden];
		for(int i = 0; i < kGuideHidden; ++i)
		{
			float acc = 0.f;
			for(int j = 0; j < kGuideOut; ++j) acc += W[kOffW3 + j * kGuideHidden + i] * d3[j];
			d2[i] = h2[i] > 0.f ? acc : 0.f;
		}
		for(int i = 0; i < kGuideHidden; ++i)
		{
			float acc = 0.f;
			for(int j = 0; j < kGuideHidden; ++j) acc += W[kOffW2 + j * kGuideHidden + i] * d2[j];
			d1[i] = h1[i] > 0.f ? acc : 0.f;
		}
		if(live)
		{
			// encoding gradient -> hash grid (trilinear weights)
			for(int l = 0; l < kGuideLevels; ++l)
			{
				float de0 = 0.f, de1 = 0.f;
				for(int j = 0; j < kGuideHidden; ++j)
				{
					de0 += W[kOffW1 + j * kGuideIn + 2 * l] * d1[j];
					de1 += W[kOffW1 + j * kGuideIn + 2 * l + 1] * d1[j];
				}
				for(int c = 0; c < 8; ++c)
				{
					const float wc = cw[l * 8 + c];
					const size_t off = cidx[l * 8 + c];
					atomicAdd(grid_grad + 2 * off, wc * de0);
					atomicAdd(grid_grad + 2 * off + 1, wc * de1);
				}
			}
		}
		for(int i = 0; i < kGuideIn; ++i) E[t * kGuideIn + i] = e[i];
		for(int i = 0; i < kGuideHidden; ++i)
		{
			H1[t * kGuideHidden + i] = h1[i]; H2[t * kGuideHidden + i] = h2[i];
			D1[t * kGuideHidden + i] = d1[i]; D2[t * kGuideHidden + i] = d2[i];
		}
		for(int i = 0; i < kGuideOut; ++i) D3[t * kGuideOut + i] = d3[i];
		__syncthreads();
		// weight gradients: sum over the 64 records of the chunk
		for(int idx = t; idx < kMlpParams; idx += kGradThreads)
		{
			float acc = 0.f;
			if(idx < kOffB1)      { const int j = idx / kGuideIn, i = idx % kGuideIn; for(int s = 0; s < kGradThreads; ++s) acc += D1[s * kGuideHidden + j] * E[s * kGuideIn + i]; }
			else if(idx < kOffW2) { const int j = idx - kOffB1; for(int s = 0; s < kGradThreads; ++s) acc += D1[s * kGuideHidden + j]; }
			else if(idx < kOffB2) { const int k = idx - kOffW2, j = k / kGuideHidden, i = k % kGuideHidden; for(int s = 0; s < kGradThreads; ++s) acc += D2[s * kGuideHidden + j] * H1[s * kGuideHidden + i]; }
			else if(idx < kOffW3) { const int j = idx - kOffB2; for(int s = 0; s < kGradThreads; ++s) acc += D2[s * kGuideHidden + j]; }
			else if(idx < kOffB3) { const int k = idx - kOffW3, j = k / kGuideHidden, i = k % kGuideHidden; for(int s = 0; s < kGradThreads; ++s) acc += D3[s * kGuideOut + j] * H2[s * kGuideHidden + i]; }
			else                  { const int j = idx - kOffB3; for(int s = 0; s < kGradThreads; ++s) acc += D3[s * kGuideOut + j]; }
			G[idx] += acc;
		}
		__syncthreads();
	}
	for(int i = t; i < kMlpParams; i += blockDim.x) partial[static_cast<size_t>(blockIdx.x) * kMlpParams + i] = G[i];
	for(int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
	if((t & 31) == 0) atomicAdd(loss_out, loss);
}

__global__ void k_weight_sum(const float *__restrict__ rec, uint32_t n, float *__restrict__ out)
{
	float acc = 0.f;
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += rec[8ull * i + 6];
	for(int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
	if((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

__global__ void k_reduce(const float *__restrict__ partial, int nblk, float *__restrict__ grad)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= kMlpParams) return;
	float acc = 0.f;
	for(int b = 0; b < nblk; ++b) acc += partial[static_cast<size_t>(b) * kMlpParams + i];
	grad[i] = acc;
}

__global__ void k_adam(float *__restrict__ p, float *__restrict__ g, float *__restrict__ m, float *__restrict__ v, size_t n,
                       float lr, float b1, float b2, float eps, float c1, float c2, int sparse)
{
	for(size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
	{
		const float gi = g[i];
		if(sparse && gi == 0.f) continue;     // untouched hash entries keep their moments
		const float mi = b1 * m[i] + (1.f - b1) * gi;
		const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi; v[i] = vi;
		p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		g[i] = 0.f;
	}
}


// ---- tensor-core forward pass ------------------------------------------------
// One CTA (4 warps) evaluates tiles of 128 positions: the encoding (hash-grid
// gathers, one position per thread) is written as BF16 into shared memory,
// then each layer is one tcgen05 MMA chain (M = 128, N = 64 / 64 / 48,
// K = 32 / 64 / 64) into TMEM, and the epilogue (bias, ReLU, BF16) reads each
// thread's TMEM lane and writes the next layer's operand.
constexpr int kTcThreads = 128;
constexpr uint32_t kTcCols = 128;              // TMEM columns: D1 [0,64), D2 [64,128), D3 reuses [0,48)
constexpr uint32_t kTcWaitIters = 1u << 24;    // bounded mbarrier wait
constexpr uint32_t kSmA0 = 0, kSmA1 = 16384, kSmB1 = 32768, kSmB2 = 36864, kSmB3 = 45056, kSmBias = 51200;
constexpr uint32_t kSmMbar = 51904, kSmSlot = 51912, kSmTotal = 51968;

__device__ __forceinline__ void tc_load_weights(const float *__restrict__ mlp, uint8_t *smem, float *bias)
{
	for(int i = threadIdx.x; i < kGuideHidden * kGuideIn; i += blockDim.x)
	{
		const int r = i / kGuideIn, k = i % kGuideIn;
		*reinterpret_cast<__nv_bfloat16 *>(smem + kSmB1 + tc::kmajor_offset(r, k, kGuideIn)) = __float2bfloat16_rn(mlp[kOffW1 + i]);
	}
	for(int i = threadIdx.x; i < kGuideHidden * kGuideHidden; i += blockDim.x)
	{
		const int r = i / kGuideHidden, k = i % kGuideHidden;
		*reinterpret_cast<__nv_bfloat16 *>(smem + kSmB2 + tc::kmajor_offset(r, k, kGuideHidden)) = __float2bfloat16_rn(mlp[kOffW2 + i]);
	}
	for(int i = threadIdx.x; i < kGuideOutPad * kGuideHidden; i += blockDim.x)
	{
		const int r = i / kGuideHidden, k = i % kGuideHidden;
		const float w = r < kGuideOut ? mlp[kOffW3 + r * kGuideHidden + k] : 0.f;
		*reinterpret_cast<__nv_bfloat16 *>(smem + kSmB3 + tc::kmajor_offset(r, k, kGuideHidden)) = __float2bfloat16_rn(w);
	}
	for(int i = threadIdx.x; i < 2 * kGuideHidden + kGuideOutPad; i += blockDim.x)
	{
		float b;
		if(i < kGuideHidden) b = mlp[kOffB1 + i];
		else if(i < 2 * kGuideHidden) b = mlp[kOffB2 + i - kGuideHidden];
		else b = (i - 2 * kGuideHidden) < kGuideOut ? mlp[kOffB3 + i - 2 * kGuideHidden] : 0.f;
		bias[i] = b;
	}
}

// Issue a K-chain of MMAs (K/16 instructions) and commit to the mbarrier.
__device__ __forceinline__ void tc_layer(uint32_t d_tmem, uint32_t a_saddr, uint32_t b_saddr, uint32_t K, uint32_t N, uint64_t *mbar)
{
	const uint32_t sbo = (K / 8) * 128u;
	const uint32_t idesc = tc::idesc_bf16(128, N);
	for(uint32_t kk = 0; kk < K / 16; ++kk)
		tc::mma_bf16(d_tmem, tc::smem_desc(a_saddr + kk * 256u, 128u, sbo), tc::smem_desc(b_saddr + kk * 256u, 128u, sbo), idesc, kk > 0 ? 1u : 0u);
	tc::mma_commit(mbar);
}

// The hash-grid encoding of a queue of positions as BF16 rows of kGuideIn
// features (64 B), one position per thread.  Kept apart from the tensor-core
// kernel, whose TMEM and shared memory allow 4 CTAs per SM: here every SM
// holds enough warps to keep its 128 gathers per position in flight.
constexpr int kEncThreads = 256;
__global__ void __launch_bounds__(kEncThreads) k_guide_encode(GuideGrid g, const float *__restrict__ table, const float *__restrict__ pos,
                                                              uint32_t n, const uint32_t *__restrict__ n_dev, uint4 *__restrict__ enc)
{
	const uint32_t count = n_dev ? min(*n_dev, n) : n;
	for(uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x)
	{
		const float p[3] = {pos[3ull * s], pos[3ull * s + 1], pos[3ull * s + 2]};
		float e[kGuideIn];
		encode(g, table, p, e, nullptr, nullptr);
		uint32_t w[kGuideIn / 2];
		for(int i = 0; i < kGuideIn / 2; ++i)
		{
			const __nv_bfloat162 b = __floats2bfloat162_rn(e[2 * i], e[2 * i + 1]);
			w[i] = *reinterpret_cast<const uint32_t *>(&b);
		}
		uint4 *row = enc + static_cast<size_t>(s) * (kGuideIn / 8);
		for(int i = 0; i < kGuideIn / 8; ++i) row[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
	}
}

// enc: the positions' encodings (k_guide_encode), or null to encode here.
__global__ void __launch_bounds__(kTcThreads) k_guide_eval_tc(GuideGrid g, const float *__restrict__ table, const float *__restrict__ mlp,
                                                              const float *__restrict__ pos, uint32_t n, const uint32_t *__restrict__ n_dev,
                                                              float *__restrict__ lobes, uint32_t *__restrict__ err, const uint4 *__restrict__ enc)
{
	extern __shared__ __align__(1024) uint8_t smem[];
	float *bias = reinterpret_cast<float *>(smem + kSmBias);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kSmMbar);
	uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSmSlot);
	const int t = threadIdx.x, warp = t >> 5;
	tc_load_weights(mlp, smem, bias);
	if(t == 0) { tc::mbar_init(mbar, 1); tc::fence_mbar_init(); }
	if(warp == 0) tc::tmem_alloc(slot, kTcCols);
	tc::fence_smem_async();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tbase = *slot;
	const uint32_t lane_addr = tbase + (static_cast<uint32_t>(warp * 32) << 16);
	const uint32_t sA0 = tc::smem_addr(smem + kSmA0), sA1 = tc::smem_addr(smem + kSmA1);
	const uint32_t sB1 = tc::smem_addr(smem + kSmB1), sB2 = tc::smem_addr(smem + kSmB2), sB3 = tc::smem_addr(smem + kSmB3);
	const uint32_t count = n_dev ? min(*n_dev, n) : n;
	uint32_t phase = 0;
	bool ok = true;
	for(uint32_t tile = blockIdx.x; tile * 128u < count; tile += gridDim.x)
	{
		const uint32_t s = tile * 128u + t;
		const bool live = s < count;
		float v[kGuideOutPad];
		if(live && enc)
		{
			const uint4 *row = enc + static_cast<size_t>(s) * (kGuideIn / 8);
			for(int i = 0; i < kGuideIn / 8; ++i)
			{
				const uint4 q = __ldg(row + i);
				const uint32_t w[4] = {q.x, q.y, q.z, q.w};
				for(int k = 0; k < 4; ++k)
				{
					const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&w[k]));
					v[8 * i + 2 * k] = f.x;
					v[8 * i + 2 * k + 1] = f.y;
				}
			}
		}
		else if(live)
		{
			const float p[3] = {pos[3ull * s], pos[3ull * s + 1], pos[3ull * s + 2]};
			encode(g, table, p, v, nullptr, nullptr);
		}
		else
			for(int i = 0; i < kGuideIn; ++i) v[i] = 0.f;
		tc::store_bf16_row(smem + kSmA0, t, kGuideIn, v, 0, kGuideIn);
		tc::fence_smem_async();
		__syncthreads();
		// layer 1: D1 = E W1^T
		if(t == 0) { tc::fence_after_sync(); tc_layer(tbase, sA0, sB1, kGuideIn, kGuideHidden, mbar); }
		ok = __syncthreads_and(tc::mbar_wait(mbar, phase, kTcWaitIters));
		phase ^= 1u;
		if(!ok) break;
		tc::fence_after_sync();
		for(int c = 0; c < kGuideHidden / 16; ++c)
		{
			tc::tmem_ld16(lane_addr + 16u * c, v);
			for(int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + bias[16 * c + i], 0.f);
			tc::store_bf16_row(smem + kSmA1, t, kGuideHidden, v, 16u * c, 16);
		}
		tc::fence_before_sync();
		tc::fence_smem_async();
		__syncthreads();
		// layer 2: D2 = H1 W2^T
		if(t == 0) { tc::fence_after_sync(); tc_layer(tbase + 64u, sA1, sB2, kGuideHidden, kGuideHidden, mbar); }
		ok = __syncthreads_and(tc::mbar_wait(mbar, phase, kTcWaitIters));
		phase ^= 1u;
		if(!ok) break;
		tc::fence_after_sync();
		for(int c = 0; c < kGuideHidden / 16; ++c)
		{
			tc::tmem_ld16(lane_addr + 64u + 16u * c, v);
			for(int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + bias[kGuideHidden + 16 * c + i], 0.f);
			tc::store_bf16_row(smem + kSmA0, t, kGuideHidden, v, 16u * c, 16);
		}
		tc::fence_before_sync();
		tc::fence_smem_async();
		__syncthreads();
		// layer 3: D3 = H2 W3^T (40 outputs padded to 48), into columns [0, 48)
		if(t == 0) { tc::fence_after_sync(); tc_layer(tbase, sA0, sB3, kGuideHidden, kGuideOutPad, mbar); }
		ok = __syncthreads_and(tc::mbar_wait(mbar, phase, kTcWaitIters));
		phase ^= 1u;
		if(!ok) break;
		tc::fence_after_sync();
		for(int c = 0; c < kGuideOutPad / 16; ++c)
		{
			tc::tmem_ld16(lane_addr + 16u * c, v + 16 * c);
			for(int i = 0; i < 16; ++i) v[16 * c + i] += bias[2 * kGuideHidden + 16 * c + i];
		}
		if(live)
		{
			float lo[kGuideOut];
			raw_to_lobes(v, lo);
			float4 *out = reinterpret_cast<float4 *>(lobes + static_cast<size_t>(kGuideOut) * s);
			for(int k = 0; k < kGuideOut / 4; ++k) out[k] = make_float4(lo[4 * k], lo[4 * k + 1], lo[4 * k + 2], lo[4 * k + 3]);
		}
		tc::fence_before_sync();
		__syncthreads();
	}
	if(!ok)
	{
		if(t == 0) atomicOr(err, 1u);
		tc::mbar_wait(mbar, phase ^ 1u, kTcWaitIters);   // the phase that timed out: let its MMAs finish before freeing TMEM
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if(warp == 0) tc::tmem_dealloc(tbase, kTcCols);
}

// Self-test of the tcgen05 path: D[128][N] = A[128][K] B[N][K]^T in BF16 with
// FP32 accumulation, through the same layouts, descriptors and TMEM loads.
__global__ void __launch_bounds__(kTcThreads) k_tc_selftest(const float *__restrict__ A, const float *__restrict__ B, uint32_t N, uint32_t K,
                                                            float *__restrict__ D, uint32_t *__restrict__ err)
{
	extern __shared__ __align__(1024) uint8_t smem[];
	uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kSmMbar);
	uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSmSlot);
	const int t = threadIdx.x, warp = t >> 5;
	for(uint32_t i = t; i < 128u * K; i += blockDim.x)
		*reinterpret_cast<__nv_bfloat16 *>(smem + kSmA0 + tc::kmajor_offset(i / K, i % K, K)) = __float2bfloat16_rn(A[i]);
	for(uint32_t i = t; i < N * K; i += blockDim.x)
		*reinterpret_cast<__nv_bfloat16 *>(smem + kSmA1 + tc::kmajor_offset(i / K, i % K, K)) = __float2bfloat16_rn(B[i]);
	if(t == 0) { tc::mbar_init(mbar, 1); tc::fence_mbar_init(); }
	if(warp == 0) tc::tmem_alloc(slot, kTcCols);
	tc::fence_smem_async();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tbase = *slot;
	if(t == 0) { tc::fence_after_sync(); tc_layer(tbase, tc::smem_addr(smem + kSmA0), tc::smem_addr(smem + kSmA1), K, N, mbar); }
	const bool ok = __syncthreads_and(tc::mbar_wait(mbar, 0, kTcWaitIters));
	tc::fence_after_sync();
	if(ok)
	{
		float v[16];
		for(uint32_t c = 0; c < N / 16; ++c)
		{
			tc::tmem_ld16(tbase + (static_cast<uint32_t>(warp * 32) << 16) + 16u * c, v);
			for(int i = 0; i < 16; ++i) D[static_cast<size_t>(t) * N + 16u * c + i] = v[i];
		}
	}
	else
	{
		if(t == 0) atomicOr(err, 1u);
		tc::mbar_wait(mbar, 0, kTcWaitIters);
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if(warp == 0) tc::tmem_dealloc(tbase, kTcCols);
}

// ---- tensor-core training step ----------------------------------------------
// One CTA per SM, tiles of 128 records.  Per tile, six tcgen05 stages:
//   L1..L3   forward (as in k_guide_eval_tc), activations kept in shared
//            memory twice: [record][feature] (A operand of the next layer)
//            and [feature][record] (operand of the weight-gradient GEMMs)
//   dH2      dO  [128x48] . W3  -> ReLU mask -> dA2
//   dH1      dA2 [128x64] . W2  -> ReLU mask -> dA1
//   dE       dA1 [128x64] . W1  -> scattered into the hash-grid gradient
// with the weight gradients accumulated in TMEM over all tiles of the CTA:
//   G1 [128 x 112] += [dA2^T ; dA1^T] . [H1^T ; E^T ; 1]^T
//        rows 0-63:  dW2 (cols 0-63), db2 (col 96)
//        rows 64-127: dW1 (cols 64-95), db1 (col 96)
//   G2 [128 x 48]  += [H2^T ; 1] . dO
//        rows 0-63: dW3^T, rows 64-127: db3
// The cross blocks of G1 (dA2^T E, dA1^T H1) are computed and ignored.
constexpr uint32_t kTrThreads = 128;
constexpr uint32_t kTrCols = 256;
constexpr uint32_t kTrW1 = 0, kTrW2 = 4096, kTrW3 = 12288, kTrW3T = 18432, kTrW2T = 24576, kTrW1T = 32768;
constexpr uint32_t kTrCH0 = 36864, kTrCH1 = 53248;                       // [128][<=64] chain operands
constexpr uint32_t kTrH2T = 69632, kTrOne64 = 86016;                     // G2 A: rows 0-63, 64-127
constexpr uint32_t kTrDA2T = 102400, kTrDA1T = 118784;                   // G1 A: rows 0-63, 64-127
constexpr uint32_t kTrH1T = 135168, kTrET = 151552, kTrOne16 = 159744;   // G1 B: rows 0-63, 64-95, 96-111
constexpr uint32_t kTrDOT = 163840;                                      // G2 B: rows 0-47 (40-47 zero)
constexpr uint32_t kTrBias = 176128, kTrMbar = 176832, kTrSlot = 176840, kTrTotal = 176896;
constexpr uint32_t kTrColG1 = 64, kTrColG2 = 192;                        // TMEM: scratch [0,64), G1, G2

__device__ __forceinline__ void st_bf16(uint8_t *smem, uint32_t off, float x)
{
	*reinterpret_cast<__nv_bfloat16 *>(smem + off) = __float2bfloat16_rn(x);
}

// [feature][record] copy of one record's row (K = 128 records).
__device__ __forceinline__ void store_bf16_col(uint8_t *base, uint32_t rec, const float *v, uint32_t nfeat)
{
	for(uint32_t f = 0; f < nfeat; ++f) st_bf16(base, tc::kmajor_offset(f, rec, 128), v[f]);
}

// Hash-grid gradient: corner weights x dL/de, as in encode.
__device__ __forceinline__ void scatter_grid_grad(const GuideGrid &g, const float p[3], const float de[kGuideIn], float *__restrict__ grid_grad)
{
	float x[3];
	for(int a = 0; a < 3; ++a) x[a] = fminf(fmaxf((p[a] - g.lo[a]) * g.inv_ext[a], 0.f), 1.f);
#pragma unroll 1
	for(int l = 0; l < kGuideLevels; ++l)
	{
		const float r = g.res[l];
		float fx[3];
		uint32_t ix[3];
		for(int a = 0; a < 3; ++a)
		{
			const float s = x[a] * r;
			const float fl = fminf(floorf(s), r - 1.f);
			ix[a] = static_cast<uint32_t>(fl);
			fx[a] = s - fl;
		}
		const float d0 = de[2 * l], d1 = de[2 * l + 1];
		for(int c = 0; c < 8; ++c)
		{
			const uint32_t dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
			const float w = (dx ? fx[0] : 1.f - fx[0]) * (dy ? fx[1] : 1.f - fx[1]) * (dz ? fx[2] : 1.f - fx[2]);
			const size_t off = (static_cast<size_t>(l) << g.log2_table) + grid_index(g, l, ix[0] + dx, ix[1] + dy, ix[2] + dz);
			atomicAdd(reinterpret_cast<float2 *>(grid_grad) + off, make_float2(w * d0, w * d1));
		}
	}
}

// A K-chain of MMAs (K/16 instructions) without commit; the operand row
// strides are given separately for A and B (both K-major, no swizzle).
__device__ __forceinline__ void tc_chain(uint32_t d_tmem, uint32_t a_saddr, uint32_t b_saddr, uint32_t K, uint32_t N, bool accumulate)
{
	const uint32_t sbo = (K / 8) * 128u;
	const uint32_t idesc = tc::idesc_bf16(128, N);
	for(uint32_t kk = 0; kk < K / 16; ++kk)
		tc::mma_bf16(d_tmem, tc::smem_desc(a_saddr + kk * 256u, 128u, sbo), tc::smem_desc(b_saddr + kk * 256u, 128u, sbo), idesc,
		             (accumulate || kk > 0) ? 1u : 0u);
}

__global__ void __launch_bounds__(kTrThreads, 1) k_guide_train_tc(GuideGrid g, const float *__restrict__ table, const float *__restrict__ mlp,
                                                                  const float *__restrict__ rec, uint32_t n, const float *__restrict__ wsum,
                                                                  float *__restrict__ partial, float *__restrict__ grid_grad,
                                                                  float *__restrict__ loss_out, uint32_t *__restrict__ err)
{
	extern __shared__ __align__(1024) uint8_t smem[];
	float *bias = reinterpret_cast<float *>(smem + kTrBias);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kTrMbar);
	uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kTrSlot);
	const int t = threadIdx.x, warp = t >> 5;
	// weights in both orientations, biases, constant blocks
	for(int i = t; i < kGuideHidden * kGuideIn; i += blockDim.x)
	{
		const int j = i / kGuideIn, f = i % kGuideIn;
		st_bf16(smem, kTrW1 + tc::kmajor_offset(j, f, kGuideIn), mlp[kOffW1 + i]);
		st_bf16(smem, kTrW1T + tc::kmajor_offset(f, j, kGuideHidden), mlp[kOffW1 + i]);
	}
	for(int i = t; i < kGuideHidden * kGuideHidden; i += blockDim.x)
	{
		const int j = i / kGuideHidden, k = i % kGuideHidden;
		st_bf16(smem, kTrW2 + tc::kmajor_offset(j, k, kGuideHidden), mlp[kOffW2 + i]);
		st_bf16(smem, kTrW2T + tc::kmajor_offset(k, j, kGuideHidden), mlp[kOffW2 + i]);
	}
	for(int i = t; i < kGuideOutPad * kGuideHidden; i += blockDim.x)
	{
		const int o = i / kGuideHidden, j = i % kGuideHidden;
		const float w = o < kGuideOut ? mlp[kOffW3 + o * kGuideHidden + j] : 0.f;
		st_bf16(smem, kTrW3 + tc::kmajor_offset(o, j, kGuideHidden), w);
		st_bf16(smem, kTrW3T + tc::kmajor_offset(j, o, kGuideOutPad), w);
	}
	for(int i = t; i < 2 * kGuideHidden + kGuideOutPad; i += blockDim.x)
	{
		float b;
		if(i < kGuideHidden) b = mlp[kOffB1 + i];
		else if(i < 2 * kGuideHidden) b = mlp[kOffB2 + i - kGuideHidden];
		else b = (i - 2 * kGuideHidden) < kGuideOut ? mlp[kOffB3 + i - 2 * kGuideHidden] : 0.f;
		bias[i] = b;
	}
	{
		const uint32_t one2 = 0x3F803F80u;   // two BF16 ones
		uint32_t *o64 = reinterpret_cast<uint32_t *>(smem + kTrOne64), *o16 = reinterpret_cast<uint32_t *>(smem + kTrOne16);
		uint32_t *dot = reinterpret_cast<uint32_t *>(smem + kTrDOT);
		for(int i = t; i < 16384 / 4; i += blockDim.x) o64[i] = one2;
		for(int i = t; i < 4096 / 4; i += blockDim.x) o16[i] = one2;
		for(int i = t; i < 12288 / 4; i += blockDim.x) dot[i] = 0u;
	}
	if(t == 0) { tc::mbar_init(mbar, 1); tc::fence_mbar_init(); }
	if(warp == 0) tc::tmem_alloc(slot, kTrCols);
	tc::fence_smem_async();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tbase = *slot;
	const uint32_t lane_addr = tbase + (static_cast<uint32_t>(warp * 32) << 16);
	const uint32_t s0 = tc::smem_addr(smem);
	const float inv_norm = *wsum > 0.f ? 1.f / *wsum : 0.f;
	const uint32_t ntiles = (n + 127u) / 128u;
	uint32_t phase = 0;
	bool ok = true, first = true;
	float loss = 0.f;
	// one MMA stage: make the shared-memory operands visible to the tensor
	// core, issue from thread 0, wait (bounded) for completion
	auto stage = [&](auto issue) -> bool {
		tc::fence_smem_async();
		tc::fence_before_sync();
		__syncthreads();
		if(t == 0) { tc::fence_after_sync(); issue(); tc::mma_commit(mbar); }
		const bool done = __syncthreads_and(tc::mbar_wait(mbar, phase, kTcWaitIters));
		phase ^= 1u;
		tc::fence_after_sync();
		return done;
	};
	for(uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
	{
		const uint32_t r = tile * 128u + t;
		const bool live = r < n;
		float p[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 1.f}, c = 0.f;
		float v[kGuideHidden];
		uint32_t m1lo = 0, m1hi = 0, m2lo = 0, m2hi = 0;   // ReLU masks
		if(live)
		{
			const float4 a = *reinterpret_cast<const float4 *>(rec + 8ull * r);
			const float4 b = *reinterpret_cast<const float4 *>(rec + 8ull * r + 4);
			p[0] = a.x; p[1] = a.y; p[2] = a.z; w[0] = a.w; w[1] = b.x; w[2] = b.y;
			c = b.z * inv_norm;
			encode(g, table, p, v, nullptr, nullptr);
		}
		else
			for(int i = 0; i < kGuideIn; ++i) v[i] = 0.f;
		tc::store_bf16_row(smem + kTrCH0, t, kGuideIn, v, 0, kGuideIn);
		store_bf16_col(smem + kTrET, t, v, kGuideIn);
		// L1
		if(!(ok = stage([&] { tc_chain(tbase, s0 + kTrCH0, s0 + kTrW1, kGuideIn, kGuideHidden, false); }))) break;
		for(int cc = 0; cc < 4; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		for(int i = 0; i < kGuideHidden; ++i)
		{
			const float a = v[i] + bias[i];
			v[i] = fmaxf(a, 0.f);
			if(a > 0.f) { if(i < 32) m1lo |= 1u << i; else m1hi |= 1u << (i - 32); }
		}
		tc::store_bf16_row(smem + kTrCH1, t, kGuideHidden, v, 0, kGuideHidden);
		store_bf16_col(smem + kTrH1T, t, v, kGuideHidden);
		// L2
		if(!(ok = stage([&] { tc_chain(tbase, s0 + kTrCH1, s0 + kTrW2, kGuideHidden, kGuideHidden, false); }))) break;
		for(int cc = 0; cc < 4; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		for(int i = 0; i < kGuideHidden; ++i)
		{
			const float a = v[i] + bias[kGuideHidden + i];
			v[i] = fmaxf(a, 0.f);
			if(a > 0.f) { if(i < 32) m2lo |= 1u << i; else m2hi |= 1u << (i - 32); }
		}
		tc::store_bf16_row(smem + kTrCH0, t, kGuideHidden, v, 0, kGuideHidden);
		store_bf16_col(smem + kTrH2T, t, v, kGuideHidden);
		// L3 + loss head
		if(!(ok = stage([&] { tc_chain(tbase, s0 + kTrCH0, s0 + kTrW3, kGuideHidden, kGuideOutPad, false); }))) break;
		for(int cc = 0; cc < 3; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		{
			float o[kGuideOut], d3[kGuideOut];
			for(int i = 0; i < kGuideOut; ++i) o[i] = v[i] + bias[2 * kGuideHidden + i];
			if(live) loss += head_grad(o, w, c, d3);
			else for(int i = 0; i < kGuideOut; ++i) d3[i] = 0.f;
			for(int i = 0; i < kGuideOut; ++i) v[i] = d3[i];
			for(int i = kGuideOut; i < kGuideOutPad; ++i) v[i] = 0.f;
		}
		tc::store_bf16_row(smem + kTrCH1, t, kGuideOutPad, v, 0, kGuideOutPad);
		store_bf16_col(smem + kTrDOT, t, v, kGuideOut);
		// dH2 = dO W3, ReLU mask of layer 2
		if(!(ok = stage([&] { tc_chain(tbase, s0 + kTrCH1, s0 + kTrW3T, kGuideOutPad, kGuideHidden, false); }))) break;
		for(int cc = 0; cc < 4; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		for(int i = 0; i < kGuideHidden; ++i)
			if(!(((i < 32 ? m2lo : m2hi) >> (i & 31)) & 1u)) v[i] = 0.f;
		tc::store_bf16_row(smem + kTrCH0, t, kGuideHidden, v, 0, kGuideHidden);
		store_bf16_col(smem + kTrDA2T, t, v, kGuideHidden);
		// dH1 = dA2 W2, ReLU mask of layer 1
		if(!(ok = stage([&] { tc_chain(tbase, s0 + kTrCH0, s0 + kTrW2T, kGuideHidden, kGuideHidden, false); }))) break;
		for(int cc = 0; cc < 4; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		for(int i = 0; i < kGuideHidden; ++i)
			if(!(((i < 32 ? m1lo : m1hi) >> (i & 31)) & 1u)) v[i] = 0.f;
		tc::store_bf16_row(smem + kTrCH1, t, kGuideHidden, v, 0, kGuideHidden);
		store_bf16_col(smem + kTrDA1T, t, v, kGuideHidden);
		// dE = dA1 W1, and the weight-gradient GEMMs of this tile
		const bool acc = !first;
		if(!(ok = stage([&] {
			tc_chain(tbase, s0 + kTrCH1, s0 + kTrW1T, kGuideHidden, kGuideIn, false);
			tc_chain(tbase + kTrColG1, s0 + kTrDA2T, s0 + kTrH1T, 128, 112, acc);
			tc_chain(tbase + kTrColG2, s0 + kTrH2T, s0 + kTrDOT, 128, kGuideOutPad, acc);
		}))) break;
		first = false;
		for(int cc = 0; cc < 2; ++cc) tc::tmem_ld16(lane_addr + 16u * cc, v + 16 * cc);
		if(live) scatter_grid_grad(g, p, v, grid_grad);
	}
	float *out = partial + static_cast<size_t>(blockIdx.x) * kMlpParams;
	if(!ok)
	{
		if(t == 0) atomicOr(err, 1u);
		tc::mbar_wait(mbar, phase ^ 1u, kTcWaitIters);
		for(int i = t; i < kMlpParams; i += blockDim.x) out[i] = 0.f;
	}
	else if(first)
		for(int i = t; i < kMlpParams; i += blockDim.x) out[i] = 0.f;
	else
	{
		float v[16];
		if(warp < 2)
		{
			for(int cc = 0; cc < 4; ++cc)
			{
				tc::tmem_ld16(lane_addr + kTrColG1 + 16u * cc, v);
				for(int i = 0; i < 16; ++i) out[kOffW2 + t * kGuideHidden + 16 * cc + i] = v[i];
			}
			tc::tmem_ld16(lane_addr + kTrColG1 + 96u, v);
			out[kOffB2 + t] = v[0];
			for(int cc = 0; cc < 3; ++cc)
			{
				tc::tmem_ld16(lane_addr + kTrColG2 + 16u * cc, v);
				for(int i = 0; i < 16; ++i)
					if(16 * cc + i < kGuideOut) out[kOffW3 + (16 * cc + i) * kGuideHidden + t] = v[i];
			}
		}
		else
		{
			const int j = t - kGuideHidden;
			for(int cc = 0; cc < 2; ++cc)
			{
				tc::tmem_ld16(lane_addr + kTrColG1 + 64u + 16u * cc, v);
				for(int i = 0; i < 16; ++i) out[kOffW1 + j * kGuideIn + 16 * cc + i] = v[i];
			}
			tc::tmem_ld16(lane_addr + kTrColG1 + 96u, v);
			out[kOffB1 + j] = v[0];
			for(int cc = 0; cc < 3; ++cc)
			{
				tc::tmem_ld16(lane_addr + kTrColG2 + 16u * cc, v);
				if(j == 0)
					for(int i = 0; i < 16; ++i)
						if(16 * cc + i < kGuideOut) out[kOffB3 + 16 * cc + i] = v[i];
			}
		}
	}
	for(int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
	if((t & 31) == 0 && loss != 0.f) atomicAdd(loss_out, loss);
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if(warp == 0) tc::tmem_dealloc(tbase, kTrCols);
}

} // namespace

struct gbrt_guide {
	int device = 0;
	GuideGrid grid{};
	gbrt_guide_params params{};
	size_t table_floats = 0;
	float *table = nullptr, *table_g = nullptr, *table_m = nullptr, *table_v = nullptr;
	float *mlp = nullptr, *mlp_g = nullptr, *mlp_m = nullptr, *mlp_v = nullptr;
	float *partial = nullptr;
	size_t partial_blocks = 0;
	float *loss = nullptr;    // [0] loss, [1] record weight sum
	uint32_t *tc_err = nullptr; // set by the tensor-core kernels when an MMA wait times out
	uint4 *enc = nullptr;       // BF16 encodings of the eval queue (stream-ordered, grown on demand)
	size_t enc_cap = 0;
	int eval_mode = GBRT_GUIDE_EVAL_TENSOR;
	int step = 0;
	int n_sm = 0;
};

namespace {

int guide_alloc(gbrt_guide *G)
{
	const size_t T = G->table_floats;
	float **bufs[] = {&G->table, &G->table_g, &G->table_m, &G->table_v};
	for(float **b : bufs) GBRT_CK(cudaMalloc(b, T * sizeof(float)));
	float **mb[] = {&G->mlp, &G->mlp_g, &G->mlp_m, &G->mlp_v};
	for(float **b : mb) GBRT_CK(cudaMalloc(b, kMlpParams * sizeof(float)));
	GBRT_CK(cudaMalloc(&G->loss, 2 * sizeof(float)));
	GBRT_CK(cudaMalloc(&G->tc_err, sizeof(uint32_t)));
	GBRT_CK(cudaMemset(G->tc_err, 0, sizeof(uint32_t)));
	return GBRT_OK;
}

// Forward pass of a queue of positions on the selected units.
int launch_eval(gbrt_guide *G, const float *pos, uint32_t cap, const uint32_t *count_dev, float *lobes, cudaStream_t s)
{
	if(G->eval_mode == GBRT_GUIDE_EVAL_TENSOR)
	{
		static bool attr = false;
		if(!attr) { GBRT_CK(cudaFuncSetAttribute(k_guide_eval_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmTotal))); attr = true; }
		if(cap > G->enc_cap)
		{
			if(G->enc) GBRT_CK(cudaFreeAsync(G->enc, s));
			G->enc = nullptr;
			GBRT_CK(cudaMallocAsync(reinterpret_cast<void **>(&G->enc), static_cast<size_t>(cap) * (kGuideIn * 2), s));
			G->enc_cap = cap;
		}
		const unsigned egrid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((static_cast<size_t>(cap) + kEncThreads - 1) / kEncThreads,
		                                                                                static_cast<size_t>(G->n_sm) * 8)));
		k_guide_encode<<<egrid, kEncThreads, 0, s>>>(G->grid, G->table, pos, cap, count_dev, G->enc);
		const size_t tiles = (static_cast<size_t>(cap) + 127) / 128;
		const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(tiles, static_cast<size_t>(G->n_sm) * 4)));
		k_guide_eval_tc<<<grid, kTcThreads, kSmTotal, s>>>(G->grid, G->table, G->mlp, pos, cap, count_dev, lobes, G->tc_err, G->enc);
	}
	else
	{
		const unsigned grid = static_cast<unsigned>(std::min<size_t>((cap + kEvalThreads - 1) / kEvalThreads, static_cast<size_t>(G->n_sm) * 8));
		k_guide_eval<<<std::max(1u, grid), kEvalThreads, 0, s>>>(G->grid, G->table, G->mlp, pos, cap, count_dev, lobes);
	}
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

size_t grad_smem_bytes()
{
	return sizeof(float) * (2 * kMlpParams + kGradThreads * (kGuideIn + 4 * kGuideHidden + kGuideOut));
}

} // namespace

namespace {
GuideGrid make_grid(const float bound[6], const gbrt_guide_params &p);
gbrt_guide_params defaults(const gbrt_guide_params *params);
} // namespace

extern "C" {

int gbrt_guide_create(const float bound[6], const gbrt_guide_params *params, gbrt_guide **out)
{
	if(!out || !bound) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_create: NULL argument");
	*out = nullptr;
	const gbrt_guide_params p = defaults(params);
	if(p.log2_table < 8 || p.log2_table > 24) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_create: log2_table %u out of [8, 24]", p.log2_table);
	gbrt_guide *G = new gbrt_guide();
	G->params = p;
	G->grid = make_grid(bound, p);
	G->table_floats = static_cast<size_t>(kGuideLevels) * kGuideFeatures << p.log2_table;
	cudaGetDevice(&G->device);
	cudaDeviceGetAttribute(&G->n_sm, cudaDevAttrMultiProcessorCount, G->device);
	if(int rc = guide_alloc(G)) { gbrt_guide_destroy(G); return rc; }
	// init: table U[-1e-4, 1e-4], MLP uniform(+-sqrt(6/fan_in)) (He), zero biases
	std::mt19937 rng(p.seed ? p.seed : 1234u);
	std::vector<float> tab(G->table_floats);
	std::uniform_real_distribution<float> ut(-1e-4f, 1e-4f);
	for(auto &x : tab) x = ut(rng);
	std::vector<float> w(kMlpParams, 0.f);
	auto fill = [&](int off, int rows, int cols, float scale) {
		std::uniform_real_distribution<float> u(-scale, scale);
		for(int i = 0; i < rows * cols; ++i) w[off + i] = u(rng);
	};
	fill(kOffW1, kGuideHidden, kGuideIn, std::sqrt(6.f / kGuideIn));
	fill(kOffW2, kGuideHidden, kGuideHidden, std::sqrt(6.f / kGuideHidden));
	fill(kOffW3, kGuideOut, kGuideHidden, 0.5f * std::sqrt(6.f / kGuideHidden));
	// mean-direction biases spread over the sphere, small kappa, equal weights
	for(int k = 0; k < kGuideLobes; ++k)
	{
		const float z = 1.f - 2.f * (k + 0.5f) / kGuideLobes, phi = 2.399963f * k, r = std::sqrt(std::max(0.f, 1.f - z * z));
		w[kOffB3 + 5 * k + 0] = r * std::cos(phi);
		w[kOffB3 + 5 * k + 1] = r * std::sin(phi);
		w[kOffB3 + 5 * k + 2] = z;
	}
	cudaError_t e;
	if((e = cudaMemcpy(G->table, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
	   (e = cudaMemcpy(G->mlp, w.data(), kMlpParams * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
	   (e = cudaMemset(G->table_g, 0, G->table_floats * 4)) != cudaSuccess || (e = cudaMemset(G->table_m, 0, G->table_floats * 4)) != cudaSuccess ||
	   (e = cudaMemset(G->table_v, 0, G->table_floats * 4)) != cudaSuccess || (e = cudaMemset(G->mlp_g, 0, kMlpParams * 4)) != cudaSuccess ||
	   (e = cudaMemset(G->mlp_m, 0, kMlpParams * 4)) != cudaSuccess || (e = cudaMemset(G->mlp_v, 0, kMlpParams * 4)) != cudaSuccess)
	{
		gbrt_guide_destroy(G);
		return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_guide_create: %s", cudaGetErrorString(e));
	}
	*out = G;
	return GBRT_OK;
}

int gbrt_guide_destroy(gbrt_guide *G)
{
	if(!G) return GBRT_OK;
	void *ptrs[] = {G->table, G->table_g, G->table_m, G->table_v, G->mlp, G->mlp_g, G->mlp_m, G->mlp_v, G->partial, G->loss, G->tc_err};
	if(G->enc) { cudaDeviceSynchronize(); cudaFree(G->enc); }
	for(void *p : ptrs) if(p) cudaFree(p);
	delete G;
	return GBRT_OK;
}

int gbrt_guide_get_params(const gbrt_guide *G, float *mlp_out, float *table_out)
{
	if(!G) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_get_params: NULL");
	if(mlp_out) GBRT_CK(cudaMemcpy(mlp_out, G->mlp, kMlpParams * 4, cudaMemcpyDeviceToHost));
	if(table_out) GBRT_CK(cudaMemcpy(table_out, G->table, G->table_floats * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_guide_set_params(gbrt_guide *G, const float *mlp, const float *table)
{
	if(!G) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_set_params: NULL");
	if(mlp) GBRT_CK(cudaMemcpy(G->mlp, mlp, kMlpParams * 4, cudaMemcpyHostToDevice));
	if(table) GBRT_CK(cudaMemcpy(G->table, table, G->table_floats * 4, cudaMemcpyHostToDevice));
	return GBRT_OK;
}

int gbrt_guide_eval(gbrt_guide *G, const float *pos_dev, uint32_t n, float *lobes_dev, void *stream)
{
	if(!G || (n && (!pos_dev || !lobes_dev))) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_eval: NULL argument");
	if(n == 0) return GBRT_OK;
	return launch_eval(G, pos_dev, n, nullptr, lobes_dev, static_cast<cudaStream_t>(stream));
}

int gbrt_guide_set_eval_mode(gbrt_guide *G, int mode)
{
	if(!G) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_set_eval_mode: NULL");
	if(mode != GBRT_GUIDE_EVAL_TENSOR && mode != GBRT_GUIDE_EVAL_FP32)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_set_eval_mode: unknown mode %d", mode);
	G->eval_mode = mode;
	return GBRT_OK;
}

int gbrt_guide_status(gbrt_guide *G, uint32_t *flags)
{
	if(!G || !flags) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_status: NULL");
	GBRT_CK(cudaMemcpy(flags, G->tc_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
	GBRT_CK(cudaMemset(G->tc_err, 0, sizeof(uint32_t)));
	return GBRT_OK;
}

int gbrt_tc_selftest(const float *A, const float *B, uint32_t N, uint32_t K, float *D)
{
	if(!A || !B || !D) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_tc_selftest: NULL argument");
	if(N < 16 || N > 64 || N % 16 || K < 16 || K > 64 || K % 16)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_tc_selftest: N=%u K=%u (each a multiple of 16 in [16, 64])", N, K);
	float *dA = nullptr, *dB = nullptr, *dD = nullptr;
	uint32_t *dErr = nullptr, herr = 0;
	cudaError_t e = cudaMalloc(&dA, 128ull * K * 4);
	if(e == cudaSuccess) e = cudaMalloc(&dB, static_cast<size_t>(N) * K * 4);
	if(e == cudaSuccess) e = cudaMalloc(&dD, 128ull * N * 4);
	if(e == cudaSuccess) e = cudaMalloc(&dErr, 4);
	if(e == cudaSuccess) e = cudaMemset(dErr, 0, 4);
	if(e == cudaSuccess) e = cudaMemcpy(dA, A, 128ull * K * 4, cudaMemcpyHostToDevice);
	if(e == cudaSuccess) e = cudaMemcpy(dB, B, static_cast<size_t>(N) * K * 4, cudaMemcpyHostToDevice);
	if(e == cudaSuccess) e = cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmTotal));
	if(e == cudaSuccess)
	{
		k_tc_selftest<<<1, kTcThreads, kSmTotal>>>(dA, dB, N, K, dD, dErr);
		e = cudaGetLastError();
	}
	if(e == cudaSuccess) e = cudaMemcpy(D, dD, 128ull * N * 4, cudaMemcpyDeviceToHost);
	if(e == cudaSuccess) e = cudaMemcpy(&herr, dErr, 4, cudaMemcpyDeviceToHost);
	cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dErr);
	if(e != cudaSuccess) return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_tc_selftest: %s", cudaGetErrorString(e));
	if(herr) return gbrt_set_error(GBRT_ERR_CUDA, "gbrt_tc_selftest: MMA completion wait timed out");
	return GBRT_OK;
}

// Gradient of the batch loss into the gradient buffers (no update).
int gbrt_guide_grad(gbrt_guide *G, const float *records_dev, uint32_t n, float *loss_out, void *stream)
{
	if(!G || (n && !records_dev)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_grad: NULL argument");
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	const size_t per_block = static_cast<size_t>(kGradThreads) * kGradChunks;
	const size_t nblk = std::max<size_t>({1, (n + per_block - 1) / per_block, static_cast<size_t>(G->n_sm)});
	if(nblk > G->partial_blocks)
	{
		if(G->partial) cudaFree(G->partial);
		GBRT_CK(cudaMalloc(&G->partial, nblk * kMlpParams * sizeof(float)));
		G->partial_blocks = nblk;
	}
	static bool attr = false;
	if(!attr)
	{
		GBRT_CK(cudaFuncSetAttribute(k_guide_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(grad_smem_bytes())));
		GBRT_CK(cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTrTotal)));
		attr = true;
	}
	GBRT_CK(cudaMemsetAsync(G->loss, 0, 2 * sizeof(float), s));
	k_weight_sum<<<std::max(1, std::min(G->n_sm * 4, static_cast<int>((n + 255) / 256))), 256, 0, s>>>(records_dev, n, G->loss + 1);
	size_t used = nblk;
	if(G->eval_mode == GBRT_GUIDE_EVAL_TENSOR)
	{
		// one CTA per SM (176 KB of shared memory, 256 TMEM columns each)
		const size_t tiles = (static_cast<size_t>(n) + 127) / 128;
		used = std::min<size_t>(tiles, static_cast<size_t>(G->n_sm));
		if(used)
			k_guide_train_tc<<<static_cast<unsigned>(used), kTrThreads, kTrTotal, s>>>(G->grid, G->table, G->mlp, records_dev, n, G->loss + 1,
			                                                                          G->partial, G->table_g, G->loss, G->tc_err);
	}
	else
		k_guide_grad<<<static_cast<unsigned>(nblk), kGradThreads, grad_smem_bytes(), s>>>(G->grid, G->table, G->mlp, records_dev, n, G->loss + 1,
		                                                                                  G->partial, G->table_g, G->loss);
	k_reduce<<<(kMlpParams + 255) / 256, 256, 0, s>>>(G->partial, static_cast<int>(used), G->mlp_g);
	GBRT_CK(cudaGetLastError());
	if(loss_out)
	{
		GBRT_CK(cudaMemcpyAsync(loss_out, G->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
		GBRT_CK(cudaStreamSynchronize(s));
	}
	return GBRT_OK;
}

int gbrt_guide_get_grads(const gbrt_guide *G, float *mlp_grad, float *table_grad)
{
	if(!G) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_get_grads: NULL");
	if(mlp_grad) GBRT_CK(cudaMemcpy(mlp_grad, G->mlp_g, kMlpParams * 4, cudaMemcpyDeviceToHost));
	if(table_grad) GBRT_CK(cudaMemcpy(table_grad, G->table_g, G->table_floats * 4, cudaMemcpyDeviceToHost));
	return GBRT_OK;
}

int gbrt_guide_step(gbrt_guide *G, const float *records_dev, uint32_t n, float *loss_out, void *stream)
{
	if(int rc = gbrt_guide_grad(G, records_dev, n, loss_out, stream)) return rc;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	G->step += 1;
	const float b1 = 0.9f, b2 = 0.99f;
	const float c1 = 1.f - std::pow(b1, static_cast<float>(G->step)), c2 = 1.f - std::pow(b2, static_cast<float>(G->step));
	const float lr = G->params.learning_rate;
	k_adam<<<64, 256, 0, s>>>(G->mlp, G->mlp_g, G->mlp_m, G->mlp_v, kMlpParams, lr, b1, b2, 1e-8f, c1, c2, 0);
	const unsigned gblocks = static_cast<unsigned>(std::min<size_t>((G->table_floats + 255) / 256, static_cast<size_t>(G->n_sm) * 16));
	k_adam<<<gblocks, 256, 0, s>>>(G->table, G->table_g, G->table_m, G->table_v, G->table_floats, lr, b1, b2, 1e-15f, c1, c2, 1);
	GBRT_CK(cudaGetLastError());
	return GBRT_OK;
}

int gbrt_guide_info(const gbrt_guide *G, uint32_t *n_mlp_params, uint64_t *n_table_params)
{
	if(!G) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_info: NULL");
	if(n_mlp_params) *n_mlp_params = kMlpParams;
	if(n_table_params) *n_table_params = G->table_floats;
	return GBRT_OK;
}

} // extern "C"

// Host build of the same forward pass (no CUDA calls): tests compare it with
// the FP64 oracle without a GPU, and with the device kernel on one.
namespace {
GuideGrid make_grid(const float bound[6], const gbrt_guide_params &p)
{
	GuideGrid g{};
	for(int a = 0; a < 3; ++a)
	{
		const float ext = bound[3 + a] - bound[a];
		g.lo[a] = bound[a];
		g.inv_ext[a] = ext > 0.f ? 1.f / ext : 0.f;
	}
	g.log2_table = p.log2_table;
	const double b = std::exp((std::log(static_cast<double>(p.max_resolution)) - std::log(static_cast<double>(p.base_resolution))) / (kGuideLevels - 1));
	for(int l = 0; l < kGuideLevels; ++l)
	{
		g.res[l] = std::floor(static_cast<float>(static_cast<double>(p.base_resolution) * std::pow(b, l)));
		const double cells = std::pow(g.res[l] + 1.0, 3.0);
		g.dense[l] = cells <= static_cast<double>(1u << p.log2_table) ? 1u : 0u;
	}
	return g;
}
gbrt_guide_params defaults(const gbrt_guide_params *params)
{
	gbrt_guide_params p{};
	if(params) p = *params;
	if(p.log2_table == 0) p.log2_table = 19;
	if(p.base_resolution <= 0.f) p.base_resolution = 16.f;
	if(p.max_resolution <= 0.f) p.max_resolution = 2048.f;
	if(p.learning_rate <= 0.f) p.learning_rate = 5e-3f;
	return p;
}
} // namespace

extern "C" int gbrt_guide_forward_host(const float bound[6], const gbrt_guide_params *params, const float *mlp, const float *table,
                                       const float *pos, uint32_t n, float *lobes)
{
	if(!bound || !mlp || !table || (n && (!pos || !lobes))) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_forward_host: NULL argument");
	const gbrt_guide_params p = defaults(params);
	if(p.log2_table < 8 || p.log2_table > 24) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_guide_forward_host: log2_table out of range");
	const GuideGrid g = make_grid(bound, p);
	for(uint32_t s = 0; s < n; ++s)
	{
		float e[kGuideIn], h1[kGuideHidden], h2[kGuideHidden], o[kGuideOut];
		encode(g, table, pos + 3ull * s, e, nullptr, nullptr);
		mlp_forward(mlp, e, h1, h2, o);
		raw_to_lobes(o, lobes + static_cast<size_t>(kGuideOut) * s);
	}
	return GBRT_OK;
}

// Used by the path tracer: lobes for the hit points of a queue.
int gbrt_guide_eval_queue(gbrt_guide *G, const float *pos_dev, uint32_t cap, const uint32_t *count_dev, float *lobes_dev, cudaStream_t s)
{
	return launch_eval(G, pos_dev, cap, count_dev, lobes_dev, s);
}
