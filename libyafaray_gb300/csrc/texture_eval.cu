// Procedural texture defaults and the diagnostics entry gbrt_texture_eval:
// a texture's getColor / getFloat at given texture-space points, on the
// host or in a kernel, with the same code the renderer's texture lookups
// run (procedural.cuh).  Compiled without floating-point contraction.
#include "gbrt.h"
#include "gbrt_internal.cuh"
#include "procedural.cuh"

#include <cstring>
#include <vector>

namespace {

__global__ void k_texture_eval(gbrt::ProcTex t, gbrt::NoiseTables T, const float *__restrict__ pts, uint32_t n, float4 *__restrict__ rgba,
                               float *__restrict__ val)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float p[3] = {pts[3ull * i], pts[3ull * i + 1], pts[3ull * i + 2]};
	float c[4];
	gbrt::proc_color(T, t, p, c);
	rgba[i] = make_float4(c[0], c[1], c[2], c[3]);
	val[i] = gbrt::proc_float(T, t, p);
}

} // namespace

extern "C" {

void gbrt_procedural_defaults(gbrt_procedural_desc *d)
{
	if(!d) return;
	std::memset(d, 0, sizeof *d);
	d->noise_type = d->noise_type2 = GBRT_NOISE_NEWPERLIN;
	for(int k = 0; k < 3; ++k) { d->color1[k] = 0.f; d->color2[k] = 1.f; }
	d->size = 1.f;
	d->depth = 2;
	d->sharpness = 1.f;
	d->turbulence = 1.f;
	d->weight[0] = 1.f;
	d->mk_exponent = 2.5f;
	d->intensity = 1.f;
	d->h = 1.f; d->lacunarity = 2.f; d->octaves = 2.f; d->offset = 1.f; d->gain = 1.f;
	d->distort = 1.f;
}

int gbrt_texture_eval(const gbrt_texture_desc *texture, const gbrt_noise_tables *tables, const float *points, uint32_t n, float *rgba,
                      float *value, int on_device)
{
	if(!texture || !tables || !tables->hash || !tables->hashpntf || !tables->hashvectf || !tables->stdp_p || !tables->stdp_g ||
	   (n && (!points || !rgba || !value)))
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_texture_eval: NULL argument");
	if(texture->kind == GBRT_TEX_IMAGE || texture->kind > GBRT_TEX_RGB_CUBE)
		return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_texture_eval: kind %u is not procedural", texture->kind);
	gbrt::ProcTex t;
	if(!gbrt::proc_from_desc(*texture, t)) return gbrt_set_error(GBRT_ERR_INVALID, "gbrt_texture_eval: ramp of %d items", texture->proc.ramp_n);
	if(n == 0) return GBRT_OK;
	if(!on_device)
	{
		const gbrt::NoiseTables T{tables->hash, tables->hashpntf, tables->hashvectf, tables->stdp_p, tables->stdp_g};
		for(uint32_t i = 0; i < n; ++i)
		{
			gbrt::proc_color(T, t, points + 3ull * i, rgba + 4ull * i);
			value[i] = gbrt::proc_float(T, t, points + 3ull * i);
		}
		return GBRT_OK;
	}
	// device: the tables, points and outputs in one temporary allocation
	const size_t b_tab = 512 + 520 + 4 * (768 + 768 + 514 * 3);
	const size_t o_pts = (b_tab + 255) & ~size_t(255), o_rgba = o_pts + ((12ull * n + 255) & ~size_t(255)),
	             o_val = o_rgba + 16ull * n, total = o_val + 4ull * n;
	std::vector<uint8_t> tab(b_tab, 0);
	std::memcpy(tab.data(), tables->hash, 512);
	std::memcpy(tab.data() + 512, tables->stdp_p, 514);
	std::memcpy(tab.data() + 1032, tables->hashpntf, 4 * 768);
	std::memcpy(tab.data() + 1032 + 4 * 768, tables->hashvectf, 4 * 768);
	std::memcpy(tab.data() + 1032 + 8 * 768, tables->stdp_g, 4 * 514 * 3);
	uint8_t *dev = nullptr;
	GBRT_CK(cudaMalloc(reinterpret_cast<void **>(&dev), total));
	cudaError_t e = cudaMemcpy(dev, tab.data(), b_tab, cudaMemcpyHostToDevice);
	if(e == cudaSuccess) e = cudaMemcpy(dev + o_pts, points, 12ull * n, cudaMemcpyHostToDevice);
	if(e == cudaSuccess)
	{
		const float *f = reinterpret_cast<const float *>(dev + 1032);
		const gbrt::NoiseTables T{dev, f, f + 768, dev + 512, f + 1536};
		k_texture_eval<<<(n + 127) / 128, 128>>>(t, T, reinterpret_cast<const float *>(dev + o_pts), n, reinterpret_cast<float4 *>(dev + o_rgba),
		                                         reinterpret_cast<float *>(dev + o_val));
		e = cudaGetLastError();
	}
	if(e == cudaSuccess) e = cudaMemcpy(rgba, dev + o_rgba, 16ull * n, cudaMemcpyDeviceToHost);
	if(e == cudaSuccess) e = cudaMemcpy(value, dev + o_val, 4ull * n, cudaMemcpyDeviceToHost);
	cudaFree(dev);
	GBRT_CK(e);
	return GBRT_OK;
}

} // extern "C"
