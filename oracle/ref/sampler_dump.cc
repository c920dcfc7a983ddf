// Test-oracle harness: evaluates the reference's sampling primitives
// (include/sampler/sample.h, src/sampler/halton.cc, include/math/math.h)
// on a fixed grid of inputs and writes them out, so the restated device
// versions can be compared value by value.  Only
// tests/golden/make_render_golden.py runs it.
// Output (binary, little endian):
//   i32 n_dims(=49), n_idx;  f64 lds[dims 1..49][n_idx]      Halton::lowDiscrepancySampling(dim, n)
//   f32 vdc[n_idx], lp[n_idx], s[n_idx]                        riVdC(n), riLp(n), riS(n)
//   u32 fnv[n_idx]                                            fnv32ABuf(n * 2654435761u)
//   f32 h2[n_idx], h3[n_idx]                                  Halton(2/3, start=1000).getNext() x n_idx
//   i32 n_ang; f32 ang[n_ang], sin[n_ang], cos[n_ang]          math::sin / math::cos (FAST_TRIG)
//   i32 n_pow; f32 base[n_pow], expo[n_pow], pow[n_pow]        math::pow (FAST_MATH exp2(log2(a) * b))
#include "sampler/halton.h"
#include "sampler/sample.h"
#include "math/random.h"
#include "math/math.h"
#include <cstdio>
#include <vector>

using namespace yafaray;

int main(int argc, char **argv)
{
	if(argc != 2) { fprintf(stderr, "usage: %s out.bin\n", argv[0]); return 2; }
	FILE *f = fopen(argv[1], "wb");
	if(!f) { perror("out"); return 2; }
	const int n_dims = 49, n_idx = 4096;
	fwrite(&n_dims, 4, 1, f);
	fwrite(&n_idx, 4, 1, f);
	FastRandom fr;
	for(int dim = 1; dim <= n_dims; ++dim)
		for(int n = 0; n < n_idx; ++n)
		{
			const unsigned int idx = static_cast<unsigned int>(n) * 7919u + static_cast<unsigned int>(dim);
			const double v = Halton::lowDiscrepancySampling(fr, dim, idx);
			fwrite(&v, 8, 1, f);
		}
	std::vector<float> a(n_idx), b(n_idx), c(n_idx);
	std::vector<unsigned int> h(n_idx);
	for(int n = 0; n < n_idx; ++n)
	{
		const unsigned int idx = static_cast<unsigned int>(n) * 2654435761u;
		a[n] = sample::riVdC(idx);
		b[n] = sample::riLp(idx);
		c[n] = sample::riS(idx);
		h[n] = sample::fnv32ABuf(idx);
	}
	fwrite(a.data(), 4, n_idx, f); fwrite(b.data(), 4, n_idx, f); fwrite(c.data(), 4, n_idx, f);
	fwrite(h.data(), 4, n_idx, f);
	Halton h2(2, 1000), h3(3, 1000);
	for(int n = 0; n < n_idx; ++n) { a[n] = h2.getNext(); b[n] = h3.getNext(); }
	fwrite(a.data(), 4, n_idx, f); fwrite(b.data(), 4, n_idx, f);
	const int n_ang = 20001;
	fwrite(&n_ang, 4, 1, f);
	std::vector<float> ang(n_ang), s(n_ang), co(n_ang);
	for(int i = 0; i < n_ang; ++i)
	{
		ang[i] = -20.f + 40.f * static_cast<float>(i) / static_cast<float>(n_ang - 1);
		s[i] = math::sin(ang[i]);
		co[i] = math::cos(ang[i]);
	}
	fwrite(ang.data(), 4, n_ang, f); fwrite(s.data(), 4, n_ang, f); fwrite(co.data(), 4, n_ang, f);
	const int n_pow = 8192;
	fwrite(&n_pow, 4, 1, f);
	std::vector<float> pb(n_pow), pe(n_pow), pv(n_pow);
	for(int i = 0; i < n_pow; ++i)
	{
		pb[i] = -0.2f + 1.2f * static_cast<float>(i % 1024) / 1023.f;
		const float exps[8] = {1.f / 51.f, 1.f / 101.f, 1.f / 501.f, 0.5f, 50.f, 100.f, 500.f, 3.3f};
		pe[i] = exps[i / 1024];
		pv[i] = math::pow(pb[i], pe[i]);
	}
	fwrite(pb.data(), 4, n_pow, f); fwrite(pe.data(), 4, n_pow, f); fwrite(pv.data(), 4, n_pow, f);
	fclose(f);
	return 0;
}
