// Device helpers of the guiding mixture (shared by the network kernels and
// the path tracer): lobe parameters, vMF density and sampling.
#pragma once

#include "guide_common.cuh"

#include <cmath>

namespace gbrt {

GBRT_GHD float softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

// raw network outputs -> per lobe {mu xyz (unit), kappa, weight (softmax)}
GBRT_GHD void raw_to_lobes(const float o[kGuideOut], float out[kGuideOut])
{
	float mx = -1e30f;
	for(int k = 0; k < kGuideLobes; ++k) mx = fmaxf(mx, o[5 * k + 4]);
	float sum = 0.f;
	for(int k = 0; k < kGuideLobes; ++k) { out[5 * k + 4] = expf(o[5 * k + 4] - mx); sum += out[5 * k + 4]; }
	const float inv = 1.f / sum;
	for(int k = 0; k < kGuideLobes; ++k)
	{
		out[5 * k + 4] *= inv;
		const float m0 = o[5 * k], m1 = o[5 * k + 1], m2 = o[5 * k + 2];
		const float len = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
		if(len > 1e-20f) { out[5 * k] = m0 / len; out[5 * k + 1] = m1 / len; out[5 * k + 2] = m2 / len; }
		else { out[5 * k] = 0.f; out[5 * k + 1] = 0.f; out[5 * k + 2] = 1.f; }
		out[5 * k + 3] = fminf(softplus(o[5 * k + 3]) + kKappaMin, kKappaMax);
	}
}

// log of the von Mises-Fisher density on the sphere:
// kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa (mu.w - 1))
GBRT_GHD float vmf_log_pdf(const float mu[3], float kappa, const float w[3])
{
	const float mw = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
	return logf(kappa) - logf(kTwoPiF) - logf(-expm1f(-2.f * kappa)) + kappa * (mw - 1.f);
}

GBRT_GHD float mixture_pdf(const float *lobes, const float w[3])
{
	float p = 0.f;
	for(int k = 0; k < kGuideLobes; ++k)
		p += lobes[5 * k + 4] * expf(vmf_log_pdf(&lobes[5 * k], lobes[5 * k + 3], w));
	return p;
}

// Sample the mixture: lobe by u0, then the vMF by (u1, u2) with the
// numerically stable inversion w = 1 + log(u1 + (1 - u1) exp(-2 kappa)) / kappa.
GBRT_GHD void mixture_sample(const float *lobes, float u0, float u1, float u2, float out[3])
{
	int k = kGuideLobes - 1;
	float acc = 0.f;
	for(int j = 0; j < kGuideLobes; ++j)
	{
		acc += lobes[5 * j + 4];
		if(u0 < acc) { k = j; break; }
	}
	const float *mu = &lobes[5 * k];
	const float kap = lobes[5 * k + 3];
	float wz = 1.f + logf(u1 + (1.f - u1) * expf(-2.f * kap)) / kap;
	wz = fminf(fmaxf(wz, -1.f), 1.f);
	const float r = sqrtf(fmaxf(0.f, 1.f - wz * wz));
	float sphi, cphi;
	sincosf(kTwoPiF * u2, &sphi, &cphi);
	// orthonormal frame around mu (Duff et al. 2017)
	const float sgn = copysignf(1.f, mu[2]);
	const float a = -1.f / (sgn + mu[2]);
	const float b = mu[0] * mu[1] * a;
	const float t[3] = {1.f + sgn * mu[0] * mu[0] * a, sgn * b, -sgn * mu[0]};
	const float bt[3] = {b, sgn + mu[1] * mu[1] * a, -mu[1]};
	for(int c = 0; c < 3; ++c) out[c] = r * cphi * t[c] + r * sphi * bt[c] + wz * mu[c];
}

} // namespace gbrt
