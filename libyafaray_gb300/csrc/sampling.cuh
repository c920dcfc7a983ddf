// Sample streams of the reference path integrator, restated for host and
// device with the reference's exact float/double operation order (explicit
// round-to-nearest intrinsics on the device, so no multiply-add fusion):
//   - riVdC / riLp / riS base-2 sequences and fnv32ABuf pixel hashing
//     (include/sampler/sample.h:100-148)
//   - radical inverse in base b as Halton::getNext produces it
//     (include/sampler/halton.h:59-85)
//   - Faure-scrambled Halton "lowDiscrepancySampling" (src/sampler/halton.cc:419-439),
//     with the permutations generated by Faure's recursive construction and
//     1/p rounded to nine decimals as the reference tabulates it
//   - the FAST_TRIG parabolic sine/cosine approximation (include/math/math.h:228-265),
//     the published two-term parabola with the 0.225 refinement
#pragma once

#include <cstdint>
#include <cmath>
#include <cstring>
#include <vector>

#if defined(__CUDACC__)
#define GBRT_HD __host__ __device__ __forceinline__
#else
#define GBRT_HD inline
#endif

namespace gbrt {

constexpr int kLdsDims = 50;           // dims 1..49 are tabulated (dim 0 is unused)

// Device-resident tables for lowDiscrepancySampling.
struct LdsTables {
	const uint16_t *perm;              // concatenated permutations
	const uint32_t *perm_offset;       // [kLdsDims]
	const uint32_t *base;              // [kLdsDims]
	const double *inv;                 // [kLdsDims] 1/base rounded to 9 decimals
};

GBRT_HD float fmul(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fmul_rn(a, b);
#else
	return a * b;
#endif
}
GBRT_HD float fadd(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fadd_rn(a, b);
#else
	return a + b;
#endif
}
GBRT_HD float fsub(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fsub_rn(a, b);
#else
	return a - b;
#endif
}
GBRT_HD double dmul(double a, double b)
{
#if defined(__CUDA_ARCH__)
	return __dmul_rn(a, b);
#else
	return a * b;
#endif
}
GBRT_HD double dadd(double a, double b)
{
#if defined(__CUDA_ARCH__)
	return __dadd_rn(a, b);
#else
	return a + b;
#endif
}

GBRT_HD float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }

constexpr double kTwoPowMinus32 = 0.00000000023283064365386962890625;

GBRT_HD uint32_t bit_reverse(uint32_t b)
{
#if defined(__CUDA_ARCH__)
	return __brev(b);
#else
	b = (b << 16) | (b >> 16);
	b = ((b & 0x00ff00ffu) << 8) | ((b & 0xff00ff00u) >> 8);
	b = ((b & 0x0f0f0f0fu) << 4) | ((b & 0xf0f0f0f0u) >> 4);
	b = ((b & 0x33333333u) << 2) | ((b & 0xccccccccu) >> 2);
	b = ((b & 0x55555555u) << 1) | ((b & 0xaaaaaaaau) >> 1);
	return b;
#endif
}

// van der Corput: bit-reversed index as a fraction
GBRT_HD float ri_vdc(uint32_t bits, uint32_t r = 0)
{
	return clamp01(static_cast<float>(dmul(static_cast<double>(bit_reverse(bits) ^ r), kTwoPowMinus32)));
}

// Larcher & Pillichshammer
GBRT_HD float ri_lp(uint32_t i, uint32_t r = 0)
{
	for(uint32_t v = 1u << 31; i; i >>= 1, v |= v >> 1)
		if(i & 1u) r ^= v;
	return clamp01(static_cast<float>(dmul(static_cast<double>(r), kTwoPowMinus32)));
}

// Sobol' second dimension
GBRT_HD float ri_s(uint32_t i, uint32_t r = 0)
{
	for(uint32_t v = 1u << 31; i; i >>= 1, v ^= v >> 1)
		if(i & 1u) r ^= v;
	return clamp01(static_cast<float>(dmul(static_cast<double>(r), kTwoPowMinus32)));
}

// FNV-1a over the four bytes of a 32-bit value, lowest byte first
GBRT_HD uint32_t fnv32(uint32_t value)
{
	uint32_t h = 0x811c9dc5u;
	for(int k = 0; k < 4; ++k)
	{
		h ^= (value >> (8 * k)) & 0xffu;
		h *= 0x01000193u;
	}
	return h;
}

// Radical inverse of n in base b (the value Halton(b, n - 1).getNext() returns).
GBRT_HD float radical_inverse(uint32_t n, uint32_t b)
{
	const double inv = 1.0 / static_cast<double>(b);
	double f = inv, v = 0.0;
	while(n > 0)
	{
		v = dadd(v, dmul(static_cast<double>(n % b), f));
		n /= b;
		f = dmul(f, inv);
	}
	return clamp01(static_cast<float>(v));
}

// Faure-scrambled Halton, digit extraction with the 9-decimal inverse as the
// reference does it (so multiples of the base round like the reference).
GBRT_HD double low_discrepancy(const LdsTables &t, int dim, uint32_t n)
{
	const uint16_t *sigma = t.perm + t.perm_offset[dim];
	const uint32_t base = t.base[dim];
	const double f = t.inv[dim];
	if(base < 2) return 0.0;
	double value = 0.0, dn = static_cast<double>(n), factor = f;
	while(n > 0)
	{
		value = dadd(value, dmul(static_cast<double>(sigma[n % base]), factor));
		dn = dmul(dn, f);
		n = static_cast<uint32_t>(dn);
		factor = dmul(factor, f);
	}
	return value;
}

// FAST_TRIG sine: wrap to [-pi, pi], parabola 4/pi x - 4/pi^2 x|x|, then the
// 0.225 blend towards the squared parabola; clamped to [-1, 1].
GBRT_HD float fast_sin(float x)
{
	const float two_pi = 6.28318530717958647692f, inv_two_pi = 0.15915494309189533577f, pi = 3.14159265358979323846f;
	const float c1 = 1.27323954473516268615f, c2 = 0.40528473456935108578f;
	if(x > two_pi || x < -two_pi) x = fsub(x, fmul(static_cast<float>(static_cast<int>(fmul(x, inv_two_pi))), two_pi));
	if(x < -pi) x = fadd(x, two_pi);
	else if(x > pi) x = fsub(x, two_pi);
	x = fsub(fmul(c1, x), fmul(fmul(c2, x), fabsf(x)));
	const float r = fadd(fmul(0.225f, fsub(fmul(x, fabsf(x)), x)), x);
	if(r <= -1.f) return -1.f;
	if(r >= 1.f) return 1.f;
	return r;
}
GBRT_HD float fast_cos(float x) { return fast_sin(fadd(x, 1.57079632679489661923f)); }

// FAST_MATH pow (include/math/math.h:116-146, 177-183): exp2(log2(a) * b)
// with fifth-degree polynomial approximations of exp2 on the fractional part
// and of log2 on the mantissa (exponent bits taken directly).
GBRT_HD float bits_to_float(int32_t i)
{
#if defined(__CUDA_ARCH__)
	return __int_as_float(i);
#else
	float f;
	std::memcpy(&f, &i, 4);
	return f;
#endif
}
GBRT_HD int32_t float_to_bits(float f)
{
#if defined(__CUDA_ARCH__)
	return __float_as_int(f);
#else
	int32_t i;
	std::memcpy(&i, &f, 4);
	return i;
#endif
}
GBRT_HD float poly_exp2(float x)
{
	return fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, 1.8775767e-3f), 8.9893397e-3f)), 5.5826318e-2f)), 2.4015361e-1f)), 6.9315308e-1f)), 9.9999994e-1f);
}
GBRT_HD float fast_exp2(float x)
{
	const float xl = fmaxf(fminf(x, 129.00000f), -126.99999f);
	const int32_t ipart = static_cast<int32_t>(fsub(xl, 0.5f));
	const float fpart = fsub(xl, static_cast<float>(ipart));
	return fmul(bits_to_float((ipart + 127) << 23), poly_exp2(fpart));
}
GBRT_HD float poly_log2(float x)
{
	return fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, fadd(fmul(x, -3.4436006e-2f), 3.1821337e-1f)), -1.2315303f)), 2.5988452f)), -3.3241990f)), 3.1157899f);
}
GBRT_HD float fast_log2(float x)
{
	const int32_t i = float_to_bits(x);
	const float m = bits_to_float((i & 0x7FFFFF) | float_to_bits(1.f));
	const float e = static_cast<float>(((i & 0x7F800000) >> 23) - 127);
	return fadd(fmul(poly_log2(m), fsub(m, 1.f)), e);
}
GBRT_HD float fast_pow(float a, float b) { return fast_exp2(fmul(fast_log2(a), b)); }

// ---- host-side table construction -------------------------------------------
inline std::vector<uint32_t> lds_bases()
{
	std::vector<uint32_t> b = {1u};
	for(uint32_t p = 2; b.size() < static_cast<size_t>(kLdsDims); ++p)
	{
		bool prime = true;
		for(uint32_t q = 2; q * q <= p; ++q)
			if(p % q == 0) { prime = false; break; }
		if(prime) b.push_back(p);
	}
	return b;
}

// Faure's permutation of {0..b-1}: sigma_2 = (0,1); even b = 2c: (2 sigma_c,
// 2 sigma_c + 1); odd b = 2c + 1: sigma_{2c} with every value >= c raised by
// one and c inserted in the middle.
inline std::vector<uint16_t> faure_permutation(uint32_t b)
{
	if(b <= 1) return {0};
	if(b == 2) return {0, 1};
	if(b % 2 == 0)
	{
		const auto s = faure_permutation(b / 2);
		std::vector<uint16_t> r;
		for(auto v : s) r.push_back(static_cast<uint16_t>(2 * v));
		for(auto v : s) r.push_back(static_cast<uint16_t>(2 * v + 1));
		return r;
	}
	const uint32_t c = (b - 1) / 2;
	auto s = faure_permutation(b - 1);
	for(auto &v : s) if(v >= c) ++v;
	s.insert(s.begin() + c, static_cast<uint16_t>(c));
	return s;
}

struct LdsHostTables {
	std::vector<uint16_t> perm;
	std::vector<uint32_t> offset, base;
	std::vector<double> inv;
};

inline LdsHostTables make_lds_tables()
{
	LdsHostTables t;
	const auto bases = lds_bases();
	for(int d = 0; d < kLdsDims; ++d)
	{
		const uint32_t b = bases[d];
		t.offset.push_back(static_cast<uint32_t>(t.perm.size()));
		t.base.push_back(b);
		t.inv.push_back(std::round(1e9 / static_cast<double>(b)) / 1e9);
		const auto p = faure_permutation(b < 2 ? 2 : b);
		t.perm.insert(t.perm.end(), p.begin(), p.end());
	}
	return t;
}

} // namespace gbrt
