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
	// sigma[d] x factor_k as the reference's loop forms them (factor_0 = inv,
	// factor_{k+1} = factor_k x inv, both rounded in double): [digit k][d]
	const double *sfac;
	const uint32_t *sfac_offset;       // [kLdsDims]
	const uint32_t *sfac_digits;       // [kLdsDims] digits tabulated
	// integer tables of the FP64-free evaluation (low_discrepancy_f,
	// radical_inverse3_f): fixed-point terms at the sfac indices, then from
	// fx_dims one entry per dimension {reciprocal of the base (64 bits),
	// mantissa of inv (53 bits) with its exponent + 128 in the top byte},
	// and from fx_rad3 the base-3 radical-inverse terms
	const uint4 *fx;
	uint32_t fx_dims, fx_rad3;
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

// x * 2^-32 rounded to float: the reference forms it in double (exact, x <
// 2^32) and rounds once, which equals rounding x to float and scaling by
// the power of two.
GBRT_HD float u32_fraction(uint32_t x) { return clamp01(static_cast<float>(x) * 2.3283064365386962890625e-10f); }

// van der Corput: bit-reversed index as a fraction
GBRT_HD float ri_vdc(uint32_t bits, uint32_t r = 0)
{
	return u32_fraction(bit_reverse(bits) ^ r);
}

// Larcher & Pillichshammer
GBRT_HD float ri_lp(uint32_t i, uint32_t r = 0)
{
	for(uint32_t v = 1u << 31; i; i >>= 1, v |= v >> 1)
		if(i & 1u) r ^= v;
	return u32_fraction(r);
}

// Sobol' second dimension
GBRT_HD float ri_s(uint32_t i, uint32_t r = 0)
{
	for(uint32_t v = 1u << 31; i; i >>= 1, v ^= v >> 1)
		if(i & 1u) r ^= v;
	return u32_fraction(r);
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

// 3^-(k+1) as the loop below forms it in double (f_0 = 1/3, f_{k+1} = f_k / 3
// rounded), k = 0 .. 20.
#define GBRT_INV3_POW {0x1.5555555555555p-2, 0x1.c71c71c71c71cp-4, 0x1.2f684bda12f68p-5, 0x1.948b0fcd6e9e0p-7, \
	0x1.0db20a88f4695p-8, 0x1.67980e0bf08c6p-10, 0x1.df75680feb65dp-12, 0x1.3fa39ab547993p-13, 0x1.aa2f78f1b4cc4p-15, \
	0x1.1c1fa5f678882p-16, 0x1.7ad4dd48a0b58p-18, 0x1.f91bd1b62b9cap-20, 0x1.50bd367972686p-21, 0x1.c0fc48a1ede08p-23, \
	0x1.2b52db169e95ap-24, 0x1.8f19241e28c78p-26, 0x1.0a10c2bec5da5p-27, 0x1.62c103a907cdcp-29, 0x1.d9015a36b5125p-31, \
	0x1.3b563c2478b6ep-32, 0x1.a472fadb4b9e8p-34}
#if defined(__CUDACC__)
static __constant__ double c_inv3_pow[21] = GBRT_INV3_POW;
#endif
static constexpr double h_inv3_pow[21] = GBRT_INV3_POW;
GBRT_HD double inv3_pow(int k)
{
#if defined(__CUDA_ARCH__)
	return c_inv3_pow[k];
#else
	return h_inv3_pow[k];
#endif
}

// Radical inverse of n in base b (the value Halton(b, n - 1).getNext() returns).
// In base 2 every term and partial sum is exact in double, so the value is
// bitrev(n) x 2^-32 rounded once to float; in base 3 the digit products
// (0, 1 or 2 x 3^-(k+1)) are exact and only the additions round.  Both give
// the general loop's result bit for bit with far less FP64 work.
GBRT_HD float radical_inverse(uint32_t n, uint32_t b)
{
	if(b == 2) return clamp01(static_cast<float>(bit_reverse(n)) * 2.3283064365386962890625e-10f);
	if(b == 3)
	{
		double v = 0.0;
		for(int k = 0; n > 0; ++k)
		{
			const uint32_t d = n % 3u;
			n /= 3u;
			if(d) v = dadd(v, d == 1u ? inv3_pow(k) : 2.0 * inv3_pow(k));
		}
		return clamp01(static_cast<float>(v));
	}
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
	const uint32_t base = t.base[dim];
	if(base < 2) return 0.0;
	const double f = t.inv[dim];
	const double *sf = t.sfac + t.sfac_offset[dim];
	const uint32_t nd = t.sfac_digits[dim];
	double value = 0.0, dn = static_cast<double>(n);
	for(uint32_t k = 0; n > 0; ++k)
	{
		double term;
		if(k < nd) term = sf[k * base + n % base];
		else
		{
			// past the tabulated digits (not reached for 32-bit n): form the factor
			double factor = f;
			for(uint32_t j = 0; j < k; ++j) factor = dmul(factor, f);
			term = dmul(static_cast<double>(t.perm[t.perm_offset[dim] + n % base]), factor);
		}
		value = dadd(value, term);
		dn = dmul(dn, f);
		n = static_cast<uint32_t>(dn);
	}
	return value;
}

// ---- FP64-free evaluation of the same streams ------------------------------
// The integrators use lowDiscrepancySampling and the base-3 radical inverse
// as floats.  Here both are formed with integer arithmetic only: the digit
// chain dn *= f with the double multiply's rounding emulated on 53-bit
// mantissas (so every digit is the reference's), the digit terms (the
// reference's double terms, converted exactly) summed in 128-bit fixed
// point, then one rounding to float.  The reference's double sum differs
// from the exact sum by at most one rounding per addition, so the float
// equals (float) of the reference's double unless the exact sum lies within
// K 2^-53 of a float rounding midpoint (K = terms added); those inputs,
// about four in a million, take the double loop instead.

// 128-bit fixed point: value = (hi 2^64 + lo) x 2^-127
struct Fx128 {
	uint64_t hi, lo;
};

GBRT_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
	return __umul64hi(a, b);
#else
	return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

GBRT_HD int clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
	return __clzll(static_cast<long long>(x));
#else
	return x ? __builtin_clzll(x) : 64;
#endif
}

GBRT_HD Fx128 fx_load(const uint4 &e) { return Fx128{(static_cast<uint64_t>(e.w) << 32) | e.z, (static_cast<uint64_t>(e.y) << 32) | e.x}; }
GBRT_HD uint64_t fx_u64(uint32_t lo, uint32_t hi) { return (static_cast<uint64_t>(hi) << 32) | lo; }

GBRT_HD void fx_add(Fx128 &a, const Fx128 &b)
{
	a.lo += b.lo;
	a.hi += b.hi + (a.lo < b.lo ? 1u : 0u);
}

// The float nearest to the exact sum z, or false when the sum of k double
// roundings could move the reference's value across a rounding midpoint.
GBRT_HD bool fx_to_float(const Fx128 &z, uint32_t k, float &out)
{
	if(z.hi == 0 && z.lo == 0) { out = 0.f; return true; }
	// every term is >= 2^-64 here, so the leading bit lies in hi
	if(z.hi == 0) return false;
	const int p = 127 - clz64(z.hi);           // leading bit index of the 128-bit integer
	const int u = p - 23;                      // ulp bit index, >= 40
	// the bits below the ulp, compared with half an ulp: bits u-1 .. 0
	// (u > 64: all of lo and the low u - 64 bits of hi)
	uint64_t rem_hi, rem_lo;                   // remainder as (rem_hi:rem_lo) with u bits
	uint32_t mant;                             // the top 24 bits
	if(u >= 64)
	{
		rem_hi = u > 64 ? (z.hi & ((1ull << (u - 64)) - 1ull)) : 0ull;
		rem_lo = z.lo;
		mant = static_cast<uint32_t>(z.hi >> (u - 64));
	}
	else
	{
		rem_hi = 0ull;
		rem_lo = z.lo & ((1ull << u) - 1ull);
		mant = static_cast<uint32_t>((z.hi << (64 - u)) | (z.lo >> u));
	}
	// |remainder - half| in units of 2^(u - 40): the tolerance k 2^-53 x 2^(p+1)
	// = k 2^(u - 29) is k 2^11 such units
	const int sh = u - 40;                     // >= 0
	const uint64_t r40 = sh >= 64 ? (rem_hi >> (sh - 64)) : ((rem_hi << (64 - sh)) | (rem_lo >> sh));
	const uint64_t half40 = 1ull << 39;
	const uint64_t dist = r40 > half40 ? r40 - half40 : half40 - r40;
	if(dist <= (static_cast<uint64_t>(k) << 11) + 1ull) return false;
	const uint32_t m = mant + (r40 > half40 ? 1u : 0u);
	// value = m x 2^(u - 127), m in [2^23, 2^24]: biased exponent u + 23
	// (m = 2^24 carries into the exponent)
	const uint32_t fb = (static_cast<uint32_t>(u + 23) << 23) + (m - (1u << 23));
	std::memcpy(&out, &fb, 4);
	return true;
}

GBRT_HD int clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
	return __clz(static_cast<int>(x));
#else
	return x ? __builtin_clz(x) : 32;
#endif
}

GBRT_HD float low_discrepancy_f(const LdsTables &t, int dim, uint32_t n)
{
	const uint32_t b = t.base[dim];
	if(b < 2 || n == 0) return 0.f;
	const uint4 de = t.fx[t.fx_dims + dim];
	const uint64_t recip = fx_u64(de.x, de.y);
	const uint64_t mf = fx_u64(de.z, de.w & 0x1FFFFFu);           // f = mf 2^ef, mf in [2^52, 2^53)
	const int ef = static_cast<int>(de.w >> 24) - 128;
	const uint4 *term = t.fx + t.sfac_offset[dim];
	const uint32_t nd = t.sfac_digits[dim];
	// dn = (double)n = dm 2^dexp, then dn *= f rounded as the double multiply
	// rounds (53-bit mantissas, product to nearest even): the reference's
	// digit chain n_k = (unsigned)dn, exactly
	const int msb = 31 - clz32(n);
	uint64_t dm = static_cast<uint64_t>(n) << (52 - msb);
	int dexp = msb - 52;
	Fx128 z{0ull, 0ull};
	uint32_t m = n, k = 0;
	for(; m > 0; ++k)
	{
		if(k >= nd) return static_cast<float>(low_discrepancy(t, dim, n));   // not reached for 32-bit n
		const uint32_t q = static_cast<uint32_t>(mulhi64(m, recip));      // floor(m / b)
		fx_add(z, fx_load(term[k * b + (m - q * b)]));
		const uint64_t plo = dm * mf, phi = mulhi64(dm, mf);               // 106-bit product
		const int sh = 52 + static_cast<int>((phi >> 41) & 1u);            // its top bit is 104 or 105
		uint64_t nm = (phi << (64 - sh)) | (plo >> sh);
		const uint64_t rem = plo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
		if(rem > half || (rem == half && (nm & 1ull))) ++nm;
		dexp += ef + sh;
		if(nm >> 53) { nm >>= 1; ++dexp; }
		dm = nm;
		m = -dexp >= 64 ? 0u : static_cast<uint32_t>(dm >> (-dexp));   // dn < 2^32, so dexp < -20
	}
	float out;
	if(fx_to_float(z, k, out)) return out;
	return static_cast<float>(low_discrepancy(t, dim, n));
}

// radical_inverse(n, 3) as a float, the same way (exact digits, exact sum).
GBRT_HD float radical_inverse3_f(const LdsTables &t, uint32_t n)
{
	const uint4 *term = t.fx + t.fx_rad3;
	Fx128 z{0ull, 0ull};
	uint32_t k = 0, adds = 0;
	for(uint32_t m = n; m > 0; ++k)
	{
		const uint32_t q = m / 3u, d = m - 3u * q;
		if(d) { fx_add(z, fx_load(term[2 * k + (d - 1)])); ++adds; }
		m = q;
	}
	float out;
	if(fx_to_float(z, adds, out)) return clamp01(out);
	return radical_inverse(n, 3);
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
	std::vector<double> sfac;
	std::vector<uint32_t> sfac_offset, sfac_digits;
	std::vector<uint4> fx;
	uint32_t fx_dims = 0, fx_rad3 = 0;
	LdsTables view() const
	{
		return LdsTables{perm.data(), offset.data(), base.data(), inv.data(), sfac.data(), sfac_offset.data(), sfac_digits.data(),
		                 fx.data(), fx_dims, fx_rad3};
	}
};

// A double in [0, 2) as 128-bit fixed point (units of 2^-127), exactly:
// every tabulated term is at least 2^-74.
inline uint4 fx_of_double(double t)
{
	uint4 e{0u, 0u, 0u, 0u};
	if(t == 0.0) return e;
	int ex = 0;
	const double fr = std::frexp(t, &ex);                       // t = fr 2^ex, fr in [0.5, 1)
	const uint64_t m53 = static_cast<uint64_t>(std::ldexp(fr, 53));
	const int sh = ex + 74;                                     // t = m53 2^(ex - 53) = (m53 << (ex + 74)) 2^-127
	const unsigned __int128 z = static_cast<unsigned __int128>(m53) << sh;
	const uint64_t hi = static_cast<uint64_t>(z >> 64), lo = static_cast<uint64_t>(z);
	e.x = static_cast<uint32_t>(lo); e.y = static_cast<uint32_t>(lo >> 32);
	e.z = static_cast<uint32_t>(hi); e.w = static_cast<uint32_t>(hi >> 32);
	return e;
}

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
		// digits a 32-bit index can have in base b, plus margin
		uint32_t nd = 2;
		for(double x = 4294967296.0; x >= 1.0; x /= static_cast<double>(b < 2 ? 2 : b)) ++nd;
		t.sfac_offset.push_back(static_cast<uint32_t>(t.sfac.size()));
		t.sfac_digits.push_back(b < 2 ? 0u : nd);
		if(b >= 2)
		{
			const double f = t.inv.back();
			double factor = f;
			for(uint32_t k = 0; k < nd; ++k)
			{
				for(uint32_t d = 0; d < b; ++d) t.sfac.push_back(static_cast<double>(p[d]) * factor);
				factor = factor * f;
			}
		}
	}
	// FP64-free tables: the terms at the sfac indices, per-dimension entries,
	// base-3 radical-inverse terms
	for(double v : t.sfac) t.fx.push_back(fx_of_double(v));
	t.fx_dims = static_cast<uint32_t>(t.fx.size());
	t.fx.resize(t.fx.size() + kLdsDims);
	for(int d = 0; d < kLdsDims; ++d)
	{
		const uint32_t b = t.base[d];
		uint4 &e = t.fx[t.fx_dims + d];
		e = uint4{0u, 0u, 0u, 0u};
		if(b < 2) continue;
		// floor(2^64 / b) + 1: floor(m / b) = mulhi(m, this) for every m < 2^32
		const uint64_t recip = static_cast<uint64_t>((~static_cast<unsigned __int128>(0) >> 64) / b) + 1u;
		// f = mf 2^ef with a 53-bit mantissa
		int ex = 0;
		const double fr = std::frexp(t.inv[d], &ex);
		const uint64_t mf = static_cast<uint64_t>(std::ldexp(fr, 53));
		const int ef = ex - 53;
		e.x = static_cast<uint32_t>(recip); e.y = static_cast<uint32_t>(recip >> 32);
		e.z = static_cast<uint32_t>(mf);
		e.w = static_cast<uint32_t>(mf >> 32) | (static_cast<uint32_t>(ef + 128) << 24);
	}
	t.fx_rad3 = static_cast<uint32_t>(t.fx.size());
	for(int k = 0; k < 21; ++k)
	{
		t.fx.push_back(fx_of_double(h_inv3_pow[k]));
		t.fx.push_back(fx_of_double(2.0 * h_inv3_pow[k]));
	}
	return t;
}

} // namespace gbrt
