// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2
// (48 significant bits, relative rounding ~2^-47 per operation).  GB300 issues FP64 at ~1.6 lanes per clock per
// SM against ~128 for FP32, so pointwise physics in double-float runs several times faster than in FP64 while
// staying within ~1e-14 of it.  The building blocks are the error-free transformations TwoSum (Knuth), FastTwoSum
// (Dekker) and the FMA-based TwoProd; addition, multiplication and division follow the "double-word" algorithms
// analysed by Joldes, Muller and Popescu (ACM TOMS 44, 2017: AccurateDWPlusDW, DWTimesDW, DWDivDW); the square
// root is one Newton step in double-float from the FP32 root (its correction term by the fast FP32 division).  The
// conversion to FP64 and the digit extraction of the tensor-core path avoid FP64 instructions (integer and FP32
// operations only).
#pragma once
#include <cstdint>

namespace dpg {
namespace df {

struct df64 {
	float hi, lo;
};

__device__ __forceinline__ df64 mk(float h, float l = 0.f) { return df64{h, l}; }
__device__ __forceinline__ df64 from2(float2 v) { return df64{v.x, v.y}; }
__device__ __forceinline__ float2 to2(df64 a) { return make_float2(a.hi, a.lo); }

__device__ __forceinline__ df64 two_sum(float a, float b)
{
	const float s = a + b, bb = s - a;
	return df64{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b)   // |a| >= |b| (or a == 0)
{
	const float s = a + b;
	return df64{s, b - (s - a)};
}
__device__ __forceinline__ df64 neg(df64 a) { return df64{-a.hi, -a.lo}; }
__device__ __forceinline__ df64 add(df64 x, df64 y)
{
	df64 s = two_sum(x.hi, y.hi);
	const df64 t = two_sum(x.lo, y.lo);
	s.lo += t.hi;
	s = fast_two_sum(s.hi, s.lo);
	s.lo += t.lo;
	return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 sub(df64 x, df64 y) { return add(x, neg(y)); }
// x + y for an FP32 y: TwoSum of the leading parts, the trailing part folded in (error ~2^-48 of the result).
__device__ __forceinline__ df64 add_f(df64 x, float y)
{
	const df64 s = two_sum(x.hi, y);
	return fast_two_sum(s.hi, s.lo + x.lo);
}
// "Sloppy" addition (one TwoSum instead of two): absolute error within ~2^-47 max(|x|, |y|), no relative bound
// under cancellation, i.e. the forward-error behaviour of FP64 arithmetic at 48 bits.  The flux kernels use it.
__device__ __forceinline__ df64 add_s(df64 x, df64 y)
{
	const df64 s = two_sum(x.hi, y.hi);
	return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ df64 sub_s(df64 x, df64 y) { return add_s(x, neg(y)); }
__device__ __forceinline__ df64 mul(df64 x, df64 y)
{
	const float p = x.hi * y.hi;
	float e = fmaf(x.hi, y.hi, -p);
	const float t = fmaf(x.lo, y.hi, x.hi * y.lo);
	e += t;
	return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 mulf(df64 x, float y)
{
	const float p = x.hi * y;
	float e = fmaf(x.hi, y, -p);
	e = fmaf(x.lo, y, e);
	return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 scale(df64 x, float pow2) { return df64{x.hi * pow2, x.lo * pow2}; }   // exact
__device__ __forceinline__ df64 div(df64 x, df64 y)
{
	const float th = __fdiv_rn(x.hi, y.hi);
	const df64 r = mulf(y, th);
	const float pi = x.hi - r.hi;   // exact (Sterbenz)
	const float d = (pi - r.lo) + (x.lo);
	const float tl = __fdiv_rn(d, y.hi);
	return fast_two_sum(th, tl);
}
// 1 / y: the correctly rounded FP32 reciprocal of hi, then one Newton step r + r (1 - y r) whose residual is formed
// with FMAs (exact for the hi part); relative error below 2^-45.
__device__ __forceinline__ df64 rcp(df64 y)
{
	const float r = __frcp_rn(y.hi);
	float e = fmaf(-y.hi, r, 1.f);
	e = fmaf(-y.lo, r, e);
	return fast_two_sum(r, r * e);
}
__device__ __forceinline__ df64 sqrt(df64 x)
{
	if (!(x.hi > 0.f)) return mk(0.f);
	const float s = __fsqrt_rn(x.hi);
	const float p = s * s;
	const float e = fmaf(s, s, -p);
	const float r = ((x.hi - p) - e) + x.lo;
	return fast_two_sum(s, __fdividef(r, 2.f * s));   // the correction term needs ~24 bits: 2-ulp division
}
__device__ __forceinline__ bool gt0(df64 a) { return a.hi > 0.f || (a.hi == 0.f && a.lo > 0.f); }
__device__ __forceinline__ df64 absd(df64 a) { return a.hi < 0.f ? neg(a) : a; }
__device__ __forceinline__ bool abs_less(df64 a, df64 b)   // |a| < |b|
{
	const df64 x = absd(a), y = absd(b);
	return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo);
}

// x * 2^e, exact while the result stays in the FP32 normal range (two factors when 2^e itself is outside it).
__device__ __forceinline__ df64 scale_pow2(df64 x, int e)
{
	const int e1 = max(min(e, 127), -126), e2 = max(min(e - e1, 127), -126);
	const float f1 = __uint_as_float((uint32_t)(e1 + 127) << 23), f2 = __uint_as_float((uint32_t)(e2 + 127) << 23);
	return df64{x.hi * f1 * f2, x.lo * f1 * f2};
}

// Double-float nearest to a double (host and device: used on the host to pre-split geometry).
__host__ __device__ inline float2 split_double(double v)
{
	const float h = (float)v;
	return make_float2(h, (float)(v - (double)h));
}

// hi + lo rounded to the nearest double without an FP64 instruction: the double of hi by exponent rebias, then lo
// added as k = round(lo / spacing) steps of the double spacing at hi (|lo| <= ulp(hi)/2 keeps the sum in hi's binade,
// or just below it when hi is a power of two and lo has the opposite sign: spacing halved there).  lo / spacing is
// an exact FP32 scaling by a power of two (two factors when it leaves the FP32 range), |k| <= 2^29, and the
// round-to-nearest-even of the conversion is that of the double (k carries the parity of its last bit).  A
// subnormal or zero hi (|x| < 2^-126) gives 0.
__device__ __forceinline__ double to_double(df64 x)
{
	const uint32_t bh = __float_as_uint(x.hi), ah = bh & 0x7FFFFFFFu;
	const int eh = (int)(ah >> 23);
	const bool opp = ((__float_as_uint(x.lo) ^ bh) >> 31) != 0u;
	const int se = 306 - eh + ((opp && (ah & 0x7FFFFFu) == 0u) ? 1 : 0);   // biased exponent of 1 / spacing
	float f = x.lo * __uint_as_float((uint32_t)min(se, 254) << 23);
	if (se > 254) f *= __uint_as_float((uint32_t)(se - 254 + 127) << 23);
	int k = __float2int_rn(f);
	k = (bh >> 31) ? -k : k;
	const uint32_t hw = ((ah >> 3) + ((1023u - 127u) << 20)) | (bh & 0x80000000u), lw = ah << 29;
	const double y = __longlong_as_double((long long)((((unsigned long long)hw << 32) | lw) + (unsigned long long)(long long)k));
	return ah < 0x00800000u ? 0.0 : y;
}

// |x| < 2^result for the double-float x (hi carries the exponent: |lo| <= ulp(hi)/2 keeps hi + lo below the next
// power of two); -4000 for zero.
__device__ __forceinline__ int exp_bound(df64 x)
{
	const uint32_t b = __float_as_uint(x.hi);
	const int be = (int)((b >> 23) & 0xFF);
	return be == 0 ? -4000 : be - 126;
}

// round(f * 2^sc) for an FP32 value f, |f 2^sc| < 2^62, with integer operations.
__device__ __forceinline__ long long f32_scaled(float f, int sc)
{
	const uint32_t b = __float_as_uint(f);
	const int be = (int)((b >> 23) & 0xFF);
	if (be == 0) return 0;
	const long long mant = (long long)((b & 0x7FFFFFu) | 0x800000u);
	const int sh = be - 150 + sc;
	long long m = 0;
	if (sh >= 0) m = mant << sh;
	else if (sh > -26) m = (mant + (1ll << (-sh - 1))) >> (-sh);
	return (b & 0x80000000u) ? -m : m;
}

// (hi + lo) * 2^sc rounded to an integer (each part rounded: at most one unit off).
__device__ __forceinline__ long long scaled_mantissa(df64 x, int sc) { return f32_scaled(x.hi, sc) + f32_scaled(x.lo, sc); }

} // namespace df
} // namespace dpg
