// kg_num.cuh -- arithmetic types of the sweeps and storage conversions.
//
// The stencil bodies are written once, as templates over a number type N, in
// the reference's own association order (C++ and C share precedence and
// left-to-right associativity of + - * /).  N fixes the rounding:
//   SD  FP64, every operation an IEEE round-to-nearest intrinsic; the compiler
//       cannot contract a*b+c into an FMA, so results equal a strict IEEE
//       build of the reference kernel bit for bit.
//   FD  FP64, plain operators: nvcc contracts products into DFMA like the
//       suite's gcc -ffast-math build does on FMA hardware.
//   FF  FP32 arithmetic (used for FP32, BF16 and FP16 storage).
#pragma once

#include <type_traits>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace kg {

struct SD {
	double v;
	__host__ __device__ constexpr SD() : v(0) {}
	__host__ __device__ constexpr explicit SD(double x) : v(x) {}
};
__device__ __forceinline__ SD operator+(SD a, SD b) { return SD(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator-(SD a, SD b) { return SD(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator*(SD a, SD b) { return SD(__dmul_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator/(SD a, SD b) { return SD(__ddiv_rn(a.v, b.v)); }

// SE: the same strict FP64 semantics as SD, computed on the integer pipes.
// Additions, subtractions and multiplications are exact IEEE round-to-
// nearest-even operations built from 32-bit integer arithmetic (53-bit
// mantissas in two words, 106-bit products from four 32x32 multiplies,
// guard/round/sticky rounding), so their bits equal the FP64 unit's; se_div
// (below) divides.  Zeros, subnormals, infinities, NaNs and results leaving
// the normal range take a rarely used branch to the FP64 unit.  GB300 issues
// FP64 arithmetic at 1/72 of its FP32 rate while the integer pipes sit idle
// in these sweeps: measured, a thread that interleaves independent native
// and integer multiplies reaches 1.9x the FP64 unit's multiply rate, and
// additions 1.3x, bit for bit the same.  The strict sweeps form their
// products (pm), quotients (pdiv) and a share of every sum's additions (nsum)
// this way, within each thread; whole warps computing in SE beside warps in
// SD were slower.
struct SE {
	double v;
	__host__ __device__ constexpr SE() : v(0) {}
	__host__ __device__ constexpr explicit SE(double x) : v(x) {}
};

// a < b for 64-bit unsigned integers from 32-bit comparisons of their words:
// a 64-bit integer comparison issues to the FP64 pipe on GB300, which the
// integer-pipe arithmetic below exists to leave to the native operations.
__device__ __forceinline__ bool se_lt_u64(unsigned long long a, unsigned long long b)
{
	unsigned lt_hi, eq_hi, lt_lo;
	asm("set.lt.u32.u32 %0, %1, %2;" : "=r"(lt_hi) : "r"((unsigned)(a >> 32)), "r"((unsigned)(b >> 32)));
	asm("set.eq.u32.u32 %0, %1, %2;" : "=r"(eq_hi) : "r"((unsigned)(a >> 32)), "r"((unsigned)(b >> 32)));
	asm("set.lt.u32.u32 %0, %1, %2;" : "=r"(lt_lo) : "r"((unsigned)a), "r"((unsigned)b));
	return (lt_hi | (eq_hi & lt_lo)) != 0;
}

static __device__ __noinline__ double se_native_mul(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double se_native_add(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ double se_mul(double a, double b)
{
	const unsigned long long A = (unsigned long long)__double_as_longlong(a);
	const unsigned long long B = (unsigned long long)__double_as_longlong(b);
	const unsigned ahw = (unsigned)(A >> 32), bhw = (unsigned)(B >> 32);
	const int ea = (ahw >> 20) & 0x7ff, eb = (bhw >> 20) & 0x7ff;
	const unsigned ah = (ahw & 0xfffffu) | 0x100000u, bh = (bhw & 0xfffffu) | 0x100000u;
	const unsigned al = (unsigned)A, bl = (unsigned)B;
	// 53 x 53 -> 106-bit product P = ah bh 2^64 + (ah bl + al bh) 2^32 + al bl
	const unsigned long long p0 = (unsigned long long)al * bl;
	const unsigned long long p1 = (unsigned long long)ah * bl;
	const unsigned long long p2 = (unsigned long long)al * bh;
	const unsigned long long p3 = (unsigned long long)ah * bh;
	const unsigned long long mid = p1 + p2 + (p0 >> 32);
	const unsigned long long hi = (p3 << 22) + (mid >> 10);          // P >> 42, in [2^62, 2^64)
	const bool low_nz = ((unsigned)(mid & 0x3ffu) | (unsigned)p0) != 0;
	const int top = (int)(hi >> 63);                                 // P >= 2^105
	const int sh = 10 + top;
	unsigned long long mant = hi >> sh;                              // 53 bits
	const unsigned long long rnd = (hi >> (sh - 1)) & 1;
	const bool stk = low_nz || (hi & ((1ull << (sh - 1)) - 1)) != 0;
	mant += rnd & ((unsigned long long)stk | (mant & 1));
	const int E = ea + eb - 1023 + top;
	const bool ok = (unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && E >= 1 && E <= 2045;
	if (__builtin_expect(!ok, 0)) return se_native_mul(a, b);
	const unsigned long long sign = (A ^ B) & 0x8000000000000000ull;
	return __longlong_as_double((long long)(sign | (((unsigned long long)(E - 1) << 52) + mant)));
}

// Exact a + b.  Branch-free apart from the rare fallback, so warps whose
// lanes add operands of mixed signs do not diverge: both the same-sign sum
// and the opposite-sign difference are formed and one is selected.
// Measured on GB300 (independent additions): 0.26e12/s alone against the
// FP64 unit's 0.50e12; a quarter or three eighths of them here and the rest
// on the FP64 unit, 0.65 and 0.66e12/s together (with the magnitude
// comparison as one 64-bit integer comparison, which issues to the FP64
// pipe, mixing gained nothing: 0.49e12/s).
__device__ __forceinline__ double se_add(double a, double b)
{
	const unsigned long long A = (unsigned long long)__double_as_longlong(a);
	const unsigned long long B = (unsigned long long)__double_as_longlong(b);
	const bool sw = se_lt_u64(A & 0x7fffffffffffffffull, B & 0x7fffffffffffffffull);   // |a| < |b|
	const unsigned long long X = sw ? B : A, Y = sw ? A : B;         // |X| >= |Y|
	const int ex = (int)(X >> 52) & 0x7ff, ey = (int)(Y >> 52) & 0x7ff;
	const bool ok_in = (unsigned)(ex - 1) < 2046u && (unsigned)(ey - 1) < 2046u;
	const int dd = ex - ey;
	// mantissas with the hidden bit at bit 62; Y aligned to X, lost bits as sticky
	const unsigned long long Mx = ((X & 0xfffffffffffffull) | 0x10000000000000ull) << 10;
	const unsigned long long My0 = ((Y & 0xfffffffffffffull) | 0x10000000000000ull) << 10;
	const int ds = dd < 63 ? dd : 63;
	const unsigned long long My = My0 >> ds;
	const unsigned long long stk_in = ds == 0 ? 0ull : (unsigned long long)((My0 << (64 - ds)) != 0);
	const bool sub = ((X ^ Y) >> 63) != 0;
	// same signs: S in [2^62, 2^64); keep a bit shifted out as sticky
	const unsigned long long Sa = Mx + My;
	const int ca = (int)(Sa >> 63);
	const unsigned long long Sa_n = (Sa >> ca) | (Sa & (unsigned long long)ca);
	// opposite signs: Y truncated, so the exact difference lies in (Ss - 1, Ss]
	const unsigned long long Ss = Mx - My - stk_in;
	const int lz = Ss ? __clzll((long long)Ss) - 1 : 0;
	const unsigned long long S = sub ? (Ss << lz) : Sa_n;
	const int E = ex + (sub ? -lz : ca);
	const unsigned long long mant0 = S >> 10;
	const unsigned long long rnd = (S >> 9) & 1;
	const unsigned long long stk = stk_in | (unsigned long long)((S & 0x1ff) != 0);
	const unsigned long long mant = mant0 + (rnd & (stk | (mant0 & 1)));
	// zeros, subnormals, inf/nan, exact cancellation, far-apart operands and
	// results out of the normal range go to the FP64 unit
	const bool ok = ok_in && dd <= 60 && !(sub && Ss == 0 && stk_in == 0) && E >= 1 && E <= 2045;
	if (__builtin_expect(!ok, 0)) return se_native_add(a, b);
	return __longlong_as_double((long long)((X & 0x8000000000000000ull) | (((unsigned long long)(E - 1) << 52) + mant)));
}

static __device__ __noinline__ double se_native_div(double a, double b) { return __ddiv_rn(a, b); }

// Small integers <-> FP32 without a conversion instruction: for |t| < 2^22
// the float 1.5 * 2^23 + t has ulp 1, so its bit pattern is that of
// 1.5 * 2^23 plus t (and a float x of magnitude below 2^22, added to
// 1.5 * 2^23, is rounded to the nearest integer in the same way).
__device__ __forceinline__ float se_i2f(int t) { return __fsub_rn(__int_as_float(0x4b400000 + t), 12582912.0f); }
__device__ __forceinline__ int se_f2i_rn(float x) { return __float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4b400000; }

// Exact a / b, round to nearest even, by digit recurrence on the integer
// significands: with N = ma or 2 ma (so that N / mb lies in [1, 2)), the 54-
// bit floor Q of N 2^53 / mb is formed as three signed digits of 20, 20 and
// 13 bits, Q = d1 2^33 + d2 2^13 + d3.  Each digit is estimated in FP32 from
// the leading bits of the running remainder times an approximate reciprocal
// of mb (rcp.approx of its leading 24 bits, relative error below 2^-22), and
// the remainder is then updated exactly, R' = R 2^k - d mb, in 64-bit
// integer arithmetic modulo 2^64 (the true remainders stay below 3.2 mb <
// 2^55 in magnitude, so the wrapped values are exact).  The digit errors are
// at most 2.2, 3.2 and 0.53 units, so one correction of the last digit makes
// Q the exact floor and R its remainder in [0, mb).  Q's last bit is the
// rounding bit; a tie (rounding bit set and R = 0) cannot occur for normal
// operands but is rounded to even all the same.  Zeros, subnormals,
// infinities, NaNs and quotients leaving the normal range go to the FP64
// unit.
__device__ __forceinline__ double se_div(double a, double b)
{
	const unsigned long long A = (unsigned long long)__double_as_longlong(a);
	const unsigned long long B = (unsigned long long)__double_as_longlong(b);
	const int ea = (int)(A >> 52) & 0x7ff, eb = (int)(B >> 52) & 0x7ff;
	const unsigned long long ma = (A & 0xfffffffffffffull) | 0x10000000000000ull;
	const unsigned long long mb = (B & 0xfffffffffffffull) | 0x10000000000000ull;
	const int sh = se_lt_u64(ma, mb) ? 1 : 0;
	const unsigned long long N = ma << sh;                            // N / mb in [1, 2)
	const int E = ea - eb - sh + 1023;
	// rb ~ 2^52 / mb
	float rb;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(__int_as_float(0x3f800000 | (int)((mb >> 29) & 0x7fffff))));
	const int d1 = se_f2i_rn(__fmul_rn(se_i2f((int)(N >> 32)), rb));                 // ~ N 2^20 / mb
	const unsigned long long R1 = (N << 20) - (unsigned long long)(long long)d1 * mb;
	const int d2 = se_f2i_rn(__fmul_rn(se_i2f((int)((long long)R1 >> 33)), 2.0f * rb));      // ~ R1 2^20 / mb
	const unsigned long long R2 = (R1 << 20) - (unsigned long long)(long long)d2 * mb;
	const int d3 = se_f2i_rn(__fmul_rn(se_i2f((int)((long long)R2 >> 33)), 0.015625f * rb)); // ~ R2 2^13 / mb
	const unsigned long long R3 = (R2 << 13) - (unsigned long long)(long long)d3 * mb;
	const unsigned long long neg = (unsigned long long)((long long)R3 < 0);
	const unsigned long long Q = ((unsigned long long)(long long)d1 << 33) + ((unsigned long long)(long long)d2 << 13) +
		(unsigned long long)(long long)d3 - neg;
	const unsigned long long R = R3 + (neg ? mb : 0ull);
	const unsigned long long mant0 = Q >> 1;
	const unsigned long long mant = mant0 + ((Q & 1) & ((unsigned long long)(R != 0) | (mant0 & 1)));
	const bool ok = (unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && E >= 1 && E <= 2045;
	if (__builtin_expect(!ok, 0)) return se_native_div(a, b);
	const unsigned long long sign = (A ^ B) & 0x8000000000000000ull;
	return __longlong_as_double((long long)(sign | (((unsigned long long)(E - 1) << 52) + mant)));
}

__device__ __forceinline__ SE operator+(SE a, SE b) { return SE(se_add(a.v, b.v)); }
__device__ __forceinline__ SE operator-(SE a, SE b)
{
	return SE(se_add(a.v, __longlong_as_double(__double_as_longlong(b.v) ^ (long long)0x8000000000000000ull)));
}
__device__ __forceinline__ SE operator*(SE a, SE b) { return SE(se_mul(a.v, b.v)); }
__device__ __forceinline__ SE operator/(SE a, SE b) { return SE(__ddiv_rn(a.v, b.v)); }

struct FD {
	double v;
	__host__ __device__ constexpr FD() : v(0) {}
	__host__ __device__ constexpr explicit FD(double x) : v(x) {}
};
__device__ __forceinline__ FD operator+(FD a, FD b) { return FD(a.v + b.v); }
__device__ __forceinline__ FD operator-(FD a, FD b) { return FD(a.v - b.v); }
__device__ __forceinline__ FD operator*(FD a, FD b) { return FD(a.v * b.v); }
__device__ __forceinline__ FD operator/(FD a, FD b) { return FD(a.v / b.v); }

struct FF {
	float v;
	__host__ __device__ constexpr FF() : v(0) {}
	__host__ __device__ constexpr explicit FF(double x) : v((float)x) {}
	__host__ __device__ constexpr explicit FF(float x, int) : v(x) {}
};
__device__ __forceinline__ FF mkf(float x) { return FF(x, 0); }
__device__ __forceinline__ FF operator+(FF a, FF b) { return mkf(a.v + b.v); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return mkf(a.v - b.v); }
__device__ __forceinline__ FF operator*(FF a, FF b) { return mkf(a.v * b.v); }
__device__ __forceinline__ FF operator/(FF a, FF b) { return mkf(a.v / b.v); }

// H16<S>: a BF16 or FP16 value still in its half of a 32-bit word of a
// loaded vector, as the vector TMA engine reads 16-bit storage.  Used as FF
// it is widened (a shift or mask for BF16, a conversion for FP16); added to
// an FP32 sum it needs no widening at all: GB300's mixed-precision add takes
// the 16-bit operand from its half of the register (add.rn.f32.bf16 /
// add.rn.f32.f16, the exact sum of the widened value and the FP32 operand
// rounded to nearest: the same bits as widening first).
template <class S> struct H16 {
	uint32_t w;
	int hi;   // 1: the upper 16 bits
	__device__ __forceinline__ operator FF() const {
		if constexpr (std::is_same<S, __nv_bfloat16>::value)
			return mkf(__uint_as_float(hi ? (w & 0xffff0000u) : (w << 16)));
		else
			return mkf(__half2float(__ushort_as_half((unsigned short)(hi ? (w >> 16) : (w & 0xffffu)))));
	}
};
template <class T> struct IsH16 : std::false_type {};
template <class S> struct IsH16<H16<S>> : std::true_type {};

// acc + x with x taken from its half-word by the mixed-precision add
template <class S> __device__ __forceinline__ FF add_h16(FF acc, H16<S> x)
{
	float d;
	if constexpr (std::is_same<S, __nv_bfloat16>::value) {
		if (x.hi) asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.bf16 %0, h, %2; }" : "=f"(d) : "r"(x.w), "f"(acc.v));
		else asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.bf16 %0, l, %2; }" : "=f"(d) : "r"(x.w), "f"(acc.v));
	} else {
		if (x.hi) asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.f16 %0, h, %2; }" : "=f"(d) : "r"(x.w), "f"(acc.v));
		else asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; add.rn.f32.f16 %0, l, %2; }" : "=f"(d) : "r"(x.w), "f"(acc.v));
	}
	return mkf(d);
}
// x - c with x taken from its half-word by the mixed-precision subtraction
template <class S> __device__ __forceinline__ FF sub_h16(H16<S> x, FF c)
{
	float d;
	if constexpr (std::is_same<S, __nv_bfloat16>::value) {
		if (x.hi) asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; sub.rn.f32.bf16 %0, h, %2; }" : "=f"(d) : "r"(x.w), "f"(c.v));
		else asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; sub.rn.f32.bf16 %0, l, %2; }" : "=f"(d) : "r"(x.w), "f"(c.v));
	} else {
		if (x.hi) asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; sub.rn.f32.f16 %0, h, %2; }" : "=f"(d) : "r"(x.w), "f"(c.v));
		else asm("{ .reg .b16 l, h; mov.b32 {l, h}, %1; sub.rn.f32.f16 %0, l, %2; }" : "=f"(d) : "r"(x.w), "f"(c.v));
	}
	return mkf(d);
}
__device__ __forceinline__ FF to_ff(FF x) { return x; }
template <class S> __device__ __forceinline__ FF to_ff(H16<S> x) { return FF(x); }
// The sum or difference of two 16-bit values (no product for nvcc to
// contract with it): one operand widened, the other taken from its half-word.
// Every other operation widens the 16-bit operand first and is the FF
// operation itself, so nvcc forms (and contracts) exactly the expression it
// forms with FF operands.
template <class S> __device__ __forceinline__ FF operator+(H16<S> a, H16<S> b) { return add_h16(FF(a), b); }
template <class S> __device__ __forceinline__ FF operator+(H16<S> a, FF b) { return FF(a) + b; }
template <class S> __device__ __forceinline__ FF operator+(FF a, H16<S> b) { return a + FF(b); }
template <class S> __device__ __forceinline__ FF operator-(H16<S> a, H16<S> b) { return sub_h16(a, FF(b)); }
template <class S> __device__ __forceinline__ FF operator-(H16<S> a, FF b) { return FF(a) - b; }
template <class S> __device__ __forceinline__ FF operator-(FF a, H16<S> b) { return a - FF(b); }
template <class S> __device__ __forceinline__ FF operator*(H16<S> a, H16<S> b) { return FF(a) * FF(b); }
template <class S> __device__ __forceinline__ FF operator*(H16<S> a, FF b) { return FF(a) * b; }
template <class S> __device__ __forceinline__ FF operator*(FF a, H16<S> b) { return a * FF(b); }

// FF2: an FP64 value carried as an unevaluated sum hi + lo of two FP32
// numbers ("float-float"), computed on the FP32 pipes with error-free
// transformations: TwoSum (Knuth) for additions, the FMA product error for
// multiplications.  About 44-48 significant bits survive an operation, so a
// stencil sweep stays within ~1e-14 of FP64 normwise, while GB300 issues FP32
// FMAs at 72x its FP64 rate.  Intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn)
// keep nvcc from re-associating or contracting the compensation terms.
struct FF2 {
	float hi, lo;
	__host__ __device__ constexpr FF2() : hi(0.f), lo(0.f) {}
	__host__ __device__ constexpr FF2(float h, float l) : hi(h), lo(l) {}
	// A double constant or coefficient, split once (on the host or folded).
	__host__ __device__ constexpr explicit FF2(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
};
__device__ __forceinline__ FF2 ff2_fast_two_sum(float a, float b)
{
	const float s = __fadd_rn(a, b);
	return FF2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ FF2 operator+(FF2 a, FF2 b)
{
	const float s = __fadd_rn(a.hi, b.hi);
	const float bb = __fsub_rn(s, a.hi);
	const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
	return ff2_fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF2 operator-(FF2 b) { return FF2(-b.hi, -b.lo); }
__device__ __forceinline__ FF2 operator-(FF2 a, FF2 b) { return a + (-b); }
__device__ __forceinline__ FF2 operator*(FF2 a, FF2 b)
{
	const float p = __fmul_rn(a.hi, b.hi);
	float e = __fmaf_rn(a.hi, b.hi, -p);
	e = __fmaf_rn(a.hi, b.lo, e);
	e = __fmaf_rn(a.lo, b.hi, e);
	return ff2_fast_two_sum(p, e);
}
// Quotient: q1 ~ a.hi / b.hi (fast approximate FP32 division, ~2 ulp), the
// remainder a - b q1 in float-float, and its quotient q2 as the correction;
// q1 + q2 is within ~2^-44 of a / b.
__device__ __forceinline__ FF2 operator/(FF2 a, FF2 b)
{
	const float q1 = __fdividef(a.hi, b.hi);
	const FF2 r = a - b * FF2(q1, 0.f);
	const float q2 = __fdividef(r.hi, b.hi);
	return ff2_fast_two_sum(q1, q2);
}

// FP64 <-> FF2 without the FP64 pipe.  On GB300 the F2F conversions between
// double and float issue to the FP64 pipe (2 per clock per SM), so both
// directions are built from the IEEE bit fields with integer and FP32 ops.
//
// Split: hi = x truncated to 24 significant bits (exponent rebiased, top 23
// fraction bits); lo = the 29 remaining fraction bits r, rounded to 24 bits,
// times 2^(e-1075), with x's sign.  r is converted exactly in two 23-bit
// pieces with the 2^23 magic-number trick.  |x| below 2^-74 keeps only hi
// (lo underflows), below 2^-126 becomes a signed zero; inf and nan pass; x
// above FP32's range becomes inf.
__device__ __forceinline__ FF2 ff2_from_double(double x)
{
	const unsigned long long b = (unsigned long long)__double_as_longlong(x);
	const unsigned bh = (unsigned)(b >> 32), bl = (unsigned)b;
	const unsigned sign = bh & 0x80000000u;
	const int e = (int)((bh >> 20) & 0x7ff);
	const unsigned fh = ((bh & 0xfffffu) << 3) | (bl >> 29);
	if (e >= 897 && e <= 1150) {
		const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | fh);
		float lo = 0.f;
		if (e >= 949) {
			const unsigned r = bl & 0x1fffffffu;
			const float f0 = __fsub_rn(__uint_as_float(0x4b000000u | (r & 0x7fffffu)), 8388608.0f);
			const float f1 = __fsub_rn(__uint_as_float(0x4b000000u | (r >> 23)), 8388608.0f);
			const float rf = __fmaf_rn(f1, 8388608.0f, f0);
			const float scale = __uint_as_float((unsigned)(e - 948) << 23);  // 2^(e - 1075)
			lo = __uint_as_float(__float_as_uint(__fmul_rn(rf, scale)) | sign);
		}
		return FF2(hi, lo);
	}
	if (e < 897) return FF2(__uint_as_float(sign), 0.f);
	const unsigned nan = (e == 0x7ff && ((bh & 0xfffffu) | bl)) ? 0x400000u : 0u;
	return FF2(__uint_as_float(sign | 0x7f800000u | nan), 0.f);
}

// Merge: hi's bit fields give its exact FP64 bit pattern; lo, in units of
// hi's FP64 ulp (an integer below 2^30 for a normalised pair), is added to
// or subtracted from that pattern.  Below a power-of-two hi the ulp halves,
// so a subtraction there counts twice.  Bits of lo under hi's FP64 ulp are
// dropped (error below one FP64 ulp).
__device__ __forceinline__ double ff2_to_double(FF2 v)
{
	const unsigned hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
	const int eh = (int)((hb >> 23) & 0xff), el = (int)((lb >> 23) & 0xff);
	const unsigned long long sgn = (unsigned long long)(hb & 0x80000000u) << 32;
	if (eh == 0) return __longlong_as_double((long long)sgn);  // zero (or FP32-subnormal) hi
	if (eh == 0xff)
		return __longlong_as_double((long long)(sgn | 0x7ff0000000000000ULL | ((hb & 0x7fffffu) ? 0x8000000000000ULL : 0)));
	const unsigned long long dh = sgn | ((unsigned long long)(eh + 896) << 52) | ((unsigned long long)(hb & 0x7fffffu) << 29);
	if (el == 0) return __longlong_as_double((long long)dh);
	const int sh = el - eh + 29;
	const unsigned long long ml = (unsigned long long)((lb & 0x7fffffu) | 0x800000u);
	unsigned long long l;
	if (sh >= 0) l = ml << (sh > 34 ? 34 : sh);
	else if (sh > -25) l = ml >> (-sh);
	else return __longlong_as_double((long long)dh);
	const bool same = ((hb ^ lb) & 0x80000000u) == 0;
	if (same) return __longlong_as_double((long long)(dh + l));
	if ((hb & 0x7fffffu) == 0) l <<= 1;
	return __longlong_as_double((long long)(dh - l));
}

// ---- storage <-> arithmetic -------------------------------------------------

template <class N, class S> struct Conv;

template <> struct Conv<SD, double> {
	static __device__ __forceinline__ SD ld(const double* p) { return SD(__ldg(p)); }
	static __device__ __forceinline__ SD from(double x) { return SD(x); }
	static __device__ __forceinline__ double to(SD x) { return x.v; }
};
template <> struct Conv<SE, double> {
	static __device__ __forceinline__ SE ld(const double* p) { return SE(__ldg(p)); }
	static __device__ __forceinline__ SE from(double x) { return SE(x); }
	static __device__ __forceinline__ double to(SE x) { return x.v; }
};
template <> struct Conv<FD, double> {
	static __device__ __forceinline__ FD ld(const double* p) { return FD(__ldg(p)); }
	static __device__ __forceinline__ FD from(double x) { return FD(x); }
	static __device__ __forceinline__ double to(FD x) { return x.v; }
};
template <> struct Conv<FF2, double> {
	static __device__ __forceinline__ FF2 ld(const double* p) { return ff2_from_double(__ldg(p)); }
	static __device__ __forceinline__ FF2 from(double x) { return ff2_from_double(x); }
	static __device__ __forceinline__ double to(FF2 x) { return ff2_to_double(x); }
};
template <> struct Conv<FF, float> {
	static __device__ __forceinline__ FF ld(const float* p) { return mkf(__ldg(p)); }
	static __device__ __forceinline__ FF from(float x) { return mkf(x); }
	static __device__ __forceinline__ float to(FF x) { return x.v; }
};
template <> struct Conv<FF, __nv_bfloat16> {
	static __device__ __forceinline__ FF ld(const __nv_bfloat16* p) { return mkf(__bfloat162float(__ldg(p))); }
	static __device__ __forceinline__ FF from(__nv_bfloat16 x) { return mkf(__bfloat162float(x)); }
	static __device__ __forceinline__ __nv_bfloat16 to(FF x) { return __float2bfloat16_rn(x.v); }
};
template <> struct Conv<FF, __half> {
	static __device__ __forceinline__ FF ld(const __half* p) { return mkf(__half2float(__ldg(p))); }
	static __device__ __forceinline__ FF from(__half x) { return mkf(__half2float(x)); }
	static __device__ __forceinline__ __half to(FF x) { return __float2half_rn(x.v); }
};

}  // namespace kg
