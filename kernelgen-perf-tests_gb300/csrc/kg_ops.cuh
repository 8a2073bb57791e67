// kg_ops.cuh -- the eleven stencil bodies, each in the reference's own term
// and association order (see kg_num.cuh for why that makes KG_F64 bitwise).
//
// Every op declares its update domain as [L, n-1-H] per axis and reads its
// inputs through `at(p, dx, dy, dz)`, an accessor centred on the point.  The
// engine (kg_engine.cuh) supplies the accessor and the iteration.
#pragma once

#include <type_traits>

#include "kg_num.cuh"

namespace kg {

// Slot roles in kg_problem.arr (reference argument order).
struct Slots {
	int in[6];
	int nin;
	int out[3];
	int nout;
};

// Neighbour reach of one input: how far back (x0, y0, z0) and ahead (x1, y1,
// z1) of the updated point the body reads it.  All zero: read at the point
// only (the staged engine then reads it from global memory directly).
struct Halo {
	int x0, x1, y0, y1, z0, z1;
	__host__ __device__ constexpr bool center() const { return !(x0 | x1 | y0 | y1 | z0 | z1); }
};

// pm(a, b): a * b; in strict FP64 formed by the exact integer multiply (the
// same bits as the FP64 unit's product), so the coefficient products of a
// sweep run on the integer pipes beside the FP64 unit's sums.  Measured on
// GB300 (strict sweeps, 512x256x256 / 512x65536, ms; none / half / all of the
// products moved): laplacian 0.508 / 0.445 / 0.383, divergence 0.508 / 0.385
// / 0.323, gradient 0.384 / 0.263 / 0.245, uxx1 1.910 / 1.722 / 1.406,
// wave13pt 0.992 / 0.870 / 0.808, jacobi 0.704 / 0.580 / 0.517, lapgsrb 1.729
// / 1.609 / 1.488, gaussblur 1.974 / 1.723 / 1.540, gameoflife 1.127 / 1.065
// / 1.000.  A share of each sum's additions moves too (nsum<K>, below).
template <class N> __device__ __forceinline__ N pm(N a, N b)
{
	if constexpr (std::is_same<N, SD>::value) return SD(se_mul(a.v, b.v));
	else return a * b;
}
template <class S> __device__ __forceinline__ FF pm(FF a, H16<S> b) { return a * FF(b); }
template <class S> __device__ __forceinline__ FF pm(H16<S> a, FF b) { return FF(a) * b; }

// pdiv(a, b): a / b; in strict FP64 formed by the exact digit-recurrence
// division on the integer and FP32 pipes (se_div; the same bits as the FP64
// unit's quotient), which takes the division off the FP64 unit.
template <class N> __device__ __forceinline__ N pdiv(N a, N b)
{
	if constexpr (std::is_same<N, SD>::value) return SD(se_div(a.v, b.v));
	else return a / b;
}

// nsum(a, b, ...): a + b + ... added left to right, as written in the
// reference.  For float-float, the terms' high parts go through a chain of
// error-free TwoSums whose errors collect, with the low parts, in one FP32
// accumulator, renormalised once at the end (8 instead of 10 FP32 operations
// per term; the same ~2^-48 relative bound).  Other types: plain binary adds,
// the same operations as the expression (bit for bit).
// Strict FP64: the first K additions of the chain on the integer pipes
// (se_add), the rest on the FP64 unit; the same bits either way.  Each op
// picks K per sum (measured at 512x256x256 / 512x65536, ms per sweep, K = 0 ->
// 1 -> 2 for every sum of the op: laplacian 0.383 / 0.322 / 0.398, uxx1
// 0.958 / 0.931 / 1.166, wave13pt 0.809 / 0.689 / 0.723, jacobi 0.517 / 0.456
// / 0.684, lapgsrb 1.490 / 1.302 / 1.150, gaussblur 1.541 / 1.230 / 1.644,
// gameoflife 0.704 / 0.647 / 0.594; then per sum: uxx1's density sum 0 (0.921),
// wave13pt's first sum 2 (0.666), jacobi's first 0 (0.453), gaussblur's
// 8-term sum 2 (1.209), lapgsrb's 12-term sum 3 and gameoflife's 3 slower): a
// sum's chain shares the FP64 unit with the integer pipes, which also form the
// products.
// A translation unit whose sweeps are bound by load latency rather than by the
// FP64 unit (the batch's small tiles) defines KG_SUMS_ON_FP64_UNIT: the
// integer additions' longer latency would then cost more than they save
// (256-problem FP64 batch: 40.9 -> 32.9 Gpts/s with them).
#ifndef KG_SUMS_ON_FP64_UNIT
#define KG_SUMS_ON_FP64_UNIT 0
#endif
template <int I, int K> __device__ __forceinline__ double nsum_sd(double acc) { return acc; }
template <int I, int K, class... T> __device__ __forceinline__ double nsum_sd(double acc, SD x, T... rest)
{
	if constexpr (I < K && !KG_SUMS_ON_FP64_UNIT) acc = se_add(acc, x.v);
	else acc = __dadd_rn(acc, x.v);
	return nsum_sd<I + 1, K>(acc, rest...);
}

// FF sums with 16-bit terms (the vector engine's BF16/FP16 reads): each
// 16-bit term joins by the mixed-precision add (no widening instruction) where
// the sum so far cannot be a product that nvcc would contract with the
// addition (any sum after the first addition, or a first term read from
// storage); otherwise the FF addition, as the expression is written.
template <bool SAFE> __device__ __forceinline__ FF nsum_h16(FF acc) { return acc; }
template <bool SAFE, class X, class... T> __device__ __forceinline__ FF nsum_h16(FF acc, X x, T... rest)
{
	if constexpr (IsH16<X>::value && SAFE) acc = add_h16(acc, x);
	else acc = acc + to_ff(x);
	return nsum_h16<true>(acc, rest...);
}

template <int K = 0, class N, class... T> __device__ __forceinline__ auto nsum(N a, T... rest)
{
	if constexpr (IsH16<N>::value || (IsH16<T>::value || ...)) {
		return nsum_h16<IsH16<N>::value>(to_ff(a), rest...);
	} else if constexpr (std::is_same<N, SD>::value) {
		return SD(nsum_sd<0, K>(a.v, rest...));
	} else if constexpr (std::is_same<N, FF2>::value) {
		float s = a.hi, e = a.lo;
		auto add = [&](FF2 x) {
			const float t = __fadd_rn(s, x.hi);
			const float bb = __fsub_rn(t, s);
			e = __fadd_rn(e, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(x.hi, bb)), x.lo));
			s = t;
		};
		(add(rest), ...);
		return ff2_fast_two_sum(s, e);
	} else {
		N acc = a;
		((acc = acc + rest), ...);
		return acc;
	}
}

// laplacian/laplacian.c:81-97
template <class N> struct OpLaplacian {
	static constexpr int LX = 1, HX = 1, LY = 1, HY = 1, LZ = 1, HZ = 1;
	static constexpr Slots slots() { return {{0}, 1, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 1, 1, 1, 1, 1}}; return h[q]; }
	N alpha, beta;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int w0 = 0;
		o[0] = pm(alpha, at(w0, 0, 0, 0)) + pm(beta, nsum<1>(
			at(w0, 1, 0, 0), at(w0, -1, 0, 0),
			at(w0, 0, 1, 0), at(w0, 0, -1, 0),
			at(w0, 0, 0, 1), at(w0, 0, 0, -1)));
	}
};

// divergence/divergence.c:84-97 (u written from ux, uy, uz)
template <class N> struct OpDivergence {
	static constexpr int LX = 1, HX = 1, LY = 1, HY = 1, LZ = 1, HZ = 1;
	static constexpr Slots slots() { return {{1, 2, 3}, 3, {0}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 1, 0, 0, 0, 0}, {0, 0, 1, 1, 0, 0}, {0, 0, 0, 0, 1, 1}}; return h[q]; }
	N alpha, beta, gamma;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int ux = 0, uy = 1, uz = 2;
		o[0] = pm(alpha, at(ux, 1, 0, 0) - at(ux, -1, 0, 0)) +
		       pm(beta, at(uy, 0, 1, 0) - at(uy, 0, -1, 0)) +
		       pm(gamma, at(uz, 0, 0, 1) - at(uz, 0, 0, -1));
	}
};

// gradient/gradient.c:85-98 (ux, uy, uz written from u)
template <class N> struct OpGradient {
	static constexpr int LX = 1, HX = 1, LY = 1, HY = 1, LZ = 1, HZ = 1;
	static constexpr Slots slots() { return {{0}, 1, {1, 2, 3}, 3}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 1, 1, 1, 1, 1}}; return h[q]; }
	N alpha, beta, gamma;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int u = 0;
		o[0] = pm(alpha, at(u, 1, 0, 0) - at(u, -1, 0, 0));
		o[1] = pm(beta, at(u, 0, 1, 0) - at(u, 0, -1, 0));
		o[2] = pm(gamma, at(u, 0, 0, 1) - at(u, 0, 0, -1));
	}
};

// uxx1/uxx1.c:70,83-106; dth = 1./nx is computed by the launcher (host IEEE
// division, the same value as the reference's per-call computation).
template <class N> struct OpUxx1 {
	static constexpr int LX = 2, HX = 1, LY = 2, HY = 1, LZ = 2, HZ = 1;
	static constexpr Slots slots() { return {{0, 2, 3, 4, 5}, 5, {1}, 1}; }
	// d1's reach; float-float reads d1 only through raw() (below), so the
	// staged engines leave it in global memory
	static constexpr Halo halo(int q) {
		constexpr Halo h[] = {{0, 0, 0, 0, 0, 0}, {0, 0, 1, 0, 1, 0}, {2, 1, 0, 0, 0, 0}, {0, 0, 2, 1, 0, 0}, {0, 0, 0, 0, 2, 1}};
		return (q == 1 && std::is_same<N, FF2>::value) ? Halo{0, 0, 0, 0, 0, 0} : h[q];
	}
	N c1, c2, dth;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int u0 = 0, d1 = 1, xx = 2, xy = 3, xz = 4;
		N d;
		if constexpr (std::is_same<N, FF2>::value) {
			// The density average can cancel (the reference draws d1 in
			// [-1,1]); FF2's 2^-48 input rounding would then dominate the
			// quotient, so it is formed from the FP64 values in FP64 and
			// rounded to FF2 once, relative to its own size.
			d = ff2_from_double(0.25 * (
				at.raw(d1, 0, 0, 0) + at.raw(d1, 0, -1, 0) +
				at.raw(d1, 0, 0, -1) + at.raw(d1, 0, -1, -1)));
		} else {
			d = pm(N(0.25), nsum<0>(
				at(d1, 0, 0, 0), at(d1, 0, -1, 0),
				at(d1, 0, 0, -1), at(d1, 0, -1, -1)));
		}
		o[0] = at(u0, 0, 0, 0) + pm(pdiv(dth, d), nsum<1>(
			pm(c1, at(xx, 0, 0, 0) - at(xx, -1, 0, 0)),
			pm(c2, at(xx, 1, 0, 0) - at(xx, -2, 0, 0)),
			pm(c1, at(xy, 0, 0, 0) - at(xy, 0, -1, 0)),
			pm(c2, at(xy, 0, 1, 0) - at(xy, 0, -2, 0)),
			pm(c1, at(xz, 0, 0, 0) - at(xz, 0, 0, -1)),
			pm(c2, at(xz, 0, 0, 1) - at(xz, 0, 0, -2))));
	}
};

// wave13pt/wave13pt.c:640-651 (plain branch), domain wave13pt.c:146-154,214
template <class N> struct OpWave13pt {
	static constexpr int LX = 2, HX = 2, LY = 2, HY = 2, LZ = 2, HZ = 2;
	static constexpr Slots slots() { return {{0, 1}, 2, {2}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{0, 0, 0, 0, 0, 0}, {2, 2, 2, 2, 2, 2}}; return h[q]; }
	N m0, m1, m2;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int w0 = 0, w1 = 1;
		o[0] = pm(m0, at(w1, 0, 0, 0)) - at(w0, 0, 0, 0) +
			pm(m1, nsum<2>(
				at(w1, 1, 0, 0), at(w1, -1, 0, 0),
				at(w1, 0, 1, 0), at(w1, 0, -1, 0),
				at(w1, 0, 0, 1), at(w1, 0, 0, -1))) +
			pm(m2, nsum<1>(
				at(w1, 2, 0, 0), at(w1, -2, 0, 0),
				at(w1, 0, 2, 0), at(w1, 0, -2, 0),
				at(w1, 0, 0, 2), at(w1, 0, 0, -2)));
	}
};

// Float-float product left unnormalised: the pair (p, e) with p the FP32
// product of the high parts and e its FMA error plus the cross terms.
__device__ __forceinline__ FF2 ff2_mul_pair(FF2 a, FF2 b)
{
	const float p = __fmul_rn(a.hi, b.hi);
	float e = __fmaf_rn(a.hi, b.hi, -p);
	e = __fmaf_rn(a.hi, b.lo, e);
	e = __fmaf_rn(a.lo, b.hi, e);
	return FF2(p, e);
}

// tricubic/tricubic.c:1041-1054: cubic Lagrange weights, same association
// (float-float: the same polynomials, operation order free within its bound).
template <class N> __device__ __forceinline__ void tricubic_weights(N a, N* w) {
	if constexpr (std::is_same<N, FF2>::value) {
		// float-float: the three pairwise products shared by the four
		// weights, unnormalised intermediates, +-1/2 applied exactly
		const FF2 ap = a + FF2(1.f, 0.f), a2 = a + FF2(2.f, 0.f), am = a - FF2(1.f, 0.f);
		const FF2 p1 = ff2_mul_pair(a, ap), p2 = ff2_mul_pair(am, a), p3 = ff2_mul_pair(am, ap);
		const FF2 c6(1.0 / 6.0);
		const FF2 h1 = ff2_mul_pair(p3, a2), h2 = ff2_mul_pair(p2, a2);
		const FF2 g0 = ff2_mul_pair(c6, ff2_mul_pair(p1, a2)), g3 = ff2_mul_pair(c6, ff2_mul_pair(p2, ap));
		w[0] = ff2_fast_two_sum(g0.hi, g0.lo);
		w[1] = ff2_fast_two_sum(-0.5f * h1.hi, -0.5f * h1.lo);
		w[2] = ff2_fast_two_sum(0.5f * h2.hi, 0.5f * h2.lo);
		w[3] = ff2_fast_two_sum(-g3.hi, -g3.lo);
		return;
	}
	const N one(1.0), two(2.0);
	w[0] = N(1.0 / 6.0) * a * (a + one) * (a + two);
	w[1] = N(-0.5) * (a - one) * (a + one) * (a + two);
	w[2] = N(0.5) * (a - one) * a * (a + two);
	w[3] = N(-1.0 / 6.0) * (a - one) * a * (a + one);
}

// Strict FP64 tricubic: of the four x-neighbours ii of every (jj, kk) row,
// the first kTricubicEmuW have their *wc product and the first
// kTricubicEmuU their *u0 product formed by the exact integer multiply
// (se_mul).  Measured on GB300 (512x256x256, ms per sweep): all on the FP64
// unit 15.85; 1 of 4 13.65; 2 of 4 12.22; 3 of 4 11.9; 4 of 4 25.6; 4 and 3
// 12.5; 3 and 4 12.3.  The kernel holds 116 registers (two CTAs of 256
// threads per SM); capping it at 85 (three CTAs) gave 14.0, letting it take
// 156 (one CTA) 21.1.  Moving part of the in-order sum, the weight
// polynomials or the wa*wb products as well was slower (those are
// dependent chains, and the integer operations' latency then shows).
constexpr int kTricubicEmuW = 3, kTricubicEmuU = 3;

// tricubic/tricubic.c:1062-1145 (64 terms, t0 + t1 + ... + t63, x fastest)
// and tricubic2/tricubic2.c:98-102 (u1 = 0; u1 += t_n, same term order).
template <class N, bool FROM_ZERO> struct OpTricubicT {
	static constexpr int LX = FROM_ZERO ? 2 : 1, HX = 2;
	static constexpr int LY = FROM_ZERO ? 2 : 1, HY = 2;
	static constexpr int LZ = FROM_ZERO ? 2 : 1, HZ = 2;
	static constexpr Slots slots() { return {{0, 2, 3, 4}, 4, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 2, 1, 2, 1, 2}, {0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}}; return h[q]; }
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int u0 = 0, pa = 1, pb = 2, pc = 3;
		N wa[4], wb[4], wc[4];
		tricubic_weights(N(at(pa, 0, 0, 0)), wa);
		tricubic_weights(N(at(pb, 0, 0, 0)), wb);
		tricubic_weights(N(at(pc, 0, 0, 0)), wc);
		if constexpr (std::is_same<N, SD>::value) {
			// Strict FP64: the same products and sum, but a share of the 128
			// products (wa*wb)*wc and (...)*u0 is formed by the exact integer
			// multiply of SE (bitwise equal to the FP64 unit's).  The 64 terms
			// are independent, so each thread keeps both the FP64 pipe and the
			// integer pipes busy; the sum stays on the FP64 pipe, in order.
			double wab[16];
#pragma unroll
			for (int jj = 0; jj < 4; jj++)
#pragma unroll
				for (int ii = 0; ii < 4; ii++)
					wab[jj * 4 + ii] = __dmul_rn(wa[ii].v, wb[jj].v);
			double s = 0.0;
#pragma unroll
			for (int kk = 0; kk < 4; kk++)
#pragma unroll
				for (int jj = 0; jj < 4; jj++)
#pragma unroll
					for (int ii = 0; ii < 4; ii++) {
						const double u = at(u0, ii - 1, jj - 1, kk - 1).v;
						const double w = wab[jj * 4 + ii];
						const double pw = ii < kTricubicEmuW ? se_mul(w, wc[kk].v) : __dmul_rn(w, wc[kk].v);
						const double t = ii < kTricubicEmuU ? se_mul(pw, u) : __dmul_rn(pw, u);
						if (kk == 0 && jj == 0 && ii == 0)
							s = FROM_ZERO ? __dadd_rn(0.0, t) : t;
						else
							s = __dadd_rn(s, t);
					}
			o[0] = N(s);
			return;
		}
		if constexpr (std::is_same<N, FF2>::value) {
			// Float-float, a form whose operation order is free within its
			// bound: s = sum_kk wc[kk] * (sum_jj,ii (wa[ii] wb[jj]) u0), each
			// dot product accumulated as one chain of TwoSums whose errors
			// collect, with the products' FMA error terms, in one FP32
			// accumulator (as nsum), renormalised once per dot product; the
			// products are left unnormalised (12 FP32 operations per term,
			// and the 64 products wab * wc are not formed).
			FF2 wab[16];
#pragma unroll
			for (int jj = 0; jj < 4; jj++)
#pragma unroll
				for (int ii = 0; ii < 4; ii++) wab[jj * 4 + ii] = wa[ii] * wb[jj];
			auto chain = [](float& s, float& e, FF2 t) {
				const float n = __fadd_rn(s, t.hi);
				const float bb = __fsub_rn(n, s);
				e = __fadd_rn(e, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(n, bb)), __fsub_rn(t.hi, bb)), t.lo));
				s = n;
			};
			float S = 0.f, E = 0.f;
#pragma unroll
			for (int kk = 0; kk < 4; kk++) {
				float s = 0.f, e = 0.f;
#pragma unroll
				for (int jj = 0; jj < 4; jj++)
#pragma unroll
					for (int ii = 0; ii < 4; ii++) {
						const FF2 t = ff2_mul_pair(wab[jj * 4 + ii], at(u0, ii - 1, jj - 1, kk - 1));
						if (jj == 0 && ii == 0) {
							s = t.hi;
							e = t.lo;
						} else {
							chain(s, e, t);
						}
					}
				const FF2 t = ff2_mul_pair(wc[kk], ff2_fast_two_sum(s, e));
				if (kk == 0) {
					S = t.hi;
					E = t.lo;
				} else {
					chain(S, E, t);
				}
			}
			o[0] = ff2_fast_two_sum(S, E);
			return;
		}
		N s;
#pragma unroll
		for (int kk = 0; kk < 4; kk++)
#pragma unroll
			for (int jj = 0; jj < 4; jj++)
#pragma unroll
				for (int ii = 0; ii < 4; ii++) {
					N t = wa[ii] * wb[jj] * wc[kk] * at(u0, ii - 1, jj - 1, kk - 1);
					if (kk == 0 && jj == 0 && ii == 0)
						s = FROM_ZERO ? N(0.0) + t : t;
					else
						s = s + t;
				}
		o[0] = s;
	}
};
template <class N> using OpTricubic = OpTricubicT<N, false>;
template <class N> using OpTricubic2 = OpTricubicT<N, true>;

// jacobi/jacobi.F90:60-67, Fortran (i,j) in [2,n-1] -> 0-based [1,n-2].
template <class N> struct OpJacobi {
	static constexpr int LX = 1, HX = 1, LY = 1, HY = 1, LZ = 0, HZ = 0;
	static constexpr Slots slots() { return {{0}, 1, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 1, 1, 1, 0, 0}}; return h[q]; }
	N c0, c1, c2;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int w0 = 0;
		o[0] = pm(c0, at(w0, 0, 0, 0)) +
			pm(c1, nsum<0>(at(w0, -1, 0, 0), at(w0, 0, -1, 0), at(w0, 1, 0, 0), at(w0, 0, 1, 0))) +
			pm(c2, nsum<1>(at(w0, -1, -1, 0), at(w0, -1, 1, 0), at(w0, 1, -1, 0), at(w0, 1, 1, 0)));
	}
};

// lapgsrb/lapgsrb.c:93-117
template <class N> struct OpLapgsrb {
	static constexpr int LX = 2, HX = 2, LY = 2, HY = 2, LZ = 2, HZ = 2;
	static constexpr Slots slots() { return {{0}, 1, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{2, 2, 2, 2, 2, 2}}; return h[q]; }
	N c0, c1, c2, c3;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int w = 0;
		o[0] = pm(c0, at(w, 0, 0, 0)) +
			pm(c1, nsum<2>(
				at(w, 1, 0, 0), at(w, -1, 0, 0),
				at(w, 0, 1, 0), at(w, 0, -1, 0),
				at(w, 0, 0, 1), at(w, 0, 0, -1))) +
			pm(c2, nsum<2>(
				at(w, 1, 1, 0), at(w, 1, 0, 1), at(w, 1, 0, -1), at(w, 1, -1, 0),
				at(w, 0, 1, 1), at(w, 0, 1, -1), at(w, 0, -1, 1), at(w, 0, -1, -1),
				at(w, -1, 1, 0), at(w, -1, 0, 1), at(w, -1, 0, -1), at(w, -1, -1, 0))) +
			pm(c3, nsum<2>(
				at(w, 2, 0, 0), at(w, -2, 0, 0),
				at(w, 0, 2, 0), at(w, 0, -2, 0),
				at(w, 0, 0, 2), at(w, 0, 0, -2)));
	}
};

// gaussblur/gaussblur.c:65,85-92; f = 1/(s0+4(s1+s2+s4+s8)+8 s5) is computed
// by the launcher (host, no contraction: the reference's per-call value).
template <class N> struct OpGaussblur {
	static constexpr int LX = 2, HX = 2, LY = 2, HY = 2, LZ = 0, HZ = 0;
	static constexpr Slots slots() { return {{0}, 1, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{2, 2, 2, 2, 0, 0}}; return h[q]; }
	N s0, s1, s2, s4, s5, s8, f;
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int w = 0;
		o[0] = pm(f, (
			pm(s0, at(w, 0, 0, 0)) +
			pm(s1, nsum<1>(at(w, -1, 0, 0), at(w, 1, 0, 0), at(w, 0, -1, 0), at(w, 0, 1, 0))) +
			pm(s2, nsum<1>(at(w, -1, -1, 0), at(w, 1, -1, 0), at(w, -1, 1, 0), at(w, 1, 1, 0))) +
			pm(s4, nsum<1>(at(w, -2, 0, 0), at(w, 2, 0, 0), at(w, 0, -2, 0), at(w, 0, 2, 0))) +
			pm(s5, nsum<2>(at(w, -2, -1, 0), at(w, -1, -2, 0), at(w, 1, -2, 0), at(w, 2, -1, 0),
			      at(w, -2, 1, 0), at(w, -1, 2, 0), at(w, 1, 2, 0), at(w, 2, 1, 0))) +
			pm(s8, nsum<1>(at(w, -2, -2, 0), at(w, 2, -2, 0), at(w, -2, 2, 0), at(w, 2, 2, 0)))));
	}
};

// gameoflife/gameoflife.c:81-91
template <class N> struct OpGameoflife {
	static constexpr int LX = 1, HX = 1, LY = 1, HY = 1, LZ = 0, HZ = 0;
	static constexpr Slots slots() { return {{0}, 1, {1}, 1}; }
	static constexpr Halo halo(int q) { constexpr Halo h[] = {{1, 1, 1, 1, 0, 0}}; return h[q]; }
	template <class A> __device__ __forceinline__ void point(const A& at, N* o) const {
		const int u0 = 0;
		const N C(100000000000000000000.);
		N L = nsum<2>(
			at(u0, -1, -1, 0), at(u0, 0, -1, 0), at(u0, 1, -1, 0),
			at(u0, -1, 0, 0),                    at(u0, 1, 0, 0),
			at(u0, -1, 1, 0), at(u0, 0, 1, 0), at(u0, 1, 1, 0));
		o[0] = pdiv(N(1.), N(1.) + pm(pm(at(u0, 0, 0, 0) + L - N(3.), L - N(3.)), C));
	}
};

}  // namespace kg
