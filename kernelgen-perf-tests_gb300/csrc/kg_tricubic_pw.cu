// kg_tricubic_pw.cu -- tricubic programs with their loop-invariant weights
// computed once.
//
// In a tricubic / tricubic2 program the offsets a, b, c never change during
// the nt-sweep time loop (tricubic/tricubic.c:293-303 rotates only u0 and
// u1), so the 64 weight products of every point, pw = (wa[ii] * wb[jj]) *
// wc[kk], are the same in every sweep.  A program (a plan or
// kg_program_run) therefore evaluates them once, with the same operations in
// the same order as the sweep (tricubic/tricubic.c:1041-1145), into 64
// planes, and each sweep reads them and forms only sum_n pw[n] * u0[n] in
// the reference's term order.  The result is bit for bit the sweep's: every
// product and sum is the same IEEE operation on the same operands.
//
// The strict sweep then needs 64 products and 64 additions per point instead
// of 252 FP64 operations; a share of the products runs on the integer pipes
// (se_mul), as in the per-sweep kernel.  The planes cost 512 bytes per point,
// so the path is taken only where they fit (tricubic_pw_bytes).
#include <cstdint>

#include "kg_engine.cuh"
#include "kg_internal.h"

namespace kg {

// Products pw * u0 formed by the exact integer multiply: x-neighbours ii <
// kTriPwEmu of every (jj, kk) row.  Measured on GB300 (512x256x256, weights
// once + 10 sweeps, ms, all additions on the FP64 unit): 0 of 4: 85.6; 1:
// 75.7; 2: 65.9; 3: 56.7; 4: 61.5 (10 sweeps computing the weights inline:
// 118.7).  Between 3 and 4, x-neighbour 3 of the first 1, 2 or 3 rows jj of
// every kk as well (tricubic / tricubic2 programs, ms, against 56.2 / 56.7):
// 57.8 / 57.7, 60.2 / 59.8 and, with no integer additions, 56.6 / 57.0 (one
// row), 58.3 / 58.1 (two), 60.8 / 60.4 (three): the integer multiply's extra
// instructions cost issue slots the FP64 unit's queue would have hidden.
#ifndef KG_PW_EMU
#define KG_PW_EMU 3
#endif
constexpr int kTriPwEmu = KG_PW_EMU;

#ifndef KG_PW_ADD_INT
#define KG_PW_ADD_INT 1
#endif
// Additions of the in-order sum on the integer pipes (se_add): the first
// kTriPwAddInt of every run of 16 terms (one kk).  Measured (ms per sweep,
// tricubic / tricubic2, products on the integer pipes 3 of 4): 0 additions
// 5.686 / 5.824, 1: 5.652 / 5.698, 2: 5.787 / 5.780; with 2 of 4 products
// and 2 or 4 additions 6.104 / 6.272 and 5.822 / 5.903; with all 4 products
// and 0 or 1 addition (ms per 10-sweep program, weights included) 61.5 /
// 61.0 and 63.9 / 63.4 against 56.1 / 56.7.
constexpr int kTriPwAddInt = KG_PW_ADD_INT;

constexpr int kPwBX = 32, kPwBY = 8, kPwKC = 8;

// Layout of the planes: the points are taken in runs of 32 along x (one warp's
// points), and the 64 products of a run are stored term after term, 32
// doubles per term: a warp reads each term as one 256-byte line and a run's
// 64 terms lie in one 16 KB block.  Run (bx, j, k) is block (k ny + j) tx + bx
// with tx = ceil(nx / 32).
__device__ __forceinline__ size_t pw_at(int bx, int j, int k, int ny, int tx, int m, int lane)
{
	return ((((size_t)k * ny + j) * tx + bx) * 64 + m) * 32 + lane;
}

template <class N, bool FROM_ZERO>
__global__ void __launch_bounds__(kPwBX * kPwBY, 2) tricubic_pw_kernel(int nx, int ny, int ns,
	const double* __restrict__ pa, const double* __restrict__ pb, const double* __restrict__ pc,
	double* __restrict__ pw)
{
	using Op = OpTricubicT<N, FROM_ZERO>;
	const int i = Op::LX + blockIdx.x * kPwBX + threadIdx.x;
	const int j = Op::LY + blockIdx.y * kPwBY + threadIdx.y;
	if (i >= nx - Op::HX || j >= ny - Op::HY) return;
	const int tx = (nx + kPwBX - 1) / kPwBX;
	const int k0 = Op::LZ + blockIdx.z * kPwKC, k1 = min(k0 + kPwKC, ns - Op::HZ);
#pragma unroll 1
	for (int k = k0; k < k1; k++) {
		const size_t c = i + (size_t)nx * j + (size_t)nx * ny * k;
		N wa[4], wb[4], wc[4];
		tricubic_weights(N(__ldg(pa + c)), wa);
		tricubic_weights(N(__ldg(pb + c)), wb);
		tricubic_weights(N(__ldg(pc + c)), wc);
#pragma unroll 1
		for (int kk = 0; kk < 4; kk++)
#pragma unroll
			for (int jj = 0; jj < 4; jj++)
#pragma unroll
				for (int ii = 0; ii < 4; ii++) {
					double v;
					if constexpr (std::is_same<N, SD>::value) {
						const double wab = __dmul_rn(wa[ii].v, wb[jj].v);
						v = (ii & 1) ? se_mul(wab, wc[kk].v) : __dmul_rn(wab, wc[kk].v);
					} else {
						v = (wa[ii] * wb[jj] * wc[kk]).v;
					}
					__stcs(pw + pw_at(blockIdx.x, j, k, ny, tx, kk * 16 + jj * 4 + ii, threadIdx.x), v);
				}
	}
}

template <class N, bool FROM_ZERO>
__global__ void __launch_bounds__(kPwBX * kPwBY, 3) tricubic_pw_sweep_kernel(int nx, int ny, int ns,
	const double* __restrict__ u0, double* __restrict__ u1, const double* __restrict__ pw)
{
	using Op = OpTricubicT<N, FROM_ZERO>;
	const int i = Op::LX + blockIdx.x * kPwBX + threadIdx.x;
	const int j = Op::LY + blockIdx.y * kPwBY + threadIdx.y;
	if (i >= nx - Op::HX || j >= ny - Op::HY) return;
	const int tx = (nx + kPwBX - 1) / kPwBX;
	const long long sy = nx, sz = (long long)nx * ny;
	const int k0 = Op::LZ + blockIdx.z * kPwKC, k1 = min(k0 + kPwKC, ns - Op::HZ);
#pragma unroll 1
	for (int k = k0; k < k1; k++) {
		const size_t c = i + (size_t)nx * j + (size_t)nx * ny * k;
		const double* w = pw + pw_at(blockIdx.x, j, k, ny, tx, 0, threadIdx.x);
		N s;
#pragma unroll 1
		for (int kk = 0; kk < 4; kk++)
#pragma unroll
			for (int jj = 0; jj < 4; jj++)
#pragma unroll
				for (int ii = 0; ii < 4; ii++) {
					const int m = kk * 16 + jj * 4 + ii;
					const double wv = __ldcs(w + m * 32);
					const double u = __ldg(u0 + c + (ii - 1) + (jj - 1) * sy + (kk - 1) * sz);
					N t;
					if constexpr (std::is_same<N, SD>::value)
						t = SD(ii < kTriPwEmu ? se_mul(wv, u) : __dmul_rn(wv, u));
					else
						t = N(wv) * N(u);
					if (m == 0) s = FROM_ZERO ? N(0.0) + t : t;
					else if constexpr (std::is_same<N, SD>::value)
						s = SD((m & 15) != 0 && (m & 15) <= kTriPwAddInt ? se_add(s.v, t.v) : __dadd_rn(s.v, t.v));
					else s = s + t;
				}
		u1[c] = s.v;
	}
}

static dim3 pw_grid(int stencil, int nx, int ny, int ns)
{
	const int l = stencil == KG_TRICUBIC2 ? 2 : 1;   // domain [l, n-3] per axis
	auto t = [&](int d, int b) { return std::max(0, (d - l - 2 + b - 1) / b); };
	return dim3(t(nx, kPwBX), (unsigned)std::min(t(ny, kPwBY), 65535), (unsigned)std::min(t(ns, kPwKC), 65535));
}

// Device bytes of the 64 weight planes of p, 0 where the path does not
// apply (not tricubic / tricubic2, not KG_F64 or KG_F64_FMA, or a grid
// beyond the launch limits).
size_t tricubic_pw_bytes(const kg_problem& p)
{
	if (p.stencil != KG_TRICUBIC && p.stencil != KG_TRICUBIC2) return 0;
	if (p.dtype != KG_F64 && p.dtype != KG_F64_FMA) return 0;
	if (p.nx < 5 || p.ny < 5 || p.ns < 5) return 0;
	if ((p.ny + kPwBY - 1) / kPwBY > 65535 || (p.ns + kPwKC - 1) / kPwKC > 65535) return 0;
	return (size_t)((p.nx + kPwBX - 1) / kPwBX) * p.ny * p.ns * 64 * kPwBX * sizeof(double);
}

template <class F> static cudaError_t by_form(const kg_problem& p, F&& f)
{
	const bool z = p.stencil == KG_TRICUBIC2;
	if (p.dtype == KG_F64) return z ? f(SD{}, std::true_type{}) : f(SD{}, std::false_type{});
	return z ? f(FD{}, std::true_type{}) : f(FD{}, std::false_type{});
}

// The 64 planes of p (arrays in the reference's argument order: u0, u1, a, b, c).
cudaError_t tricubic_pw_precompute(const kg_problem& p, double* pw, cudaStream_t st)
{
	return by_form(p, [&](auto nv, auto zv) {
		using N = decltype(nv);
		constexpr bool Z = decltype(zv)::value;
		tricubic_pw_kernel<N, Z><<<pw_grid(p.stencil, p.nx, p.ny, p.ns), dim3(kPwBX, kPwBY), 0, st>>>(
			p.nx, p.ny, p.ns, (const double*)p.arr[2], (const double*)p.arr[3], (const double*)p.arr[4], pw);
		return cudaGetLastError();
	});
}

// One sweep of p (current roles of u0, u1) from the planes.
cudaError_t tricubic_pw_sweep(const kg_problem& p, const double* pw, cudaStream_t st)
{
	return by_form(p, [&](auto nv, auto zv) {
		using N = decltype(nv);
		constexpr bool Z = decltype(zv)::value;
		tricubic_pw_sweep_kernel<N, Z><<<pw_grid(p.stencil, p.nx, p.ny, p.ns), dim3(kPwBX, kPwBY), 0, st>>>(
			p.nx, p.ny, p.ns, (const double*)p.arr[0], (double*)p.arr[1], pw);
		return cudaGetLastError();
	});
}

}  // namespace kg
