// kg_engine.cuh -- iteration engine of the sweeps.
//
// One thread owns one (i, j) column and walks a run of KC consecutive planes
// k, so neighbouring threads of a warp touch consecutive x addresses (full
// 128-byte lines per warp for FP32, two per warp for FP64) and the z
// neighbours of plane k are the centre values of planes k+-1 that the same
// thread has just read (served from L1).  Rims [0,L) and (n-1-H, n-1] of every
// axis are never written, as in the reference loops.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <type_traits>

#include "../../include/kg_b200.h"
#include "kg_ops.cuh"

namespace kg {

template <class S> struct Ptrs {
	const S* in[6];
	S* out[3];
};

template <class N, class S> struct GAcc {
	const S* const* in;
	long long c, sy, sz;
	__device__ __forceinline__ N operator()(int q, int dx, int dy, int dz) const {
		return Conv<N, S>::ld(in[q] + c + dx + dy * sy + dz * sz);
	}
	// The stored value itself, without conversion to N.
	__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const {
		return __ldg(in[q] + c + dx + dy * sy + dz * sz);
	}
};

constexpr int kBX = 32, kBY = 8;


// One tile: BX x BY columns (threadIdx.x, threadIdx.y) of the update domain,
// planes [LZ + tz*KC, LZ + (tz+1)*KC).  2D ops (LZ = HZ = 0, ns = 1) walk KC
// rows instead, BY apart, so a tile covers BX x (BY*KC) points either way.
// The z loop is unrolled UK times so that a thread has the loads of UK
// planes in flight at once (measured on GB300: FP32 wave13pt 213 -> 348
// Gpts/s going from 1 to 2).
template <class Op, class N, class S, int BX, int BY, int KC, int UK = 2>
__device__ __forceinline__ void sweep_tile(const Op& op, const Ptrs<S>& p, int nx, int ny, int ns,
	int tx, int ty, int tz)
{
	constexpr Slots sl = Op::slots();
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	const int i = Op::LX + tx * BX + (int)threadIdx.x;
	if (i >= nx - Op::HX) return;
	const long long sy = nx, sz = (long long)nx * ny;
	if (k2d) {
		const int j0 = Op::LY + ty * (BY * KC) + (int)threadIdx.y;
#pragma unroll 1
		for (int r = 0; r < KC; r++) {
			const int j = j0 + r * BY;
			if (j >= ny - Op::HY) break;
			const long long c = i + sy * j;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	} else {
		const int j = Op::LY + ty * BY + (int)threadIdx.y;
		if (j >= ny - Op::HY) return;
		const int k0 = Op::LZ + tz * KC, k1 = min(k0 + KC, ns - Op::HZ);
#pragma unroll UK
		for (int k = k0; k < k1; k++) {
			const long long c = i + sy * j + sz * k;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	}
}

// Tiles of a domain along each axis for the (BX, BY, KC) tile shape.
template <class Op> struct TileCount {
	static __host__ __device__ int x(int nx, int bx) { return max(0, (nx - Op::LX - Op::HX + bx - 1) / bx); }
	static __host__ __device__ int y(int ny, int by, int kc) {
		const int d = ny - Op::LY - Op::HY;
		const int t = (Op::LZ == 0 && Op::HZ == 0) ? by * kc : by;
		return max(0, (d + t - 1) / t);
	}
	static __host__ __device__ int z(int ns, int kc) {
		if (Op::LZ == 0 && Op::HZ == 0) return 1;
		return max(0, (ns - Op::LZ - Op::HZ + kc - 1) / kc);
	}
};

template <class Op, class N, class S, int KC>
__global__ void __launch_bounds__(kBX * kBY) sweep_kernel(Op op, Ptrs<S> p, int nx, int ny, int ns)
{
	const int tyn = TileCount<Op>::y(ny, kBY, KC), tzn = TileCount<Op>::z(ns, KC);
	for (int ty = blockIdx.y; ty < tyn; ty += gridDim.y)
		for (int tz = blockIdx.z; tz < tzn; tz += gridDim.z)
			sweep_tile<Op, N, S, kBX, kBY, KC>(op, p, nx, ny, ns, blockIdx.x, ty, tz);
}

template <class Op, class N, class S>
struct Launch {
	static constexpr int KC = 8;
	static const void* func() { return (const void*)sweep_kernel<Op, N, S, KC>; }
	static cudaError_t run(const Op& op, const kg_problem& pr, cudaStream_t st) {
		constexpr Slots sl = Op::slots();
		Ptrs<S> p{};
		for (int q = 0; q < sl.nin; q++) p.in[q] = (const S*)pr.arr[sl.in[q]];
		for (int q = 0; q < sl.nout; q++) p.out[q] = (S*)pr.arr[sl.out[q]];
		const int tx = TileCount<Op>::x(pr.nx, kBX), ty = TileCount<Op>::y(pr.ny, kBY, KC),
			tz = TileCount<Op>::z(pr.ns, KC);
		if (tx <= 0 || ty <= 0 || tz <= 0) return cudaSuccess;  // empty domain: nothing to write
		dim3 block(kBX, kBY, 1);
		dim3 grid(tx, (unsigned)min(ty, 65535), (unsigned)min(tz, 65535));
		sweep_kernel<Op, N, S, KC><<<grid, block, 0, st>>>(op, p, pr.nx, pr.ny, pr.ns);
		return cudaGetLastError();
	}
};

// Builds the op of pr.stencil with coefficients converted to N, then calls
// F::template go<Op>(op).
template <class N, class F>
cudaError_t with_op(const kg_problem& pr, F&& f)
{
	const double* k = pr.coef;
	switch (pr.stencil) {
	case KG_LAPLACIAN: return f(OpLaplacian<N>{N(k[0]), N(k[1])});
	case KG_DIVERGENCE: return f(OpDivergence<N>{N(k[0]), N(k[1]), N(k[2])});
	case KG_GRADIENT: return f(OpGradient<N>{N(k[0]), N(k[1]), N(k[2])});
	case KG_UXX1: return f(OpUxx1<N>{N(k[0]), N(k[1]), N(1. / pr.nx)});
	case KG_WAVE13PT: return f(OpWave13pt<N>{N(k[0]), N(k[1]), N(k[2])});
	case KG_TRICUBIC: return f(OpTricubic<N>{});
	case KG_TRICUBIC2: return f(OpTricubic2<N>{});
	case KG_JACOBI: return f(OpJacobi<N>{N(k[0]), N(k[1]), N(k[2])});
	case KG_LAPGSRB: return f(OpLapgsrb<N>{N(k[0]), N(k[1]), N(k[2]), N(k[3])});
	case KG_GAUSSBLUR: {
		// gaussblur/gaussblur.c:65, evaluated on the host without contraction
		const double fnorm = 1. / (k[0] + 4 * (k[1] + k[2] + k[3] + k[5]) + 8 * k[4]);
		return f(OpGaussblur<N>{N(k[0]), N(k[1]), N(k[2]), N(k[3]), N(k[4]), N(k[5]), N(fnorm)});
	}
	case KG_GAMEOFLIFE: return f(OpGameoflife<N>{});
	default: return cudaErrorInvalidValue;
	}
}

}  // namespace kg
