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
};

constexpr int kBX = 32, kBY = 8;

template <class Op, class N, class S, int KC>
__global__ void __launch_bounds__(kBX * kBY) sweep_kernel(Op op, Ptrs<S> p, int nx, int ny, int ns)
{
	constexpr Slots sl = Op::slots();
	const int i = Op::LX + blockIdx.x * kBX + threadIdx.x;
	const int iend = nx - Op::HX, jend = ny - Op::HY, kend = ns - Op::HZ;
	if (i >= iend) return;
	const long long sy = nx, sz = (long long)nx * ny;
	for (int j = Op::LY + blockIdx.y * kBY + threadIdx.y; j < jend; j += gridDim.y * kBY) {
		for (int k0 = Op::LZ + blockIdx.z * KC; k0 < kend; k0 += gridDim.z * KC) {
			const int k1 = min(k0 + KC, kend);
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
}

template <class Op, class N, class S>
struct Launch {
	static constexpr int KC = (Op::LZ == 0 && Op::HZ == 0) ? 1 : 8;
	static const void* func() { return (const void*)sweep_kernel<Op, N, S, KC>; }
	static cudaError_t run(const Op& op, const kg_problem& pr, cudaStream_t st) {
		constexpr Slots sl = Op::slots();
		Ptrs<S> p{};
		for (int q = 0; q < sl.nin; q++) p.in[q] = (const S*)pr.arr[sl.in[q]];
		for (int q = 0; q < sl.nout; q++) p.out[q] = (S*)pr.arr[sl.out[q]];
		const int dx = pr.nx - Op::LX - Op::HX, dy = pr.ny - Op::LY - Op::HY, dz = pr.ns - Op::LZ - Op::HZ;
		if (dx <= 0 || dy <= 0 || dz <= 0) return cudaSuccess;  // empty domain: nothing to write
		dim3 block(kBX, kBY, 1);
		dim3 grid((dx + kBX - 1) / kBX, (unsigned)min((dy + kBY - 1) / kBY, 65535),
			(unsigned)min((dz + KC - 1) / KC, 65535));
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

template <class N, class S>
cudaError_t sweep_typed(const kg_problem& pr, cudaStream_t st)
{
	return with_op<N>(pr, [&](const auto& op) {
		using Op = std::decay_t<decltype(op)>;
		return Launch<Op, N, S>::run(op, pr, st);
	});
}

template <class N, class S>
cudaError_t regs_typed(const kg_problem& pr, int* nregs)
{
	return with_op<N>(pr, [&](const auto& op) {
		using Op = std::decay_t<decltype(op)>;
		cudaFuncAttributes a;
		cudaError_t e = cudaFuncGetAttributes(&a, Launch<Op, N, S>::func());
		if (e == cudaSuccess) *nregs = a.numRegs;
		return e;
	});
}

}  // namespace kg
