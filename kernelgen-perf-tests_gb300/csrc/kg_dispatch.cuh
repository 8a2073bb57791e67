// kg_dispatch.cuh -- which engine runs a sweep of a given arithmetic.
//
// Engines (kg_problem.engine, KG_ENGINE_AUTO picks per arithmetic):
//   direct (kg_engine.cuh)  one thread per (i, j) column, neighbours through L1;
//   staged (kg_staged.cuh)  halo planes in shared memory, loaded by all threads
//                           and converted once to the arithmetic's pair;
//   tma    (kg_tma.cuh)     halo planes in shared memory, moved by tiled bulk
//                           copies, own column in registers.
// Strict and contracted FP64 (SD, FD) are bound by the FP64 pipe and run
// direct by default; FP32 arithmetic (FF) is bound by memory and runs on the
// TMA engine for the stencils where that measured faster on GB300, where the
// arrays allow it, and direct for the rest.  Same-run Gpts/s, direct -> TMA,
// FP32 512x256x256: laplacian 443 -> 583, divergence 343 -> 402, gradient
// 238 -> 325, uxx1 171 -> 224, lapgsrb 260 -> 289, wave13pt 340 -> 344,
// tricubic 95 -> 86; 1024x512x512: laplacian 443 -> 681, uxx1 170 -> 234,
// wave13pt 351 -> 377; BF16 1024x512x512: laplacian 482 -> 636, uxx1 162 ->
// 264, wave13pt 354 -> 341.  tricubic, tricubic2 and the 2D stencils stay
// direct, and wave13pt takes TMA for 4-byte storage only.  Float-float (FF2)
// is bound by issue slots and runs staged, which splits each value once
// instead of once per use.
#pragma once

#include <type_traits>

#include "kg_engine.cuh"
#include "kg_staged.cuh"
#include "kg_tma.cuh"
#include "kg_tmavec.cuh"

namespace kg {

// KG_FF_STAGED=1 at build time compiles the staged engine for FP32 too.
#ifndef KG_FF_STAGED
#define KG_FF_STAGED 0
#endif

template <class N> struct Engines {
	static constexpr bool ff2 = std::is_same<N, FF2>::value;
	static constexpr bool ff = std::is_same<N, FF>::value;
	static constexpr bool direct = !ff2;
	static constexpr bool staged = ff2 || (ff && KG_FF_STAGED);
	static constexpr bool tma = true;
	static constexpr bool tma_vec = ff;
	static constexpr int automatic = ff2 ? KG_ENGINE_STAGED : ff ? KG_ENGINE_TMA : KG_ENGINE_DIRECT;
};

// FP32 arithmetic: the stencils that run on the vector TMA engine by default
// (where its arrays allow it, else the TMA or direct engine).  The 2D ones
// walk bands of rows: measured at 512x65536 (Gpts/s, direct / vector TMA),
// FP32 jacobi 362 / 616, gaussblur 255 / 479, gameoflife 355 / 604; BF16
// 380 / 955, 258 / 627, 371 / 708.  tricubic (compute-bound) at 512x256x256:
// FP32 95 (TMA engine) / 112, BF16 85 / 116.
inline bool tma_vec_preferred(int stencil)
{
	return stencil == KG_LAPLACIAN || stencil == KG_DIVERGENCE || stencil == KG_GRADIENT ||
		stencil == KG_UXX1 || stencil == KG_LAPGSRB || stencil == KG_WAVE13PT || stencil == KG_JACOBI ||
		stencil == KG_GAUSSBLUR || stencil == KG_GAMEOFLIFE || stencil == KG_TRICUBIC || stencil == KG_TRICUBIC2;
}

inline bool tma_preferred(int stencil, int elem_bytes)
{
	return stencil == KG_LAPLACIAN || stencil == KG_DIVERGENCE || stencil == KG_GRADIENT ||
		stencil == KG_UXX1 || stencil == KG_LAPGSRB || (stencil == KG_WAVE13PT && elem_bytes == 4);
}

template <class N, class S> int automatic_engine(int stencil)
{
	const int e = Engines<N>::automatic;
	// float-float: the staged engine splits each value once, which pays where
	// values are used many times; divergence and uxx1 read most inputs along
	// one axis only, and the TMA copies win there (FF2 Gpts/s at 512x256x256,
	// staged -> TMA: divergence 88.6 -> 93.6, uxx1 45.2 -> 48.7; laplacian
	// 130.8 -> 101.6, wave13pt 80.7 -> 62.7, tricubic 13.3 -> 6.6)
	if (e == KG_ENGINE_STAGED) return (stencil == KG_DIVERGENCE || stencil == KG_UXX1) ? KG_ENGINE_TMA : e;
	return e == KG_ENGINE_TMA && !tma_preferred(stencil, (int)sizeof(S)) ? KG_ENGINE_DIRECT : e;
}

template <class Op, class N, class S>
int resolve_engine(const kg_problem& pr)
{
	if (pr.engine != KG_ENGINE_AUTO) return pr.engine;
	if constexpr (Engines<N>::tma_vec)
		if (tma_vec_preferred(pr.stencil) && TmaVecLaunch<Op, N, S>::usable(pr)) return KG_ENGINE_TMA_VEC;
	const int e = automatic_engine<N, S>(pr.stencil);
	if (e == KG_ENGINE_TMA && !TmaLaunch<Op, N, S>::usable(pr))
		return Engines<N>::ff2 ? KG_ENGINE_STAGED : KG_ENGINE_DIRECT;
	return e;
}

template <class N, class S>
cudaError_t sweep_typed(const kg_problem& pr, cudaStream_t st)
{
	return with_op<N>(pr, [&](const auto& op) -> cudaError_t {
		using Op = std::decay_t<decltype(op)>;
		const int e = resolve_engine<Op, N, S>(pr);
		if constexpr (Engines<N>::tma_vec)
			if (e == KG_ENGINE_TMA_VEC)
				return TmaVecLaunch<Op, N, S>::usable(pr) ? TmaVecLaunch<Op, N, S>::run(op, pr, st) : cudaErrorInvalidValue;
		if constexpr (Engines<N>::tma)
			if (e == KG_ENGINE_TMA)
				return TmaLaunch<Op, N, S>::usable(pr) ? TmaLaunch<Op, N, S>::run(op, pr, st) : cudaErrorInvalidValue;
		if constexpr (Engines<N>::staged)
			if (e == KG_ENGINE_STAGED) return StagedLaunch<Op, N, S>::run(op, pr, st);
		if constexpr (Engines<N>::direct)
			if (e == KG_ENGINE_DIRECT) return Launch<Op, N, S>::run(op, pr, st);
		return cudaErrorNotSupported;
	});
}

// Registers per thread of the kernel the automatic choice runs on aligned arrays.
template <class N, class S>
cudaError_t regs_typed(const kg_problem& pr, int* nregs)
{
	return with_op<N>(pr, [&](const auto& op) -> cudaError_t {
		using Op = std::decay_t<decltype(op)>;
		const void* f = nullptr;
		int e = automatic_engine<N, S>(pr.stencil);
		if constexpr (Engines<N>::tma_vec)
			if (tma_vec_preferred(pr.stencil) && TmaVecLaunch<Op, N, S>::built) {
				f = TmaVecLaunch<Op, N, S>::func();
				e = -1;
			}
		if constexpr (Engines<N>::tma)
			if (e == KG_ENGINE_TMA) f = TmaLaunch<Op, N, S>::func();
		if constexpr (Engines<N>::staged)
			if (e == KG_ENGINE_STAGED) f = StagedLaunch<Op, N, S>::func();
		if constexpr (Engines<N>::direct)
			if (e == KG_ENGINE_DIRECT) f = Launch<Op, N, S>::func();
		cudaFuncAttributes a;
		cudaError_t err = cudaFuncGetAttributes(&a, f);
		if (err == cudaSuccess) *nregs = a.numRegs;
		return err;
	});
}

// Engines built for a storage type (bit e set: engine e available).
constexpr int engines_mask_ff() { return (1 << KG_ENGINE_DIRECT) | (1 << KG_ENGINE_TMA) | (KG_FF_STAGED ? 1 << KG_ENGINE_STAGED : 0); }

}  // namespace kg
