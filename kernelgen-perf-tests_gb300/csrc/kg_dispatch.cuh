// kg_dispatch.cuh -- which engine runs a sweep of a given arithmetic.
//
// Strict and contracted FP64 (SD, FD) are bound by the FP64 pipe and FP32
// (FF) by memory; they use the direct engine (kg_engine.cuh), whose neighbour
// loads hit L1.  Float-float arithmetic (FF2) is bound by issue slots; it uses
// the staged engine (kg_staged.cuh), which moves each value into shared
// memory once and splits it into its pair once instead of once per use.
#pragma once

#include <type_traits>

#include "kg_engine.cuh"
#include "kg_staged.cuh"

namespace kg {

// KG_FF_STAGED=1 at build time moves FP32 arithmetic to the staged engine too.
#ifndef KG_FF_STAGED
#define KG_FF_STAGED 0
#endif
template <class Op, class N, class S>
using LaunchFor = typename std::conditional<std::is_same<N, FF2>::value || (KG_FF_STAGED && std::is_same<N, FF>::value),
	StagedLaunch<Op, N, S>, Launch<Op, N, S>>::type;

template <class N, class S>
cudaError_t sweep_typed(const kg_problem& pr, cudaStream_t st)
{
	return with_op<N>(pr, [&](const auto& op) {
		using Op = std::decay_t<decltype(op)>;
		return LaunchFor<Op, N, S>::run(op, pr, st);
	});
}

template <class N, class S>
cudaError_t regs_typed(const kg_problem& pr, int* nregs)
{
	return with_op<N>(pr, [&](const auto& op) {
		using Op = std::decay_t<decltype(op)>;
		cudaFuncAttributes a;
		cudaError_t e = cudaFuncGetAttributes(&a, LaunchFor<Op, N, S>::func());
		if (e == cudaSuccess) *nregs = a.numRegs;
		return e;
	});
}

}  // namespace kg
