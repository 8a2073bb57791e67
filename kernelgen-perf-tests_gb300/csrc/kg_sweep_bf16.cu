// kg_sweep_bf16.cu -- sweeps with storage __nv_bfloat16, arithmetic FF (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_bf16(const kg_problem& p, cudaStream_t s) { return sweep_typed<FF, __nv_bfloat16>(p, s); }
cudaError_t regs_bf16(const kg_problem& p, int* nregs) { return regs_typed<FF, __nv_bfloat16>(p, nregs); }
}  // namespace kg
