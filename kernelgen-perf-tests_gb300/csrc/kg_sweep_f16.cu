// kg_sweep_f16.cu -- sweeps with storage __half, arithmetic FF (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_f16(const kg_problem& p, cudaStream_t s) { return sweep_typed<FF, __half>(p, s); }
cudaError_t regs_f16(const kg_problem& p, int* nregs) { return regs_typed<FF, __half>(p, nregs); }
}  // namespace kg
