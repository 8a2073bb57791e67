// kg_sweep_f32.cu -- sweeps with storage float, arithmetic FF (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_f32(const kg_problem& p, cudaStream_t s) { return sweep_typed<FF, float>(p, s); }
cudaError_t regs_f32(const kg_problem& p, int* nregs) { return regs_typed<FF, float>(p, nregs); }
}  // namespace kg
