// kg_sweep_f64.cu -- sweeps with storage double, arithmetic SD (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_f64(const kg_problem& p, cudaStream_t s) { return sweep_typed<SD, double>(p, s); }
cudaError_t regs_f64(const kg_problem& p, int* nregs) { return regs_typed<SD, double>(p, nregs); }
}  // namespace kg
