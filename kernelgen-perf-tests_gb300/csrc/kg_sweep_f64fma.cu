// kg_sweep_f64fma.cu -- sweeps with storage double, arithmetic FD (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_f64fma(const kg_problem& p, cudaStream_t s) { return sweep_typed<FD, double>(p, s); }
cudaError_t regs_f64fma(const kg_problem& p, int* nregs) { return regs_typed<FD, double>(p, nregs); }
}  // namespace kg
