// kg_sweep_f64ff.cu -- sweeps with FP64 storage and float-float arithmetic (kg_num.cuh).
#include "kg_dispatch.cuh"
#include "kg_internal.h"

namespace kg {
cudaError_t sweep_f64ff(const kg_problem& p, cudaStream_t s) { return sweep_typed<FF2, double>(p, s); }
cudaError_t regs_f64ff(const kg_problem& p, int* nregs) { return regs_typed<FF2, double>(p, nregs); }
}  // namespace kg
