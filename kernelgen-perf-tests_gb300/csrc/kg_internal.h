// kg_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/kg_b200.h"

namespace kg {

// One sweep / register count of the sweep kernel, per storage type (one
// translation unit each, compiled in parallel).
cudaError_t sweep_f64(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_f64fma(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_f64ff(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_f32(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_bf16(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_f16(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_u8(const kg_problem& p, cudaStream_t s);
cudaError_t regs_f64(const kg_problem& p, int* nregs);
cudaError_t regs_f64fma(const kg_problem& p, int* nregs);
cudaError_t regs_f64ff(const kg_problem& p, int* nregs);
cudaError_t sweep_uxx1_mix(const kg_problem& p, cudaStream_t s);
cudaError_t sweep_wave13pt_mix(const kg_problem& p, cudaStream_t s);
cudaError_t regs_wave13pt_mix(int* nregs);
cudaError_t regs_uxx1_mix(int* nregs);
cudaError_t regs_f32(const kg_problem& p, int* nregs);
cudaError_t regs_bf16(const kg_problem& p, int* nregs);
cudaError_t regs_f16(const kg_problem& p, int* nregs);
cudaError_t regs_u8(const kg_problem& p, int* nregs);

// Per-thread last error message.
kg_status fail(kg_status s, const char* fmt, ...);
kg_status fail_cuda(cudaError_t e, const char* what);
void clear_error();

size_t dtype_size(int dt);

// The library's stream-ordered pool on the current device (kg_runtime.cu):
// memory stays cached between calls up to a threshold.
cudaError_t program_pool(cudaMemPool_t* out);

// Tricubic programs with loop-invariant weights (kg_tricubic_pw.cu).
size_t tricubic_pw_bytes(const kg_problem& p);
cudaError_t tricubic_pw_precompute(const kg_problem& p, double* pw, cudaStream_t st);
cudaError_t tricubic_pw_sweep(const kg_problem& p, const double* pw, cudaStream_t st);

}  // namespace kg
