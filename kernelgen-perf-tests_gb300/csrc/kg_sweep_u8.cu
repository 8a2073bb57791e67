// kg_sweep_u8.cu -- gameoflife on 0/1 byte cells (B3/S23).
//
// Fed 0/1 doubles, the reference rule of gameoflife/gameoflife.c:81-91 gives
// exactly 1.0 when (u + L - 3) * (L - 3) == 0 and a value below 1e-19
// otherwise, and those tiny values never change a later neighbour count once
// rounded; so this integer rule, thresholded, equals the reference sweep for
// sweep on such inputs.  Domain [1,n-2]^2, rims untouched.
//
// One thread per cell; a warp reads 34 consecutive bytes of each of the three
// rows it needs.
#include <cstdint>

#include "kg_internal.h"

namespace kg {

__device__ __forceinline__ uint32_t cell(const uint8_t* __restrict__ u, long long c) { return __ldg(u + c); }

__global__ void __launch_bounds__(256) conway_u8_kernel(const uint8_t* __restrict__ u0,
	uint8_t* __restrict__ u1, int nx, int ny)
{
	const int i = 1 + blockIdx.x * 32 + threadIdx.x;
	if (i >= nx - 1) return;
	for (int j = 1 + blockIdx.y * 8 + threadIdx.y; j < ny - 1; j += gridDim.y * 8) {
		const long long c = i + (long long)nx * j;
		const uint32_t L =
			cell(u0, c - nx - 1) + cell(u0, c - nx) + cell(u0, c - nx + 1) +
			cell(u0, c - 1) + cell(u0, c + 1) +
			cell(u0, c + nx - 1) + cell(u0, c + nx) + cell(u0, c + nx + 1);
		const int u = (int)cell(u0, c);
		const int l = (int)L;
		u1[c] = (uint8_t)((u + l - 3) * (l - 3) == 0);
	}
}

cudaError_t sweep_u8(const kg_problem& p, cudaStream_t s)
{
	const int nx = p.nx, ny = p.ny * p.ns;
	if (nx < 3 || ny < 3) return cudaSuccess;
	dim3 block(32, 8);
	dim3 grid((nx - 2 + 31) / 32, (unsigned)min((ny - 2 + 7) / 8, 65535));
	conway_u8_kernel<<<grid, block, 0, s>>>((const uint8_t*)p.arr[0], (uint8_t*)p.arr[1], nx, ny);
	return cudaGetLastError();
}

cudaError_t regs_u8(const kg_problem&, int* nregs)
{
	cudaFuncAttributes a;
	cudaError_t e = cudaFuncGetAttributes(&a, (const void*)conway_u8_kernel);
	if (e == cudaSuccess) *nregs = a.numRegs;
	return e;
}

}  // namespace kg
