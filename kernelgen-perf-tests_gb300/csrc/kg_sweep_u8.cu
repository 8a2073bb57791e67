// kg_sweep_u8.cu -- gameoflife on 0/1 byte cells (B3/S23).
//
// Fed 0/1 doubles, the reference rule of gameoflife/gameoflife.c:81-91 gives
// exactly 1.0 when (u + L - 3) * (L - 3) == 0 and a value below 1e-19
// otherwise, and those tiny values never change a later neighbour count once
// rounded; so this integer rule, thresholded, equals the reference sweep for
// sweep on such inputs.  Domain [1,n-2]^2, rims untouched.
//
// Rows of a multiple of 16 bytes (16-byte aligned arrays): a lane holds 16
// consecutive cells of a row as one 16-byte vector and walks a run of rows
// down, keeping the rows above and at the point in registers (one vector
// load a row).  The neighbour count is formed 4 cells at a time in the
// bytes of 32-bit words (values below 10: no carries between bytes): the
// column sums of the three rows, then each byte's left and right column by
// byte shifts, with the bytes beyond the lane's vector taken from the
// neighbouring lanes by warp shuffles (the warp's end lanes load the column
// next to theirs); the rule is three byte compares.  Rim cells keep their
// values.  Other rows: one thread per cell, a warp reading 34 consecutive
// bytes of each of the three rows it needs.
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

constexpr int kU8Rows = 16;   // rows a lane walks

// B3/S23 on the 4 cells of a word: L the neighbour counts, u the cells.
__device__ __forceinline__ uint32_t conway4(uint32_t L, uint32_t u)
{
	const uint32_t born = __vcmpeq4(L, 0x03030303u), stay = __vcmpeq4(L, 0x02020202u) & __vcmpeq4(u, 0x01010101u);
	return (born | stay) & 0x01010101u;
}

// Sum of the three cells of column x at rows r-1, r, r+1.
__device__ __forceinline__ uint32_t col3(const uint8_t* __restrict__ u, int nx, int x, int r)
{
	return (uint32_t)__ldg(u + (size_t)(r - 1) * nx + x) + __ldg(u + (size_t)r * nx + x) + __ldg(u + (size_t)(r + 1) * nx + x);
}

__global__ void __launch_bounds__(256) conway_u8_vec_kernel(const uint8_t* __restrict__ u0,
	uint8_t* __restrict__ u1, int nx, int ny)
{
	const int lane = threadIdx.x;
	const int nvx = nx / 16;
	const int xv = blockIdx.x * 32 + lane;
	const bool live = xv < nvx;
	const int x0 = xv * 16;
	const int r0 = 1 + (blockIdx.y * blockDim.y + threadIdx.y) * kU8Rows;   // the same for the warp
	if (r0 >= ny - 1) return;
	const int r1 = min(r0 + kU8Rows, ny - 1);
	auto ld = [&](int r) {
		return live ? __ldg(reinterpret_cast<const uint4*>(u0 + (size_t)r * nx + x0)) : make_uint4(0, 0, 0, 0);
	};
	uint4 up = ld(r0 - 1), mid = ld(r0);
	for (int r = r0; r < r1; r++) {
		const uint4 dn = ld(r + 1);
		// column sums (bytes <= 3)
		const uint32_t v0 = up.x + mid.x + dn.x, v1 = up.y + mid.y + dn.y, v2 = up.z + mid.z + dn.z,
			v3 = up.w + mid.w + dn.w;
		// the column left of the vector (top byte of vl) and right of it (low byte of vr)
		uint32_t vl = __shfl_up_sync(0xffffffffu, v3, 1), vr = __shfl_down_sync(0xffffffffu, v0, 1);
		if (lane == 0) vl = (live && x0 > 0) ? col3(u0, nx, x0 - 1, r) << 24 : 0u;
		if (lane == 31 || xv + 1 >= nvx) vr = (live && x0 + 16 < nx) ? col3(u0, nx, x0 + 16, r) : 0u;
		// nine-cell sums minus the cell: the neighbour counts (bytes <= 8)
		const uint32_t l0 = v0 + ((v0 << 8) | (vl >> 24)) + ((v0 >> 8) | (v1 << 24)) - mid.x;
		const uint32_t l1 = v1 + ((v1 << 8) | (v0 >> 24)) + ((v1 >> 8) | (v2 << 24)) - mid.y;
		const uint32_t l2 = v2 + ((v2 << 8) | (v1 >> 24)) + ((v2 >> 8) | (v3 << 24)) - mid.z;
		const uint32_t l3 = v3 + ((v3 << 8) | (v2 >> 24)) + ((v3 >> 8) | (vr << 24)) - mid.w;
		uint4 o = make_uint4(conway4(l0, mid.x), conway4(l1, mid.y), conway4(l2, mid.z), conway4(l3, mid.w));
		if (live) {
			uint8_t* dst = u1 + (size_t)r * nx + x0;
			if (x0 == 0 || x0 + 16 == nx) {
				// the rim columns 0 and nx - 1 keep their values
				const uint4 old = *reinterpret_cast<const uint4*>(dst);
				if (x0 == 0) o.x = (o.x & 0xffffff00u) | (old.x & 0xffu);
				if (x0 + 16 == nx) o.w = (o.w & 0x00ffffffu) | (old.w & 0xff000000u);
			}
			*reinterpret_cast<uint4*>(dst) = o;
		}
		up = mid;
		mid = dn;
	}
}

cudaError_t sweep_u8(const kg_problem& p, cudaStream_t s)
{
	const int nx = p.nx, ny = p.ny * p.ns;
	if (nx < 3 || ny < 3) return cudaSuccess;
	if (nx % 16 == 0 && (uintptr_t)p.arr[0] % 16 == 0 && (uintptr_t)p.arr[1] % 16 == 0) {
		const int nvx = nx / 16, chunks = (ny - 2 + kU8Rows - 1) / kU8Rows;
		dim3 block(32, 8);
		for (int c0 = 0; c0 < chunks; c0 += 65535 * 8) {
			// each launch takes up to 65535 * 8 chunks of rows (rows 1 + c0 kU8Rows on)
			const int n = min(chunks - c0, 65535 * 8);
			dim3 g((unsigned)((nvx + 31) / 32), (unsigned)((n + 7) / 8));
			const size_t off = (size_t)c0 * kU8Rows * nx;
			conway_u8_vec_kernel<<<g, block, 0, s>>>((const uint8_t*)p.arr[0] + off, (uint8_t*)p.arr[1] + off, nx,
				min(ny - c0 * kU8Rows, n * kU8Rows + 2));
			cudaError_t e = cudaGetLastError();
			if (e != cudaSuccess) return e;
		}
		return cudaSuccess;
	}
	dim3 block(32, 8);
	dim3 grid((nx - 2 + 31) / 32, (unsigned)min((ny - 2 + 7) / 8, 65535));
	conway_u8_kernel<<<grid, block, 0, s>>>((const uint8_t*)p.arr[0], (uint8_t*)p.arr[1], nx, ny);
	return cudaGetLastError();
}

// Registers of the kernel the suite's rows (multiples of 16 bytes) take.
cudaError_t regs_u8(const kg_problem&, int* nregs)
{
	cudaFuncAttributes a;
	cudaError_t e = cudaFuncGetAttributes(&a, (const void*)conway_u8_vec_kernel);
	if (e == cudaSuccess) *nregs = a.numRegs;
	return e;
}

}  // namespace kg
