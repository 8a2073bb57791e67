// kg_solve.cu -- Poisson solves A u = f with the 7-point Laplacian
// (A u = 6 u(c) - sum of the 6 face neighbours, Dirichlet u = 0 on the
// outer planes), by red-black SOR or Jacobi sweeps.
//
// KG_SOLVE_SOR_F64: red-black SOR on u in FP64 until ||f - A u||_2 <=
//   rtol ||f||_2.
// KG_SOLVE_IR_SOR_F32 / KG_SOLVE_IR_JACOBI_F32: iterative refinement.  The
//   residual r = f - A u and its norm are formed in FP64; A e = r is
//   relaxed by `sweeps_per_check` FP32 sweeps from e = 0; u += e in FP64.
//   A red-black SOR (or Jacobi) sweep is a stationary linear iteration
//   x' = M x + N b, so relaxing A e = r from e = 0 and adding e to u is the
//   same step as relaxing A u = f from u: refinement keeps the FP64
//   iteration's convergence rate while every sweep moves FP32 data, and the
//   FP32 rounding is relative to the current residual, so the final accuracy
//   is that of the FP64 residual.
// The residual is checked every `sweeps_per_check` sweeps in both modes.
// Past `max_sweeps` the solve stops with KG_ETIMEOUT (an iteration cap
// counted on the host; no kernel waits on anything).
//
// This solver has no counterpart in the reference: lapgsrb there is an
// out-of-place 25-point sweep, not red-black SOR (lapgsrb/lapgsrb.c:81-117).
#include <chrono>
#include <cmath>
#include <cstring>

#include "kg_internal.h"

namespace kg {

constexpr int kSX = 32, kSY = 8;
constexpr int kNormBlocks = 1184;  // 152 SMs x 8

// Points of colour `color` ((i + j + k) % 2 == color) in the interior.
// Thread t of a row takes i = i0 + 2t, so every lane has work.
template <class T>
__global__ void __launch_bounds__(kSX * kSY) rb_sor_kernel(T* __restrict__ u, const T* __restrict__ rhs,
	int nx, int ny, int ns, T omega, int color)
{
	const long long sy = nx, sz = (long long)nx * ny;
	const T sixth = T(1.0 / 6.0);
	const int t = blockIdx.x * kSX + threadIdx.x;
	for (int k = 1 + blockIdx.z; k < ns - 1; k += gridDim.z) {
		for (int j = 1 + blockIdx.y * kSY + threadIdx.y; j < ny - 1; j += gridDim.y * kSY) {
			const int i0 = ((1 + j + k) & 1) == color ? 1 : 2;
			const int i = i0 + 2 * t;
			if (i >= nx - 1) continue;
			const long long c = i + sy * j + sz * k;
			const T s = u[c - 1] + u[c + 1] + u[c - sy] + u[c + sy] + u[c - sz] + u[c + sz];
			const T old = u[c];
			u[c] = old + omega * ((s + rhs[c]) * sixth - old);
		}
	}
}

// The FP32 correction of refinement is stored split by colour: point
// (i, j, k) of colour c = (i + j + k) & 1 lives in array c, row (j, k),
// position i >> 1 (rows of nh >= (nx + 1) / 2 elements, a multiple of 4).  In row (j, k) the
// points of colour c are i = p + 2m, p = (c + j + k) & 1; their six
// neighbours all have the other colour: (i - 1, j, k) and (i + 1, j, k) at
// positions m - 1 + p and m + p of the other array's same row, the four
// others at position m of its neighbouring rows.  A colour's sweep then
// reads the other colour's array, its own and its right-hand side with
// unit stride and writes only its own: 16 bytes a point per red-black sweep,
// where the interleaved layout moves 24 (the stride-2 writes and
// right-hand-side reads of each colour touch every sector of the array).
// Same operands, order and expression as rb_sor_kernel.
// A lane takes kSV consecutive positions of a row as one 16-byte vector of
// each array (rows of nh elements, nh a multiple of kSV, so every vector is
// aligned); the one x neighbour outside its vector is the last value of the
// previous lane's (p = 0) or the first of the next lane's (p = 1) other-colour
// vector, exchanged by a warp shuffle; the first and last lane of the warp
// load theirs.  The warp's lanes share j and k, so p, the shuffles and the
// loop trip counts are uniform across the warp.  Positions outside the
// interior keep their values (the lane writes its whole vector: no other
// thread writes that colour's positions in this pass).
constexpr int kSV = 4;
// Resident blocks of 256 threads per SM the vector sweeps are compiled for
// (registers capped to fit them; a few spill).  Measured at 768x768x512 (ms
// a refinement sweep, residuals included, SOR / Jacobi): uncapped (54 and 48
// registers) 1.098 / 0.816, 6 blocks (40) 0.930 / 0.804, 8 blocks 1.665 /
// 0.982.
#ifndef KG_SOLVE_MINB
#define KG_SOLVE_MINB 6
#endif
__global__ void __launch_bounds__(kSX * kSY, KG_SOLVE_MINB) rb_sor_split_kernel(float* __restrict__ own,
	const float* __restrict__ oth, const float* __restrict__ rhs, int nx, int ny, int ns, int nh, float omega,
	int color)
{
	const long long rz = (long long)ny * nh;
	const float sixth = 1.0f / 6.0f;
	const int lane = threadIdx.x;
	const int m0 = (blockIdx.x * kSX + lane) * kSV;
	const bool inrow = m0 < nh;
	auto ld = [](const float* q) { return *reinterpret_cast<const float4*>(q); };
	for (int k = 1 + blockIdx.z; k < ns - 1; k += gridDim.z) {
		for (int j = 1 + blockIdx.y * kSY + threadIdx.y; j < ny - 1; j += gridDim.y * kSY) {
			const int p = (color + j + k) & 1;
			const int mlo = 1 - p, mhi = (nx - 2 - p) >> 1;   // interior positions: i = p + 2m in [1, nx-2]
			const long long rb = (long long)k * rz + (long long)j * nh;
			float4 c = make_float4(0.f, 0.f, 0.f, 0.f), jm = c, jp = c, km = c, kp = c, o = c, r = c;
			if (inrow) {
				c = ld(oth + rb + m0);
				jm = ld(oth + rb - nh + m0);
				jp = ld(oth + rb + nh + m0);
				km = ld(oth + rb - rz + m0);
				kp = ld(oth + rb + rz + m0);
				o = ld(own + rb + m0);
				r = ld(rhs + rb + m0);
			}
			float left = __shfl_up_sync(0xffffffffu, c.w, 1), right = __shfl_down_sync(0xffffffffu, c.x, 1);
			if (lane == 0 && p == 0 && m0 > 0 && inrow) left = oth[rb + m0 - 1];
			if (lane == kSX - 1 && p == 1 && m0 + kSV < nh) right = oth[rb + m0 + kSV];
			if (!inrow || m0 > mhi || m0 + kSV - 1 < mlo) continue;
			// x neighbours (i - 1, i + 1) of position m0 + v: other-colour
			// positions m0 + v - 1 + p and m0 + v + p
			const float xl[kSV] = {p ? c.x : left, p ? c.y : c.x, p ? c.z : c.y, p ? c.w : c.z};
			const float xr[kSV] = {p ? c.y : c.x, p ? c.z : c.y, p ? c.w : c.z, p ? right : c.w};
			const float cj0[kSV] = {jm.x, jm.y, jm.z, jm.w}, cj1[kSV] = {jp.x, jp.y, jp.z, jp.w};
			const float ck0[kSV] = {km.x, km.y, km.z, km.w}, ck1[kSV] = {kp.x, kp.y, kp.z, kp.w};
			const float rr[kSV] = {r.x, r.y, r.z, r.w};
			float ov[kSV] = {o.x, o.y, o.z, o.w};
#pragma unroll
			for (int v = 0; v < kSV; v++) {
				const int m = m0 + v;
				if (m < mlo || m > mhi) continue;
				const float s = xl[v] + xr[v] + cj0[v] + cj1[v] + ck0[v] + ck1[v];
				ov[v] = ov[v] + omega * ((s + rr[v]) * sixth - ov[v]);
			}
			*reinterpret_cast<float4*>(own + rb + m0) = make_float4(ov[0], ov[1], ov[2], ov[3]);
		}
	}
}

// e1 = (sum of e0's face neighbours + rhs) / 6 on the interior.
__global__ void __launch_bounds__(kSX * kSY) jacobi_kernel(const float* __restrict__ e0, float* __restrict__ e1,
	const float* __restrict__ rhs, int nx, int ny, int ns)
{
	const long long sy = nx, sz = (long long)nx * ny;
	const int i = 1 + blockIdx.x * kSX + threadIdx.x;
	if (i >= nx - 1) return;
	for (int k = 1 + blockIdx.z; k < ns - 1; k += gridDim.z) {
		for (int j = 1 + blockIdx.y * kSY + threadIdx.y; j < ny - 1; j += gridDim.y * kSY) {
			const long long c = i + sy * j + sz * k;
			const float s = __ldg(e0 + c - 1) + __ldg(e0 + c + 1) + __ldg(e0 + c - sy) + __ldg(e0 + c + sy) +
				__ldg(e0 + c - sz) + __ldg(e0 + c + sz);
			e1[c] = (s + __ldg(rhs + c)) * (1.0f / 6.0f);
		}
	}
}

// The same sweep with a lane on 4 consecutive points of a row as 16-byte
// vectors (rows of a multiple of 4 elements, 16-byte aligned arrays): the x
// neighbours outside the vector come from the neighbouring lanes by warp
// shuffles (the warp's end lanes load theirs).  The outer planes of e1 stay
// 0 (positions 0 and nx - 1 of a row are written as 0, their value).  Same
// operands, order and expression as jacobi_kernel.
__global__ void __launch_bounds__(kSX * kSY, KG_SOLVE_MINB) jacobi_vec_kernel(const float* __restrict__ e0, float* __restrict__ e1,
	const float* __restrict__ rhs, int nx, int ny, int ns)
{
	const long long sy = nx, sz = (long long)nx * ny;
	const int lane = threadIdx.x;
	const int i0 = (blockIdx.x * kSX + lane) * kSV;
	const bool inrow = i0 < nx;
	auto ld = [](const float* q) { return __ldg(reinterpret_cast<const float4*>(q)); };
	for (int k = 1 + blockIdx.z; k < ns - 1; k += gridDim.z) {
		for (int j = 1 + blockIdx.y * kSY + threadIdx.y; j < ny - 1; j += gridDim.y * kSY) {
			const long long c = i0 + sy * j + sz * k;
			float4 m = make_float4(0.f, 0.f, 0.f, 0.f), ym = m, yp = m, zm = m, zp = m, r = m;
			if (inrow) {
				m = ld(e0 + c);
				ym = ld(e0 + c - sy);
				yp = ld(e0 + c + sy);
				zm = ld(e0 + c - sz);
				zp = ld(e0 + c + sz);
				r = ld(rhs + c);
			}
			float left = __shfl_up_sync(0xffffffffu, m.w, 1), right = __shfl_down_sync(0xffffffffu, m.x, 1);
			if (lane == 0 && inrow && i0 > 0) left = __ldg(e0 + c - 1);
			if (lane == kSX - 1 && inrow && i0 + kSV < nx) right = __ldg(e0 + c + kSV);
			if (!inrow) continue;
			const float xl[kSV] = {left, m.x, m.y, m.z}, xr[kSV] = {m.y, m.z, m.w, right};
			const float y0[kSV] = {ym.x, ym.y, ym.z, ym.w}, y1[kSV] = {yp.x, yp.y, yp.z, yp.w};
			const float z0[kSV] = {zm.x, zm.y, zm.z, zm.w}, z1[kSV] = {zp.x, zp.y, zp.z, zp.w};
			const float rr[kSV] = {r.x, r.y, r.z, r.w};
			float o[kSV];
#pragma unroll
			for (int v = 0; v < kSV; v++) {
				const int i = i0 + v;
				const float s = xl[v] + xr[v] + y0[v] + y1[v] + z0[v] + z1[v];
				o[v] = (i > 0 && i < nx - 1) ? (s + rr[v]) * (1.0f / 6.0f) : 0.0f;
			}
			*reinterpret_cast<float4*>(e1 + c) = make_float4(o[0], o[1], o[2], o[3]);
		}
	}
}

// r = f - A u on the interior (FP64); r32 = (float) r (0 on the outer
// planes), interleaved (nh = 0) or split by colour (rows of nh elements);
// partial[b] = this block's sum of r^2.
__global__ void __launch_bounds__(256) residual_kernel(const double* __restrict__ u, const double* __restrict__ f,
	float* __restrict__ r32, double* __restrict__ partial, int nx, int ny, int ns, int nh)
{
	const long long half = (long long)nh * ny * ns;
	__shared__ double sh[256];
	const long long sy = nx, sz = (long long)nx * ny;
	const long long n = sz * ns;
	double acc = 0.0;
	for (long long c = blockIdx.x * 256LL + threadIdx.x; c < n; c += (long long)gridDim.x * 256) {
		const int i = (int)(c % nx);
		const long long jk = c / nx;
		const int j = (int)(jk % ny), k = (int)(jk / ny);
		double r = 0.0;
		if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < ns - 1) {
			const double au = 6.0 * u[c] - (u[c - 1] + u[c + 1] + u[c - sy] + u[c + sy] + u[c - sz] + u[c + sz]);
			r = f[c] - au;
		}
		if (r32) {
			if (nh) r32[((i + j + k) & 1) * half + jk * nh + (i >> 1)] = (float)r;
			else r32[c] = (float)r;
		}
		acc += r * r;
	}
	sh[threadIdx.x] = acc;
	__syncthreads();
	for (int s = 128; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
		__syncthreads();
	}
	if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// Sum of squares of f over the interior.
__global__ void __launch_bounds__(256) norm2_kernel(const double* __restrict__ f, double* __restrict__ partial,
	int nx, int ny, int ns)
{
	__shared__ double sh[256];
	const long long sz = (long long)nx * ny, n = sz * ns;
	double acc = 0.0;
	for (long long c = blockIdx.x * 256LL + threadIdx.x; c < n; c += (long long)gridDim.x * 256) {
		const int i = (int)(c % nx);
		const long long jk = c / nx;
		const int j = (int)(jk % ny), k = (int)(jk / ny);
		if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < ns - 1) acc += f[c] * f[c];
	}
	sh[threadIdx.x] = acc;
	__syncthreads();
	for (int s = 128; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
		__syncthreads();
	}
	if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(256) sum_partials(const double* __restrict__ partial, int g, double* out)
{
	__shared__ double sh[256];
	double acc = 0.0;
	for (int b = threadIdx.x; b < g; b += 256) acc += partial[b];
	sh[threadIdx.x] = acc;
	__syncthreads();
	for (int s = 128; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
		__syncthreads();
	}
	if (threadIdx.x == 0) *out = sh[0];
}

// u += e on every point (e is 0 on the outer planes), e interleaved
// (nh = 0) or split by colour (rows of nh elements).
__global__ void axpy_kernel(double* __restrict__ u, const float* __restrict__ e, int nx, int ny, int ns, int nh)
{
	const long long n = (long long)nx * ny * ns, half = (long long)nh * ny * ns;
	for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
		if (nh) {
			const int i = (int)(c % nx);
			const long long jk = c / nx;
			const int j = (int)(jk % ny), k = (int)(jk / ny);
			u[c] += (double)e[((i + j + k) & 1) * half + jk * nh + (i >> 1)];
		} else {
			u[c] += (double)e[c];
		}
	}
}

struct Grid3 { dim3 grid, block; };

static Grid3 sweep_grid(int nx, int ny, int ns, bool pairs, int kz = 1)
{
	const int wx = pairs ? (nx - 2 + 1) / 2 : nx - 2;
	Grid3 g;
	g.block = dim3(kSX, kSY, 1);
	g.grid = dim3((unsigned)std::max(1, (wx + kSX - 1) / kSX), (unsigned)std::min(std::max(1, (ny - 2 + kSY - 1) / kSY), 65535),
		(unsigned)std::min(std::max(1, (ns - 2 + kz - 1) / kz), 65535));
	return g;
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_poisson_solve(int nx, int ny, int ns, const double* f, double* u,
	const kg_solve_opts* opts, kg_solve_report* rep, kg_stream_t stream)
{
	clear_error();
	if (!f || !u || !opts || nx < 3 || ny < 3 || ns < 3)
		return fail(KG_EINVAL, "kg_poisson_solve: need f, u, opts and a grid of at least 3^3");
	if (opts->kind < KG_SOLVE_SOR_F64 || opts->kind > KG_SOLVE_IR_JACOBI_F32)
		return fail(KG_EINVAL, "kg_poisson_solve: unknown kind %d", opts->kind);
	if (!(opts->omega > 0.0 && opts->omega < 2.0) || !(opts->rtol > 0.0) || opts->sweeps_per_check < 1 ||
		opts->max_sweeps < 1)
		return fail(KG_EINVAL, "kg_poisson_solve: need 0 < omega < 2, rtol > 0, sweeps_per_check >= 1, max_sweeps >= 1");
	const long long n = (long long)nx * ny * ns;
	cudaStream_t st = (cudaStream_t)stream;
	const bool ir = opts->kind != KG_SOLVE_SOR_F64;
	const bool jac = opts->kind == KG_SOLVE_IR_JACOBI_F32;
	// refinement around SOR keeps e and its right-hand side split by colour
	const int nh = ir && !jac ? ((nx + 1) / 2 + kSV - 1) / kSV * kSV : 0;
	const long long half = (long long)nh * ny * ns;
	const long long ne = nh ? 2 * half : n;

	float *e = nullptr, *e2 = nullptr, *r32 = nullptr;
	double *partial = nullptr, *norm = nullptr;
	kg_solve_report R;
	memset(&R, 0, sizeof(R));
	kg_status s = KG_OK;
	cudaError_t err = cudaMallocAsync((void**)&partial, sizeof(double) * (kNormBlocks + 2), st);
	if (err == cudaSuccess && ir) err = cudaMallocAsync((void**)&e, sizeof(float) * ne, st);
	if (err == cudaSuccess && ir) err = cudaMallocAsync((void**)&r32, sizeof(float) * ne, st);
	if (err == cudaSuccess && jac) err = cudaMallocAsync((void**)&e2, sizeof(float) * n, st);
	if (err != cudaSuccess) {
		s = fail_cuda(err, "kg_poisson_solve: work arrays");
		goto out;
	}
	norm = partial + kNormBlocks;
	{
		auto t0 = std::chrono::steady_clock::now();
		double host[2] = {0, 0};
		norm2_kernel<<<kNormBlocks, 256, 0, st>>>(f, partial, nx, ny, ns);
		sum_partials<<<1, 256, 0, st>>>(partial, kNormBlocks, norm);
		err = cudaMemcpyAsync(host, norm, sizeof(double), cudaMemcpyDeviceToHost, st);
		if (err == cudaSuccess) err = cudaStreamSynchronize(st);
		if (err != cudaSuccess) { s = fail_cuda(err, "kg_poisson_solve: ||f||"); goto out; }
		const double fnorm = std::sqrt(host[0]);
		R.fnorm = fnorm;
		const Grid3 gp = sweep_grid(nx, ny, ns, true), gj = sweep_grid(nx, ny, ns, false);
		// Jacobi sweeps on 16-byte vectors where rows allow them (the work
		// arrays come from cudaMallocAsync: 256-byte aligned)
		const bool jvec = nx % kSV == 0;
		Grid3 gv = sweep_grid(nx, ny, ns, false);
		gv.grid.x = (unsigned)std::max(1, (nx + kSX * kSV - 1) / (kSX * kSV));
		Grid3 gs = sweep_grid(nx, ny, ns, true);
		gs.grid.x = (unsigned)std::max(1, (nh + kSX * kSV - 1) / (kSX * kSV));
		long long sweeps = 0;
		for (;;) {
			// FP64 residual (and, for refinement, its FP32 copy as the right-hand side)
			residual_kernel<<<kNormBlocks, 256, 0, st>>>(u, f, ir ? r32 : nullptr, partial, nx, ny, ns, nh);
			sum_partials<<<1, 256, 0, st>>>(partial, kNormBlocks, norm);
			err = cudaMemcpyAsync(host, norm, sizeof(double), cudaMemcpyDeviceToHost, st);
			if (err == cudaSuccess) err = cudaStreamSynchronize(st);
			if (err != cudaSuccess) { s = fail_cuda(err, "kg_poisson_solve: residual"); break; }
			const double rel = fnorm > 0 ? std::sqrt(host[0]) / fnorm : 0.0;
			if (R.nhistory < KG_SOLVE_HISTORY) {
				R.history_sweeps[R.nhistory] = sweeps;
				R.history_rel[R.nhistory] = rel;
				R.nhistory++;
			}
			R.rel_residual = rel;
			if (rel <= opts->rtol) break;
			if (sweeps >= opts->max_sweeps) {
				s = fail(KG_ETIMEOUT, "kg_poisson_solve: %lld sweeps, relative residual %.3e > %.3e",
					sweeps, rel, opts->rtol);
				break;
			}
			const int m = (int)std::min<long long>(opts->sweeps_per_check, opts->max_sweeps - sweeps);
			if (ir) {
				cudaMemsetAsync(e, 0, sizeof(float) * ne, st);
				if (jac) cudaMemsetAsync(e2, 0, sizeof(float) * n, st);
				for (int it = 0; it < m; it++) {
					if (jac) {
						if (jvec) jacobi_vec_kernel<<<gv.grid, gv.block, 0, st>>>(e, e2, r32, nx, ny, ns);
						else jacobi_kernel<<<gj.grid, gj.block, 0, st>>>(e, e2, r32, nx, ny, ns);
						float* t = e; e = e2; e2 = t;
					} else {
						const float w = (float)opts->omega;
						rb_sor_split_kernel<<<gs.grid, gs.block, 0, st>>>(e, e + half, r32, nx, ny, ns, nh, w, 0);
						rb_sor_split_kernel<<<gs.grid, gs.block, 0, st>>>(e + half, e, r32 + half, nx, ny, ns, nh, w, 1);
					}
				}
				const long long nb = std::min<long long>((n + 255) / 256, 152 * 16);
				axpy_kernel<<<(unsigned)nb, 256, 0, st>>>(u, e, nx, ny, ns, nh);
				R.outer++;
			} else {
				for (int it = 0; it < m; it++) {
					rb_sor_kernel<double><<<gp.grid, gp.block, 0, st>>>(u, f, nx, ny, ns, opts->omega, 0);
					rb_sor_kernel<double><<<gp.grid, gp.block, 0, st>>>(u, f, nx, ny, ns, opts->omega, 1);
				}
			}
			if ((err = cudaGetLastError()) != cudaSuccess) { s = fail_cuda(err, "kg_poisson_solve: sweeps"); break; }
			sweeps += m;
		}
		R.sweeps = sweeps;
		R.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
	}
out:
	if (e) cudaFreeAsync(e, st);
	if (e2) cudaFreeAsync(e2, st);
	if (r32) cudaFreeAsync(r32, st);
	if (partial) cudaFreeAsync(partial, st);
	if (rep) *rep = R;
	return s;
}
