// kg_mix.cu -- the KG_F64_MIX form of the incremental updates, uxx1 and
// wave13pt: FP64 state, the update's small part in FP32 arithmetic, combined
// with the state in FP64.
//
// uxx1 advances u by an increment each step (uxx1/uxx1.c:83-106):
//   u1 = u0 + (dth / d) * (c1 (xx - xx[x-1]) + c2 (xx[x+1] - xx[x-2]) + ...y, z)
// with d the average of four density values.  The increment is computed in
// FP32 and added to u0 in FP64, so the state keeps FP64 precision and the
// error of a step is FP32's relative error of the increment alone (FP32
// storage instead rounds u itself every step).  The density sum, whose terms
// can cancel, and the final addition run on the FP64 unit: three additions a
// point, the pair sum of plane k reused as plane k+1's previous pair (the
// mixed form is not bound to the reference's association order).  Doubles
// enter FP32 truncated to 24 significant bits by integer operations (the
// conversion instruction would issue to the FP64 unit); the increment goes
// back to FP64 by exact widening, also from its bit fields.
//
// wave13pt (wave13pt/wave13pt.c:640-651) is rewritten around the centre value
// c = w1[i]: w2 = (m0 + 6 m1 + 6 m2) c - w0 + m1 D1 + m2 D2, with D1, D2 the
// sums of the differences w1[neighbour] - c over the six neighbours at
// distance 1 and 2.  The differences are formed in FP32 from the float-float
// split of each value (hi parts subtract exactly when the values are within a
// factor of two, the low parts add the rest), so they carry FP32's relative
// error of the difference, not of w; m1 D1 + m2 D2 is FP32 and the rest one
// FP64 FMA and one addition.
#include <cstdint>

#include "kg_internal.h"
#include "kg_num.cuh"

namespace kg {

// x truncated to FP32 (24 significant bits); |x| below FP32's normal range
// gives a signed zero, above it infinity; infinities and NaNs pass.
__device__ __forceinline__ float mix_f32(double x)
{
	const unsigned long long b = (unsigned long long)__double_as_longlong(x);
	const unsigned bh = (unsigned)(b >> 32), bl = (unsigned)b;
	const unsigned sign = bh & 0x80000000u;
	const int e = (int)((bh >> 20) & 0x7ff);
	if (e >= 897 && e <= 1150)
		return __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((bh & 0xfffffu) << 3) | (bl >> 29));
	if (e < 897) return __uint_as_float(sign);
	const unsigned nan = (e == 0x7ff && ((bh & 0xfffffu) | bl)) ? 0x400000u : 0u;
	return __uint_as_float(sign | 0x7f800000u | nan);
}

// f widened to FP64 exactly; zeros, subnormals, infinities and NaNs take the
// conversion instruction.
__device__ __forceinline__ double mix_f64(float f)
{
	const unsigned u = __float_as_uint(f);
	const unsigned e = (u >> 23) & 0xffu;
	if (e == 0 || e == 0xff) return (double)f;
	const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
	return __hiloint2double((int)hi, (int)((u & 7u) << 29));
}

constexpr int kMixBX = 32, kMixBY = 8, kMixKC = 16;

// The loads of one plane of a thread's column.
struct MixPlane {
	double xx0, xxm1, xx1, xxm2, xy0, xym1, xy1, xym2, xz1, d0, dm, u;
};

__device__ __forceinline__ MixPlane mix_load(long long c, long long sy, long long sz, const double* __restrict__ u0,
	const double* __restrict__ d1, const double* __restrict__ xx, const double* __restrict__ xy,
	const double* __restrict__ xz)
{
	MixPlane p;
	p.xx0 = __ldg(xx + c);
	p.xxm1 = __ldg(xx + c - 1);
	p.xx1 = __ldg(xx + c + 1);
	p.xxm2 = __ldg(xx + c - 2);
	p.xy0 = __ldg(xy + c);
	p.xym1 = __ldg(xy + c - sy);
	p.xy1 = __ldg(xy + c + sy);
	p.xym2 = __ldg(xy + c - 2 * sy);
	p.xz1 = __ldg(xz + c + sz);
	p.d0 = __ldg(d1 + c);
	p.dm = __ldg(d1 + c - sy);
	p.u = __ldg(u0 + c);
	return p;
}

// One thread per (i, j) column, kMixKC planes of it, the next plane's loads
// in flight while the current one is evaluated; arrays in the reference's
// argument order: u0, u1, d1, xx, xy, xz.
__global__ void __launch_bounds__(kMixBX * kMixBY) uxx1_mix_kernel(int nx, int ny, int ns, float c1, float c2,
	float dth, const double* __restrict__ u0, double* __restrict__ u1, const double* __restrict__ d1,
	const double* __restrict__ xx, const double* __restrict__ xy, const double* __restrict__ xz)
{
	const int i = 2 + blockIdx.x * kMixBX + threadIdx.x;
	if (i >= nx - 1) return;
	const long long sy = nx, sz = (long long)nx * ny;
	const int tyn = (ny - 3 + kMixBY - 1) / kMixBY, tzn = (ns - 3 + kMixKC - 1) / kMixKC;
	for (int ty = blockIdx.y; ty < tyn; ty += gridDim.y) {
		const int j = 2 + ty * kMixBY + threadIdx.y;
		if (j >= ny - 1) continue;
		for (int tz = blockIdx.z; tz < tzn; tz += gridDim.z) {
			const int k0 = 2 + tz * kMixKC, k1 = min(k0 + kMixKC, ns - 1);
			long long c = i + sy * j + sz * k0;
			// the column of xz (planes k-2 .. k+1) and the previous plane's density pair
			float z0 = mix_f32(__ldg(xz + c - 2 * sz)), z1 = mix_f32(__ldg(xz + c - sz)), z2 = mix_f32(__ldg(xz + c));
			double prev = __dadd_rn(__ldg(d1 + c - sz), __ldg(d1 + c - sz - sy));
			MixPlane cur = mix_load(c, sy, sz, u0, d1, xx, xy, xz);
			for (int k = k0; k < k1; k++, c += sz) {
				MixPlane nxt = cur;
				if (k + 1 < k1) nxt = mix_load(c + sz, sy, sz, u0, d1, xx, xy, xz);
				const float z3 = mix_f32(cur.xz1);
				const double pair = __dadd_rn(cur.d0, cur.dm);
				const float d = 0.25f * mix_f32(__dadd_rn(pair, prev));
				prev = pair;
				const float s = c1 * (mix_f32(cur.xx0) - mix_f32(cur.xxm1)) + c2 * (mix_f32(cur.xx1) - mix_f32(cur.xxm2)) +
					c1 * (mix_f32(cur.xy0) - mix_f32(cur.xym1)) + c2 * (mix_f32(cur.xy1) - mix_f32(cur.xym2)) +
					c1 * (z2 - z1) + c2 * (z3 - z0);
				const float inc = __fdividef(dth, d) * s;
				u1[c] = __dadd_rn(cur.u, mix_f64(inc));
				z0 = z1;
				z1 = z2;
				z2 = z3;
				cur = nxt;
			}
		}
	}
}

// ---- wave13pt ------------------------------------------------------------

// x as a float pair: hi = x truncated to 24 significant bits (mix_f32), lo =
// the remaining 29 bits rounded to FP32 (one integer-to-float conversion,
// which issues to the otherwise idle XU pipe, scaled by 2^(e-1075)).  Values
// outside FP32's normal range keep only hi, as ff2_from_double does.
__device__ __forceinline__ FF2 mix_split(double x)
{
	const unsigned long long b = (unsigned long long)__double_as_longlong(x);
	const unsigned bh = (unsigned)(b >> 32), bl = (unsigned)b;
	const int e = (int)((bh >> 20) & 0x7ff);
	const float hi = mix_f32(x);
	if (e < 949 || e > 1150) return FF2(hi, 0.f);
	const float scale = __uint_as_float((unsigned)(e - 948) << 23);   // 2^(e - 1075)
	const float lo = __uint_as_float(__float_as_uint(__fmul_rn(__uint2float_rn(bl & 0x1fffffffu), scale)) |
		(bh & 0x80000000u));
	return FF2(hi, lo);
}

constexpr int kWmBX = 32, kWmBY = 8, kWmKC = 16;

struct WavePlane {
	double x1, xm1, x2, xm2, y1, ym1, y2, ym2, z2, w0;
};

__device__ __forceinline__ WavePlane wave_load(long long c, long long sy, long long sz,
	const double* __restrict__ w0, const double* __restrict__ w1)
{
	WavePlane p;
	p.x1 = __ldg(w1 + c + 1);
	p.xm1 = __ldg(w1 + c - 1);
	p.x2 = __ldg(w1 + c + 2);
	p.xm2 = __ldg(w1 + c - 2);
	p.y1 = __ldg(w1 + c + sy);
	p.ym1 = __ldg(w1 + c - sy);
	p.y2 = __ldg(w1 + c + 2 * sy);
	p.ym2 = __ldg(w1 + c - 2 * sy);
	p.z2 = __ldg(w1 + c + 2 * sz);
	p.w0 = __ldg(w0 + c);
	return p;
}

// (a - c) + (b - c) + ... for float-float values against the centre (hi, lo)
__device__ __forceinline__ float wave_diffs(FF2 c, FF2 a, FF2 b, FF2 d, FF2 e, FF2 f, FF2 g)
{
	const float h = (((((a.hi - c.hi) + (b.hi - c.hi)) + (d.hi - c.hi)) + (e.hi - c.hi)) + (f.hi - c.hi)) + (g.hi - c.hi);
	const float l = (a.lo + b.lo + d.lo + e.lo + f.lo + g.lo) - 6.0f * c.lo;
	return h + l;
}

// One thread per (i, j) column, kWmKC planes of it, the next plane's loads in
// flight; arrays in the reference's argument order: w0, w1, w2.
__global__ void __launch_bounds__(kWmBX * kWmBY) wave13pt_mix_kernel(int nx, int ny, int ns, double M, float m1,
	float m2, const double* __restrict__ w0, const double* __restrict__ w1, double* __restrict__ w2)
{
	const int i = 2 + blockIdx.x * kWmBX + threadIdx.x;
	if (i >= nx - 2) return;
	const long long sy = nx, sz = (long long)nx * ny;
	const int tyn = (ny - 4 + kWmBY - 1) / kWmBY, tzn = (ns - 4 + kWmKC - 1) / kWmKC;
	for (int ty = blockIdx.y; ty < tyn; ty += gridDim.y) {
		const int j = 2 + ty * kWmBY + threadIdx.y;
		if (j >= ny - 2) continue;
		for (int tz = blockIdx.z; tz < tzn; tz += gridDim.z) {
			const int k0 = 2 + tz * kWmKC, k1 = min(k0 + kWmKC, ns - 2);
			long long c = i + sy * j + sz * k0;
			// the column of w1, planes k-2 .. k+1 (raw centre, split pairs)
			FF2 zm2 = mix_split(__ldg(w1 + c - 2 * sz)), zm1 = mix_split(__ldg(w1 + c - sz));
			double zc = __ldg(w1 + c), zc1 = __ldg(w1 + c + sz);
			FF2 z0 = mix_split(zc), zp1 = mix_split(zc1);
			WavePlane cur = wave_load(c, sy, sz, w0, w1);
			for (int k = k0; k < k1; k++, c += sz) {
				WavePlane nxt = cur;
				if (k + 1 < k1) nxt = wave_load(c + sz, sy, sz, w0, w1);
				const FF2 zp2 = mix_split(cur.z2);
				const float d1 = wave_diffs(z0, mix_split(cur.x1), mix_split(cur.xm1), mix_split(cur.y1),
					mix_split(cur.ym1), zp1, zm1);
				const float d2 = wave_diffs(z0, mix_split(cur.x2), mix_split(cur.xm2), mix_split(cur.y2),
					mix_split(cur.ym2), zp2, zm2);
				const float inc = m1 * d1 + m2 * d2;
				w2[c] = __dadd_rn(__fma_rn(M, zc, -cur.w0), mix_f64(inc));
				// the column moves one plane on
				zm2 = zm1;
				zm1 = z0;
				z0 = zp1;
				zp1 = zp2;
				zc = zc1;
				zc1 = cur.z2;
				cur = nxt;
			}
		}
	}
}

cudaError_t sweep_wave13pt_mix(const kg_problem& p, cudaStream_t st)
{
	if (p.nx < 5 || p.ny < 5 || p.ns < 5) return cudaSuccess;   // empty domain [2, n-3]
	const int tx = (p.nx - 4 + kWmBX - 1) / kWmBX, ty = (p.ny - 4 + kWmBY - 1) / kWmBY,
		tz = (p.ns - 4 + kWmKC - 1) / kWmKC;
	dim3 grid(tx, (unsigned)std::min(ty, 65535), (unsigned)std::min(tz, 65535));
	const double m0 = p.coef[0], m1 = p.coef[1], m2 = p.coef[2];
	wave13pt_mix_kernel<<<grid, dim3(kWmBX, kWmBY), 0, st>>>(p.nx, p.ny, p.ns, m0 + 6.0 * m1 + 6.0 * m2, (float)m1,
		(float)m2, (const double*)p.arr[0], (const double*)p.arr[1], (double*)p.arr[2]);
	return cudaGetLastError();
}

cudaError_t sweep_uxx1_mix(const kg_problem& p, cudaStream_t st)
{
	if (p.nx < 4 || p.ny < 4 || p.ns < 4) return cudaSuccess;   // empty domain [2, n-2]
	const int tx = (p.nx - 3 + kMixBX - 1) / kMixBX, ty = (p.ny - 3 + kMixBY - 1) / kMixBY,
		tz = (p.ns - 3 + kMixKC - 1) / kMixKC;
	dim3 grid(tx, (unsigned)std::min(ty, 65535), (unsigned)std::min(tz, 65535));
	uxx1_mix_kernel<<<grid, dim3(kMixBX, kMixBY), 0, st>>>(p.nx, p.ny, p.ns, (float)p.coef[0], (float)p.coef[1],
		(float)(1.0 / p.nx), (const double*)p.arr[0], (double*)p.arr[1], (const double*)p.arr[2],
		(const double*)p.arr[3], (const double*)p.arr[4], (const double*)p.arr[5]);
	return cudaGetLastError();
}

cudaError_t regs_uxx1_mix(int* nregs)
{
	cudaFuncAttributes a;
	cudaError_t e = cudaFuncGetAttributes(&a, (const void*)uxx1_mix_kernel);
	if (e == cudaSuccess) *nregs = a.numRegs;
	return e;
}

cudaError_t regs_wave13pt_mix(int* nregs)
{
	cudaFuncAttributes a;
	cudaError_t e = cudaFuncGetAttributes(&a, (const void*)wave13pt_mix_kernel);
	if (e == cudaSuccess) *nregs = a.numRegs;
	return e;
}

}  // namespace kg
