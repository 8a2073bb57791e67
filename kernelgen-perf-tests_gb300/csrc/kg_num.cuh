// kg_num.cuh -- arithmetic types of the sweeps and storage conversions.
//
// The stencil bodies are written once, as templates over a number type N, in
// the reference's own association order (C++ and C share precedence and
// left-to-right associativity of + - * /).  N fixes the rounding:
//   SD  FP64, every operation an IEEE round-to-nearest intrinsic; the compiler
//       cannot contract a*b+c into an FMA, so results equal a strict IEEE
//       build of the reference kernel bit for bit.
//   FD  FP64, plain operators: nvcc contracts products into DFMA like the
//       suite's gcc -ffast-math build does on FMA hardware.
//   FF  FP32 arithmetic (used for FP32, BF16 and FP16 storage).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace kg {

struct SD {
	double v;
	__host__ __device__ constexpr SD() : v(0) {}
	__host__ __device__ constexpr explicit SD(double x) : v(x) {}
};
__device__ __forceinline__ SD operator+(SD a, SD b) { return SD(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator-(SD a, SD b) { return SD(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator*(SD a, SD b) { return SD(__dmul_rn(a.v, b.v)); }
__device__ __forceinline__ SD operator/(SD a, SD b) { return SD(__ddiv_rn(a.v, b.v)); }

struct FD {
	double v;
	__host__ __device__ constexpr FD() : v(0) {}
	__host__ __device__ constexpr explicit FD(double x) : v(x) {}
};
__device__ __forceinline__ FD operator+(FD a, FD b) { return FD(a.v + b.v); }
__device__ __forceinline__ FD operator-(FD a, FD b) { return FD(a.v - b.v); }
__device__ __forceinline__ FD operator*(FD a, FD b) { return FD(a.v * b.v); }
__device__ __forceinline__ FD operator/(FD a, FD b) { return FD(a.v / b.v); }

struct FF {
	float v;
	__host__ __device__ constexpr FF() : v(0) {}
	__host__ __device__ constexpr explicit FF(double x) : v((float)x) {}
	__host__ __device__ constexpr explicit FF(float x, int) : v(x) {}
};
__device__ __forceinline__ FF mkf(float x) { return FF(x, 0); }
__device__ __forceinline__ FF operator+(FF a, FF b) { return mkf(a.v + b.v); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return mkf(a.v - b.v); }
__device__ __forceinline__ FF operator*(FF a, FF b) { return mkf(a.v * b.v); }
__device__ __forceinline__ FF operator/(FF a, FF b) { return mkf(a.v / b.v); }

// ---- storage <-> arithmetic -------------------------------------------------

template <class N, class S> struct Conv;

template <> struct Conv<SD, double> {
	static __device__ __forceinline__ SD ld(const double* p) { return SD(__ldg(p)); }
	static __device__ __forceinline__ SD from(double x) { return SD(x); }
	static __device__ __forceinline__ double to(SD x) { return x.v; }
};
template <> struct Conv<FD, double> {
	static __device__ __forceinline__ FD ld(const double* p) { return FD(__ldg(p)); }
	static __device__ __forceinline__ FD from(double x) { return FD(x); }
	static __device__ __forceinline__ double to(FD x) { return x.v; }
};
template <> struct Conv<FF, float> {
	static __device__ __forceinline__ FF ld(const float* p) { return mkf(__ldg(p)); }
	static __device__ __forceinline__ FF from(float x) { return mkf(x); }
	static __device__ __forceinline__ float to(FF x) { return x.v; }
};
template <> struct Conv<FF, __nv_bfloat16> {
	static __device__ __forceinline__ FF ld(const __nv_bfloat16* p) { return mkf(__bfloat162float(__ldg(p))); }
	static __device__ __forceinline__ FF from(__nv_bfloat16 x) { return mkf(__bfloat162float(x)); }
	static __device__ __forceinline__ __nv_bfloat16 to(FF x) { return __float2bfloat16_rn(x.v); }
};
template <> struct Conv<FF, __half> {
	static __device__ __forceinline__ FF ld(const __half* p) { return mkf(__half2float(__ldg(p))); }
	static __device__ __forceinline__ FF from(__half x) { return mkf(__half2float(x)); }
	static __device__ __forceinline__ __half to(FF x) { return __float2half_rn(x.v); }
};

}  // namespace kg
