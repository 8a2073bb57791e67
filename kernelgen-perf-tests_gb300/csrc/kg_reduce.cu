// kg_reduce.cu -- FP64 checksums, error statistics and type conversion.
//
// The checksums stand for the reference's "initial mean"/"final mean" loops
// (laplacian/laplacian.c:158-165,374-377): per index the arrays are added
// left to right in FP64 and the per-index values accumulated.  The GPU sum is
// a fixed two-level tree (the block count depends on n only), so its bits are
// the same on every run; it differs from the reference's serial loop only by
// summation order (relative 1e-16 of the sum of magnitudes), far below the
// %f resolution of the printed mean.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <mutex>
#include <type_traits>

#include "kg_internal.h"

namespace kg {

constexpr int kRB = 256;    // threads per first-level block
constexpr int kRG = 2048;   // most first-level blocks
constexpr int kRF = 1024;   // threads of the final block

template <class S> __device__ __forceinline__ double to_f64(S x);
template <> __device__ __forceinline__ double to_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_f64<float>(float x) { return (double)x; }
template <> __device__ __forceinline__ double to_f64<__nv_bfloat16>(__nv_bfloat16 x) { return (double)__bfloat162float(x); }
template <> __device__ __forceinline__ double to_f64<__half>(__half x) { return (double)__half2float(x); }
template <> __device__ __forceinline__ double to_f64<uint8_t>(uint8_t x) { return (double)x; }

struct Arrs { const void* a[6]; int narr; };

int reduce_blocks(size_t n)
{
	size_t g = (n + (size_t)kRB * 4 - 1) / ((size_t)kRB * 4);
	if (g < 1) g = 1;
	if (g > (size_t)kRG) g = kRG;
	return (int)g;
}

template <int W>
__device__ __forceinline__ void block_reduce(double (&v)[W], double (*sh)[W], bool maxof[W])
{
	const int t = threadIdx.x;
#pragma unroll
	for (int q = 0; q < W; q++) sh[t][q] = v[q];
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1) {
		if (t < s) {
#pragma unroll
			for (int q = 0; q < W; q++)
				sh[t][q] = maxof[q] ? fmax(sh[t][q], sh[t + s][q]) : sh[t][q] + sh[t + s][q];
		}
		__syncthreads();
	}
#pragma unroll
	for (int q = 0; q < W; q++) v[q] = sh[0][q];
}

template <class S>
__global__ void __launch_bounds__(kRB) checksum_l1(Arrs A, size_t n, size_t chunk, double* partial)
{
	__shared__ double sh[kRB][1];
	bool mx[1] = {false};
	const size_t b0 = (size_t)blockIdx.x * chunk;
	const size_t b1 = min(b0 + chunk, n);
	double acc[1] = {0.0};
	for (size_t e = b0 + threadIdx.x; e < b1; e += kRB) {
		double v = to_f64<S>(((const S*)A.a[0])[e]);
		for (int q = 1; q < A.narr; q++) v = v + to_f64<S>(((const S*)A.a[q])[e]);
		acc[0] += v;
	}
	block_reduce<1>(acc, sh, mx);
	if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

template <int W>
__global__ void __launch_bounds__(kRF) reduce_l2(const double* partial, int g, double* out, int maxmask)
{
	__shared__ double sh[kRF][W];
	bool mx[W];
	double acc[W];
#pragma unroll
	for (int q = 0; q < W; q++) { mx[q] = (maxmask >> q) & 1; acc[q] = 0.0; }
	for (int b = threadIdx.x; b < g; b += kRF)
#pragma unroll
		for (int q = 0; q < W; q++)
			acc[q] = mx[q] ? fmax(acc[q], partial[(size_t)b * W + q]) : acc[q] + partial[(size_t)b * W + q];
	block_reduce<W>(acc, sh, mx);
	if (threadIdx.x == 0)
#pragma unroll
		for (int q = 0; q < W; q++) out[q] = acc[q];
}

template <class S>
__global__ void __launch_bounds__(kRB) errstats_l1(const S* x, const double* ref, size_t n, size_t chunk, double* partial)
{
	__shared__ double sh[kRB][4];
	bool mx[4] = {true, false, true, false};
	const size_t b0 = (size_t)blockIdx.x * chunk;
	const size_t b1 = min(b0 + chunk, n);
	double acc[4] = {0.0, 0.0, 0.0, 0.0};
	for (size_t e = b0 + threadIdx.x; e < b1; e += kRB) {
		const double r = ref[e];
		const double d = to_f64<S>(x[e]) - r;
		acc[0] = fmax(acc[0], fabs(d));
		acc[1] += d * d;
		acc[2] = fmax(acc[2], fabs(r));
		acc[3] += r * r;
	}
	block_reduce<4>(acc, sh, mx);
	if (threadIdx.x == 0)
		for (int q = 0; q < 4; q++) partial[(size_t)blockIdx.x * 4 + q] = acc[q];
}

template <class D, class S>
__global__ void convert_kernel(D* dst, const S* src, size_t n)
{
	for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
		const double v = to_f64<S>(src[e]);
		if constexpr (std::is_same<D, double>::value) dst[e] = v;
		else if constexpr (std::is_same<D, float>::value) dst[e] = (float)v;
		else if constexpr (std::is_same<D, __nv_bfloat16>::value) dst[e] = __double2bfloat16(v);
		else if constexpr (std::is_same<D, __half>::value) dst[e] = __double2half(v);
		else dst[e] = (uint8_t)(v > 0.5);
	}
}

template <class S>
static cudaError_t checksum_t(size_t n, const Arrs& A, double* out, cudaStream_t st)
{
	const int g = reduce_blocks(n);
	const size_t chunk = (n + g - 1) / g;
	double* partial = nullptr;
	cudaError_t e = cudaMallocAsync((void**)&partial, sizeof(double) * g, st);
	if (e != cudaSuccess) return e;
	checksum_l1<S><<<g, kRB, 0, st>>>(A, n, chunk, partial);
	reduce_l2<1><<<1, kRF, 0, st>>>(partial, g, out, 0);
	e = cudaGetLastError();
	cudaError_t f = cudaFreeAsync(partial, st);
	return e != cudaSuccess ? e : f;
}

template <class S>
static cudaError_t errstats_t(size_t n, const void* x, const double* ref, double* out, cudaStream_t st)
{
	const int g = reduce_blocks(n);
	const size_t chunk = (n + g - 1) / g;
	double* partial = nullptr;
	cudaError_t e = cudaMallocAsync((void**)&partial, sizeof(double) * 4 * g, st);
	if (e != cudaSuccess) return e;
	errstats_l1<S><<<g, kRB, 0, st>>>((const S*)x, ref, n, chunk, partial);
	reduce_l2<4><<<1, kRF, 0, st>>>(partial, g, out, 0x5);
	e = cudaGetLastError();
	cudaError_t f = cudaFreeAsync(partial, st);
	return e != cudaSuccess ? e : f;
}

template <class D, class S>
static cudaError_t convert_t(void* dst, const void* src, size_t n, cudaStream_t st)
{
	if (n == 0) return cudaSuccess;
	size_t blocks = (n + 255) / 256;
	if (blocks > 152 * 32) blocks = 152 * 32;
	convert_kernel<D, S><<<(unsigned)blocks, 256, 0, st>>>((D*)dst, (const S*)src, n);
	return cudaGetLastError();
}

// ---- kg_checksum_noalloc ------------------------------------------------------
//
// For callers that may not allocate device memory once they are running: a
// host framework that hands out all device memory from its own arena, or a
// latency-critical loop that cannot accept the device-wide synchronisation a
// cudaMalloc/cudaFree may cause.  The partial sums live in this file-scope
// array instead of the stream-ordered pool; every GPU that loads the library
// holds its 16 KiB until the process exits.  Every call shares the array and
// it keeps the previous call's partials: the first level writes every slot the
// second level reads, so nothing has to be cleared, but two calls whose
// kernels overlap on the GPU (different streams, no ordering between them)
// race on it.
static __device__ __align__(256) double g_checksum_partials[KG_CHECKSUM_NOALLOC_PARTIALS];
static_assert(KG_CHECKSUM_NOALLOC_PARTIALS >= kRG, "the first level may use kRG partials");

constexpr int kMaxDevices = 64;
static std::mutex g_partials_mu;
static double* g_partials_addr[kMaxDevices];

// The device address of g_checksum_partials on the current device.  In host
// code the array's name stands for a host-side shadow, not device memory, so
// its address is looked up once per device (with that device current) and
// cached; the first call on a device does it.
static kg_status partials_address(double** out)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail_cuda(e, "kg_checksum_noalloc: cudaGetDevice");
	if (dev < 0 || dev >= kMaxDevices) return fail(KG_EINVAL, "kg_checksum_noalloc: device %d beyond %d", dev, kMaxDevices);
	std::lock_guard<std::mutex> lock(g_partials_mu);
	if (!g_partials_addr[dev]) {
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_checksum_partials);
		if (e != cudaSuccess) return fail_cuda(e, "kg_checksum_noalloc: cudaGetSymbolAddress");
		g_partials_addr[dev] = (double*)p;
	}
	*out = g_partials_addr[dev];
	return KG_OK;
}

template <class S>
static cudaError_t checksum_static_t(size_t n, const Arrs& A, double* partial, double* out, cudaStream_t st)
{
	const int g = reduce_blocks(n);
	const size_t chunk = (n + g - 1) / g;
	checksum_l1<S><<<g, kRB, 0, st>>>(A, n, chunk, partial);
	reduce_l2<1><<<1, kRF, 0, st>>>(partial, g, out, 0);
	return cudaGetLastError();
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_checksum_noalloc(kg_dtype dt, size_t n, int narr, const void* const* arrays,
	double* out_dev, kg_stream_t stream)
{
	clear_error();
	if (narr < 1 || narr > 6 || !arrays || !out_dev)
		return fail(KG_EINVAL, "kg_checksum_noalloc: narr must be 1..6, pointers non-null");
	if (n > (size_t)KG_CHECKSUM_NOALLOC_MAX_N)
		return fail(KG_EINVAL, "kg_checksum_noalloc: n = %zu exceeds the maximum of %zu elements",
			n, (size_t)KG_CHECKSUM_NOALLOC_MAX_N);
	Arrs A{};
	A.narr = narr;
	for (int q = 0; q < narr; q++) {
		if (!arrays[q] && n) return fail(KG_EINVAL, "kg_checksum_noalloc: array %d is null", q);
		A.a[q] = arrays[q];
	}
	cudaStream_t st = (cudaStream_t)stream;
	if (n == 0) return fail_cuda(cudaMemsetAsync(out_dev, 0, sizeof(double), st), "kg_checksum_noalloc");
	double* partial = nullptr;
	kg_status s = partials_address(&partial);
	if (s != KG_OK) return s;
	cudaError_t e;
	switch (dt) {
	case KG_F64: case KG_F64_FMA: case KG_F64_FF: case KG_F64_MIX: e = checksum_static_t<double>(n, A, partial, out_dev, st); break;
	case KG_F32: e = checksum_static_t<float>(n, A, partial, out_dev, st); break;
	case KG_BF16: e = checksum_static_t<__nv_bfloat16>(n, A, partial, out_dev, st); break;
	case KG_F16: e = checksum_static_t<__half>(n, A, partial, out_dev, st); break;
	case KG_U8: e = checksum_static_t<uint8_t>(n, A, partial, out_dev, st); break;
	default: return fail(KG_EINVAL, "kg_checksum_noalloc: unknown dtype %d", (int)dt);
	}
	return fail_cuda(e, "kg_checksum_noalloc");
}

extern "C" kg_status kg_checksum(kg_dtype dt, size_t n, int narr, const void* const* arrays,
	double* out_dev, kg_stream_t stream)
{
	clear_error();
	if (narr < 1 || narr > 6 || !arrays || !out_dev) return fail(KG_EINVAL, "kg_checksum: narr must be 1..6, pointers non-null");
	Arrs A{};
	A.narr = narr;
	for (int q = 0; q < narr; q++) {
		if (!arrays[q] && n) return fail(KG_EINVAL, "kg_checksum: array %d is null", q);
		A.a[q] = arrays[q];
	}
	if (n == 0) return fail_cuda(cudaMemsetAsync(out_dev, 0, sizeof(double), (cudaStream_t)stream), "kg_checksum");
	cudaStream_t st = (cudaStream_t)stream;
	cudaError_t e;
	switch (dt) {
	case KG_F64: case KG_F64_FMA: case KG_F64_FF: case KG_F64_MIX: e = checksum_t<double>(n, A, out_dev, st); break;
	case KG_F32: e = checksum_t<float>(n, A, out_dev, st); break;
	case KG_BF16: e = checksum_t<__nv_bfloat16>(n, A, out_dev, st); break;
	case KG_F16: e = checksum_t<__half>(n, A, out_dev, st); break;
	case KG_U8: e = checksum_t<uint8_t>(n, A, out_dev, st); break;
	default: return fail(KG_EINVAL, "kg_checksum: unknown dtype %d", (int)dt);
	}
	return fail_cuda(e, "kg_checksum");
}

extern "C" kg_status kg_error_stats(kg_dtype dt, size_t n, const void* x, const double* ref,
	double* out_dev, kg_stream_t stream)
{
	clear_error();
	if (!out_dev || (n && (!x || !ref))) return fail(KG_EINVAL, "kg_error_stats: null pointer");
	cudaStream_t st = (cudaStream_t)stream;
	if (n == 0) return fail_cuda(cudaMemsetAsync(out_dev, 0, 4 * sizeof(double), st), "kg_error_stats");
	cudaError_t e;
	switch (dt) {
	case KG_F64: case KG_F64_FMA: case KG_F64_FF: case KG_F64_MIX: e = errstats_t<double>(n, x, ref, out_dev, st); break;
	case KG_F32: e = errstats_t<float>(n, x, ref, out_dev, st); break;
	case KG_BF16: e = errstats_t<__nv_bfloat16>(n, x, ref, out_dev, st); break;
	case KG_F16: e = errstats_t<__half>(n, x, ref, out_dev, st); break;
	case KG_U8: e = errstats_t<uint8_t>(n, x, ref, out_dev, st); break;
	default: return fail(KG_EINVAL, "kg_error_stats: unknown dtype %d", (int)dt);
	}
	return fail_cuda(e, "kg_error_stats");
}

extern "C" kg_status kg_convert(kg_dtype dst_t, void* dst, kg_dtype src_t, const void* src,
	size_t n, kg_stream_t stream)
{
	clear_error();
	if (n && (!dst || !src)) return fail(KG_EINVAL, "kg_convert: null pointer");
	cudaStream_t st = (cudaStream_t)stream;
	auto is64 = [](kg_dtype t) { return t == KG_F64 || t == KG_F64_FMA || t == KG_F64_FF || t == KG_F64_MIX; };
	cudaError_t e = cudaErrorInvalidValue;
	if (is64(src_t)) {
		switch (dst_t) {
		case KG_F64: case KG_F64_FMA: case KG_F64_FF: case KG_F64_MIX: e = convert_t<double, double>(dst, src, n, st); break;
		case KG_F32: e = convert_t<float, double>(dst, src, n, st); break;
		case KG_BF16: e = convert_t<__nv_bfloat16, double>(dst, src, n, st); break;
		case KG_F16: e = convert_t<__half, double>(dst, src, n, st); break;
		case KG_U8: e = convert_t<uint8_t, double>(dst, src, n, st); break;
		default: return fail(KG_EINVAL, "kg_convert: unknown dtype");
		}
	} else if (is64(dst_t)) {
		switch (src_t) {
		case KG_F32: e = convert_t<double, float>(dst, src, n, st); break;
		case KG_BF16: e = convert_t<double, __nv_bfloat16>(dst, src, n, st); break;
		case KG_F16: e = convert_t<double, __half>(dst, src, n, st); break;
		case KG_U8: e = convert_t<double, uint8_t>(dst, src, n, st); break;
		default: return fail(KG_EINVAL, "kg_convert: unknown dtype");
		}
	} else {
		return fail(KG_ENOTSUP, "kg_convert: one side must be FP64");
	}
	return fail_cuda(e, "kg_convert");
}
