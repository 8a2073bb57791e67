// kg_tma.cu -- host side of the TMA engine: tensor maps and the wait flag.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "kg_internal.h"
#include "kg_tma.cuh"

namespace kg {

// Raised (set to 1) by a TMA-engine kernel whose wait for a copy gave up.
static __device__ int g_tma_error;

// The compute warps' wait limit passed to kernels launched from now on
// (process-wide; negative: the default).
static std::atomic<long long> g_tma_wait{-1};

long long tma_wait_limit()
{
	const long long w = g_tma_wait.load(std::memory_order_relaxed);
	return w < 0 ? kTmaWaitCycles : w;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn(cudaError_t* err)
{
	static std::once_flag once;
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	static cudaError_t status = cudaSuccess;
	std::call_once(once, [] {
		void* f = nullptr;
		cudaDriverEntryPointQueryResult q;
		status = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q);
		if (status == cudaSuccess && q != cudaDriverEntryPointSuccess) status = cudaErrorSymbolNotFound;
		fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
	});
	*err = status;
	return fn;
}

// A rank-3 tiled map over an nx x ny x ns array (x fastest) with boxes of
// box_w x box_h x 1 elements, zero fill outside the array.
cudaError_t tma_encode_3d(CUtensorMap* map, CUtensorMapDataType type, const void* base, uint64_t nx,
	uint64_t ny, uint64_t ns, int elem_bytes, int box_w, int box_h)
{
	cudaError_t e;
	PFN_cuTensorMapEncodeTiled_v12000 encode = encode_fn(&e);
	if (!encode) return e != cudaSuccess ? e : cudaErrorSymbolNotFound;
	const cuuint64_t dims[3] = {nx, ny, ns};
	const cuuint64_t strides[2] = {nx * elem_bytes, nx * ny * elem_bytes};
	const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
	const cuuint32_t estr[3] = {1, 1, 1};
	CUresult r = encode(map, type, 3, const_cast<void*>(base), dims, strides, box, estr,
		CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
		CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// A rank-2 tiled map over an FP32 array of `outer` rows of `inner` elements
// (rows contiguous, inner * 4 a multiple of 16 bytes) with boxes of
// box_inner x box_outer elements in the 128- or 64-byte swizzle (box_inner *
// 4 <= that), zero fill outside the array.
cudaError_t tma_encode_2d_swizzled(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, int box_inner,
	int box_outer, int swizzle_bytes)
{
	cudaError_t e;
	PFN_cuTensorMapEncodeTiled_v12000 encode = encode_fn(&e);
	if (!encode) return e != cudaSuccess ? e : cudaErrorSymbolNotFound;
	const cuuint64_t dims[2] = {inner, outer};
	const cuuint64_t strides[1] = {inner * 4};
	const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
	const cuuint32_t estr[2] = {1, 1};
	CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
		CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
		CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
		CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// The device address of g_tma_error on the current device, looked up once per
// device and cached (it does not survive cudaDeviceReset).
int* tma_error_flag()
{
	static std::mutex m;
	static int* addr[64];
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
	std::lock_guard<std::mutex> g(m);
	if (!addr[dev]) {
		void* a = nullptr;
		if (cudaGetSymbolAddress(&a, g_tma_error) != cudaSuccess) return nullptr;
		addr[dev] = (int*)a;
	}
	return addr[dev];
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_set_tma_wait_limit(long long cycles)
{
	clear_error();
	g_tma_wait.store(cycles < 0 ? -1 : cycles, std::memory_order_relaxed);
	return KG_OK;
}

extern "C" kg_status kg_engine_status(kg_stream_t stream)
{
	clear_error();
	cudaStream_t st = (cudaStream_t)stream;
	int* flag = tma_error_flag();
	if (!flag) return fail(KG_ECUDA, "kg_engine_status: no device flag");
	int v = 0;
	kg_status s = fail_cuda(cudaMemcpyAsync(&v, flag, sizeof(int), cudaMemcpyDeviceToHost, st), "kg_engine_status");
	if (s == KG_OK) s = fail_cuda(cudaStreamSynchronize(st), "kg_engine_status");
	if (s != KG_OK) return s;
	if (v) {
		const int zero = 0;
		s = fail_cuda(cudaMemcpyAsync(flag, &zero, sizeof(int), cudaMemcpyHostToDevice, st), "kg_engine_status");
		if (s == KG_OK) s = fail_cuda(cudaStreamSynchronize(st), "kg_engine_status");
		if (s != KG_OK) return s;
		return fail(KG_ETIMEOUT, "a sweep's wait for its tile copies gave up; its output is incomplete");
	}
	return KG_OK;
}
