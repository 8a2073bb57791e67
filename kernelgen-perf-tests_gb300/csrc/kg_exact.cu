// kg_exact.cu -- element-wise access to the strict sweeps' FP64 arithmetic
// on the integer pipes (se_add, se_mul, se_div in kg_num.cuh) and, for
// comparison, to the FP64 unit's, so that tests can check the former bit for
// bit against IEEE arithmetic on any operands.
#include "kg_internal.h"
#include "kg_num.cuh"

namespace kg {

template <int OP>
__global__ void __launch_bounds__(256) exact_arith_kernel(size_t n, const double* __restrict__ a,
	const double* __restrict__ b, double* __restrict__ out)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const double x = a[i], y = b[i];
		double r;
		if (OP == KG_ARITH_ADD) r = se_add(x, y);
		else if (OP == KG_ARITH_MUL) r = se_mul(x, y);
		else if (OP == KG_ARITH_DIV) r = se_div(x, y);
		else if (OP == KG_ARITH_NATIVE_ADD) r = __dadd_rn(x, y);
		else if (OP == KG_ARITH_NATIVE_MUL) r = __dmul_rn(x, y);
		else r = __ddiv_rn(x, y);
		out[i] = r;
	}
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_exact_arith(int op, size_t n, const double* a, const double* b, double* out,
	kg_stream_t stream)
{
	clear_error();
	if (op < KG_ARITH_ADD || op > KG_ARITH_NATIVE_DIV) return fail(KG_EINVAL, "kg_exact_arith: unknown op %d", op);
	if (n == 0) return KG_OK;
	if (!a || !b || !out) return fail(KG_EINVAL, "kg_exact_arith: null array");
	int dev = 0, sms = 152;
	if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const size_t want = (n + 255) / 256, cap = (size_t)sms * 16;
	const unsigned grid = (unsigned)(want < cap ? want : cap);
	cudaStream_t st = (cudaStream_t)stream;
	switch (op) {
	case KG_ARITH_ADD: exact_arith_kernel<KG_ARITH_ADD><<<grid, 256, 0, st>>>(n, a, b, out); break;
	case KG_ARITH_MUL: exact_arith_kernel<KG_ARITH_MUL><<<grid, 256, 0, st>>>(n, a, b, out); break;
	case KG_ARITH_DIV: exact_arith_kernel<KG_ARITH_DIV><<<grid, 256, 0, st>>>(n, a, b, out); break;
	case KG_ARITH_NATIVE_ADD: exact_arith_kernel<KG_ARITH_NATIVE_ADD><<<grid, 256, 0, st>>>(n, a, b, out); break;
	case KG_ARITH_NATIVE_MUL: exact_arith_kernel<KG_ARITH_NATIVE_MUL><<<grid, 256, 0, st>>>(n, a, b, out); break;
	default: exact_arith_kernel<KG_ARITH_NATIVE_DIV><<<grid, 256, 0, st>>>(n, a, b, out); break;
	}
	return fail_cuda(cudaGetLastError(), "kg_exact_arith");
}
