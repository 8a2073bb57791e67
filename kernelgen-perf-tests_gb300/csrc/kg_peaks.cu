// kg_peaks.cu -- issue-rate calibration of the arithmetic pipes.
//
// The FP64 sweeps are bound by GB300's FP64 pipe, not by HBM, so their
// roofline denominator is the FP64 operation rate.  These kernels measure it
// (and the FP32/INT32 rates for comparison) with eight independent
// dependency chains per thread on every SM, timed with CUDA events.
#include "kg_internal.h"

namespace kg {

constexpr int kPeakIters = 4096;
constexpr int kPeakThreads = 256;

__global__ void __launch_bounds__(kPeakThreads) peak_dfma(double* out, double a, double b)
{
	double x[8];
#pragma unroll
	for (int q = 0; q < 8; q++) x[q] = threadIdx.x + q;
	for (int i = 0; i < kPeakIters; i++)
#pragma unroll
		for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
	double s = 0;
#pragma unroll
	for (int q = 0; q < 8; q++) s += x[q];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(kPeakThreads) peak_ffma(float* out, float a, float b)
{
	float x[8];
#pragma unroll
	for (int q = 0; q < 8; q++) x[q] = threadIdx.x + q;
	for (int i = 0; i < kPeakIters; i++)
#pragma unroll
		for (int q = 0; q < 8; q++) x[q] = fmaf(x[q], a, b);
	float s = 0;
#pragma unroll
	for (int q = 0; q < 8; q++) s += x[q];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(kPeakThreads) peak_imad(unsigned* out, unsigned a, unsigned b)
{
	unsigned x[8];
#pragma unroll
	for (int q = 0; q < 8; q++) x[q] = threadIdx.x + q;
	for (int i = 0; i < kPeakIters; i++)
#pragma unroll
		for (int q = 0; q < 8; q++) x[q] = x[q] * a + b;
	unsigned s = 0;
#pragma unroll
	for (int q = 0; q < 8; q++) s += x[q];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_measure_peaks(kg_peaks* out, kg_stream_t stream)
{
	clear_error();
	if (!out) return fail(KG_EINVAL, "kg_measure_peaks: null output");
	cudaStream_t st = (cudaStream_t)stream;
	int dev = 0, sms = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e != cudaSuccess) return fail_cuda(e, "kg_measure_peaks");
	const int blocks = sms * 8;
	void* buf = nullptr;
	if ((e = cudaMallocAsync(&buf, sizeof(double) * blocks * kPeakThreads, st)) != cudaSuccess)
		return fail_cuda(e, "kg_measure_peaks");
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	const double ops = (double)blocks * kPeakThreads * kPeakIters * 8;
	double best[3] = {0, 0, 0};
	for (int rep = 0; rep < 3; rep++) {
		for (int k = 0; k < 3; k++) {
			cudaEventRecord(a, st);
			if (k == 0) peak_dfma<<<blocks, kPeakThreads, 0, st>>>((double*)buf, 1.0000001, 1e-9);
			else if (k == 1) peak_ffma<<<blocks, kPeakThreads, 0, st>>>((float*)buf, 1.0000001f, 1e-9f);
			else peak_imad<<<blocks, kPeakThreads, 0, st>>>((unsigned*)buf, 1664525u, 1013904223u);
			cudaEventRecord(b, st);
			if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
			float ms = 0;
			cudaEventElapsedTime(&ms, a, b);
			const double r = ops / (ms * 1e-3);
			if (rep > 0 && r > best[k]) best[k] = r;  // first round warms up
		}
	}
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	cudaFreeAsync(buf, st);
	if (e != cudaSuccess) return fail_cuda(e, "kg_measure_peaks");
	if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "kg_measure_peaks");
	out->fp64_ops = best[0];
	out->fp32_ops = best[1];
	out->int32_ops = best[2];
	out->sms = sms;
	return KG_OK;
}
