// kg_extra.cu -- the suite's tests that are not stencil sweeps: vecadd,
// matvec, matmul, sincos and whispering, each behind an entry point with the
// reference kernel's arguments.
//
// The arithmetic types are those of the sweeps (kg_num.cuh): KG_F64 strict
// IEEE (bit for bit the reference's expression), KG_F64_FMA contracted FP64,
// KG_F32.  matvec and matmul accumulate every output in the reference's loop
// order (a sequential sum per output), so their strict FP64 form is bound by
// GB300's FP64 issue rate; like the strict tricubic, they form a share of the
// products with the exact integer multiply (se_mul), which gives the same
// bits as the FP64 unit.
#include <cstdint>
#include <cstring>

#include "kg_internal.h"
#include "kg_num.cuh"

namespace kg {

// Product a*b; for strict FP64 on the integer pipes when `integer` is set.
template <class N> __device__ __forceinline__ N mul_on(N a, N b, bool integer)
{
	if constexpr (std::is_same<N, SD>::value) return integer ? SD(se_mul(a.v, b.v)) : a * b;
	else return a * b;
}

// Quotient a/b; for strict FP64 by the exact division on the integer and
// FP32 pipes (se_div, the FP64 unit's bits).
template <class N> __device__ __forceinline__ N div_on(N a, N b)
{
	if constexpr (std::is_same<N, SD>::value) return SD(se_div(a.v, b.v));
	else return a / b;
}

// ---- vecadd/vecadd.c:38-84: w2 = w0 + w1 -----------------------------------

template <class N, class S>
__global__ void __launch_bounds__(256) vecadd_kernel(size_t n, const S* __restrict__ w0,
	const S* __restrict__ w1, S* __restrict__ w2)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
		w2[i] = Conv<N, S>::to(Conv<N, S>::ld(w0 + i) + Conv<N, S>::ld(w1 + i));
}

// Two 16-byte vectors per thread and step (arrays 16-byte aligned).
template <class S, class V>
__global__ void __launch_bounds__(256) vecadd_vec_kernel(size_t nv, const V* __restrict__ w0,
	const V* __restrict__ w1, V* __restrict__ w2)
{
	constexpr int L = sizeof(V) / sizeof(S);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
		const V a = __ldg(w0 + i), b = __ldg(w1 + i);
		V c;
		const S* pa = reinterpret_cast<const S*>(&a);
		const S* pb = reinterpret_cast<const S*>(&b);
		S* pc = reinterpret_cast<S*>(&c);
#pragma unroll
		for (int l = 0; l < L; l++) {
			if constexpr (std::is_same<S, double>::value) pc[l] = __dadd_rn(pa[l], pb[l]);
			else pc[l] = __fadd_rn(pa[l], pb[l]);
		}
		w2[i] = c;
	}
}

static int grid_for(size_t work, int threads)
{
	int dev = 0, sms = 152;
	if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const size_t want = (work + threads - 1) / threads;
	const size_t cap = (size_t)sms * 8;
	return (int)(want < cap ? (want ? want : 1) : cap);
}

template <class N, class S>
cudaError_t vecadd_run(size_t n, const void* w0, const void* w1, void* w2, cudaStream_t st)
{
	using V = typename std::conditional<std::is_same<S, double>::value, double2, float4>::type;
	const bool aligned = ((uintptr_t)w0 | (uintptr_t)w1 | (uintptr_t)w2) % 16 == 0;
	constexpr int L = sizeof(V) / sizeof(S);
	size_t done = 0;
	if (aligned && n >= (size_t)L) {
		const size_t nv = n / L;
		vecadd_vec_kernel<S, V><<<grid_for(nv, 256), 256, 0, st>>>(nv, (const V*)w0, (const V*)w1, (V*)w2);
		done = nv * L;
	}
	if (done < n)
		vecadd_kernel<N, S><<<grid_for(n - done, 256), 256, 0, st>>>(n - done, (const S*)w0 + done,
			(const S*)w1 + done, (S*)w2 + done);
	return cudaGetLastError();
}

// ---- matvec/matvec.c:37-71: y[j] = 0; y[j] += A[i + nx j] * x[i], i = 0.. ----
//
// A CTA owns ROWS rows; column chunks of A (KC per row) and x go through
// shared memory with coalesced loads, the next chunk's loads in flight in
// registers while the current one is summed, and each thread sums its row in
// order.  Strict FP64 forms the products on the integer pipes, so the FP64
// unit only adds.

// 8 CTAs of 64 threads per SM (measured, 512 x 65536 strict FP64: 0.152 ms
// with no register cap, 0.139 with this one, 0.181 with 12 CTAs; FP32 0.039,
// 0.035, 0.033).
constexpr int kMvRows = 64, kMvKC = 32, kMvMinBlocks = 8;
// Columns a chunk for 4-byte elements (the in-order sums do not depend on it):
// measured on GB300, FP32 512 x 65536 0.0351 ms with 32, 0.0292 with 64 (4.6
// TB/s); 4096 x 65536 0.235 and 0.199.
#ifndef KG_MV_KC32
#define KG_MV_KC32 64
#endif
static_assert(KG_MV_KC32 <= kMvRows, "x's chunk is loaded one element a thread");

template <class N, class S>
__global__ void __launch_bounds__(kMvRows, kMvMinBlocks) matvec_kernel(int nx, int ny, const S* __restrict__ A,
	const S* __restrict__ x, S* __restrict__ y)
{
	constexpr int KC = sizeof(S) == 4 ? KG_MV_KC32 : kMvKC;   // columns a chunk
	__shared__ S tile[kMvRows][KC + 1];
	__shared__ S xs[KC];
	constexpr int PER = KC;                    // elements per thread per chunk (kMvRows rows, kMvRows threads)
	const int t = threadIdx.x;
	const int j0 = blockIdx.x * kMvRows, j = j0 + t;
	S v[PER], xv{};
	auto fetch = [&](int i0) {
#pragma unroll
		for (int q = 0; q < PER; q++) {
			const int e = t + q * kMvRows, r = e / KC, c = e - r * KC;
			v[q] = (j0 + r < ny && i0 + c < nx) ? __ldg(A + (size_t)(j0 + r) * nx + i0 + c) : S{};
		}
		xv = (t < KC && i0 + t < nx) ? __ldg(x + i0 + t) : S{};
	};
	N s = N(0.0);
	if (nx > 0) fetch(0);
	for (int i0 = 0; i0 < nx; i0 += KC) {
#pragma unroll
		for (int q = 0; q < PER; q++) {
			const int e = t + q * kMvRows, r = e / KC, c = e - r * KC;
			tile[r][c] = v[q];
		}
		if (t < KC) xs[t] = xv;
		__syncthreads();
		if (i0 + KC < nx) fetch(i0 + KC);
		const int kc = min(KC, nx - i0);
		if (j < ny) {
			if (kc == KC) {
#pragma unroll
				for (int c = 0; c < KC; c++)
					s = s + mul_on(Conv<N, S>::from(tile[t][c]), Conv<N, S>::from(xs[c]), true);
			} else {
				for (int c = 0; c < kc; c++)
					s = s + mul_on(Conv<N, S>::from(tile[t][c]), Conv<N, S>::from(xs[c]), true);
			}
		}
		__syncthreads();
	}
	if (j < ny) y[j] = Conv<N, S>::to(s);
}

// FP32 with 16-byte aligned rows and x (nx a multiple of 4): the chunks reach
// shared memory by 16-byte cp.async copies, which hold no registers, through a
// ring of kMvaStages chunks of kMvaKC columns, so a CTA has the next chunks in
// flight while it sums one.  Rows of kMvaLd floats: a thread reads its own row
// 16 bytes at a time, and the eight threads of each quarter-warp then fall on
// eight distinct groups of four banks.  Same sums in the same order as
// matvec_kernel.  Measured on GB300 (ms, 512 x 65536 and 4096 x 65536; the
// register-staged kernel 0.0290 and 0.195): 32 columns, 2 stages, 8 CTAs per
// SM 0.0254 and 0.176; 3 stages (7 CTAs) 0.0268 and 0.178; 4 stages (5)
// 0.0297 and 0.216; 64 columns, 2 stages (6) 0.0270 and 0.192; 16 columns,
// 6 stages 0.0297 and 0.199; 8 columns, 12 stages 0.048 and 0.330.  Deeper
// rings of narrower row segments keep more bytes in flight but spread them
// over more DRAM pages at once.
#ifndef KG_MVA_KC
#define KG_MVA_KC 32
#endif
#ifndef KG_MVA_STAGES
#define KG_MVA_STAGES 2
#endif
#ifndef KG_MVA_MINB
#define KG_MVA_MINB 8
#endif
constexpr int kMvaKC = KG_MVA_KC, kMvaStages = KG_MVA_STAGES, kMvaLd = kMvaKC + 4;
constexpr int kMvaMinBlocks = KG_MVA_MINB;   // 65536 rows of 512: one wave of 64-row CTAs on 152 SMs

__device__ __forceinline__ void mv_cp16(void* dst, const void* src, int src_bytes)
{
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}

template <class N>
__global__ void __launch_bounds__(kMvRows, kMvaMinBlocks) matvec_ring_kernel(int nx, int ny,
	const float* __restrict__ A, const float* __restrict__ x, float* __restrict__ y)
{
	__shared__ __align__(16) float tile[kMvaStages][kMvRows][kMvaLd];
	__shared__ __align__(16) float xs[kMvaStages][kMvaKC];
	constexpr int V = kMvaKC / 4;   // 16-byte copies a row of a chunk
	const int t = threadIdx.x, j0 = blockIdx.x * kMvRows, j = j0 + t;
	const int nch = (nx + kMvaKC - 1) / kMvaKC;
	// chunk ch into its ring slot; rows past ny and columns past nx are
	// zero-filled (no bytes read) and never summed
	auto issue = [&](int ch) {
		if (ch < nch) {
			const int st = ch % kMvaStages, i0 = ch * kMvaKC;
#pragma unroll
			for (int q = 0; q < kMvRows * V / kMvRows; q++) {
				const int e = t + q * kMvRows, r = e / V, c = 4 * (e % V);
				const bool ok = j0 + r < ny && i0 + c < nx;
				mv_cp16(&tile[st][r][c], ok ? A + (size_t)(j0 + r) * nx + i0 + c : A, ok ? 16 : 0);
			}
			if (t < V) {
				const bool ok = i0 + 4 * t < nx;
				mv_cp16(&xs[st][4 * t], ok ? x + i0 + 4 * t : x, ok ? 16 : 0);
			}
		}
		asm volatile("cp.async.commit_group;" ::: "memory");   // one group per chunk, empty past the end
	};
#pragma unroll
	for (int ch = 0; ch < kMvaStages - 1; ch++) issue(ch);
	N s = N(0.0);
	for (int ch = 0; ch < nch; ch++) {
		issue(ch + kMvaStages - 1);   // into the slot summed in the step before (freed by its barrier)
		asm volatile("cp.async.wait_group %0;" ::"n"(kMvaStages - 1) : "memory");
		__syncthreads();
		const int st = ch % kMvaStages, kc = min(kMvaKC, nx - ch * kMvaKC);
		if (j < ny) {
			const float4* row = reinterpret_cast<const float4*>(&tile[st][t][0]);
			const float4* xv = reinterpret_cast<const float4*>(&xs[st][0]);
			auto step4 = [&](int c4) {
				const float4 a = row[c4], b = xv[c4];
				s = s + mul_on(mkf(a.x), mkf(b.x), true);
				s = s + mul_on(mkf(a.y), mkf(b.y), true);
				s = s + mul_on(mkf(a.z), mkf(b.z), true);
				s = s + mul_on(mkf(a.w), mkf(b.w), true);
			};
			if (kc == kMvaKC) {
#pragma unroll
				for (int c4 = 0; c4 < V; c4++) step4(c4);
			} else {
				for (int c4 = 0; c4 < kc / 4; c4++) step4(c4);
			}
		}
		__syncthreads();
	}
	asm volatile("cp.async.wait_group 0;" ::: "memory");
	if (j < ny) y[j] = s.v;
}

// ---- matmul/matmul.F90:56-68: C(i,j) = C(i,j) + A(i,k) * B(k,j), k = 1..ny --
//
// Column-major: A(i,k) at A[i + nx k], B(k,j) at B[k + ny j], C(i,j) at
// C[i + nx j].  A CTA of 32 x 8 threads owns a 32 x 32 tile of C, each thread
// four outputs 8 columns apart; k runs in chunks of 16 through shared
// memory, and every output accumulates its products in k order.

constexpr int kMmTI = 32, kMmTJ = 32, kMmKC = 16;
// Of each thread's four products per k, the first kMmInt on the integer
// pipes (strict FP64; 512x256x256, ms: 2 of 4 0.131, 3 of 4 0.113, 4 of 4
// 0.119).
constexpr int kMmInt = 3;

template <class N, class S>
__global__ void __launch_bounds__(256) matmul_kernel(int nx, int ny, int ns, const S* __restrict__ A,
	const S* __restrict__ B, S* __restrict__ C)
{
	__shared__ S As[kMmKC][kMmTI];
	__shared__ S Bs[kMmTJ][kMmKC + 1];
	const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
	const int i0 = blockIdx.x * kMmTI, j0 = blockIdx.y * kMmTJ;
	const int i = i0 + tx;
	N c[4];
#pragma unroll
	for (int m = 0; m < 4; m++) {
		const int j = j0 + ty + 8 * m;
		c[m] = (i < nx && j < ns) ? Conv<N, S>::ld(C + i + (size_t)nx * j) : N(0.0);
	}
	for (int k0 = 0; k0 < ny; k0 += kMmKC) {
		const int kc = min(kMmKC, ny - k0);
#pragma unroll
		for (int q = 0; q < 2; q++) {
			const int e = tid + 256 * q;
			const int kk = e / kMmTI, ti = e - kk * kMmTI;
			As[kk][ti] = (i0 + ti < nx && kk < kc) ? __ldg(A + (i0 + ti) + (size_t)nx * (k0 + kk)) : S{};
			const int tj = e / kMmKC, kb = e - tj * kMmKC;
			Bs[tj][kb] = (j0 + tj < ns && kb < kc) ? __ldg(B + (k0 + kb) + (size_t)ny * (j0 + tj)) : S{};
		}
		__syncthreads();
		if (kc == kMmKC) {
#pragma unroll
			for (int kk = 0; kk < kMmKC; kk++) {
				const N a = Conv<N, S>::from(As[kk][tx]);
#pragma unroll
				for (int m = 0; m < 4; m++) c[m] = c[m] + mul_on(a, Conv<N, S>::from(Bs[ty + 8 * m][kk]), m < kMmInt);
			}
		} else {
			for (int kk = 0; kk < kc; kk++) {
				const N a = Conv<N, S>::from(As[kk][tx]);
#pragma unroll
				for (int m = 0; m < 4; m++) c[m] = c[m] + mul_on(a, Conv<N, S>::from(Bs[ty + 8 * m][kk]), m < kMmInt);
			}
		}
		__syncthreads();
	}
#pragma unroll
	for (int m = 0; m < 4; m++) {
		const int j = j0 + ty + 8 * m;
		if (i < nx && j < ns) C[i + (size_t)nx * j] = Conv<N, S>::to(c[m]);
	}
}

// ---- sincos/sincos.F90:60-72: xy = sin(x) + cos(y) -------------------------

template <class N, class S>
__global__ void __launch_bounds__(256) sincos_kernel(size_t n, const S* __restrict__ x,
	const S* __restrict__ y, S* __restrict__ xy)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		if constexpr (std::is_same<S, double>::value) xy[i] = Conv<N, S>::to(N(sin(__ldg(x + i))) + N(cos(__ldg(y + i))));
		else xy[i] = Conv<N, S>::to(mkf(sinf(__ldg(x + i))) + mkf(cosf(__ldg(y + i))));
	}
}

// FP32 with 16-byte aligned arrays: four points a thread and step, so each
// thread has 32 bytes of loads in flight instead of 8 (the scalar kernel's
// loads in flight per SM are too few to cover HBM latency).  Same functions
// on the same values: the same bits.
__global__ void __launch_bounds__(256) sincos_vec_kernel(size_t nv, const float4* __restrict__ x,
	const float4* __restrict__ y, float4* __restrict__ xy)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
		const float4 a = __ldg(x + i), b = __ldg(y + i);
		float4 c;
		c.x = (mkf(sinf(a.x)) + mkf(cosf(b.x))).v;
		c.y = (mkf(sinf(a.y)) + mkf(cosf(b.y))).v;
		c.z = (mkf(sinf(a.z)) + mkf(cosf(b.z))).v;
		c.w = (mkf(sinf(a.w)) + mkf(cosf(b.w))).v;
		xy[i] = c;
	}
}

// ---- whispering/whispering.c:87-108 ------------------------------------------
//
// The reference updates e in place inside its j, i loops, and the terms ey
// and ex read e at (i, j-1) and (i-1, j), which the loops have already
// updated when those points are interior.  Every new e depends only on old
// values, so two passes give exactly the loop's result: pass 1 writes the new
// e of every interior point; pass 2 evaluates h and u_em reading e, which then
// holds new values inside and the untouched boundary values outside.  e is
// planar: component c of (i, j) at e[i + nx j + nx ny c].

template <class N, class S>
__global__ void __launch_bounds__(256) whispering_e_kernel(int nx, int ny, S* __restrict__ e,
	const S* __restrict__ h0, const S* __restrict__ ca, const S* __restrict__ cb)
{
	const int i = 1 + blockIdx.x * 32 + threadIdx.x;
	const size_t plane = (size_t)nx * ny;
	if (i >= nx - 1) return;
	for (int j = 1 + blockIdx.y * 8 + threadIdx.y; j < ny - 1; j += gridDim.y * 8) {
		const size_t c = i + (size_t)nx * j;
		using Cv = Conv<N, S>;
		auto M = [](N a, N b) { return mul_on(a, b, true); };
		const N vca = Cv::ld(ca + c), vcb = Cv::ld(cb + c), vh = Cv::ld(h0 + c);
		const N e0 = M(vca, Cv::from(e[c])) + M(vcb, Cv::ld(h0 + c + nx) - vh);
		const N e1 = M(vca, Cv::from(e[c + plane])) - M(vcb, Cv::ld(h0 + c + 1) - vh);
		e[c] = Cv::to(e0);
		e[c + plane] = Cv::to(e1);
	}
}

template <class N, class S>
__global__ void __launch_bounds__(256) whispering_h_kernel(int nx, int ny, N mu, N epsilon,
	const S* __restrict__ e, const S* __restrict__ h0, S* __restrict__ h1, const S* __restrict__ u_em0,
	S* __restrict__ u_em1, const S* __restrict__ ca, const S* __restrict__ cb, const S* __restrict__ da,
	const S* __restrict__ db)
{
	const int i = 1 + blockIdx.x * 32 + threadIdx.x;
	const size_t plane = (size_t)nx * ny;
	if (i >= nx - 1) return;
	for (int j = 1 + blockIdx.y * 8 + threadIdx.y; j < ny - 1; j += gridDim.y * 8) {
		const size_t c = i + (size_t)nx * j;
		using Cv = Conv<N, S>;
		auto M = [](N a, N b) { return mul_on(a, b, true); };
		const N vh = Cv::ld(h0 + c);
		const N e0 = Cv::ld(e + c), e1 = Cv::ld(e + c + plane);
		const N ey = M(Cv::ld(ca + c - nx), Cv::ld(e + c - nx)) + M(Cv::ld(cb + c - nx), vh - Cv::ld(h0 + c - nx));
		const N ex = M(Cv::ld(ca + c - 1), Cv::ld(e + c - 1 + plane)) - M(Cv::ld(cb + c - 1), vh - Cv::ld(h0 + c - 1));
		const N h = M(Cv::ld(da + c), vh) + M(Cv::ld(db + c), e0 - ey + ex - e1);
		h1[c] = Cv::to(h);
		u_em1[c] = Cv::to(Cv::ld(u_em0 + c) + M(N(0.5), div_on(M(h, h), mu) + M(epsilon, M(e0, e0) + M(e1, e1))));
	}
}

// ---- dispatch by storage type -------------------------------------------

template <class F> cudaError_t by_type(int dt, F&& f)
{
	switch (dt) {
	case KG_F64: return f(SD{}, double{});
	case KG_F64_FMA: return f(FD{}, double{});
	case KG_F32: return f(FF{}, float{});
	default: return cudaErrorInvalidValue;
	}
}

static bool extra_type(int dt) { return dt == KG_F64 || dt == KG_F64_FMA || dt == KG_F32; }

static bool overlaps(const void* a, size_t na, const void* b, size_t nb)
{
	const char* x = (const char*)a;
	const char* y = (const char*)b;
	return x < y + nb && y < x + na;
}

}  // namespace kg

using namespace kg;

extern "C" {

kg_status kg_vecadd(kg_dtype dt, int nx, int ny, int ns, const void* w0, const void* w1, void* w2,
	kg_stream_t stream)
{
	clear_error();
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "vecadd: dtype %d not provided (KG_F64, KG_F64_FMA, KG_F32)", dt);
	if (nx < 0 || ny < 0 || ns < 0) return fail(KG_EINVAL, "vecadd: negative size");
	const size_t n = (size_t)nx * ny * ns, bytes = n * dtype_size(dt);
	if (n == 0) return KG_OK;
	if (!w0 || !w1 || !w2) return fail(KG_EINVAL, "vecadd: null array");
	if (overlaps(w2, bytes, w0, bytes) || overlaps(w2, bytes, w1, bytes))
		return fail(KG_EINVAL, "vecadd: output array overlaps an input");
	return fail_cuda(by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		return vecadd_run<N, S>(n, w0, w1, w2, (cudaStream_t)stream);
	}), "vecadd");
}

kg_status kg_matvec(kg_dtype dt, int nx, int ny, const void* A, const void* x, void* y, kg_stream_t stream)
{
	clear_error();
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "matvec: dtype %d not provided (KG_F64, KG_F64_FMA, KG_F32)", dt);
	if (nx < 0 || ny < 0) return fail(KG_EINVAL, "matvec: negative size");
	if (ny == 0) return KG_OK;
	if (!y || (nx > 0 && (!A || !x))) return fail(KG_EINVAL, "matvec: null array");
	const size_t es = dtype_size(dt);
	if (nx > 0 && (overlaps(y, ny * es, A, (size_t)nx * ny * es) || overlaps(y, ny * es, x, nx * es)))
		return fail(KG_EINVAL, "matvec: output array overlaps an input");
	if ((size_t)nx * ny > ((size_t)1 << 40)) return fail(KG_EINVAL, "matvec: beyond the supported size");
	return fail_cuda(by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		const unsigned grid = (unsigned)((ny + kMvRows - 1) / kMvRows);
		if constexpr (std::is_same<S, float>::value) {
			if (nx >= 4 && nx % 4 == 0 && ((uintptr_t)A | (uintptr_t)x) % 16 == 0) {
				matvec_ring_kernel<N><<<grid, kMvRows, 0, (cudaStream_t)stream>>>(nx, ny, (const float*)A,
					(const float*)x, (float*)y);
				return cudaGetLastError();
			}
		}
		matvec_kernel<N, S><<<grid, kMvRows, 0, (cudaStream_t)stream>>>(nx, ny, (const S*)A, (const S*)x, (S*)y);
		return cudaGetLastError();
	}), "matvec");
}

kg_status kg_matmul(kg_dtype dt, int nx, int ny, int ns, const void* A, const void* B, void* C, kg_stream_t stream)
{
	clear_error();
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "matmul: dtype %d not provided (KG_F64, KG_F64_FMA, KG_F32)", dt);
	if (nx < 0 || ny < 0 || ns < 0) return fail(KG_EINVAL, "matmul: negative size");
	if ((size_t)nx * ns == 0) return KG_OK;
	if (!C || (ny > 0 && (!A || !B))) return fail(KG_EINVAL, "matmul: null array");
	const size_t es = dtype_size(dt), cb = (size_t)nx * ns * es;
	if (ny > 0 && (overlaps(C, cb, A, (size_t)nx * ny * es) || overlaps(C, cb, B, (size_t)ny * ns * es)))
		return fail(KG_EINVAL, "matmul: output array overlaps an input");
	if ((nx + kMmTI - 1) / kMmTI > 2147483647 || (ns + kMmTJ - 1) / kMmTJ > 65535)
		return fail(KG_EINVAL, "matmul: ns beyond the supported size");
	return fail_cuda(by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		dim3 grid((nx + kMmTI - 1) / kMmTI, (ns + kMmTJ - 1) / kMmTJ);
		matmul_kernel<N, S><<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(nx, ny, ns, (const S*)A,
			(const S*)B, (S*)C);
		return cudaGetLastError();
	}), "matmul");
}

kg_status kg_sincos(kg_dtype dt, int nx, int ny, int ns, const void* x, const void* y, void* xy, kg_stream_t stream)
{
	clear_error();
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "sincos: dtype %d not provided (KG_F64, KG_F64_FMA, KG_F32)", dt);
	if (nx < 0 || ny < 0 || ns < 0) return fail(KG_EINVAL, "sincos: negative size");
	const size_t n = (size_t)nx * ny * ns, bytes = n * dtype_size(dt);
	if (n == 0) return KG_OK;
	if (!x || !y || !xy) return fail(KG_EINVAL, "sincos: null array");
	if (overlaps(xy, bytes, x, bytes) || overlaps(xy, bytes, y, bytes))
		return fail(KG_EINVAL, "sincos: output array overlaps an input");
	return fail_cuda(by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		cudaStream_t st = (cudaStream_t)stream;
		size_t done = 0;
		if constexpr (std::is_same<S, float>::value) {
			if (((uintptr_t)x | (uintptr_t)y | (uintptr_t)xy) % 16 == 0 && n >= 4) {
				const size_t nv = n / 4;
				sincos_vec_kernel<<<grid_for(nv, 256), 256, 0, st>>>(nv, (const float4*)x, (const float4*)y, (float4*)xy);
				done = nv * 4;
			}
		}
		if (done < n)
			sincos_kernel<N, S><<<grid_for(n - done, 256), 256, 0, st>>>(n - done, (const S*)x + done,
				(const S*)y + done, (S*)xy + done);
		return cudaGetLastError();
	}), "sincos");
}

kg_status kg_whispering(kg_dtype dt, int nx, int ny, double mu, double epsilon, void* e, const void* h0,
	void* h1, const void* u_em0, void* u_em1, const void* ca, const void* cb, const void* da, const void* db,
	kg_stream_t stream)
{
	clear_error();
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "whispering: dtype %d not provided (KG_F64, KG_F64_FMA, KG_F32)", dt);
	if (nx < 0 || ny < 0) return fail(KG_EINVAL, "whispering: negative size");
	const size_t n = (size_t)nx * ny, es = dtype_size(dt), bytes = n * es;
	if (n == 0) return KG_OK;
	const void* in[] = {h0, u_em0, ca, cb, da, db};
	if (!e || !h1 || !u_em1) return fail(KG_EINVAL, "whispering: null array");
	for (const void* p : in)
		if (!p) return fail(KG_EINVAL, "whispering: null array");
	// h1 and u_em1 must not overlap anything; e (two planes) only itself.
	const void* outs[] = {h1, u_em1};
	for (const void* o : outs) {
		if (overlaps(o, bytes, e, 2 * bytes)) return fail(KG_EINVAL, "whispering: output array overlaps e");
		for (const void* p : in)
			if (overlaps(o, bytes, p, bytes)) return fail(KG_EINVAL, "whispering: output array overlaps an input");
	}
	if (overlaps(h1, bytes, u_em1, bytes)) return fail(KG_EINVAL, "whispering: h1 overlaps u_em1");
	for (const void* p : in)
		if (overlaps(e, 2 * bytes, p, bytes)) return fail(KG_EINVAL, "whispering: e overlaps an input");
	if (nx < 3 || ny < 3) return KG_OK;
	return fail_cuda(by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		cudaStream_t st = (cudaStream_t)stream;
		dim3 grid((nx - 2 + 31) / 32, (unsigned)min((ny - 2 + 7) / 8, 65535));
		whispering_e_kernel<N, S><<<grid, dim3(32, 8), 0, st>>>(nx, ny, (S*)e, (const S*)h0, (const S*)ca, (const S*)cb);
		whispering_h_kernel<N, S><<<grid, dim3(32, 8), 0, st>>>(nx, ny, N(mu), N(epsilon), (const S*)e,
			(const S*)h0, (S*)h1, (const S*)u_em0, (S*)u_em1, (const S*)ca, (const S*)cb, (const S*)da, (const S*)db);
		return cudaGetLastError();
	}), "whispering");
}

kg_status kg_extra_regcount(const char* name, kg_dtype dt, int* nregs)
{
	clear_error();
	if (!name || !nregs) return fail(KG_EINVAL, "kg_extra_regcount: bad argument");
	if (!extra_type(dt)) return fail(KG_ENOTSUP, "kg_extra_regcount: dtype %d not provided", dt);
	const void* f = nullptr;
	by_type(dt, [&](auto nv, auto sv) {
		using N = decltype(nv);
		using S = decltype(sv);
		// the kernels that run on 16-byte aligned arrays
		using V = typename std::conditional<std::is_same<S, double>::value, double2, float4>::type;
		constexpr bool f32 = std::is_same<S, float>::value;
		if (!strcmp(name, "vecadd")) f = (const void*)vecadd_vec_kernel<S, V>;
		else if (!strcmp(name, "matvec")) {
			if constexpr (f32) f = (const void*)matvec_ring_kernel<N>;
			else f = (const void*)matvec_kernel<N, S>;
		} else if (!strcmp(name, "matmul")) f = (const void*)matmul_kernel<N, S>;
		else if (!strcmp(name, "sincos")) {
			if constexpr (f32) f = (const void*)sincos_vec_kernel;
			else f = (const void*)sincos_kernel<N, S>;
		}
		else if (!strcmp(name, "whispering")) f = (const void*)whispering_h_kernel<N, S>;
		return cudaSuccess;
	});
	if (!f) return fail(KG_EINVAL, "kg_extra_regcount: unknown test %s", name);
	cudaFuncAttributes a;
	kg_status s = fail_cuda(cudaFuncGetAttributes(&a, f), "kg_extra_regcount");
	if (s == KG_OK) *nregs = a.numRegs;
	return s;
}

}  // extern "C"
