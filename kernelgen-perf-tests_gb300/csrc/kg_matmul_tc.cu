// kg_matmul_tc.cu -- the suite's dense matmul on the 5th-generation tensor
// cores (tcgen05), FP32 arrays.
//
// matmul/matmul.F90:56-68 accumulates C(i,j) += A(i,k) B(k,j) (column-major:
// A(i,k) at A[i + nx k], B(k,j) at B[k + ny j], C(i,j) at C[i + nx j]).  As a
// GEMM: D (M = i, N = j) = sum over K = k of A(i,k) B(k,j), then C += D.
//
// Precision.  A kind::tf32 MMA reads 19 of an FP32 operand's 32 bits.  Each
// operand x is split x = hi + lo (hi: x rounded to TF32; lo = x - hi,
// exact), and D = lo_A hi_B + hi_A lo_B + hi_A hi_B is accumulated in FP32 in
// tensor memory; the dropped lo_A lo_B term is 2^-22 of the product.  The
// result is FP32-accurate but not the k-ordered FP32 sum of kg_matmul, so
// not bit for bit.
//
// Layout.  A pre-pass writes the splits K-major with rows padded to kp (a
// multiple of 32, zeros past ny): At_hi / At_lo [nx][kp] (A transposed) and
// B_hi / B_lo [ns][kp] (B as stored, padded).  A CTA of 4 warps owns a
// 128 x TN tile of C (TN = 128).  Warp 0 lane 0 copies 128 x 32 and
// TN x 32 boxes (128 bytes of K per row, 128-byte swizzle) of the four splits
// into a ring of stages by TMA; warp 1 lane 0 issues the MMAs (M 128, N TN,
// K 8: four K steps a box, three products each, both operands K-major) and
// commits each stage back to the producer and, after the last, to the
// epilogue; warp 2 allocates the TN tensor-memory columns of the accumulator
// (row i of D in lane i).  All four
// warps then read their 32 rows of D (tcgen05.ld 32x32b) and add them to C:
// at a fixed column, consecutive lanes hold consecutive i, so the stores
// are coalesced.
//
// Waits are bounded (the TMA engine's limit); a wait that gives up raises
// the error flag kg_engine_status reports; the CTA still waits (bounded) for
// its copies and its MMAs and releases its tensor memory before it exits.
#include <cuda.h>

#include <algorithm>
#include <atomic>

#include "kg_internal.h"
#include "kg_tma.cuh"

namespace kg {

constexpr int kTcM = 128;   // rows of C a CTA owns
#ifndef KG_TC_GROUP
#define KG_TC_GROUP 8
#endif

// Tiles of 128 x TN.  TN = 128: K stages of 32 (rows of 128 bytes, 128-byte
// swizzle), 3 stages of 64 KB.  TN = 256: K stages of 16 (rows of 64 bytes,
// 64-byte swizzle), 4 stages of 48 KB -- a third fewer operand bytes a flop
// for the tensor cores to read from shared memory, with the stages in flight
// of the narrower tile.  Measured on GB300 (ms, 128 / 256 columns): 2048^3
// 0.229 / 0.214, 4096^3 1.058 / 1.083, 8192^3 5.74 / 5.29; 256 columns with
// K stages of 32 (2 stages of 96 KB): 4096^3 1.18, 8192^3 6.40; 128 columns
// with K stages of 16 (6 stages of 32 KB): 1.19, 6.74.
template <int TN> struct TcShape {
	static constexpr int N = TN;
	static constexpr int K = TN == 128 ? 32 : 16;            // K elements a stage
	static constexpr int RowBytes = K * 4;                    // = the swizzle span
	static constexpr int BoxA = kTcM * K * 4;                 // bytes of one split of A
	static constexpr int BoxB = TN * K * 4;
	static constexpr int Stage = 2 * BoxA + 2 * BoxB;         // A_hi, A_lo, B_hi, B_lo
	static constexpr int Stages = TN == 128 ? 3 : 4;
	static constexpr int Smem = Stages * Stage + 256 + 1024;  // + barriers, + alignment slack
};

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
	asm volatile(
		"cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
		" [%0], [%1, {%2, %3}], [%4];"
		::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
		: "memory");
}

// Shared-memory matrix descriptor of a K-major box written by TMA with the
// 128-byte swizzle: rows of 128 bytes, groups of 8 rows 1024 bytes apart
// (start address, leading offset unused, stride offset, descriptor version,
// swizzle mode).  A K step inside the 128-byte row adds its byte offset to
// the start address; the swizzle applies to the full address.
template <int ROW_BYTES>
__device__ __forceinline__ uint64_t umma_desc_swizzled(uint32_t saddr)
{
	static_assert(ROW_BYTES == 128 || ROW_BYTES == 64, "128- or 64-byte swizzle");
	uint64_t d = (uint64_t)((saddr >> 4) & 0x3fff);
	d |= (uint64_t)1 << 16;
	d |= (uint64_t)((8 * ROW_BYTES) >> 4) << 32;              // 8 rows
	d |= (uint64_t)1 << 46;
	d |= (uint64_t)(ROW_BYTES == 128 ? 2 : 4) << 61;         // 128- or 64-byte swizzle
	return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5), A and B
// TF32 (bits 7-9, 10-12), both K-major (bits 15, 16 clear), N / 8 (bits
// 17-22), M / 16 (bits 24-28).
constexpr uint32_t umma_idesc_tf32(int m, int n)
{
	return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
		: "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before()
{
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after()
{
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// D (tensor memory) = A B^T + (accum ? D : 0), one elected thread.
__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
		::"r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(accum)
		: "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued so
// far has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
		: "memory");
}
// 32 consecutive columns of the warp's 32 lanes (one row per thread); the
// wait is in the same statement, so no use of the values precedes it.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
	uint32_t r[32];
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
		"%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
		"tcgen05.wait::ld.sync.aligned;"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
		  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
		  "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
		  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
		: "r"(taddr)
		: "memory");
#pragma unroll
	for (int c = 0; c < 32; c++) v[c] = __uint_as_float(r[c]);
}

// x = hi + lo: hi = x rounded to TF32 (10 fraction bits, ties away from
// zero), lo = x - hi (exact in FP32).
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo)
{
	hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
	lo = x - hi;
}

// At_hi / At_lo [i][k] (rows of kp) from A(i,k) = A[i + nx k]: 32 x 32 tiles
// through shared memory (coalesced on both sides).
__global__ void __launch_bounds__(256) tc_split_a(const float* __restrict__ A, float* __restrict__ hi,
	float* __restrict__ lo, int nx, int ny, int kp)
{
	__shared__ float t[32][33];
	const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
	for (int r = threadIdx.y; r < 32; r += blockDim.y) {
		const int i = i0 + threadIdx.x, k = k0 + r;
		t[r][threadIdx.x] = (i < nx && k < ny) ? A[i + (size_t)nx * k] : 0.f;
	}
	__syncthreads();
	for (int r = threadIdx.y; r < 32; r += blockDim.y) {
		const int i = i0 + r, k = k0 + threadIdx.x;
		if (i < nx && k < kp) {
			float h, l;
			tf32_split(t[threadIdx.x][r], h, l);
			hi[(size_t)i * kp + k] = h;
			lo[(size_t)i * kp + k] = l;
		}
	}
}

// B_hi / B_lo [j][k] (rows of kp) from B(k,j) = B[k + ny j].
__global__ void __launch_bounds__(256) tc_split_b(const float* __restrict__ B, float* __restrict__ hi,
	float* __restrict__ lo, int ny, int ns, int kp)
{
	const long long n = (long long)ns * kp;
	for (long long e = blockIdx.x * 256LL + threadIdx.x; e < n; e += (long long)gridDim.x * 256) {
		const int j = (int)(e / kp), k = (int)(e - (long long)j * kp);
		float h, l;
		tf32_split(k < ny ? B[k + (size_t)ny * j] : 0.f, h, l);
		hi[e] = h;
		lo[e] = l;
	}
}

template <int TN>
__global__ void __launch_bounds__(128, 1) matmul_tc_kernel(const __grid_constant__ CUtensorMap m_ahi,
	const __grid_constant__ CUtensorMap m_alo, const __grid_constant__ CUtensorMap m_bhi,
	const __grid_constant__ CUtensorMap m_blo, float* __restrict__ C, int nx, int ns, int nkb, int* err,
	long long wait)
{
	using T = TcShape<TN>;
	constexpr int kTcStages = T::Stages, kTcStage = T::Stage, kTcN = TN;
	extern __shared__ unsigned char tc_smem_raw[];
	// the swizzled boxes want 1024-byte aligned destinations
	unsigned char* sm = tc_smem_raw + ((1024u - (smem_addr(tc_smem_raw) & 1023u)) & 1023u);
	uint64_t* full = reinterpret_cast<uint64_t*>(sm + kTcStages * kTcStage);
	uint64_t* empty = full + kTcStages;
	uint64_t* done = empty + kTcStages;
	uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
	volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);   // the MMA issuer gave up
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	// tile order: groups of KG_TC_GROUP row tiles, each walked column tile
	// by column tile, so that the CTAs resident together share their A and B
	// panels in L2 (the launch order is blockIdx.x fastest).  Measured: 8192^3
	// 5.95 ms in row-major order, 5.79 in groups of 8 or 16; 4096^3 within 0.3 %.
	// The kernel is not bound by DRAM misses but by its stages in flight.
	int mt_i, nt_i;
	{
		const int mt = (int)gridDim.x, nt = (int)gridDim.y;
		const int b = (int)blockIdx.x + mt * (int)blockIdx.y;
		const int per = KG_TC_GROUP * nt, g = b / per;
		const int gm = min(KG_TC_GROUP, mt - g * KG_TC_GROUP), r = b - g * per;
		mt_i = g * KG_TC_GROUP + r % gm;
		nt_i = r / gm;
	}
	const int m0 = mt_i * kTcM, n0 = nt_i * kTcN;

	if (threadIdx.x == 0) {
		for (int s = 0; s < kTcStages; s++) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		mbar_init(done, 1);
		*abort = 0;
		mbar_fence_init();
	}
	if (warp == 2) {
		tmem_alloc(tslot, kTcN);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tslot;

	if (warp == 0 && lane == 0) {
		// ---- producer ----
		tma_prefetch_map(&m_ahi);
		tma_prefetch_map(&m_alo);
		tma_prefetch_map(&m_bhi);
		tma_prefetch_map(&m_blo);
		int issued = 0;
		bool ok = true;
		for (int kb = 0; kb < nkb; kb++) {
			const int s = kb % kTcStages;
			if (kb >= kTcStages && !mbar_wait(&empty[s], ((kb / kTcStages) - 1) & 1, kTmaWaitCycles, abort)) {
				ok = false;
				break;
			}
			unsigned char* st = sm + s * kTcStage;
			mbar_expect_tx(&full[s], kTcStage);
			tma_load_2d(st, &m_ahi, &full[s], kb * T::K, m0);
			tma_load_2d(st + T::BoxA, &m_alo, &full[s], kb * T::K, m0);
			tma_load_2d(st + 2 * T::BoxA, &m_bhi, &full[s], kb * T::K, n0);
			tma_load_2d(st + 2 * T::BoxA + T::BoxB, &m_blo, &full[s], kb * T::K, n0);
			issued = kb + 1;
		}
		if (!ok) {
			atomicExch(err, 1);
			// the copies issued land before the CTA's shared memory goes away
			for (int kb = std::max(0, issued - kTcStages); kb < issued; kb++)
				mbar_wait(&full[kb % kTcStages], (kb / kTcStages) & 1, kTmaWaitCycles);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer ----
		constexpr uint32_t idesc = umma_idesc_tf32(kTcM, kTcN);
		bool ok = true;
		for (int kb = 0; kb < nkb; kb++) {
			const int s = kb % kTcStages;
			if (!mbar_wait(&full[s], (kb / kTcStages) & 1, wait)) {
				ok = false;
				break;
			}
			tc_fence_after();
			const uint32_t base = smem_addr(sm + s * kTcStage);
#pragma unroll
			for (int ks = 0; ks < T::K / 8; ks++) {
				const uint32_t off = ks * 32;   // 8 TF32 values of K
				constexpr int RB = T::RowBytes;
				const uint64_t ahi = umma_desc_swizzled<RB>(base + off), alo = umma_desc_swizzled<RB>(base + T::BoxA + off);
				const uint64_t bhi = umma_desc_swizzled<RB>(base + 2 * T::BoxA + off);
				const uint64_t blo = umma_desc_swizzled<RB>(base + 2 * T::BoxA + T::BoxB + off);
				umma_tf32(tmem, alo, bhi, idesc, (kb | ks) != 0);
				umma_tf32(tmem, ahi, blo, idesc, 1);
				umma_tf32(tmem, ahi, bhi, idesc, 1);
			}
			umma_commit(&empty[s]);   // the stage is free once these MMAs are done
		}
		if (!ok) {
			atomicExch(err, 1);
			*abort = 1;               // the producer stops; the epilogue adds nothing
		}
		umma_commit(done);            // every MMA issued is done: the accumulator is ready
	}
	__syncwarp();

	// ---- epilogue: row i of D is lane i of the tensor memory ----
	const bool got = mbar_wait(done, 0, kTmaWaitCycles) && !*abort;
	tc_fence_after();
	if (__all_sync(0xffffffffu, got)) {
		const int i = m0 + warp * 32 + lane;
#pragma unroll 1
		for (int cb = 0; cb < kTcN / 32; cb++) {
			float v[32];
			tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), v);
			if (i < nx) {
#pragma unroll
				for (int c = 0; c < 32; c++) {
					const int j = n0 + cb * 32 + c;
					if (j < ns) C[i + (size_t)nx * j] += v[c];
				}
			}
		}
	} else if (lane == 0) {
		atomicExch(err, 1);
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 2) tmem_dealloc(tmem, kTcN);
}

static bool tc_overlaps(const void* a, size_t na, const void* b, size_t nb)
{
	const char *pa = (const char*)a, *pb = (const char*)b;
	return pa < pb + nb && pb < pa + na;
}

}  // namespace kg

using namespace kg;

extern "C" kg_status kg_matmul_tc(int nx, int ny, int ns, const float* A, const float* B, float* C,
	kg_stream_t stream)
{
	clear_error();
	if (nx < 0 || ny < 0 || ns < 0) return fail(KG_EINVAL, "matmul_tc: negative size");
	if (nx == 0 || ns == 0) return KG_OK;
	if (!C || (ny > 0 && (!A || !B))) return fail(KG_EINVAL, "matmul_tc: null array");
	const size_t cb = (size_t)nx * ns * sizeof(float);
	if (ny > 0 && (tc_overlaps(C, cb, A, (size_t)nx * ny * sizeof(float)) ||
	               tc_overlaps(C, cb, B, (size_t)ny * ns * sizeof(float))))
		return fail(KG_EINVAL, "matmul_tc: output array overlaps an input");
	if (ny == 0) return KG_OK;   // C += nothing
	if ((ns + 127) / 128 > 65535) return fail(KG_EINVAL, "matmul_tc: ns beyond the supported size");
	if ((ny + 31) / 32 > 65535) return fail(KG_EINVAL, "matmul_tc: ny beyond the supported size");
	int dev = 0, major = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
	if (major != 10) return fail(KG_ENOTSUP, "matmul_tc: needs a Blackwell (sm_10x) GPU");
	cudaStream_t st = (cudaStream_t)stream;
	const int kp = (ny + 31) / 32 * 32;   // a multiple of both shapes' K stage
	const size_t na = (size_t)nx * kp, nb = (size_t)ns * kp;
	float* ws = nullptr;
	// from the library's pool, whose memory stays cached between calls (the
	// device's default pool hands it back at every synchronisation)
	cudaMemPool_t pool;
	kg_status s = fail_cuda(program_pool(&pool), "matmul_tc: memory pool");
	if (s != KG_OK) return s;
	s = fail_cuda(cudaMallocFromPoolAsync((void**)&ws, sizeof(float) * 2 * (na + nb), pool, st), "matmul_tc: workspace");
	if (s != KG_OK) return s;
	float *ahi = ws, *alo = ws + na, *bhi = ws + 2 * na, *blo = ws + 2 * na + nb;
	tc_split_a<<<dim3((unsigned)((nx + 31) / 32), (unsigned)((kp + 31) / 32)), dim3(32, 8), 0, st>>>(A, ahi, alo, nx, ny, kp);
	const long long nbl = std::min<long long>(((long long)nb + 255) / 256, 152 * 16);
	tc_split_b<<<(unsigned)nbl, 256, 0, st>>>(B, bhi, blo, ny, ns, kp);
	// 256-column tiles where their waves cost less than the 128-column ones'
	// (a 256-column tile takes about 1.83 times a 128-column tile's time)
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	sms = sms > 0 ? sms : 1;
	const long long mt = (nx + kTcM - 1) / kTcM;
	const long long w128 = (mt * ((ns + 127) / 128) + sms - 1) / sms, w256 = (mt * ((ns + 255) / 256) + sms - 1) / sms;
	const bool wide = (ns + 255) / 256 <= 65535 && 1.83 * (double)w256 < (double)w128;
	int* err = tma_error_flag();
	cudaError_t e = err ? cudaSuccess : cudaErrorInvalidValue;
	if (e == cudaSuccess) {
		auto launch = [&](auto shape) {
			using T = decltype(shape);
			CUtensorMap maps[4];
			const float* bases[4] = {ahi, alo, bhi, blo};
			const int rows[4] = {nx, nx, ns, ns};
			for (int q = 0; q < 4; q++) {
				cudaError_t r = tma_encode_2d_swizzled(&maps[q], bases[q], (uint64_t)kp, (uint64_t)rows[q], T::K,
					q < 2 ? kTcM : T::N, T::RowBytes);
				if (r != cudaSuccess) return r;
			}
			// the shared-memory opt-in, once per device
			static std::atomic<bool> set[64];
			if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
			if (!set[dev].load(std::memory_order_acquire)) {
				cudaError_t r = cudaFuncSetAttribute(matmul_tc_kernel<T::N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
					T::Smem);
				if (r != cudaSuccess) return r;
				set[dev].store(true, std::memory_order_release);
			}
			dim3 grid((unsigned)((nx + kTcM - 1) / kTcM), (unsigned)((ns + T::N - 1) / T::N));
			matmul_tc_kernel<T::N><<<grid, 128, T::Smem, st>>>(maps[0], maps[1], maps[2], maps[3], C, nx, ns, kp / T::K,
				err, tma_wait_limit());
			return cudaGetLastError();
		};
		e = wide ? launch(TcShape<256>{}) : launch(TcShape<128>{});
	}
	cudaFreeAsync(ws, st);
	return fail_cuda(e, "matmul_tc");
}
