// kg_tma.cuh -- the TMA engine: halo tiles moved by the tensor memory
// accelerator into a ring of shared-memory planes, streaming along z.
//
// A CTA of TX x TY threads owns a BX x BY tile of (i, j) columns (BX = TX,
// BY = TY * PY: each thread evaluates PY points TY rows apart) and walks a
// run of planes along z.  For every input the CTA keeps a ring of R planes
// of its halo tile in shared memory.  A producer warp issues the tiled bulk
// copies (cp.async.bulk.tensor, one box per input and plane) up to L steps
// ahead of the plane being evaluated; each step's copies complete on one
// mbarrier, which the compute warps wait on before they read the step's
// planes, and each compute warp reports on a second mbarrier when it is done
// with a step, which frees the oldest plane's slot for the producer.
// The points then read their neighbours from shared memory, and the values of
// their own column at other planes (the dz neighbours) from registers, which
// shift by one plane per step (2.5D streaming): a value crosses from global
// memory about once per sweep, and each thread issues no global loads.
//
// Box geometry: a copy must start at an x that is a multiple of 16 bytes, so
// the tile origin xt is a multiple of BX and each box starts A = 16 / sizeof
// element columns to the left of it (A >= every op's left halo) and spans a
// multiple of A columns.  Boxes may reach outside the array (the copy fills
// zeros there); no point reads those values, because every neighbour of a
// domain point lies inside the array.  Inputs read only at the point itself
// are not staged: each thread loads them from global memory.
//
// Waits are bounded.  A compute warp waits for a step's copies at most
// `wait` clock cycles (a kernel argument: kTmaWaitCycles unless the host set
// another limit, kg_set_tma_wait_limit; 0 = give up unless the copies have
// already landed at the first look); when that runs out it records an error
// in a device flag (read back by kg_engine_status), raises the CTA's abort
// flag in shared memory and returns.  The producer waits for the compute
// warps at most kTmaWaitCycles and stops issuing as soon as the abort flag is
// up; either way it then waits, again at most kTmaWaitCycles, for every copy
// it issued to land before the CTA exits.
#pragma once

#include <cuda.h>
#include <cstdint>

#include "kg_engine.cuh"
#include "kg_staged.cuh"

namespace kg {

constexpr long long kTmaWaitCycles = 1ll << 31;   // ~1 s at 2 GHz

// ---- PTX wrappers ----------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t done;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(done)
		: "r"(smem_addr(bar)), "r"(parity)
		: "memory");
	return done != 0;
}

// Whether the phase with the given parity has completed, without waiting.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t done;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(done)
		: "r"(smem_addr(bar)), "r"(parity)
		: "memory");
	return done != 0;
}

// Wait for the phase with the given parity to complete, for at most `limit`
// clock cycles (0: only look once), and no longer once *abort (if given) is
// set; false if it did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit,
	const volatile int* abort = nullptr)
{
	if (limit <= 0) return mbar_test_wait(bar, parity);
	if (mbar_try_wait(bar, parity)) return true;
	const long long t0 = clock64();
	while (!mbar_try_wait(bar, parity)) {
		if (abort && *abort) return false;
		if (clock64() - t0 > limit) return false;
	}
	return true;
}

__device__ __forceinline__ void fence_proxy_async()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map)
{
	asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z)
{
	asm volatile(
		"cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
		" [%0], [%1, {%2, %3, %4}], [%5];"
		::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
		: "memory");
}

// ---- geometry -----------------------------------------------------------

constexpr int round_up(int n, int m) { return (n + m - 1) / m * m; }

// One tensor map per input slot.
struct TMaps {
	CUtensorMap m[6];
};

// Build-time choices of the ring layout (measured, see TmaDepth):
// KG_TMA_POW2 rings of a power-of-two number of planes (slot = plane & mask)
// rather than exactly NZ + L planes (slot = plane % R); KG_TMA_CENTER
// stages inputs read only at the point itself as well (else each thread
// loads them from global memory when it evaluates the point).
#ifndef KG_TMA_POW2
#define KG_TMA_POW2 0
#endif
#ifndef KG_TMA_CENTER
#define KG_TMA_CENTER 1
#endif

constexpr int pow2_at_least(int n) { int p = 1; while (p < n) p *= 2; return p; }

template <class Op, class S, int BX, int BY, int L> struct TGeo {
	static constexpr int kBY = BY;
	static constexpr int ES = (int)sizeof(S);
	static constexpr int A = 16 / ES;                       // x alignment, elements
	static constexpr int NIN = Op::slots().nin;
	static constexpr bool staged(int q) { return KG_TMA_CENTER || !Op::halo(q).center(); }
	static constexpr int XL(int q) { return Op::halo(q).x0 > 0 ? A : 0; }
	static constexpr int W(int q) { return round_up(BX + XL(q) + Op::halo(q).x1, A); }
	static constexpr int H(int q) { return BY + Op::halo(q).y0 + Op::halo(q).y1; }
	static constexpr int NZ(int q) { return Op::halo(q).z0 + Op::halo(q).z1 + 1; }
	static constexpr int R(int q) {
		return !staged(q) ? 0 : KG_TMA_POW2 ? pow2_at_least(NZ(q) + L) : NZ(q) + L;
	}
	static __device__ __forceinline__ int slot(int q, int plane) {
		if constexpr (KG_TMA_POW2) return plane & (R(q) - 1);
		else return (int)((unsigned)plane % (unsigned)R(q));
	}
	// Slot of plane k + dz from the slot v0 of plane k (|dz| < R).
	static __device__ __forceinline__ int step_slot(int q, int v0, int dz) {
		const int v = v0 + dz;
		if constexpr (KG_TMA_POW2) return v & (R(q) - 1);
		else return dz > 0 ? (v >= R(q) ? v - R(q) : v) : dz < 0 ? (v < 0 ? v + R(q) : v) : v;
	}
	static constexpr int box_bytes(int q) { return staged(q) ? W(q) * H(q) * ES : 0; }
	static constexpr int PS(int q) { return round_up(box_bytes(q), 128); }   // plane stride, bytes
	static constexpr int NB = L + 1;                                         // steps in flight
	static constexpr int kBar = 128;                          // 2 x NB mbarriers, then the abort flag
	static constexpr int kAbort = kBar - 8;
	static constexpr int offset(int q) { int o = kBar; for (int r = 0; r < q; r++) o += R(r) * PS(r); return o; }
	static constexpr int total() { return offset(NIN); }
	static constexpr int step_bytes() { int b = 0; for (int q = 0; q < NIN; q++) b += box_bytes(q); return b; }
	static constexpr int window_bytes() { int b = 0; for (int q = 0; q < NIN; q++) b += NZ(q) * box_bytes(q); return b; }
	static constexpr int NZMAX() { int m = 1; for (int q = 0; q < NIN; q++) m = NZ(q) > m ? NZ(q) : m; return m; }
	static constexpr bool fits() {
		for (int q = 0; q < NIN; q++)
			if (Op::halo(q).x0 > A || W(q) > 256 || H(q) > 256) return false;
		return L >= 1 && 2 * NB * 8 <= kAbort && step_bytes() > 0;
	}
};

// ---- accessor -----------------------------------------------------------

template <class Op, class N, class S, class G, int ZMAX> struct TAcc {
	using Rp = Rep<N, S>;
	using M = typename Rp::M;
	const unsigned char* sm;       // shared memory base
	const int* toff;               // per input: this point's byte offset inside a plane
	const int* sb;                 // per input: ring slot of plane k
	const M (*col)[ZMAX];          // per input: own column, planes k - z0 .. k + z1
	const S* const* in;
	long long c, sy, sz;
	__device__ __forceinline__ N operator()(int q, int dx, int dy, int dz) const {
		const Halo h = Op::halo(q);
		if (!G::staged(q)) return Conv<N, S>::ld(in[q] + c + dx + dy * sy + dz * sz);
		if (dx == 0 && dy == 0 && G::NZ(q) > 1) return Rp::get(col[q][dz + h.z0]);
		const int slot = G::step_slot(q, sb[q], dz);
		const int off = G::offset(q) + slot * G::PS(q) + toff[q] + (dy * G::W(q) + dx) * G::ES;
		return Rp::get(Rp::stage(*reinterpret_cast<const S*>(sm + off)));
	}
	__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const {
		return __ldg(in[q] + c + dx + dy * sy + dz * sz);
	}
};

// ---- kernel -------------------------------------------------------------

// BAND: a 2D op walked in bands of BY rows (step k = band k, rows yt + k BY
// onward; the arrays' maps are rank 3 with one plane).
template <class Op, class S, class G, bool BAND = false>
__device__ __forceinline__ void tma_issue(const TMaps& maps, unsigned char* sm, uint64_t* bar,
	int xt, int yt, int k, bool window)
{
	mbar_expect_tx(bar, window ? G::window_bytes() : G::step_bytes());
#pragma unroll
	for (int q = 0; q < G::NIN; q++) {
		if (!G::staged(q)) continue;
		const Halo h = Op::halo(q);
		const int x = xt - G::XL(q), y = yt - h.y0;
		const int p1 = k + h.z1;
		for (int p = window ? k - h.z0 : p1; p <= p1; p++) {
			if constexpr (BAND)
				tma_load_3d(sm + G::offset(q) + G::slot(q, p) * G::PS(q), &maps.m[q], bar, x, y + p * G::kBY, 0);
			else
				tma_load_3d(sm + G::offset(q) + G::slot(q, p) * G::PS(q), &maps.m[q], bar, x, y, p);
		}
	}
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// The producer of a TMA-engine CTA (one thread): issues each step's copies
// onto full[step % NB] once the step NB earlier is done (done[]), so up to
// NB - 1 = L steps of copies are in flight ahead of the compute warps; each
// run along z starts with its whole window of planes.  Waits for the compute
// warps are bounded by kTmaWaitCycles and end early once a compute warp has
// raised the CTA's abort flag; the thread then stops issuing and waits for
// every copy it issued to land before it returns.  Normally it returns after
// the compute warps are done with the last step.
// The runs of one CTA of the TMA engine: planes kb, kb + gridDim.z kc, ...
// (up to kc each) of its tile (xt, yt).
struct ZRuns {
	static constexpr bool kBand = false;
	int xt, yt, kb, kend, kc;
	__device__ __forceinline__ bool next(int& x, int& y, int& k0, int& n) {
		if (kb >= kend) return false;
		x = xt;
		y = yt;
		k0 = kb;
		n = min(kc, kend - kb);
		kb += gridDim.z * kc;
		return true;
	}
};

// The same runs over the bands of BY rows of a 2D op (band k: rows
// yt + k BY ...; the producer's copies then start at row yt + k BY - y0).
struct BandRuns : ZRuns {
	static constexpr bool kBand = true;
};

template <class Op, class S, class G, class Runs>
__device__ __forceinline__ void tma_produce(const TMaps& maps, unsigned char* sm, uint64_t* full, uint64_t* done,
	const volatile int* abort, Runs runs, int* err)
{
	constexpr int NB = G::NB, L = G::NB - 1;
#pragma unroll
	for (int q = 0; q < G::NIN; q++)
		if (G::staged(q)) tma_prefetch_map(&maps.m[q]);
	uint32_t g = 0, issued = 0;   // steps issued so far
	bool ok = true;
	int xt, yt, kb, nsteps;
	while (ok && runs.next(xt, yt, kb, nsteps)) {
		// a new run's window may reuse any slot: wait for the previous run
		if (g > 0) ok = mbar_wait(&done[(g - 1) % NB], ((g - 1) / NB) & 1, kTmaWaitCycles, abort);
		for (int t = 0; t < nsteps && ok; t++) {
			const uint32_t gt = g + t;
			if (t >= L + 1) ok = mbar_wait(&done[(gt - L - 1) % NB], ((gt - L - 1) / NB) & 1, kTmaWaitCycles, abort);
			if (!ok) break;
			fence_proxy_async();
			tma_issue<Op, S, G, Runs::kBand>(maps, sm, &full[gt % NB], xt, yt, kb + t, t == 0);
			issued = gt + 1;
		}
		g += nsteps;
	}
	// stay until the compute warps are done with the last step, or gave up
	if (ok && issued > 0) ok = mbar_wait(&done[(issued - 1) % NB], ((issued - 1) / NB) & 1, kTmaWaitCycles, abort);
	if (!ok) {
		atomicExch(err, 1);
		// Every step before the last NB issued is done (the copies of step
		// w + NB were issued only after step w was done): the copies still
		// in flight belong to those NB steps, and they land before the
		// CTA's shared memory goes away.
		for (uint32_t w = issued > NB ? issued - NB : 0; w < issued; w++)
			mbar_wait(&full[w % NB], (w / NB) & 1, kTmaWaitCycles);
	}
}

// TX*TY compute threads and one producer warp.  Step t of a run (plane kb+t)
// has two mbarriers: full[t % NB] completes when the step's copies have
// landed, done[t % NB] when every compute warp has evaluated the step.  The
// producer issues step t once step t-L-1 is done: then the planes step t
// brings in replace planes no later step needs, since each ring holds L
// planes more than a step's window.  So up to L steps of copies are in flight
// ahead of the compute warps, which never wait for each other.
template <class Op, class N, class S, int TX, int TY, int PY, int L>
__global__ void __launch_bounds__(TX * TY + 32) tma_kernel(Op op, Ptrs<S> p, const __grid_constant__ TMaps maps,
	int nx, int ny, int ns, int kc, int yt0, int* err, long long wait)
{
	constexpr int BX = TX, BY = TY * PY, NC = TX * TY;
	using G = TGeo<Op, S, BX, BY, L>;
	constexpr int NB = G::NB;
	using Rp = Rep<N, S>;
	using M = typename Rp::M;
	constexpr Slots sl = Op::slots();
	constexpr int ZMAX = 5;
	static_assert(G::fits(), "tile does not fit the TMA engine");
	static_assert(G::NZMAX() <= ZMAX, "column registers hold at most ZMAX planes");
	static_assert(NC % 32 == 0, "whole compute warps");
	extern __shared__ __align__(128) unsigned char sm[];
	uint64_t* full = reinterpret_cast<uint64_t*>(sm);
	uint64_t* done = full + NB;
	volatile int* abort = reinterpret_cast<volatile int*>(sm + G::kAbort);

	const int tid = threadIdx.x;
	const int xt = blockIdx.x * BX, yt = Op::LY + (yt0 + (int)blockIdx.y) * BY;
	const int kend = ns - Op::HZ;

	if (tid == 0) {
		for (int b = 0; b < NB; b++) {
			mbar_init(&full[b], 1);
			mbar_init(&done[b], NC / 32);
		}
		*abort = 0;
		mbar_fence_init();
	}
	__syncthreads();

	if (tid >= NC) {
		if (tid == NC)
			tma_produce<Op, S, G>(maps, sm, full, done, abort, ZRuns{xt, yt, Op::LZ + (int)blockIdx.z * kc, kend, kc}, err);
		return;
	}

	// ---- compute warps ----
	const int tx = tid % TX, ty = tid / TX;
	const int i = xt + tx;
	const long long sy = nx, sz = (long long)nx * ny;
	// per point of this thread: byte offset inside a plane of each input, and
	// whether it lies in the update domain (both fixed for the whole kernel)
	int toff[PY][6];
	bool pt_ok[PY];
#pragma unroll
	for (int r = 0; r < PY; r++) {
		const int j = yt + ty + r * TY;
		pt_ok[r] = i >= Op::LX && i < nx - Op::HX && j < ny - Op::HY;
#pragma unroll
		for (int q = 0; q < G::NIN; q++)
			toff[r][q] = ((ty + r * TY + Op::halo(q).y0) * G::W(q) + tx + G::XL(q)) * G::ES;
	}
	uint32_t g = 0;
	for (int kb = Op::LZ + blockIdx.z * kc; kb < kend; kb += gridDim.z * kc) {
		const int nsteps = min(kc, kend - kb);
		M col[PY][6][ZMAX];
		int sb[6];
		// this thread's outputs at plane kb; each step moves them one plane on
		S* outp[PY][3];
#pragma unroll
		for (int r = 0; r < PY; r++)
#pragma unroll
			for (int q = 0; q < sl.nout; q++)
				outp[r][q] = p.out[q] + (i + sy * (yt + ty + r * TY) + sz * kb);
		for (int s = 0; s < nsteps; s++) {
			const int k = kb + s;
			const uint32_t gs = g + s;
#pragma unroll
			for (int q = 0; q < G::NIN; q++)
				if (G::staged(q)) sb[q] = s == 0 ? G::slot(q, k) : G::step_slot(q, sb[q], 1);
			const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[gs % NB], (gs / NB) & 1, wait, abort));
			if (!ok) {
				if ((tid & 31) == 0) {
					*abort = 1;
					atomicExch(err, 1);
				}
				return;
			}
#pragma unroll
			for (int r = 0; r < PY; r++) {
#pragma unroll
				for (int q = 0; q < G::NIN; q++) {
					const Halo h = Op::halo(q);
					// own column: shift by one plane and read the newest (all of
					// them at the first step of a run)
					const int nz = G::NZ(q);
					if (G::staged(q) && nz > 1) {
						const unsigned char* ring = sm + G::offset(q) + toff[r][q];
						if (s == 0) {
#pragma unroll
							for (int m = 0; m < ZMAX; m++)
								if (m < nz)
									col[r][q][m] = Rp::stage(*reinterpret_cast<const S*>(
										ring + G::slot(q, k - h.z0 + m) * G::PS(q)));
						} else {
#pragma unroll
							for (int m = 0; m + 1 < ZMAX; m++)
								if (m + 1 < nz) col[r][q][m] = col[r][q][m + 1];
							col[r][q][nz - 1] = Rp::stage(*reinterpret_cast<const S*>(
								ring + G::step_slot(q, sb[q], h.z1) * G::PS(q)));
						}
					}
				}
				if (pt_ok[r]) {
					const long long c = i + sy * (yt + ty + r * TY) + sz * k;
					TAcc<Op, N, S, G, ZMAX> at{sm, toff[r], sb, col[r], p.in, c, sy, sz};
					N o[3];
					op.point(at, o);
#pragma unroll
					for (int q = 0; q < sl.nout; q++) *outp[r][q] = Conv<N, S>::to(o[q]);
				}
#pragma unroll
				for (int q = 0; q < sl.nout; q++) outp[r][q] += sz;
			}
			// this warp is done with the step's planes
			__syncwarp();
			if ((tid & 31) == 0) mbar_arrive(&done[gs % NB]);
		}
		g += nsteps;
	}
}

}  // namespace kg

// ---- host side ------------------------------------------------------------

namespace kg {

// kg_tma.cu: tensor-map encoding through the driver entry point, and the
// device flag the kernels raise when a wait gives up.
cudaError_t tma_encode_3d(CUtensorMap* map, CUtensorMapDataType type, const void* base, uint64_t nx,
	uint64_t ny, uint64_t ns, int elem_bytes, int box_w, int box_h);
cudaError_t tma_encode_2d_swizzled(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, int box_inner,
	int box_outer, int swizzle_bytes);
int* tma_error_flag();
// Clock cycles a compute warp waits for its copies (kg_set_tma_wait_limit).
long long tma_wait_limit();

// Planes per run along z: z is split into runs so that the CTAs fill whole
// waves of per_sm x sms, weighing each run's extra window planes (weight w
// each) and a fixed cost per run.
inline int tma_run_length(int per_sm, int sms, long long tiles, int dz, int nzmax, double w = 1.0, double fixed = 2.0)
{
	const long long slots = (long long)per_sm * sms;
	int nz = 1;
	double best = 1e300;
	for (int c = 1; c <= min(dz, 256); c++) {
		const long long ctas = tiles * c;
		const double waves = (double)((ctas + slots - 1) / slots);
		const int run = (dz + c - 1) / c;
		const double cost = waves * (run + w * (nzmax - 1) + fixed);
		if (cost < best * 0.999) { best = cost; nz = c; }
	}
	return (dz + nz - 1) / nz;
}

template <class S> struct TmaType;
template <> struct TmaType<float> { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; };
template <> struct TmaType<double> { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_FLOAT64; };
template <> struct TmaType<__nv_bfloat16> { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16; };
template <> struct TmaType<__half> { static constexpr CUtensorMapDataType v = CU_TENSOR_MAP_DATA_TYPE_FLOAT16; };

// Tile and pipeline depth per op: 3D tiles of 32 x 8 threads (2 points per
// thread for 4- and 2-byte elements where the rings allow it), 2D ops as rows
// of 128 points; L (steps of copies in flight) the largest, up to 6, whose
// rings fit the shared-memory budget.
// Shared memory per CTA for the rings: 40 KB keeps 5 CTAs of 288 threads per
// SM.  Measured on GB300 (FP32, 512x256x256, Gpts/s at 31 / 40 / 48 KB):
// laplacian 494 / 493 / 493, divergence 287 / 382 / 378, uxx1 215 / 213 /
// 205, lapgsrb 271 / 268 / 268; wave13pt 282 / 277 / 277 (direct engine 341).
#ifndef KG_TMA_BUDGET
#define KG_TMA_BUDGET (40 * 1024)
#endif
#ifndef KG_TMA_MIN_L2
#define KG_TMA_MIN_L2 4
#endif
template <class K, class S, int TX, int TY, int PY> struct TmaDepth {
	static constexpr int BX = TX, BY = TY * PY;
	template <int L> static constexpr int bytes() { return TGeo<K, S, BX, BY, L>::total(); }
	static constexpr int kBudget = KG_TMA_BUDGET;
	static constexpr int L = bytes<6>() <= kBudget ? 6 : bytes<5>() <= kBudget ? 5 : bytes<4>() <= kBudget ? 4
		: bytes<3>() <= kBudget ? 3 : bytes<2>() <= kBudget ? 2 : 1;
};

template <class Op, class N, class S>
struct TmaLaunch {
	static constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	using K = typename std::conditional<k2d, AsRows<Op>, Op>::type;
	static constexpr int TX = k2d ? 128 : 32, TY = k2d ? 1 : 8;
	// two points per thread where that still leaves four steps of copies in flight
	static constexpr int PY = (k2d || sizeof(S) == 8 || TmaDepth<K, S, TX, TY, 2>::L < KG_TMA_MIN_L2) ? 1 : 2;
	static constexpr int L = TmaDepth<K, S, TX, TY, PY>::L;
	static constexpr int kThreads = TX * TY + 32;
	using G = TGeo<K, S, TX, TY * PY, L>;
	static const void* func() { return (const void*)tma_kernel<K, N, S, TX, TY, PY, L>; }

	// The copies need 16-byte aligned arrays and rows.
	static bool usable(const kg_problem& pr) {
		constexpr Slots sl = Op::slots();
		if (((size_t)pr.nx * sizeof(S)) % 16) return false;
		for (int q = 0; q < sl.nin; q++)
			if ((uintptr_t)pr.arr[sl.in[q]] % 16) return false;
		return true;
	}

	static cudaError_t run(const Op& op, const kg_problem& pr, cudaStream_t st) {
		constexpr Slots sl = Op::slots();
		Ptrs<S> p{};
		for (int q = 0; q < sl.nin; q++) p.in[q] = (const S*)pr.arr[sl.in[q]];
		for (int q = 0; q < sl.nout; q++) p.out[q] = (S*)pr.arr[sl.out[q]];
		const int nx = pr.nx, ny = k2d ? 1 : pr.ny, ns = k2d ? pr.ny : pr.ns;
		const int dx = nx - K::LX - K::HX, dy = ny - K::LY - K::HY, dz = ns - K::LZ - K::HZ;
		if (dx <= 0 || dy <= 0 || dz <= 0) return cudaSuccess;
		constexpr int threads = kThreads;
		constexpr size_t smem = G::total();
		// per device: resident CTAs per SM and SMs, packed in one atomic word
		// (host threads may race to fill it; both write the same value)
		static std::atomic<int> occ_of[64];
		int dev = 0;
		cudaError_t e = cudaGetDevice(&dev);
		if (e != cudaSuccess) return e;
		if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
		int occ = occ_of[dev].load(std::memory_order_acquire);
		if (!occ) {
			if ((e = cudaFuncSetAttribute(func(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
				return e;
			int b = 0, n = 0;
			if ((e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
			if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, tma_kernel<K, N, S, TX, TY, PY, L>, threads, smem)) != cudaSuccess)
				return e;
			occ = ((b > 0 ? b : 1) << 16) | (n & 0xffff);
			occ_of[dev].store(occ, std::memory_order_release);
		}
		const int per_sm = occ >> 16, sms = occ & 0xffff;
		int* err = tma_error_flag();
		if (!err) return cudaErrorInvalidSymbol;
		const long long wait = tma_wait_limit();
		TMaps maps;
		memset(&maps, 0, sizeof(maps));
		for (int q = 0; q < sl.nin; q++) {
			if (!G::staged(q)) continue;
			e = tma_encode_3d(&maps.m[q], TmaType<S>::v, p.in[q], nx, ny, ns, (int)sizeof(S),
				G::W(q), G::H(q));
			if (e != cudaSuccess) return e;
		}
		const int gx = (nx - K::HX + TX - 1) / TX;
		const int gy = (dy + TY * PY - 1) / (TY * PY);
		const int kc = tma_run_length(per_sm, sms, (long long)gx * gy, dz, G::NZMAX());
		const int nz = (dz + kc - 1) / kc;
		K kop;
		if constexpr (k2d) kop.op = op;
		else kop = op;
		// y tiles beyond the grid's limit (65535) go to further launches
		for (int y0 = 0; y0 < gy; y0 += 65535) {
			dim3 grid(gx, (unsigned)min(gy - y0, 65535), (unsigned)min(nz, 65535));
			tma_kernel<K, N, S, TX, TY, PY, L><<<grid, threads, smem, st>>>(kop, p, maps, nx, ny, ns, kc, y0, err, wait);
			if ((e = cudaGetLastError()) != cudaSuccess) return e;
		}
		return cudaSuccess;
	}
};

}  // namespace kg
