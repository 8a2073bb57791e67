// kg_tmavec.cuh -- the TMA engine with V consecutive points per thread.
//
// The copies, rings, mbarriers and the producer are those of the TMA engine
// (kg_tma.cuh); only the compute side differs.  A compute warp owns one row
// of the CTA's tile, 32 * V consecutive columns, and each lane evaluates V
// consecutive points of it, so every neighbour row the body reads is fetched
// from shared memory as whole vectors: the V values of the lane's own
// columns (one 16-byte load for V = 4 FP32 values) and, where the body reaches
// left or right of them, the V values before or after.  The body itself is
// evaluated V times with its accessor shifted by one column each time; the
// compiler merges the identical vector loads of the V evaluations, so a
// 7-point body costs about 7 vector loads per V points instead of 7 scalar
// loads per point, and the outputs leave as one vector store per row.
//
// For ops with storage of 4 or 2 bytes (FP32, BF16, FP16; FP32 arithmetic)
// whose reach along x is at most V on either side.  3D ops stream along z;
// 2D ops stream down bands of BY rows: step k is the band of rows LY + k BY
// onward, its box grown by the op's reach in y (re-read from L2 by the
// neighbouring band), the arrays' tensor maps rank 3 with one plane.
#pragma once

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "kg_tma.cuh"

// 1: launch sweeps as programmatic dependents of the previous kernel on the
// stream (griddepcontrol), so that a launch and its prologue overlap the
// previous sweep's tail.  Measured on GB300, back-to-back sweeps at
// 512x256x256 (Gpts/s, without / with): FP32 laplacian 674 / 695,
// divergence 411 / 426, gradient 346 / 357, wave13pt 493 / 509; BF16
// laplacian 952 / 1016; at 1024x512x512 within 0-3 %.
#ifndef KG_TMAVEC_PDL
#define KG_TMAVEC_PDL 1
#endif
// 1: consecutive sweeps alternate the direction in which their runs along
// z (or bands of rows) are taken.  Measured on GB300 (ping-pong sweeps at
// 512x256x256 / 512x65536, Gpts/s, fixed / alternating): FP32 gradient 356 /
// 370, jacobi 654 / 659, wave13pt 507 / 511; BF16 gradient 521 / 544, uxx1
// 300 / 305, jacobi 994 / 1008; the others within 0.5 %.
#ifndef KG_TMAVEC_ALT
#define KG_TMAVEC_ALT 1
#endif

namespace kg {

template <class S, int V> struct alignas(V * sizeof(S)) VPack {
	S v[V];
};

// Element x (0 <= x < 3V) of the 3V stored values that start V columns left
// of the lane's first column, row_elems elements after the lane's base.
template <class S, int V>
__device__ __forceinline__ S vrow_load(const unsigned char* b, int row_elems, int x)
{
	const int chunk = x / V - 1;   // -1, 0, 1
	const VPack<S, V> pk = *reinterpret_cast<const VPack<S, V>*>(b + (row_elems + chunk * V) * (int)sizeof(S));
	return pk.v[x % V];
}

// The value as FP32 arithmetic reads it.  16-bit storage: the element stays
// in its half of the 16-byte vector's 32-bit word (H16): sums take it from
// there by the mixed-precision add, every other use widens it (for BF16, the
// upper half of an FP32 pattern, by one shift or mask: the conversion,
// exactly).
template <class N, class S, int V>
__device__ __forceinline__ auto vrow_value(const unsigned char* b, int row_elems, int x)
{
	if constexpr (sizeof(S) == 2) {
		const int chunk = x / V - 1;
		const uint4 q = *reinterpret_cast<const uint4*>(b + (row_elems + chunk * V) * (int)sizeof(S));
		const int e = x % V;
		const uint32_t w = e / 2 == 0 ? q.x : e / 2 == 1 ? q.y : e / 2 == 2 ? q.z : q.w;
		return H16<S>{w, e % 2};
	} else {
		return Conv<N, S>::from(vrow_load<S, V>(b, row_elems, x));
	}
}

// ZP: the plane of the step among the steps evaluated together (its window
// starts ZP planes after the first step's); ZS_: window entries per input.
template <class Op, class N, class S, class G, int V, int VI, int RY = 0, int ZP = 0, int ZS_ = 5> struct VAcc {
	static constexpr int ZS = ZS_;
	const unsigned char* (*base)[ZS];   // per input and dz + z0 + ZP: the lane's first column in the point's row
	const S* const* in;
	long long c, sy, sz;                      // c: the lane's first point
	__device__ __forceinline__ auto operator()(int q, int dx, int dy, int dz) const {
		return vrow_value<N, S, V>(base[q][dz + Op::halo(q).z0 + ZP], (dy + RY) * G::W(q), VI + dx + V);
	}
	__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const {
		return __ldg(in[q] + c + VI + dx + (dy + RY) * sy + dz * sz);
	}
};

// Two FP32 results rounded to the storage type as one packed pair (one
// conversion instruction for both; each rounded to nearest as alone).
template <class S> struct PairConv;
template <> struct PairConv<__nv_bfloat16> {
	static __device__ __forceinline__ __nv_bfloat162 to(float a, float b) { return __floats2bfloat162_rn(a, b); }
};
template <> struct PairConv<__half> {
	static __device__ __forceinline__ __half2 to(float a, float b) { return __floats2half2_rn(a, b); }
};

// V outputs of one lane (FP32 arithmetic) to global memory: one vector store
// where all V points are in the domain, else one store per point that is.
template <class N, class S, int V>
__device__ __forceinline__ void vstore(S* dst, const N (&o)[V], unsigned valid_mask)
{
	if (valid_mask == (1u << V) - 1) {
		VPack<S, V> pk;
		if constexpr (sizeof(S) == 2) {
			static_assert(V % 2 == 0, "pairs");
#pragma unroll
			for (int v = 0; v < V; v += 2) {
				const auto two = PairConv<S>::to(o[v].v, o[v + 1].v);
				memcpy(&pk.v[v], &two, 2 * sizeof(S));
			}
		} else {
#pragma unroll
			for (int v = 0; v < V; v++) pk.v[v] = Conv<N, S>::to(o[v]);
		}
		*reinterpret_cast<VPack<S, V>*>(dst) = pk;
	} else {
#pragma unroll
		for (int v = 0; v < V; v++)
			if ((valid_mask >> v) & 1u) dst[v] = Conv<N, S>::to(o[v]);
	}
}

template <int I, int V, class F> __device__ __forceinline__ void for_v(F&& f)
{
	if constexpr (I < V) {
		f(std::integral_constant<int, I>{});
		for_v<I + 1, V>(f);
	}
}

// NW compute warps and one producer warp.  The warps cover RB = NW RPW rows
// of the tile (BX = 128 columns, RPW = 32 V / BX rows per warp): lane l
// evaluates the V consecutive points from column (l mod BX/V) V of row
// l / (BX/V) of its warp's rows, V = 16 bytes of storage, and the same
// points PY - 1 more times, RB rows further down each time (BY = RB PY).
// PZ = 2: the warps take the steps of a run two at a time (both planes'
// points from one set of slot and address computations, the plane between
// them read once for both).
template <class Op, class N, class S, int V, int NW, int PY, int L, int PZ>
__global__ void __launch_bounds__(32 * NW + 32) tma_vec_kernel(Op op, Ptrs<S> p, const __grid_constant__ TMaps maps,
	int nx, int ny, int ns, int kc, int yt0, int* err, long long wait, int rev)
{
	constexpr int BX = 128, LPR = BX / V, RPW = 32 / LPR, RB = NW * RPW, BY = RB * PY, NC = 32 * NW;
	static_assert(LPR * RPW == 32, "a warp covers whole rows");
	using G = TGeo<Op, S, BX, BY, L>;
	constexpr int NB = G::NB;
	constexpr Slots sl = Op::slots();
	constexpr int ZS = 4 + PZ;   // window entries per input: the planes of PZ steps
	static_assert(G::fits(), "tile does not fit the TMA engine");
	static_assert(G::NZMAX() + PZ - 1 <= ZS, "at most ZS planes per window");
	static_assert(PZ == 1 || PZ == 2, "one or two steps at a time");
	extern __shared__ __align__(128) unsigned char sm[];
	uint64_t* full = reinterpret_cast<uint64_t*>(sm);
	uint64_t* done = full + NB;
	volatile int* abort = reinterpret_cast<volatile int*>(sm + G::kAbort);

	// 2D ops walk bands of BY rows instead of planes: step k covers rows
	// LY + k BY ... (one tile column per CTA in y)
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	const int tid = threadIdx.x;
	const int xt = blockIdx.x * BX, yt = Op::LY + (yt0 + (int)blockIdx.y) * BY;
	const int kend = k2d ? (ny - Op::LY - Op::HY + BY - 1) / BY : ns - Op::HZ;
	// the CTA's runs along z or down the bands (each run is a window plus steps)
	using Runs = std::conditional_t<k2d, BandRuns, ZRuns>;
	Runs runs;
	runs.xt = xt;
	runs.yt = yt;
	// rev: the runs taken from the far end of z (or of the bands) first
	runs.kb = Op::LZ + (rev ? (int)gridDim.z - 1 - (int)blockIdx.z : (int)blockIdx.z) * kc;
	runs.kend = kend;
	runs.kc = kc;

	if (KG_TMAVEC_PDL) {
		// a sweep launched after this one may start its CTAs as SMs free up
		// (all of this grid's CTAs are resident by then)
		asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
	}
	if (tid == 0) {
		for (int b = 0; b < NB; b++) {
			mbar_init(&full[b], 1);
			mbar_init(&done[b], NW);
		}
		*abort = 0;
		mbar_fence_init();
	}
	__syncthreads();
	if (KG_TMAVEC_PDL) {
		// the previous sweep's writes (this one's inputs) are complete and
		// visible, and its reads of this one's outputs are done
		asm volatile("griddepcontrol.wait;" ::: "memory");
	}

	if (tid >= NC) {
		if (tid == NC) tma_produce<Op, S, G>(maps, sm, full, done, abort, runs, err);
		return;
	}

	// ---- compute warps ----
	const int lane = tid & 31, w = tid >> 5;
	const int lx = lane % LPR, ry = w * RPW + lane / LPR;
	const long long sy = nx, sz = k2d ? (long long)nx * BY : (long long)nx * ny;
	// byte offset of the lane's first column in the point's row of a plane, per input
	int toff[6];
#pragma unroll
	for (int q = 0; q < G::NIN; q++)
		toff[q] = ((ry + Op::halo(q).y0) * G::W(q) + lx * V + G::XL(q)) * G::ES;

	const int i0 = xt + lx * V, j = yt + ry;
	unsigned cols = 0;
#pragma unroll
	for (int v = 0; v < V; v++)
		if (i0 + v >= Op::LX && i0 + v < nx - Op::HX) cols |= 1u << v;
	// rows in the domain: fixed for 3D ops, per band for 2D ones
	auto rows_valid = [&](int band, unsigned (&valid)[PY]) {
#pragma unroll
		for (int r = 0; r < PY; r++) valid[r] = j + r * RB + band * BY < ny - Op::HY ? cols : 0u;
	};
	unsigned valid[PY];
	rows_valid(0, valid);
	// step counters kept incrementally: barrier index and phase of the step,
	// and the ring slot of the step's plane of every input
	int bi = 0;
	uint32_t ph = 0;
	Runs rz = runs;
	int xr, yr, kb, nsteps;
	while (rz.next(xr, yr, kb, nsteps)) {
		int s0[6];
#pragma unroll
		for (int q = 0; q < G::NIN; q++) s0[q] = G::slot(q, kb);
		const long long c0 = i0 + sy * j + sz * kb;
		if constexpr (PZ == 1) {
		for (int s = 0; s < nsteps; s++) {
			if (k2d) rows_valid(kb + s, valid);
			const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[bi], ph, wait, abort));
			if (!ok) {
				if (lane == 0) {
					*abort = 1;
					atomicExch(err, 1);
				}
				return;
			}
			const unsigned char* base[6][ZS];
#pragma unroll
			for (int q = 0; q < G::NIN; q++) {
				const Halo h = Op::halo(q);
#pragma unroll
				for (int d = 0; d < ZS; d++)
					if (d < G::NZ(q))
						base[q][d] = sm + G::offset(q) + G::step_slot(q, s0[q], d - h.z0) * G::PS(q) + toff[q];
			}
			const long long c = c0 + sz * s;
			N o[PY][3][V];
			for_v<0, PY>([&](auto ri) {
				constexpr int R = decltype(ri)::value;
				for_v<0, V>([&](auto vi) {
					constexpr int VI = decltype(vi)::value;
					VAcc<Op, N, S, G, V, VI, R * RB, 0, ZS> at{base, p.in, c, sy, sz};
					N r[3];
					op.point(at, r);
#pragma unroll
					for (int q = 0; q < sl.nout; q++) o[R][q][VI] = r[q];
				});
			});
			// this warp is done with the step's planes
			__syncwarp();
			if (lane == 0) mbar_arrive(&done[bi]);
#pragma unroll
			for (int r = 0; r < PY; r++)
				if (valid[r]) {
#pragma unroll
					for (int q = 0; q < sl.nout; q++) vstore<N, S, V>(p.out[q] + c + r * RB * sy, o[r][q], valid[r]);
				}
			if (++bi == NB) {
				bi = 0;
				ph ^= 1;
			}
#pragma unroll
			for (int q = 0; q < G::NIN; q++) s0[q] = G::step_slot(q, s0[q], 1);
		}
		} else {
		for (int s = 0; s < nsteps;) {
			const int np = s + 1 < nsteps ? 2 : 1;
			// barrier index and phase of the second step
			const int bi1 = bi + 1 == NB ? 0 : bi + 1;
			const uint32_t ph1 = bi + 1 == NB ? ph ^ 1u : ph;
			bool ok = __all_sync(0xffffffffu, mbar_wait(&full[bi], ph, wait, abort));
			if (ok && np == 2) ok = __all_sync(0xffffffffu, mbar_wait(&full[bi1], ph1, wait, abort));
			if (!ok) {
				if (lane == 0) {
					*abort = 1;
					atomicExch(err, 1);
				}
				return;
			}
			// NP steps from one set of plane addresses: the window of step s
			// + P is entries P .. P + NZ - 1
			auto steps = [&](auto npc) {
				constexpr int NP = decltype(npc)::value;
				const unsigned char* base[6][ZS];
#pragma unroll
				for (int q = 0; q < G::NIN; q++) {
					const Halo h = Op::halo(q);
#pragma unroll
					for (int d = 0; d < ZS; d++)
						if (d < G::NZ(q) + NP - 1)
							base[q][d] = sm + G::offset(q) + G::step_slot(q, s0[q], d - h.z0) * G::PS(q) + toff[q];
				}
				N o[NP][PY][3][V];
				for_v<0, NP>([&](auto pi) {
					constexpr int P = decltype(pi)::value;
					for_v<0, PY>([&](auto ri) {
						constexpr int R = decltype(ri)::value;
						for_v<0, V>([&](auto vi) {
							constexpr int VI = decltype(vi)::value;
							VAcc<Op, N, S, G, V, VI, R * RB, P, ZS> at{base, p.in, c0 + sz * (s + P), sy, sz};
							N r[3];
							op.point(at, r);
#pragma unroll
							for (int q = 0; q < sl.nout; q++) o[P][R][q][VI] = r[q];
						});
					});
				});
				// this warp is done with the steps' planes
				__syncwarp();
				if (lane == 0) {
					mbar_arrive(&done[bi]);
					if (NP == 2) mbar_arrive(&done[bi1]);
				}
#pragma unroll
				for (int P = 0; P < NP; P++) {
					if (k2d) rows_valid(kb + s + P, valid);
					const long long c = c0 + sz * (s + P);
#pragma unroll
					for (int r = 0; r < PY; r++)
						if (valid[r]) {
#pragma unroll
							for (int q = 0; q < sl.nout; q++)
								vstore<N, S, V>(p.out[q] + c + r * RB * sy, o[P][r][q], valid[r]);
						}
				}
			};
			if (np == 2) steps(std::integral_constant<int, 2>{});
			else steps(std::integral_constant<int, 1>{});
			s += np;
			bi = np == 2 ? (bi1 + 1 == NB ? 0 : bi1 + 1) : bi1;
			ph = np == 2 ? (bi1 + 1 == NB ? ph1 ^ 1u : ph1) : ph1;
#pragma unroll
			for (int q = 0; q < G::NIN; q++) s0[q] = G::step_slot(q, s0[q], np);
		}
		}
	}
}

// Shared memory per CTA for the rings: L (steps of copies in flight) is the
// largest, up to 6, whose rings fit the budget of the storage size; the CTAs
// per SM follow from what the rings then take.  Measured on GB300 (Gpts/s at
// 512x256x256 and 1024x512x512): 2-byte storage gains from more CTAs with
// shallower rings (48 KB against 100 KB: BF16 laplacian 900 -> 985 and
// 1236 -> 1311, gradient 400 -> 482 and 575 -> 616, the others within 1 %),
// FP32 loses (laplacian 661 -> 546).
#ifndef KG_TMAVEC_BUDGET
#define KG_TMAVEC_BUDGET (100 * 1024)
#endif
#ifndef KG_TMAVEC_BUDGET16
#define KG_TMAVEC_BUDGET16 (48 * 1024)
#endif
// Rows of points per lane (each lane evaluates PY x V points per plane; 0:
// per op and storage size).  FP32: one (two measured: uxx1 279 -> 242, the
// others within 2 %).  16-bit storage with the 48 KB ring budget, measured
// on GB300 (BF16, Gpts/s at 512x256x256 or 512x65536 and 1024x512x512, two
// rows / one): laplacian 1008 / 1116 and 1413 / 1482, divergence 738 / 780
// and 829 / 864, uxx1 305 / 358 and 355 / 405, tricubic 116 / 121 at
// 1024x512x512 take one; wave13pt 758 / 742 and 899 / 864, jacobi 1010 / 959,
// gaussblur 660 / 624, gradient 545 / 537, lapgsrb 564 / 561 keep two.
#ifndef KG_TMAVEC_PY
#define KG_TMAVEC_PY 0
#endif
template <class Op> struct VecRows16 { static constexpr int v = 2; };
template <class N> struct VecRows16<OpLaplacian<N>> { static constexpr int v = 1; };
template <class N> struct VecRows16<OpDivergence<N>> { static constexpr int v = 1; };
template <class N> struct VecRows16<OpUxx1<N>> { static constexpr int v = 1; };
template <class N, bool Z> struct VecRows16<OpTricubicT<N, Z>> { static constexpr int v = 1; };
// Steps a compute warp takes at a time (0: per op; 1 or 2 for all).
#ifndef KG_TMAVEC_PZ
#define KG_TMAVEC_PZ 0
#endif
// Two at a time pays where a point reads many rows of the planes around it:
// the rows of the planes the two steps share are loaded once.  Measured on
// GB300 (Gpts/s at 512x256x256 and 1024x512x512, one step / two): FP32
// lapgsrb 356 / 442 and 382 / 485 (the same gain on every GPU measured);
// FP32 laplacian at 512x256x256 734 / 785, 733 / 790 and 786 / 769 on three
// GPUs (two steps steadier), 1024x512x512 within 1 %; the others within the
// spread between GPUs or slower (uxx1 268 / 145, tricubic 121 / 116).  With 16-bit
// storage every stencil was slower, the second step's registers costing
// resident CTAs (BF16 laplacian 1149 / 1005; 1112 with the registers capped
// for four CTAs per SM, divergence 761 against 780; lapgsrb with one row of
// points a lane instead of two 557 / 485).
template <class Op, class S> struct VecSteps { static constexpr int v = 1; };
template <class N> struct VecSteps<OpLapgsrb<N>, float> { static constexpr int v = 2; };
template <class N> struct VecSteps<OpLaplacian<N>, float> { static constexpr int v = 2; };
// Runs along z per tile column (0: the TMA engine's wave-count model).
#ifndef KG_TMAVEC_ZRUNS
#define KG_TMAVEC_ZRUNS 0
#endif
template <class Op, class S, int BX, int BY> struct TmaVecDepth {
	template <int L> static constexpr int bytes() { return TGeo<Op, S, BX, BY, L>::total(); }
	static constexpr int kBudget = sizeof(S) == 2 ? KG_TMAVEC_BUDGET16 : KG_TMAVEC_BUDGET;
	static constexpr int L = bytes<6>() <= kBudget ? 6 : bytes<5>() <= kBudget ? 5 : bytes<4>() <= kBudget ? 4
		: bytes<3>() <= kBudget ? 3 : bytes<2>() <= kBudget ? 2 : 1;
};

template <class Op, class N, class S>
struct TmaVecLaunch {
	static constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	static constexpr int V = 16 / (int)sizeof(S), NW = 8;
	static constexpr int PY = KG_TMAVEC_PY > 0 ? KG_TMAVEC_PY : (sizeof(S) == 2 ? VecRows16<Op>::v : 1);
	static constexpr int BX = 128, BY = NW * (32 * V / BX) * PY;
	static constexpr int L = TmaVecDepth<Op, S, BX, BY>::L;
	static constexpr int PZ = KG_TMAVEC_PZ > 0 ? KG_TMAVEC_PZ : VecSteps<Op, S>::v;
	static constexpr int kThreads = 32 * NW + 32;
	using G = TGeo<Op, S, BX, BY, L>;
	static constexpr bool reach_ok() {
		for (int q = 0; q < Op::slots().nin; q++)
			if (Op::halo(q).x0 > V || Op::halo(q).x1 > V) return false;
		return true;
	}
	// built for 4- and 2-byte storage where the reach along x fits (3D ops
	// along z, 2D ops down bands of BY rows)
	static constexpr bool built = (sizeof(S) == 4 || sizeof(S) == 2) && reach_ok();
	static const void* func() {
		if constexpr (built) return (const void*)tma_vec_kernel<Op, N, S, V, NW, PY, L, PZ>;
		else return nullptr;
	}

	// The copies need 16-byte aligned input arrays and rows; the vector
	// stores need V-element aligned outputs.
	static bool usable(const kg_problem& pr) {
		if constexpr (!built) return false;
		constexpr Slots sl = Op::slots();
		if (((size_t)pr.nx * sizeof(S)) % 16) return false;
		for (int q = 0; q < sl.nin; q++)
			if ((uintptr_t)pr.arr[sl.in[q]] % 16) return false;
		for (int q = 0; q < sl.nout; q++)
			if ((uintptr_t)pr.arr[sl.out[q]] % (V * sizeof(S))) return false;
		return true;
	}

	static cudaError_t run(const Op& op, const kg_problem& pr, cudaStream_t st) {
		if constexpr (!built) {
			return cudaErrorNotSupported;
		} else {
			constexpr Slots sl = Op::slots();
			Ptrs<S> p{};
			for (int q = 0; q < sl.nin; q++) p.in[q] = (const S*)pr.arr[sl.in[q]];
			for (int q = 0; q < sl.nout; q++) p.out[q] = (S*)pr.arr[sl.out[q]];
			const int nx = pr.nx, ny = pr.ny, ns = pr.ns;
			const int dx = nx - Op::LX - Op::HX, dy = ny - Op::LY - Op::HY;
			if (dx <= 0 || dy <= 0 || ns - Op::LZ - Op::HZ <= 0) return cudaSuccess;
			// 2D: one tile column in y, the bands of BY rows as the steps
			const int dz = k2d ? (dy + BY - 1) / BY : ns - Op::LZ - Op::HZ;
			constexpr size_t smem = G::total();
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
				if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, tma_vec_kernel<Op, N, S, V, NW, PY, L, PZ>, kThreads, smem)) != cudaSuccess)
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
				e = tma_encode_3d(&maps.m[q], TmaType<S>::v, p.in[q], nx, ny, ns, (int)sizeof(S), G::W(q), G::H(q));
				if (e != cudaSuccess) return e;
			}
			const int gx = (nx - Op::HX + BX - 1) / BX;
			const int gy = k2d ? 1 : (dy + BY - 1) / BY;
			// z split into runs so that the CTAs fill whole waves (all tiles
			// then walk the same planes at about the same time, and the halo
			// rows of neighbouring tiles are served from L2).  Window planes
			// weigh a quarter of a plane and a run nothing more: fitted to
			// sweeps of fixed run counts on GB300 (Gpts/s, FP32 at 512x256x256
			// and 1024x512x512, runs per tile 7-9 / 14 / 19 / 28): laplacian 657
			// / 672 / 668 / 649 and 795 / 837 / 847 / 851, gradient 318 / 338 /
			// 347 / 358 and 366 / 388 / 394 / 399, wave13pt (5-plane window)
			// 486 / 442 / 429 / 408 and 559 / 553 / 539 / 516.
			constexpr int zruns = KG_TMAVEC_ZRUNS > 0 ? KG_TMAVEC_ZRUNS : 1;
			const int kc = KG_TMAVEC_ZRUNS > 0 ? (dz + zruns - 1) / zruns
				: tma_run_length(per_sm, sms, (long long)gx * gy, dz, G::NZMAX(), 0.25, 0.0);
			const int nz = (dz + kc - 1) / kc;
			// consecutive sweeps walk z (the bands) in opposite directions:
			// a sweep then starts on the planes the one before it wrote
			// (or read) last, which are still in L2
			static std::atomic<unsigned> sweeps{0};
			const int rev = KG_TMAVEC_ALT ? (int)(sweeps.fetch_add(1, std::memory_order_relaxed) & 1u) : 0;
			for (int y0 = 0; y0 < gy; y0 += 65535) {
				dim3 grid(gx, (unsigned)min(gy - y0, 65535), (unsigned)min(nz, 65535));
				if (KG_TMAVEC_PDL) {
					// programmatic dependent launch: the launch and the prologue
					// overlap the previous kernel's tail on the stream
					cudaLaunchConfig_t cfg = {};
					cfg.gridDim = grid;
					cfg.blockDim = dim3(kThreads);
					cfg.dynamicSmemBytes = smem;
					cfg.stream = st;
					cudaLaunchAttribute at[1];
					at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
					at[0].val.programmaticStreamSerializationAllowed = 1;
					cfg.attrs = at;
					cfg.numAttrs = 1;
					e = cudaLaunchKernelEx(&cfg, tma_vec_kernel<Op, N, S, V, NW, PY, L, PZ>, op, p, maps, nx, ny, ns, kc, y0, err,
						wait, rev);
					if (e != cudaSuccess) return e;
				} else {
					tma_vec_kernel<Op, N, S, V, NW, PY, L, PZ><<<grid, kThreads, smem, st>>>(op, p, maps, nx, ny, ns, kc, y0, err,
						wait, rev);
				}
				if ((e = cudaGetLastError()) != cudaSuccess) return e;
			}
			return cudaSuccess;
		}
	}
};

}  // namespace kg
