// kg_staged.cuh -- the plane-streaming engine: halo tiles in shared memory.
//
// A CTA of BX x BY threads owns BX x BY columns of the update domain and
// walks a run of KC planes along z (the slowest axis).  For every input the
// body reads at neighbouring points, the CTA keeps a ring of the planes
// z-z0 .. z+z1 of that input's halo tile ((BY + y0 + y1) x (BX + x0 + x1)
// points) in shared memory.  Each step loads ONE new plane per input with
// coalesced loads along x, converting every value once to the arithmetic's
// representation (a float-float pair, FP32, or FP64), then every thread
// evaluates its point from shared memory.  So each input value crosses from
// global memory about once per sweep (halo rows and columns are re-read by
// the neighbouring CTA, mostly from L2) and, for the float-float arithmetic,
// is split into its pair once instead of once per use.
//
// Inputs read only at the point itself come straight from global memory.
#pragma once

#include <atomic>

#include "kg_engine.cuh"

namespace kg {

// Shared-memory representation of a stored value for the arithmetic N.
template <class N, class S> struct Rep;
template <> struct Rep<SD, double> {
	using M = double;
	static __device__ __forceinline__ M stage(double x) { return x; }
	static __device__ __forceinline__ SD get(M m) { return SD(m); }
};
template <> struct Rep<FD, double> {
	using M = double;
	static __device__ __forceinline__ M stage(double x) { return x; }
	static __device__ __forceinline__ FD get(M m) { return FD(m); }
};
template <> struct Rep<FF2, double> {
	using M = float2;
	static __device__ __forceinline__ M stage(double x) { const FF2 v = ff2_from_double(x); return make_float2(v.hi, v.lo); }
	static __device__ __forceinline__ FF2 get(M m) { return FF2(m.x, m.y); }
};
template <class S> struct Rep<FF, S> {
	using M = float;
	static __device__ __forceinline__ M stage(S x) { return Conv<FF, S>::from(x).v; }
	static __device__ __forceinline__ FF get(M m) { return mkf(m); }
};

// Ring geometry of input q of Op for a BX x BY tile.
template <class Op, int BX, int BY> struct Ring {
	static constexpr int W(int q) { return BX + Op::halo(q).x0 + Op::halo(q).x1; }
	static constexpr int H(int q) { return BY + Op::halo(q).y0 + Op::halo(q).y1; }
	static constexpr int NZ(int q) { return Op::halo(q).z0 + Op::halo(q).z1 + 1; }
	static constexpr int elems(int q) { return Op::halo(q).center() ? 0 : W(q) * H(q) * NZ(q); }
	static constexpr int offset(int q) { int o = 0; for (int r = 0; r < q; r++) o += elems(r); return o; }
	static constexpr int total() { return offset(Op::slots().nin); }
};

template <class Op, class N, class S, int BX, int BY>
struct SAcc {
	using R = Rep<N, S>;
	using M = typename R::M;
	using G = Ring<Op, BX, BY>;
	const M* sm;             // ring storage of all staged inputs
	const S* const* in;      // global inputs (for inputs read at the point only)
	long long c, sy, sz;
	int k, tx, ty;
	__device__ __forceinline__ N operator()(int q, int dx, int dy, int dz) const {
		const Halo h = Op::halo(q);
		if (h.center()) return Conv<N, S>::ld(in[q] + c + dx + dy * sy + dz * sz);
		const int nz = G::NZ(q);
		const int slot = (k + dz) % nz;
		return R::get(sm[G::offset(q) + (slot * G::H(q) + ty + h.y0 + dy) * G::W(q) + tx + h.x0 + dx]);
	}
	__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const {
		return __ldg(in[q] + c + dx + dy * sy + dz * sz);
	}
};

// Per-thread share of one plane of a staged input: the thread's elements
// e = tid, tid + BX*BY, ... of the W x H halo tile, fetched into registers
// first (so the loads are in flight while the current plane is computed) and
// written to the ring afterwards.
template <class Op, class N, class S, int BX, int BY, int Q> struct PlaneRegs {
	static constexpr int W = BX + Op::halo(Q).x0 + Op::halo(Q).x1;
	static constexpr int H = BY + Op::halo(Q).y0 + Op::halo(Q).y1;
	static constexpr int PER = Op::halo(Q).center() ? 0 : (W * H + BX * BY - 1) / (BX * BY);
	S v[PER > 0 ? PER : 1];
	__device__ __forceinline__ void fetch(const S* __restrict__ plane, int x0, int y0, int nx, int ny, long long sy, int tid) {
		constexpr Halo h = Op::halo(Q);
#pragma unroll
		for (int r = 0; r < PER; r++) {
			const int e = tid + r * BX * BY;
			const int ly = e / W, lx = e - ly * W;
			const int gx = x0 - h.x0 + lx, gy = y0 - h.y0 + ly;
			v[r] = (e < W * H && gx < nx && gy < ny) ? __ldg(plane + gx + sy * gy) : S{};
		}
	}
	__device__ __forceinline__ void commit(typename Rep<N, S>::M* dst, int tid) const {
#pragma unroll
		for (int r = 0; r < PER; r++) {
			const int e = tid + r * BX * BY;
			if (e < W * H) dst[e] = Rep<N, S>::stage(v[r]);
		}
	}
};

// The staged inputs' register shares, one member per input slot (up to 6).
template <class Op, class N, class S, int BX, int BY> struct Prefetch {
	PlaneRegs<Op, N, S, BX, BY, 0> r0;
	PlaneRegs<Op, N, S, BX, BY, (Op::slots().nin > 1 ? 1 : 0)> r1;
	PlaneRegs<Op, N, S, BX, BY, (Op::slots().nin > 2 ? 2 : 0)> r2;
	PlaneRegs<Op, N, S, BX, BY, (Op::slots().nin > 3 ? 3 : 0)> r3;
	PlaneRegs<Op, N, S, BX, BY, (Op::slots().nin > 4 ? 4 : 0)> r4;
	template <int Q> __device__ __forceinline__ auto& get() {
		if constexpr (Q == 0) return r0;
		else if constexpr (Q == 1) return r1;
		else if constexpr (Q == 2) return r2;
		else if constexpr (Q == 3) return r3;
		else return r4;
	}
	template <int Q> __device__ __forceinline__ const auto& get() const {
		if constexpr (Q == 0) return r0;
		else if constexpr (Q == 1) return r1;
		else if constexpr (Q == 2) return r2;
		else if constexpr (Q == 3) return r3;
		else return r4;
	}
};

template <class Op, class N, class S, int BX, int BY, int Q>
__device__ __forceinline__ void fetch_one(Prefetch<Op, N, S, BX, BY>& pf, const Ptrs<S>& p, int kk,
	int x0, int y0, int nx, int ny, long long sy, long long sz, int tid)
{
	if constexpr (Q < Op::slots().nin) {
		if constexpr (!Op::halo(Q).center())
			pf.template get<Q>().fetch(p.in[Q] + sz * (kk + Op::halo(Q).z1), x0, y0, nx, ny, sy, tid);
		fetch_one<Op, N, S, BX, BY, Q + 1>(pf, p, kk, x0, y0, nx, ny, sy, sz, tid);
	}
}

template <class Op, class N, class S, int BX, int BY, int Q>
__device__ __forceinline__ void commit_one(const Prefetch<Op, N, S, BX, BY>& pf, typename Rep<N, S>::M* sm,
	int kk, int tid)
{
	if constexpr (Q < Op::slots().nin) {
		if constexpr (!Op::halo(Q).center()) {
			using G = Ring<Op, BX, BY>;
			const int plane = kk + Op::halo(Q).z1;
			pf.template get<Q>().commit(sm + G::offset(Q) + (plane % G::NZ(Q)) * G::H(Q) * G::W(Q), tid);
		}
		commit_one<Op, N, S, BX, BY, Q + 1>(pf, sm, kk, tid);
	}
}

// Ring of planes along z, software-pipelined: while plane k is evaluated
// from shared memory, the loads of plane k+1's new planes are in flight.
template <class Op, class N, class S, int BX, int BY, int KC>
__device__ __forceinline__ void staged3d_body(const Op& op, const Ptrs<S>& p, int nx, int ny, int ns)
{
	using R = Rep<N, S>;
	using M = typename R::M;
	using G = Ring<Op, BX, BY>;
	constexpr Slots sl = Op::slots();
	extern __shared__ __align__(16) unsigned char smem_raw[];
	M* sm = reinterpret_cast<M*>(smem_raw);

	const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
	const int x0 = Op::LX + blockIdx.x * BX;
	const int i = x0 + tx;
	const long long sy = nx, sz = (long long)nx * ny;
	const int kend = ns - Op::HZ;
	// rows of tiles beyond the grid's y limit (65535) are taken in turn
	const int tyn = (ny - Op::LY - Op::HY + BY - 1) / BY;
	Prefetch<Op, N, S, BX, BY> pf;

	for (int yb = blockIdx.y; yb < tyn; yb += gridDim.y)
	for (int kb = Op::LZ + blockIdx.z * KC; kb < kend; kb += gridDim.z * KC) {
		const int y0 = Op::LY + yb * BY, j = y0 + ty;
		const bool mine = i < nx - Op::HX && j < ny - Op::HY;
		const int ke = min(kb + KC, kend);
		// planes kb - z0 .. kb + z1 - 1 of each staged input: plane kk + z1
		// of input q is the prefetch of step kk, so run steps kb-z0-z1 ..
		// kb-1 of the prefetch for inputs whose window reaches them.
#pragma unroll
		for (int q = 0; q < sl.nin; q++) {
			const Halo h = Op::halo(q);
			if (h.center()) continue;
			for (int kk = kb - h.z0; kk < kb + h.z1; kk++) {
				M* dst = sm + G::offset(q) + (kk % G::NZ(q)) * G::H(q) * G::W(q);
				const S* src = p.in[q] + sz * kk;
				for (int e = tid; e < G::W(q) * G::H(q); e += BX * BY) {
					const int ly = e / G::W(q), lx = e - ly * G::W(q);
					const int gx = x0 - h.x0 + lx, gy = y0 - h.y0 + ly;
					M v{};
					if (gx < nx && gy < ny) v = R::stage(__ldg(src + gx + sy * gy));
					dst[e] = v;
				}
			}
		}
		fetch_one<Op, N, S, BX, BY, 0>(pf, p, kb, x0, y0, nx, ny, sy, sz, tid);
		for (int k = kb; k < ke; k++) {
			commit_one<Op, N, S, BX, BY, 0>(pf, sm, k, tid);   // plane k + z1 of each input
			__syncthreads();
			if (k + 1 < ke) fetch_one<Op, N, S, BX, BY, 0>(pf, p, k + 1, x0, y0, nx, ny, sy, sz, tid);
			if (mine) {
				const long long c = i + sy * j + sz * k;
				SAcc<Op, N, S, BX, BY> at{sm, p.in, c, sy, sz, k, tx, ty};
				N o[3];
				op.point(at, o);
#pragma unroll
				for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
			}
			__syncthreads();
		}
	}
}

template <class Op, class N, class S, int BX, int BY, int KC>
__global__ void __launch_bounds__(BX * BY) staged3d_kernel(Op op, Ptrs<S> p, int nx, int ny, int ns)
{
	staged3d_body<Op, N, S, BX, BY, KC>(op, p, nx, ny, ns);
}

// The same kernel asked for at least four CTAs per SM (64 registers a
// thread; ptxas then also schedules more independent work in flight), for
// the ops where that measured faster (StagedOcc4).
template <class Op, class N, class S, int BX, int BY, int KC>
__global__ void __launch_bounds__(BX * BY, 4) staged3d_kernel_occ4(Op op, Ptrs<S> p, int nx, int ny, int ns)
{
	staged3d_body<Op, N, S, BX, BY, KC>(op, p, nx, ny, ns);
}

// Float-float tricubic, 512x256x256 on GB300: 1.71 -> 1.61 ms per sweep
// with four CTAs per SM; every other stencil was slower with the cap
// (laplacian 0.251 -> 0.281 ms, wave13pt 0.411 -> 0.482, gaussblur 0.476 ->
// 0.514, ...).
template <class Op> struct StagedOcc4 : std::false_type {};
template <class N, bool Z> struct StagedOcc4<OpTricubicT<N, Z>> : std::true_type {};

// A 2D op seen as a 3D op whose rows are planes: (dx, dy) -> (dx, 0, dy),
// so the same plane-streaming kernel walks down the rows of a 2D grid with
// a ring of rows, 256-point row segments per CTA.
template <class Op> struct AsRows {
	static_assert(Op::LZ == 0 && Op::HZ == 0, "AsRows is for 2D ops");
	static constexpr int LX = Op::LX, HX = Op::HX, LY = 0, HY = 0, LZ = Op::LY, HZ = Op::HY;
	static constexpr Slots slots() { return Op::slots(); }
	static constexpr Halo halo(int q) {
		return Halo{Op::halo(q).x0, Op::halo(q).x1, 0, 0, Op::halo(q).y0, Op::halo(q).y1};
	}
	Op op;
	template <class A> struct Flip {
		const A& a;
		__device__ __forceinline__ auto operator()(int q, int dx, int dy, int) const { return a(q, dx, 0, dy); }
		__device__ __forceinline__ auto raw(int q, int dx, int dy, int) const { return a.raw(q, dx, 0, dy); }
	};
	template <class A, class N> __device__ __forceinline__ void point(const A& at, N* o) const {
		op.point(Flip<A>{at}, o);
	}
};

template <class Op, class N, class S>
struct StagedLaunch {
	static constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	using K = typename std::conditional<k2d, AsRows<Op>, Op>::type;
	static constexpr int BX = k2d ? 256 : 32, BY = k2d ? 1 : 8, KC = k2d ? 64 : 16;
	using M = typename Rep<N, S>::M;
	static constexpr size_t smem() { return (size_t)Ring<K, BX, BY>::total() * sizeof(M); }
	static constexpr bool occ4 = StagedOcc4<Op>::value;
	static const void* func() {
		if constexpr (occ4) return (const void*)staged3d_kernel_occ4<K, N, S, BX, BY, KC>;
		else return (const void*)staged3d_kernel<K, N, S, BX, BY, KC>;
	}
	static cudaError_t run(const Op& op, const kg_problem& pr, cudaStream_t st) {
		constexpr Slots sl = Op::slots();
		Ptrs<S> p{};
		for (int q = 0; q < sl.nin; q++) p.in[q] = (const S*)pr.arr[sl.in[q]];
		for (int q = 0; q < sl.nout; q++) p.out[q] = (S*)pr.arr[sl.out[q]];
		// 2D: (nx, ny) runs as (nx, 1, ny)
		const int nx = pr.nx, ny = k2d ? 1 : pr.ny, ns = k2d ? pr.ny : pr.ns;
		const int dx = nx - K::LX - K::HX, dy = ny - K::LY - K::HY, dz = ns - K::LZ - K::HZ;
		if (dx <= 0 || dy <= 0 || dz <= 0) return cudaSuccess;
		constexpr size_t bytes = smem();
		static_assert(bytes <= 200 * 1024, "halo tiles exceed shared memory");
		if (bytes > 48 * 1024) {
			// the opt-in is a per-device setting of the function: once per
			// device (host threads may race to set it; setting it twice is
			// harmless, and the flag itself is atomic)
			static std::atomic<bool> set_on[64];
			int dev = 0;
			cudaError_t e = cudaGetDevice(&dev);
			if (e != cudaSuccess) return e;
			if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
			if (!set_on[dev].load(std::memory_order_acquire)) {
				e = cudaFuncSetAttribute(func(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
				if (e != cudaSuccess) return e;
				set_on[dev].store(true, std::memory_order_release);
			}
		}
		K kop;
		if constexpr (k2d) kop.op = op;
		else kop = op;
		dim3 block(BX, BY, 1);
		dim3 grid((dx + BX - 1) / BX, (unsigned)min((dy + BY - 1) / BY, 65535), (unsigned)min((dz + KC - 1) / KC, 65535));
		if constexpr (occ4) staged3d_kernel_occ4<K, N, S, BX, BY, KC><<<grid, block, bytes, st>>>(kop, p, nx, ny, ns);
		else staged3d_kernel<K, N, S, BX, BY, KC><<<grid, block, bytes, st>>>(kop, p, nx, ny, ns);
		return cudaGetLastError();
	}
};

}  // namespace kg
