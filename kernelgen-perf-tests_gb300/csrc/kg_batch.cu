// kg_batch.cu -- many independent problems of uneven sizes and mixed stencils
// advanced together: one persistent launch per time step.
//
// Layout.  A device table holds one descriptor per problem (stencil, sizes,
// coefficients, its arrays in their original roles, its tile counts and the
// index of its first tile in the global tile list).  The launch has
// ctas_per_sm x #SMs CTAs; CTA b takes tiles b, b + gridDim.x, ... of the
// global list, finds the owning problem by binary search over the prefix
// offsets (kept in shared memory) and runs that stencil's tile body -- the
// same body the single-problem sweeps use, so every problem's result equals
// its own kg_sweep bit for bit.
//
// Roles.  Array roles rotate with the step number as the reference loops
// rotate their pointers (two-buffer swap; wave13pt's three levels; none for
// divergence).  The step number lives on the device: each launch reads the
// base and adds its position in the sequence, and a one-thread kernel after
// the sequence advances the base, so a captured N-step graph can be replayed
// and continue where it stopped.
//
// Temporal tiles.  With a temporal factor T > 1 one launch advances every
// problem T steps: a CTA loads a block of the step's input expanded by T
// stencil radii into shared memory (with the rims of the other time levels
// where the block touches the domain's edge), evaluates the T steps there on
// regions that shrink by one radius per step (the halo points are evaluated
// redundantly by the neighbouring blocks), and writes the block of the time
// levels the next launch reads; so a value crosses HBM about twice per T
// steps instead of twice per step.  Each point is evaluated by the same body
// as the single-problem sweeps, so the results are those of T sweeps, bit for
// bit.  divergence (whose inputs never change) is evaluated T times from
// global memory.
//
// Tuning.  The tile shape (BX x BY x KC, or an output block and T) and the
// CTAs per SM are chosen by timing every candidate on the batch itself
// (kg_batch_tune); the choice is cached in a text file keyed by the device
// and a hash of the problem list.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <algorithm>

// the batch's small tiles are latency-bound: every sum on the FP64 unit
#define KG_SUMS_ON_FP64_UNIT 1
#include "kg_engine.cuh"
#include "kg_internal.h"
#include "kg_tma.cuh"

namespace kg {

constexpr int kBatchMax = 4096;

struct BatchDesc {
	int stencil, nx, ny, ns;
	int tiles_x, tiles_y, tiles_z, first;
	double c[8];          // coefficients in the compute type's precision (as double)
	void* a[4];           // arrays in their original roles
	void* b[4];           // temporal tiles: a second set of the rotating arrays
};

// Roles of the arrays of problem d at time step `step`.
template <class S>
__device__ __forceinline__ void batch_roles(const BatchDesc& d, long long step, Ptrs<S>& p)
{
	switch (d.stencil) {
	case KG_LAPLACIAN: case KG_GAUSSBLUR: {
		const int r = (int)(step & 1);
		p.in[0] = (const S*)d.a[r];
		p.out[0] = (S*)d.a[r ^ 1];
		break;
	}
	case KG_WAVE13PT: {
		const int r = (int)(step % 3);
		p.in[0] = (const S*)d.a[r];
		p.in[1] = (const S*)d.a[(r + 1) % 3];
		p.out[0] = (S*)d.a[(r + 2) % 3];
		break;
	}
	case KG_DIVERGENCE:
	default:
		p.out[0] = (S*)d.a[0];
		p.in[0] = (const S*)d.a[1];
		p.in[1] = (const S*)d.a[2];
		p.in[2] = (const S*)d.a[3];
		break;
	}
}

// One tile of a batch problem.  The (i, j) columns of the update domain are
// numbered row by row and a tile takes NT consecutive ones (3D: each thread
// then walks KC planes of its column; 2D: KC points NT apart), so tiles of
// narrow problems are not cut at every row end: only the last tile of a
// plane runs partly idle.
template <class Op, class N, class S, int NT, int KC, int UK>
__device__ __forceinline__ void sweep_lin(const Op& op, const Ptrs<S>& p, int nx, int ny, int ns, int tcol, int tz)
{
	constexpr Slots sl = Op::slots();
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	const int tid = threadIdx.x + threadIdx.y * blockDim.x;
	const int dxn = nx - Op::LX - Op::HX, dyn = ny - Op::LY - Op::HY;
	const long long ncol = (long long)dxn * dyn;
	const long long sy = nx, sz = (long long)nx * ny;
	if (k2d) {
#pragma unroll 1
		for (int r = 0; r < KC; r++) {
			const long long col = ((long long)tcol * KC + r) * NT + tid;
			if (col >= ncol) break;
			const int j = Op::LY + (int)(col / dxn), i = Op::LX + (int)(col - (col / dxn) * dxn);
			const long long c = i + sy * j;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	} else {
		const long long col = (long long)tcol * NT + tid;
		if (col >= ncol) return;
		const int j = Op::LY + (int)(col / dxn), i = Op::LX + (int)(col - (col / dxn) * dxn);
		const int k0 = Op::LZ + tz * KC, k1 = min(k0 + KC, ns - Op::HZ);
#pragma unroll UK
		for (int k = k0; k < k1; k++) {
			const long long c = i + sy * j + sz * k;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	}
}

// Registers capped for 2048 resident threads per SM (32 per thread; a few
// spill): the batch's small tiles are bound by load latency, and the extra
// warps hide it.  Measured on 256 FP32 problems (Gpts/s, best tile shape and
// CTAs per SM): 188 uncapped (40 registers, 6 CTAs of 256 threads), 282
// capped.
template <class N, class S, int BX, int BY, int KC>
__global__ void __launch_bounds__(BX * BY, 2048 / (BX * BY)) batch_kernel(const BatchDesc* __restrict__ desc, int nprob,
	int total, const long long* __restrict__ step_base, int local)
{
	constexpr int NT = BX * BY;
	__shared__ int first[kBatchMax + 1];
	for (int q = threadIdx.x + threadIdx.y * BX; q < nprob; q += BX * BY) first[q] = desc[q].first;
	__syncthreads();
	const long long step = *step_base + local;
	for (int item = blockIdx.x; item < total; item += gridDim.x) {
		int lo = 0, hi = nprob - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (first[mid] <= item) lo = mid;
			else hi = mid - 1;
		}
		const BatchDesc& d = desc[lo];
		const int t = item - d.first;
		const int tcol = t % d.tiles_x, tz = t / d.tiles_x;
		Ptrs<S> p{};
		batch_roles<S>(d, step, p);
		switch (d.stencil) {
		case KG_LAPLACIAN:
			sweep_lin<OpLaplacian<N>, N, S, NT, KC, 4>(OpLaplacian<N>{N(d.c[0]), N(d.c[1])}, p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_DIVERGENCE:
			sweep_lin<OpDivergence<N>, N, S, NT, KC, 4>(OpDivergence<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])},
				p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_WAVE13PT:
			sweep_lin<OpWave13pt<N>, N, S, NT, KC, 4>(OpWave13pt<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])},
				p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_GAUSSBLUR:
			sweep_lin<OpGaussblur<N>, N, S, NT, KC, 4>(OpGaussblur<N>{N(d.c[0]), N(d.c[1]), N(d.c[2]),
				N(d.c[3]), N(d.c[4]), N(d.c[5]), N(d.c[6])}, p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		default: break;
		}
	}
}

// ---- temporal tiles ----------------------------------------------------------
//
// A launch of T steps reads the time levels from one set of arrays and writes
// them to the other (the problem's own arrays a[] or its second set b[]):
// blocks of other CTAs still read the levels a block has advanced, so the
// levels cannot be written in place.  The host orders the launches of a
// sequence so that the last one writes the problem's own arrays, and copies
// the rims of the rotating arrays into the second set first (the sweeps never
// write rims, and a level is read at its rims by the blocks at the domain's
// edge).

constexpr int kTBThreads = 256;

// Bytes of the first-tile table at the start of the temporal kernel's
// dynamic shared memory (16-byte multiple).
__host__ __device__ __forceinline__ int tb_first_bytes(int nprob) { return ((nprob + 1) * 4 + 15) / 16 * 16; }

// Output block (bx x by x bz points; 2D problems: bx x (by bz) rows) and the
// steps per launch.
struct TBShape { int bx, by, bz, t; };

__device__ __forceinline__ void cp_async_elem(void* dst_smem, const void* src, int bytes)
{
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
	if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
	else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
	asm volatile("cp.async.wait_all;" ::: "memory");
}

// A box [x0, x0+ex) x [y0, y0+ey) x [z0, z0+ez) of array coordinates.
struct TBBox {
	int x0, y0, z0, ex, ey, ez;
	__device__ __forceinline__ int n() const { return ex * ey * ez; }
};

// b grown by (rx, ry, rz) on every side, clipped to [lx, hx) x [ly, hy) x [lz, hz).
__device__ __forceinline__ TBBox tb_grow(const TBBox& b, int rx, int ry, int rz, int lx, int ly, int lz, int hx,
	int hy, int hz)
{
	TBBox o;
	o.x0 = max(lx, b.x0 - rx);
	o.y0 = max(ly, b.y0 - ry);
	o.z0 = max(lz, b.z0 - rz);
	o.ex = min(hx, b.x0 + b.ex + rx) - o.x0;
	o.ey = min(hy, b.y0 + b.ey + ry) - o.y0;
	o.ez = min(hz, b.z0 + b.ez + rz) - o.z0;
	return o;
}

// Reads of a body evaluated on shared-memory time levels: input q is level
// lev[q], element c of the region is the point, (sy, sz) the region strides.
template <class N, class S> struct TBAcc {
	const S* lev[2];
	int c, sy, sz;
	__device__ __forceinline__ N operator()(int q, int dx, int dy, int dz) const {
		return Conv<N, S>::from(lev[q][c + dx + dy * sy + dz * sz]);
	}
	__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const { return lev[q][c + dx + dy * sy + dz * sz]; }
};

// Stores of the box `b` of a level (region R in shared memory) to the global array dst.
template <class S>
__device__ __forceinline__ void tb_store(S* dst, const S* src, const TBBox& R, const TBBox& b, int nx, int ny)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	for (int row = warp; row < b.ey * b.ez; row += kTBThreads / 32) {
		const int z = row / b.ey, y = row - z * b.ey;
		const int gy = b.y0 + y, gz = b.z0 + z;
		const S* s = src + ((gz - R.z0) * R.ey + (gy - R.y0)) * R.ex + (b.x0 - R.x0);
		S* d = dst + b.x0 + (long long)nx * (gy + (long long)ny * gz);
		for (int x = lane; x < b.ex; x += 32) d[x] = s[x];
	}
}

// Shared memory (elements of S) the blocks of a shape need for problems of
// a stencil: NLEV levels of the output block grown by T radii.
inline long long tb_smem_elems(int stencil, const TBShape& sh, int T)
{
	const bool k2d = stencil == KG_GAUSSBLUR;
	const int r = stencil == KG_LAPLACIAN ? 1 : 2;
	const int nlev = stencil == KG_WAVE13PT ? 3 : 2;
	if (stencil == KG_DIVERGENCE) return 0;
	const long long ex = sh.bx + 2 * r * T;
	const long long ey = (k2d ? sh.by * sh.bz : sh.by) + 2 * r * T;
	const long long ez = k2d ? 1 : sh.bz + 2 * r * T;
	return nlev * ex * ey * ez;
}

// T steps of one output block of a problem of Op with NLEV rotating time
// levels (2: the two-buffer swap; 3: wave13pt's levels).  Level i of the
// shared memory mirrors array (g + i) % NLEV of the set read (rd) over the
// region R (the block grown by T radii, clipped to the array); the levels the
// first step reads are loaded whole, the others only where R leaves the
// update domain (their rims).  Step s evaluates the block grown by T-1-s
// radii (clipped to the domain) from level s and writes level s + NLEV - 1.
// Then the block of every level the next launch reads goes to the set
// written (wr); with all_levels, every level (the arrays as the reference
// loop leaves them after the steps).
template <class Op, class N, class S, int NLEV>
__device__ void tb_block(const Op& op, const BatchDesc& d, void* const* rd, void* const* wr, long long g, int tile,
	int T, const TBShape& sh, S* sm, bool all_levels)
{
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	constexpr int r = Op::LX;   // the batch's ops reach r = LX = HX = LY = HY (= LZ = HZ) points
	const int nx = d.nx, ny = d.ny, ns = d.ns;
	const int DX0 = Op::LX, DX1 = nx - Op::HX, DY0 = Op::LY, DY1 = ny - Op::HY;
	const int DZ0 = Op::LZ, DZ1 = ns - Op::HZ;
	const int bz = k2d ? 1 : sh.bz, by = k2d ? sh.by * sh.bz : sh.by;
	const int tx = (DX1 - DX0 + sh.bx - 1) / sh.bx, ty = (DY1 - DY0 + by - 1) / by;
	const int ix = tile % tx, iy = (tile / tx) % ty, iz = tile / (tx * ty);
	TBBox O;
	O.x0 = DX0 + ix * sh.bx;
	O.y0 = DY0 + iy * by;
	O.z0 = DZ0 + iz * bz;
	O.ex = min(sh.bx, DX1 - O.x0);
	O.ey = min(by, DY1 - O.y0);
	O.ez = min(bz, DZ1 - O.z0);
	const int rz = k2d ? 0 : r;
	const TBBox R = tb_grow(O, r * T, r * T, rz * T, 0, 0, 0, nx, ny, ns);
	const int RN = R.n();
	const bool inside = R.x0 >= DX0 && R.x0 + R.ex <= DX1 && R.y0 >= DY0 && R.y0 + R.ey <= DY1 &&
		R.z0 >= DZ0 && R.z0 + R.ez <= DZ1;
	constexpr int nin0 = NLEV - 1;   // levels the first step reads
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll 1
	for (int l = 0; l < NLEV; l++) {
		if (l >= nin0 && inside) continue;
		const S* src = (const S*)rd[(int)((g + l) % NLEV)];
		S* lev = sm + l * RN;
		for (int row = warp; row < R.ey * R.ez; row += kTBThreads / 32) {
			const int z = row / R.ey, y = row - z * R.ey;
			const int gy = R.y0 + y, gz = R.z0 + z;
			const bool row_rim = gy < DY0 || gy >= DY1 || gz < DZ0 || gz >= DZ1;
			const S* srow = src + (long long)nx * (gy + (long long)ny * gz);
			for (int x = lane; x < R.ex; x += 32) {
				const int gx = R.x0 + x;
				if (l < nin0 || row_rim || gx < DX0 || gx >= DX1)
					cp_async_elem(lev + row * R.ex + x, srow + gx, (int)sizeof(S));
			}
		}
	}
	cp_async_wait_all();
	__syncthreads();
	const int sy = R.ex, szr = R.ex * R.ey;
	for (int st = 0; st < T; st++) {
		const int grow = T - 1 - st;
		const TBBox E = tb_grow(O, r * grow, r * grow, rz * grow, DX0, DY0, DZ0, DX1, DY1, DZ1);
		const S* in0 = sm + (st % NLEV) * RN;
		const S* in1 = sm + ((st + 1) % NLEV) * RN;
		S* out = sm + ((st + NLEV - 1) % NLEV) * RN;
		const int pe = E.ex * E.ey;
		const float inv_ex = 1.0f / (float)E.ex;
		for (int z = 0; z < E.ez; z++) {
			const int cz = (E.z0 - R.z0 + z) * szr + (E.y0 - R.y0) * sy + (E.x0 - R.x0);
			for (int p = threadIdx.x; p < pe; p += kTBThreads) {
				// p / E.ex through FP32: p + 1/2 lies at least 1 / (2 E.ex) from
				// a multiple of E.ex, far beyond FP32's rounding at these sizes
				const int y = __float2int_rz(((float)p + 0.5f) * inv_ex);
				const int x = p - y * E.ex;
				const int c = cz + y * sy + x;
				TBAcc<N, S> at{{in0, in1}, c, sy, szr};
				N o[3];
				op.point(at, o);
				out[c] = Conv<N, S>::to(o[0]);
			}
		}
		__syncthreads();
	}
	// level l holds array (g + l) % NLEV after the steps; the next launch
	// reads levels T .. T + nin0 - 1 (mod NLEV)
	const int nw = all_levels ? NLEV : nin0;
#pragma unroll 1
	for (int b = 0; b < nw; b++) {
		const int l = (T + b) % NLEV;
		tb_store<S>((S*)wr[(int)((g + l) % NLEV)], sm + l * RN, R, O, nx, ny);
	}
	__syncthreads();
}

// divergence: T evaluations of the block from global memory (its inputs
// never change, so each step writes the same values to the same array).
template <class N, class S>
__device__ void tb_divergence(const BatchDesc& d, int tile, int T, const TBShape& sh)
{
	using Op = OpDivergence<N>;
	const Op op{N(d.c[0]), N(d.c[1]), N(d.c[2])};
	const int nx = d.nx, ny = d.ny, ns = d.ns;
	const int dxn = nx - 2, dyn = ny - 2, dzn = ns - 2;
	const int tx = (dxn + sh.bx - 1) / sh.bx, ty = (dyn + sh.by - 1) / sh.by;
	const int ix = tile % tx, iy = (tile / tx) % ty, iz = tile / (tx * ty);
	const int x0 = 1 + ix * sh.bx, y0 = 1 + iy * sh.by, z0 = 1 + iz * sh.bz;
	const int ex = min(sh.bx, 1 + dxn - x0), ey = min(sh.by, 1 + dyn - y0), ez = min(sh.bz, 1 + dzn - z0);
	Ptrs<S> p{};
	p.out[0] = (S*)d.a[0];
	p.in[0] = (const S*)d.a[1];
	p.in[1] = (const S*)d.a[2];
	p.in[2] = (const S*)d.a[3];
	const long long sy = nx, sz = (long long)nx * ny;
	const int pe = ex * ey * ez;
	for (int st = 0; st < T; st++)
		for (int q = threadIdx.x; q < pe; q += kTBThreads) {
			const int z = q / (ex * ey), rem = q - z * ex * ey, y = rem / ex, x = rem - y * ex;
			const long long c = (x0 + x) + sy * (y0 + y) + sz * (z0 + z);
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
			p.out[0][c] = Conv<N, S>::to(o[0]);
		}
}

// One launch of T steps over the blocks of every problem: read_b selects the
// set read (0: the problems' own arrays, 1: the second set); the other set
// is written.
template <class N, class S>
__global__ void __launch_bounds__(kTBThreads) batch_tb_kernel(const BatchDesc* __restrict__ desc, int nprob, int total,
	const long long* __restrict__ step_base, int local, int T, TBShape sh, int read_b, int all_levels)
{
	// dynamic shared memory: the problems' first tiles, then the time levels
	extern __shared__ __align__(16) unsigned char tb_smem[];
	int* first = reinterpret_cast<int*>(tb_smem);
	S* sm = reinterpret_cast<S*>(tb_smem + tb_first_bytes(nprob));
	for (int q = threadIdx.x; q < nprob; q += kTBThreads) first[q] = desc[q].first;
	__syncthreads();
	const long long g = *step_base + local;
	for (int item = blockIdx.x; item < total; item += gridDim.x) {
		int lo = 0, hi = nprob - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (first[mid] <= item) lo = mid;
			else hi = mid - 1;
		}
		const BatchDesc& d = desc[lo];
		const int t = item - d.first;
		void* const* rd = read_b ? d.b : d.a;
		void* const* wr = read_b ? d.a : d.b;
		switch (d.stencil) {
		case KG_LAPLACIAN:
			tb_block<OpLaplacian<N>, N, S, 2>(OpLaplacian<N>{N(d.c[0]), N(d.c[1])}, d, rd, wr, g, t, T, sh, sm,
				all_levels != 0);
			break;
		case KG_GAUSSBLUR:
			tb_block<OpGaussblur<N>, N, S, 2>(OpGaussblur<N>{N(d.c[0]), N(d.c[1]), N(d.c[2]), N(d.c[3]), N(d.c[4]),
				N(d.c[5]), N(d.c[6])}, d, rd, wr, g, t, T, sh, sm, all_levels != 0);
			break;
		case KG_WAVE13PT:
			tb_block<OpWave13pt<N>, N, S, 3>(OpWave13pt<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])}, d, rd, wr, g, t, T, sh,
				sm, all_levels != 0);
			break;
		case KG_DIVERGENCE:
			tb_divergence<N, S>(d, t, T, sh);
			break;
		default: break;
		}
	}
}

// The rims (points outside the update domain; with `all`, every point) of
// the rotating arrays of every problem copied from its own arrays into its
// second set: CTAs per (problem, group of planes).
template <class S>
__global__ void batch_rim_copy(const BatchDesc* __restrict__ desc, int nprob, int all)
{
	for (int q = blockIdx.x; q < nprob; q += gridDim.x) {
		const BatchDesc& d = desc[q];
		int narr, r, k2d = 0;
		switch (d.stencil) {
		case KG_LAPLACIAN: narr = 2; r = 1; break;
		case KG_GAUSSBLUR: narr = 2; r = 2; k2d = 1; break;
		case KG_WAVE13PT: narr = 3; r = 2; break;
		default: continue;
		}
		const int nx = d.nx, ny = d.ny, ns = d.ns;
		const int rz = k2d ? 0 : r;
		for (int z = blockIdx.y; z < ns; z += gridDim.y) {
			const bool zrim = z < rz || z >= ns - rz;
			for (int e = threadIdx.x; e < nx * ny; e += blockDim.x) {
				const int y = e / nx, x = e - y * nx;
				if (!all && !(zrim || y < r || y >= ny - r || x < r || x >= nx - r)) continue;
				const long long c = e + (long long)nx * ny * z;
				for (int k = 0; k < narr; k++) ((S*)d.b[k])[c] = ((const S*)d.a[k])[c];
			}
		}
	}
}

// ---- bulk-staged tiles ---------------------------------------------------------
//
// The one-step tile of the batch (NT consecutive (i, j) columns of a problem,
// KC planes; 2D: KC groups of NT columns), with its inputs staged in shared
// memory by bulk copies instead of read through L1.  The NT columns of a
// plane lie in one contiguous range of the array, grown by the input's reach
// (x0 + y0 nx before, x1 + y1 nx after): one 1D bulk copy per input and plane
// (cp.async.bulk, 16-byte aligned, rounded out to 16 bytes and never past the
// array's last whole 16 bytes).  A producer warp issues each step's copies
// kBulkL steps ahead of the compute warps, onto an mbarrier per step (as the
// TMA engine does, with its bounded waits and drain); each input keeps a ring
// of NZ + kBulkL plane ranges.  The batch's small problems are bound by the
// latency of their loads; the copies put several steps of loads in flight
// without taking registers.  A step whose range the array's end cut short
// reads its inputs from global memory instead (the last up to 15 bytes of an
// array).  Every point is the same body as the other engines evaluate.

// Steps of copies in flight.  Measured on the 256-problem FP32 batch: 2
// steps make the rings small enough for 3 resident CTAs per SM, but the best
// configuration is no faster (394 against 396 Gpts/s).
#ifndef KG_BULK_L
#define KG_BULK_L 3
#endif
constexpr int kBulkL = KG_BULK_L;
constexpr int kBulkNB = kBulkL + 1;    // mbarriers per direction
constexpr int kBulkBar = 128;          // bytes: 2 x kBulkNB mbarriers, the abort flag

// Shared-memory rings of one stencil's inputs: elements per slot, byte offset.
struct BulkRings {
	int cap[4];
	int off[4];
};
struct BulkLayout {
	BulkRings k[4];    // laplacian, divergence, wave13pt, gaussblur (stencil ids 0, 1, 4, 9)
};
__host__ __device__ __forceinline__ int bulk_kind(int stencil)
{
	return stencil == KG_LAPLACIAN ? 0 : stencil == KG_DIVERGENCE ? 1 : stencil == KG_WAVE13PT ? 2 : 3;
}

__device__ __forceinline__ void bulk_copy(void* dst_smem, const void* src, unsigned bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		::"r"(smem_addr(dst_smem)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// The bulk kernel's dynamic shared memory (the first-tile table, then the
// mbarriers and the rings): named at file scope so that the tile code's
// reads are shared-memory loads with 32-bit offsets.
extern __shared__ __align__(128) unsigned char bk_smem[];

// One item (tile) of the batch as the bulk kernel walks it: NC = NT CPT
// consecutive interior columns per step (each thread takes CPT of them, NT
// apart); 3D: the same columns on KC planes; 2D: KC groups of NC columns.
// The bulk path takes problems of fewer than 2^31 - 2^16 points, so every
// index of an item (and its sums with a step's columns) is a 32-bit int.
template <class Op> struct BulkItem {
	static constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	int nx, ny, ns, dxn, ncol, col0, P, kb, nsteps;
	__device__ __forceinline__ void init(const BatchDesc& d, int t, int NC, int KC) {
		nx = d.nx;
		ny = d.ny;
		ns = d.ns;
		dxn = nx - Op::LX - Op::HX;
		ncol = dxn * (ny - Op::LY - Op::HY);
		P = nx * ny;
		const int tcol = t % d.tiles_x, tz = t / d.tiles_x;
		if (k2d) {
			col0 = tcol * KC * NC;
			kb = 0;
			nsteps = min(KC, (ncol - col0 + NC - 1) / NC);
		} else {
			col0 = tcol * NC;
			kb = Op::LZ + tz * KC;
			nsteps = min(KC, ns - Op::HZ - kb);
		}
	}
	// full index (in its plane) of interior column col
	__device__ __forceinline__ int f(int col) const {
		const int j = col / dxn;
		return Op::LX + (col - j * dxn) + nx * (Op::LY + j);
	}
};

// A column of a 2D item and its full index, moved NC columns on per step
// without a division: NC = qd dxn + rd, so a step adds rd to the column's x
// offset and qd rows, and one more row where x passes the row's end.
struct ColWalk {
	int col, i, fc;   // interior column, its x offset in the row, full index
	template <class Op> __device__ __forceinline__ void start(const BulkItem<Op>& it, int c) {
		const int j = c / it.dxn;
		col = c;
		i = c - j * it.dxn;
		fc = Op::LX + i + it.nx * (Op::LY + j);
	}
	__device__ __forceinline__ void step(int NC, int rd, int fq, int dxn, int wrap) {
		col += NC;
		i += rd;
		fc += fq;
		if (i >= dxn) {
			i -= dxn;
			fc += wrap;
		}
	}
};

// The chunk of input q of Op for a step: the element range [st, st + count)
// it copies, the 16-byte phase of its first needed element, and whether the
// array's end cut it short.
template <class Op, class S> struct BulkChunk {
	int st, count, phase;
	bool cut;
	__device__ __forceinline__ void make(int q, int fl, int fh, int pbase, int nx, int n) {
		constexpr int A = 16 / (int)sizeof(S);
		const Halo h = Op::halo(q);
		const int lo = fl - (h.x0 + h.y0 * nx) + pbase;
		const int end = fh + h.x1 + h.y1 * nx + 1 + pbase;   // exclusive
		const int nfl = n & ~(A - 1);
		phase = lo & (A - 1);
		st = lo - phase;
		const int e = min((end + A - 1) & ~(A - 1), nfl);
		count = max(0, e - st);
		cut = end > nfl || count == 0;
	}
};

template <class Op, class N, class S, int NT, int CPT, int KC>
__device__ __forceinline__ void bulk_item(const Op& op, const BatchDesc& d, int t, const Ptrs<S>& p,
	const BulkRings& rg, unsigned char* sm, int rbase, uint64_t* full, uint64_t* done, volatile int* abort,
	uint32_t& g, bool producer, int* err, long long wait, bool& ok)
{
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	constexpr Slots sl = Op::slots();
	constexpr int NIN = sl.nin;
	constexpr int ES = (int)sizeof(S);
	constexpr int A = 16 / ES;
	constexpr int NC = NT * CPT;
	BulkItem<Op> it;
	it.init(d, t, NC, KC);
	const int n = it.P * it.ns;
	auto NZ = [](int q) { return k2d ? 1 : Op::halo(q).z0 + Op::halo(q).z1 + 1; };
	auto RZ = [](int q) { return (k2d ? 1 : Op::halo(q).z0 + Op::halo(q).z1 + 1) + kBulkL; };
	// the steps' first and last columns: fixed in 3D; in 2D walked NC
	// columns on per step (the last step's last column is the domain's)
	const int qd = NC / it.dxn, rd = NC - qd * it.dxn;
	const int fq = rd + qd * it.nx, wrap = it.nx - it.dxn;
	ColWalk wl, wh;
	int fl = 0, fh = 0, flast = 0;
	if (k2d) {
		wl.start(it, it.col0);
		wh.start(it, it.col0 + NC - 1);
		flast = it.f(it.ncol - 1);
	} else {
		fl = it.f(it.col0);
		fh = it.f(min(it.col0 + NC, it.ncol) - 1);
	}
	if (producer) {
		// a new item's windows may reuse any slot: wait for the previous item
		if (g > 0 && ok) ok = mbar_wait(&done[(g - 1) % kBulkNB], ((g - 1) / kBulkNB) & 1, kTmaWaitCycles, abort);
		uint32_t issued = g;
		for (int s = 0; s < it.nsteps && ok; s++) {
			const uint32_t gs = g + s;
			if (s >= kBulkL + 1)
				ok = mbar_wait(&done[(gs - kBulkL - 1) % kBulkNB], ((gs - kBulkL - 1) / kBulkNB) & 1, kTmaWaitCycles, abort);
			if (!ok) break;
			if (k2d) {
				fl = wl.fc;
				fh = wh.col < it.ncol ? wh.fc : flast;
			}
			const int k = it.kb + s;
			// planes of this step: the window at the first step, then the
			// newest; the byte count first, then the copies
			unsigned bytes = 0;
#pragma unroll
			for (int q = 0; q < NIN; q++) {
				const Halo h = Op::halo(q);
				const int p0 = k2d ? 0 : (s == 0 ? k - h.z0 : k + h.z1);
				const int np = k2d ? 1 : (s == 0 ? NZ(q) : 1);
				for (int m = 0; m < np; m++) {
					BulkChunk<Op, S> ch;
					ch.make(q, fl, fh, k2d ? 0 : (p0 + m) * it.P, it.nx, n);
					bytes += (unsigned)ch.count * ES;
				}
			}
			mbar_expect_tx(&full[gs % kBulkNB], bytes);
			fence_proxy_async();
#pragma unroll
			for (int q = 0; q < NIN; q++) {
				const Halo h = Op::halo(q);
				const int p0 = k2d ? 0 : (s == 0 ? k - h.z0 : k + h.z1);
				const int np = k2d ? 1 : (s == 0 ? NZ(q) : 1);
				for (int m = 0; m < np; m++) {
					BulkChunk<Op, S> ch;
					ch.make(q, fl, fh, k2d ? 0 : (p0 + m) * it.P, it.nx, n);
					const int slot = (k2d ? s : p0 + m) % RZ(q);
					if (ch.count > 0)
						bulk_copy(sm + rg.off[q] + slot * rg.cap[q] * ES, p.in[q] + ch.st, (unsigned)ch.count * ES,
							&full[gs % kBulkNB]);
				}
			}
			issued = gs + 1;
			if (k2d) {
				wl.step(NC, rd, fq, it.dxn, wrap);
				wh.step(NC, rd, fq, it.dxn, wrap);
			}
		}
		if (!ok) {
			// every step before the last kBulkNB issued is done; the copies of
			// those land before the CTA's shared memory goes away
			atomicExch(err, 1);
			for (uint32_t w = issued > kBulkNB ? issued - kBulkNB : 0; w < issued; w++)
				mbar_wait(&full[w % kBulkNB], (w / kBulkNB) & 1, kTmaWaitCycles);
		}
		g += it.nsteps;
		return;
	}
	// ---- compute warps ----
	const int tid = threadIdx.x, lane = tid & 31;
	const int pm = it.P & (A - 1);
	const int nxes = it.nx * ES;
	// the thread's columns: 3D fixed for the item; 2D walked with the steps
	// (a column past the domain is evaluated at the step's first column and
	// not stored)
	ColWalk wc[CPT];
	int fc[CPT];
	bool cv[CPT];
	bool item_cut = false;
	// per input: byte offset of the chunk of the newest plane for full index
	// fl (all but the ring slot and the 16-byte phase), the newest plane's
	// slot and phase, and the offsets of the NZ planes of the step
	int qb[6], nsl[6], nph[6];
	int b[6][5];
#pragma unroll
	for (int q = 0; q < NIN; q++) {
		const Halo h = Op::halo(q);
		qb[q] = rbase + rg.off[q] + (h.x0 + h.y0 * it.nx) * ES;
	}
	if (!k2d) {
#pragma unroll
		for (int r = 0; r < CPT; r++) {
			const int col = it.col0 + tid + r * NT;
			cv[r] = col < it.ncol;
			fc[r] = it.f(cv[r] ? col : it.col0);
		}
#pragma unroll
		for (int q = 0; q < NIN; q++) {
			const Halo h = Op::halo(q);
			BulkChunk<Op, S> ch;
			ch.make(q, fl, fh, (it.kb + it.nsteps - 1 + h.z1) * it.P, it.nx, n);
			item_cut = item_cut || ch.cut;
			// the planes of step 0: kb - z0 .. kb + z1
			const int lob = fl - (h.x0 + h.y0 * it.nx);
#pragma unroll
			for (int m = 0; m < 5; m++) {
				if (m >= NZ(q)) continue;
				const int pl = it.kb - h.z0 + m;
				nph[q] = (lob + pl * pm) & (A - 1);
				nsl[q] = pl % RZ(q);
				b[q][m] = qb[q] + (nsl[q] * rg.cap[q] + nph[q]) * ES;
			}
		}
	} else {
#pragma unroll
		for (int r = 0; r < CPT; r++) wc[r].start(it, it.col0 + tid + r * NT);
	}
	for (int s = 0; s < it.nsteps; s++) {
		const uint32_t gs = g + s;
		const bool got = __all_sync(0xffffffffu, mbar_wait(&full[gs % kBulkNB], (gs / kBulkNB) & 1, wait, abort));
		if (!got) {
			if (lane == 0) {
				*abort = 1;
				atomicExch(err, 1);
			}
			ok = false;
			return;
		}
		bool cut = item_cut;
		if (k2d) {
			fl = wl.fc;
			fh = wh.col < it.ncol ? wh.fc : flast;
#pragma unroll
			for (int r = 0; r < CPT; r++) {
				cv[r] = wc[r].col < it.ncol;
				fc[r] = cv[r] ? wc[r].fc : fl;
			}
			const int slot = s % RZ(0);
#pragma unroll
			for (int q = 0; q < NIN; q++) {
				const Halo h = Op::halo(q);
				BulkChunk<Op, S> ch;
				ch.make(q, fl, fh, 0, it.nx, n);
				cut = cut || ch.cut;
				b[q][0] = qb[q] + (slot * rg.cap[q] + ch.phase) * ES;
			}
		}
		const long long pk = k2d ? 0 : (long long)(it.kb + s) * it.P;
		N o[CPT][3];
		if (!cut) {
			// input q's value at column fc, offset (dx, dy, dz), lies at byte
			// b[q][dz + z0] + (fc - fl) ES + dx ES + dy nx ES of the dynamic
			// shared memory
#pragma unroll
			for (int r = 0; r < CPT; r++) {
				struct Acc {
					const int (*b)[5];
					int rel;       // (fc - fl) ES
					int nxes;
					__device__ __forceinline__ N operator()(int q, int dx, int dy, int dz) const {
						return Conv<N, S>::from(raw(q, dx, dy, dz));
					}
					__device__ __forceinline__ S raw(int q, int dx, int dy, int dz) const {
						return *reinterpret_cast<const S*>(bk_smem + (b[q][dz + Op::halo(q).z0] + rel + dx * ES + dy * nxes));
					}
				} at{b, (fc[r] - fl) * ES, nxes};
				op.point(at, o[r]);
			}
		} else {
#pragma unroll
			for (int r = 0; r < CPT; r++) {
				GAcc<N, S> at{p.in, fc[r] + pk, it.nx, it.P};
				op.point(at, o[r]);
			}
		}
		// the step's inputs are read: this warp is done with its planes
		__syncwarp();
		if (lane == 0) mbar_arrive(&done[gs % kBulkNB]);
#pragma unroll
		for (int q = 0; q < sl.nout; q++) {
			S* out = p.out[q] + pk;
#pragma unroll
			for (int r = 0; r < CPT; r++)
				if (cv[r]) out[fc[r]] = Conv<N, S>::to(o[r][q]);
		}
		// the next step's planes: the window moves one plane on
		if (k2d) {
			wl.step(NC, rd, fq, it.dxn, wrap);
			wh.step(NC, rd, fq, it.dxn, wrap);
#pragma unroll
			for (int r = 0; r < CPT; r++) wc[r].step(NC, rd, fq, it.dxn, wrap);
		} else {
#pragma unroll
			for (int q = 0; q < NIN; q++) {
#pragma unroll
				for (int m = 0; m + 1 < 5; m++)
					if (m + 1 < NZ(q)) b[q][m] = b[q][m + 1];
				nsl[q] = nsl[q] + 1 == RZ(q) ? 0 : nsl[q] + 1;
				nph[q] = (nph[q] + pm) & (A - 1);
				b[q][NZ(q) - 1] = qb[q] + (nsl[q] * rg.cap[q] + nph[q]) * ES;
			}
		}
	}
	g += it.nsteps;
}

// Registers bounded for the CTAs per SM the rings leave room for: two of
// 512 compute threads, four of 256 with two columns each, three of 256 with
// four.
constexpr int bulk_min_blocks(int nt, int cpt) { return nt >= 512 ? 2 : cpt <= 2 ? 4 : 3; }
template <class N, class S, int NT, int CPT, int KC>
__global__ void __launch_bounds__(NT + 32, bulk_min_blocks(NT, CPT)) batch_bulk_kernel(const BatchDesc* __restrict__ desc, int nprob, int total,
	const long long* __restrict__ step_base, int local, BulkLayout lay, int* err, long long wait)
{
	int* first = reinterpret_cast<int*>(bk_smem);
	const int rbase = tb_first_bytes(nprob);   // ring offsets count from the mbarriers
	uint64_t* full = reinterpret_cast<uint64_t*>(bk_smem + tb_first_bytes(nprob));
	uint64_t* done = full + kBulkNB;
	volatile int* abort = reinterpret_cast<volatile int*>(reinterpret_cast<unsigned char*>(full) + kBulkBar - 8);
	unsigned char* rings = reinterpret_cast<unsigned char*>(full);   // ring offsets count from here
	for (int q = threadIdx.x; q < nprob; q += blockDim.x) first[q] = desc[q].first;
	if (threadIdx.x == 0) {
		for (int b = 0; b < kBulkNB; b++) {
			mbar_init(&full[b], 1);
			mbar_init(&done[b], NT / 32);
		}
		*abort = 0;
		mbar_fence_init();
	}
	__syncthreads();
	const bool producer = threadIdx.x >= NT;
	if (producer && threadIdx.x != NT) return;
	const long long step = *step_base + local;
	uint32_t g = 0;
	bool ok = true;
	for (int item = blockIdx.x; item < total && ok; item += gridDim.x) {
		int lo = 0, hi = nprob - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (first[mid] <= item) lo = mid;
			else hi = mid - 1;
		}
		const BatchDesc& d = desc[lo];
		const int t = item - d.first;
		Ptrs<S> p{};
		batch_roles<S>(d, step, p);
		const BulkRings& rg = lay.k[bulk_kind(d.stencil)];
		switch (d.stencil) {
		case KG_LAPLACIAN:
			bulk_item<OpLaplacian<N>, N, S, NT, CPT, KC>(OpLaplacian<N>{N(d.c[0]), N(d.c[1])}, d, t, p, rg, rings, rbase, full, done,
				abort, g, producer, err, wait, ok);
			break;
		case KG_DIVERGENCE:
			bulk_item<OpDivergence<N>, N, S, NT, CPT, KC>(OpDivergence<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])}, d, t, p, rg,
				rings, rbase, full, done, abort, g, producer, err, wait, ok);
			break;
		case KG_WAVE13PT:
			bulk_item<OpWave13pt<N>, N, S, NT, CPT, KC>(OpWave13pt<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])}, d, t, p, rg, rings,
				rbase, full, done, abort, g, producer, err, wait, ok);
			break;
		case KG_GAUSSBLUR:
			bulk_item<OpGaussblur<N>, N, S, NT, CPT, KC>(OpGaussblur<N>{N(d.c[0]), N(d.c[1]), N(d.c[2]), N(d.c[3]),
				N(d.c[4]), N(d.c[5]), N(d.c[6])}, d, t, p, rg, rings, rbase, full, done, abort, g, producer, err, wait, ok);
			break;
		default: break;
		}
	}
	// the producer stays until the compute warps are done with the last step
	if (producer && ok && g > 0) {
		if (!mbar_wait(&done[(g - 1) % kBulkNB], ((g - 1) / kBulkNB) & 1, kTmaWaitCycles, abort)) {
			atomicExch(err, 1);
			for (uint32_t w = g > kBulkNB ? g - kBulkNB : 0; w < g; w++)
				mbar_wait(&full[w % kBulkNB], (w / kBulkNB) & 1, kTmaWaitCycles);
		}
	}
}

__global__ void batch_advance(long long* step_base, int n)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) *step_base += n;
}

// Tile shapes the tuner tries (BX, BY, KC), one step per launch.
struct Shape { int bx, by, kc; };
static const Shape k_shapes[] = {{32, 8, 8}, {32, 4, 8}, {64, 4, 8}, {32, 8, 4}, {32, 8, 16}, {128, 2, 8},
	{32, 8, 32}, {32, 16, 16}, {32, 4, 32}, {32, 8, 64}};
static const int k_nshapes = sizeof(k_shapes) / sizeof(k_shapes[0]);
// Temporal tiles (output block, steps per launch); configuration index
// k_nshapes + i.  A shape whose shared memory a batch's stencils exceed is
// not used for that batch.
static const TBShape k_tb_shapes[] = {{32, 8, 8, 2}, {32, 8, 4, 2}, {32, 4, 4, 2}, {64, 4, 4, 2}, {64, 8, 4, 2},
	{32, 8, 8, 3}, {32, 4, 4, 3}, {64, 4, 4, 3}, {32, 8, 8, 4}, {32, 4, 4, 4}};
static const int k_ntb = sizeof(k_tb_shapes) / sizeof(k_tb_shapes[0]);
// Bulk-staged one-step tiles (NT consecutive columns, KC planes); configuration
// index k_nshapes + k_ntb + i.
struct BulkShape { int nt, cpt, kc; };
static const BulkShape k_bulk_shapes[] = {{256, 4, 32}, {512, 2, 64}, {256, 4, 64}, {512, 2, 32}, {256, 2, 64}, {256, 2, 32}};
static const int k_nbulk = sizeof(k_bulk_shapes) / sizeof(k_bulk_shapes[0]);
static const int k_bulk0 = k_nshapes + k_ntb;
static const int k_nconfigs = k_nshapes + k_ntb + k_nbulk;
static bool is_temporal(int shape) { return shape >= k_nshapes && shape < k_bulk0; }
static bool is_bulk(int shape) { return shape >= k_bulk0; }
// Steps each tuning trial times (a multiple of every temporal factor).
constexpr int kTuneSteps = 12;
constexpr int kSmemOptin = 227 * 1024;

template <class N, class S>
static cudaError_t launch_shape(int shape, dim3 grid, const BatchDesc* desc, int nprob, int total,
	const long long* base, int local, cudaStream_t st)
{
	switch (shape) {
#define KG_SHAPE_CASE(I, BX, BY, KC) \
	case I: batch_kernel<N, S, BX, BY, KC><<<grid, dim3(BX, BY), 0, st>>>(desc, nprob, total, base, local); break;
	KG_SHAPE_CASE(0, 32, 8, 8)
	KG_SHAPE_CASE(1, 32, 4, 8)
	KG_SHAPE_CASE(2, 64, 4, 8)
	KG_SHAPE_CASE(3, 32, 8, 4)
	KG_SHAPE_CASE(4, 32, 8, 16)
	KG_SHAPE_CASE(5, 128, 2, 8)
	KG_SHAPE_CASE(6, 32, 8, 32)
	KG_SHAPE_CASE(7, 32, 16, 16)
	KG_SHAPE_CASE(8, 32, 4, 32)
	KG_SHAPE_CASE(9, 32, 8, 64)
#undef KG_SHAPE_CASE
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

// Tiles of one problem for a shape: runs of bx*by columns (3D: times runs
// of kc planes; 2D: kc runs per tile).
// Resident CTAs per SM of the kernel of a shape (the persistent grid should
// not exceed one wave: a CTA that starts late runs its share of the items
// after the others have finished).
template <class N, class S>
static int shape_occupancy(int shape)
{
	int n = 0;
	switch (shape) {
#define KG_OCC_CASE(I, BX, BY, KC) \
	case I: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<N, S, BX, BY, KC>, BX * BY, 0); break;
	KG_OCC_CASE(0, 32, 8, 8)
	KG_OCC_CASE(1, 32, 4, 8)
	KG_OCC_CASE(2, 64, 4, 8)
	KG_OCC_CASE(3, 32, 8, 4)
	KG_OCC_CASE(4, 32, 8, 16)
	KG_OCC_CASE(5, 128, 2, 8)
	KG_OCC_CASE(6, 32, 8, 32)
	KG_OCC_CASE(7, 32, 16, 16)
	KG_OCC_CASE(8, 32, 4, 32)
	KG_OCC_CASE(9, 32, 8, 64)
#undef KG_OCC_CASE
	default: break;
	}
	return n > 0 ? n : 1;
}

static int tiles_of(int stencil, int nx, int ny, int ns, const Shape& s, int* tx, int* ty, int* tz)
{
	int lx, hx, ly, hy, lz, hz;
	switch (stencil) {
	case KG_LAPLACIAN: case KG_DIVERGENCE: lx = hx = ly = hy = lz = hz = 1; break;
	case KG_WAVE13PT: lx = hx = ly = hy = lz = hz = 2; break;
	case KG_GAUSSBLUR: lx = hx = ly = hy = 2; lz = hz = 0; break;
	default: return -1;
	}
	const long long nt = (long long)s.bx * s.by;
	const long long ncol = (long long)std::max(0, nx - lx - hx) * std::max(0, ny - ly - hy);
	const int dz = std::max(0, ns - lz - hz);
	*ty = 1;
	if (lz == 0 && hz == 0) {
		*tx = (int)((ncol + nt * s.kc - 1) / (nt * s.kc));
		*tz = ncol > 0 ? 1 : 0;
	} else {
		*tx = (int)((ncol + nt - 1) / nt);
		*tz = (dz + s.kc - 1) / s.kc;
	}
	return 0;
}

// Blocks of one problem for a temporal shape (2D: bx x (by bz) rows).
static long long tb_tiles_of(int stencil, int nx, int ny, int ns, const TBShape& s)
{
	int r, k2d = 0;
	switch (stencil) {
	case KG_LAPLACIAN: case KG_DIVERGENCE: r = 1; break;
	case KG_WAVE13PT: r = 2; break;
	case KG_GAUSSBLUR: r = 2; k2d = 1; break;
	default: return 0;
	}
	const long long dx = std::max(0, nx - 2 * r), dy = std::max(0, ny - 2 * r), dz = k2d ? 1 : std::max(0, ns - 2 * r);
	const long long by = k2d ? (long long)s.by * s.bz : s.by, bz = k2d ? 1 : s.bz;
	return ((dx + s.bx - 1) / s.bx) * ((dy + by - 1) / by) * ((dz + bz - 1) / bz);
}

// Dynamic shared memory of a temporal launch of T steps for these problems.
static size_t tb_smem_bytes(const std::vector<kg_problem>& probs, int es, const TBShape& sh, int T)
{
	long long m = 0;
	bool kinds[KG_NSTENCILS] = {false};
	for (const kg_problem& p : probs) kinds[p.stencil] = true;
	for (int k = 0; k < KG_NSTENCILS; k++)
		if (kinds[k]) m = std::max(m, tb_smem_elems(k, sh, T));
	return (size_t)tb_first_bytes((int)probs.size()) + (size_t)m * es;
}

template <class N, class S>
static int tb_occupancy(size_t smem)
{
	static std::atomic<bool> set[64];   // the opt-in, once per device
	int dev = 0;
	cudaGetDevice(&dev);
	if (dev >= 0 && dev < 64 && !set[dev].load(std::memory_order_acquire)) {
		cudaFuncSetAttribute(batch_tb_kernel<N, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemOptin);
		set[dev].store(true, std::memory_order_release);
	}
	int n = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_tb_kernel<N, S>, kTBThreads, smem);
	return n;
}

// Ring layout of the bulk kernel for these problems: per stencil kind and
// input, a slot holds the largest plane range any of its problems copies
// (the NT columns' span, grown by the input's reach, plus 16-byte rounding at
// both ends); NZ + kBulkL slots per input.  Returns the dynamic shared memory
// (first-tile table, mbarriers, rings), 0 if an array is not 16-byte aligned
// or a problem has 2^31 - 2^16 points or more.
template <class Op> static void bulk_rings_of(const kg_problem& p, int nt, int es, BulkRings& r, int& bytes)
{
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	constexpr Slots sl = Op::slots();
	const int A = 16 / es;
	const long long dxn = std::max(1, p.nx - Op::LX - Op::HX);
	const long long span = (nt - 1) + ((nt - 1) / dxn + 1) * (Op::LX + Op::HX);
	int off = bytes;
	for (int q = 0; q < sl.nin; q++) {
		const Halo h = Op::halo(q);
		const long long need = span + h.x0 + h.x1 + (long long)(h.y0 + h.y1) * p.nx + 1 + 2 * (A - 1);
		const int cap = (int)((need + A - 1) / A * A);
		r.cap[q] = std::max(r.cap[q], cap);
	}
	for (int q = 0; q < sl.nin; q++) {
		const int nz = k2d ? 1 : Op::halo(q).z0 + Op::halo(q).z1 + 1;
		r.off[q] = off;
		off += (nz + kBulkL) * r.cap[q] * es;
	}
	bytes = off;
}

static size_t bulk_layout(const std::vector<kg_problem>& probs, int es, int nt, BulkLayout* lay)
{
	memset(lay, 0, sizeof(*lay));
	int bytes[4] = {kBulkBar, kBulkBar, kBulkBar, kBulkBar};
	for (const kg_problem& p : probs) {
		const long long n = (long long)p.nx * p.ny * p.ns;
		if (n >= (1LL << 31) - (1LL << 16)) return 0;
		for (int k = 0; k < kg_stencil_narrays(p.stencil); k++)
			if ((uintptr_t)p.arr[k] % 16) return 0;
	}
	// caps first (maximum over the problems of a kind), then offsets
	for (int pass = 0; pass < 2; pass++)
		for (const kg_problem& p : probs) {
			const int k = bulk_kind(p.stencil);
			int b = kBulkBar;
			switch (p.stencil) {
			case KG_LAPLACIAN: bulk_rings_of<OpLaplacian<FF>>(p, nt, es, lay->k[k], b); break;
			case KG_DIVERGENCE: bulk_rings_of<OpDivergence<FF>>(p, nt, es, lay->k[k], b); break;
			case KG_WAVE13PT: bulk_rings_of<OpWave13pt<FF>>(p, nt, es, lay->k[k], b); break;
			case KG_GAUSSBLUR: bulk_rings_of<OpGaussblur<FF>>(p, nt, es, lay->k[k], b); break;
			default: break;
			}
			bytes[k] = std::max(bytes[k], b);
		}
	const int m = std::max(std::max(bytes[0], bytes[1]), std::max(bytes[2], bytes[3]));
	return (size_t)tb_first_bytes((int)probs.size()) + (size_t)m;
}

template <class N, class S, int NT, int CPT, int KC>
static int bulk_occ(size_t smem)
{
	static std::atomic<bool> set[64];   // the shared-memory opt-in, once per device
	int dev = 0;
	cudaGetDevice(&dev);
	if (dev >= 0 && dev < 64 && !set[dev].load(std::memory_order_acquire)) {
		cudaFuncSetAttribute(batch_bulk_kernel<N, S, NT, CPT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemOptin);
		set[dev].store(true, std::memory_order_release);
	}
	int n = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_bulk_kernel<N, S, NT, CPT, KC>, NT + 32, smem);
	return n;
}

template <class N, class S>
static int bulk_occupancy(int i, size_t smem)
{
	switch (i) {
	case 0: return bulk_occ<N, S, 256, 4, 32>(smem);
	case 1: return bulk_occ<N, S, 512, 2, 64>(smem);
	case 2: return bulk_occ<N, S, 256, 4, 64>(smem);
	case 3: return bulk_occ<N, S, 512, 2, 32>(smem);
	case 4: return bulk_occ<N, S, 256, 2, 64>(smem);
	case 5: return bulk_occ<N, S, 256, 2, 32>(smem);
	default: return 0;
	}
}

template <class N, class S>
static cudaError_t bulk_launch(int i, dim3 grid, size_t smem, const BatchDesc* desc, int nprob, int total,
	const long long* base, int local, const BulkLayout& lay, int* err, long long wait, cudaStream_t st)
{
	switch (i) {
	case 0: batch_bulk_kernel<N, S, 256, 4, 32><<<grid, 256 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	case 1: batch_bulk_kernel<N, S, 512, 2, 64><<<grid, 512 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	case 2: batch_bulk_kernel<N, S, 256, 4, 64><<<grid, 256 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	case 3: batch_bulk_kernel<N, S, 512, 2, 32><<<grid, 512 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	case 4: batch_bulk_kernel<N, S, 256, 2, 64><<<grid, 256 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	case 5: batch_bulk_kernel<N, S, 256, 2, 32><<<grid, 256 + 32, smem, st>>>(desc, nprob, total, base, local, lay, err, wait); break;
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

}  // namespace kg

using namespace kg;

struct kg_batch_s {
	std::vector<kg_problem> probs;
	int dtype = KG_F32;
	int sms = 0;
	int shape = 0, ctas = 4;
	int total = 0;
	long long steps_done = 0;
	BatchDesc* d_desc = nullptr;   // device table for the current shape
	long long* d_step = nullptr;   // device step base
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	int graph_steps = 0;
	void* scratch = nullptr;       // temporal tiles: the second set of the rotating arrays
	size_t tb_smem = 0;            // temporal tiles: dynamic shared memory of a launch
	size_t bulk_smem = 0;          // bulk-staged tiles: dynamic shared memory, ring layout
	BulkLayout bulk_lay;
};

static int es_of(const kg_batch_s* b) { return b->dtype == KG_F32 ? 4 : 8; }

// The second set of every problem's rotating arrays (one allocation).
static kg_status batch_scratch(kg_batch_s* b, std::vector<void*>* sets)
{
	const size_t es = (size_t)es_of(b);
	size_t total = 0;
	std::vector<size_t> off;
	for (const kg_problem& p : b->probs) {
		const int nrot = p.stencil == KG_WAVE13PT ? 3 : (p.stencil == KG_DIVERGENCE ? 0 : 2);
		for (int k = 0; k < nrot; k++) {
			off.push_back(total);
			total += ((size_t)p.nx * p.ny * p.ns * es + 255) / 256 * 256;
		}
	}
	if (!b->scratch && total) {
		cudaError_t e = cudaMalloc(&b->scratch, total);
		if (e != cudaSuccess) {
			b->scratch = nullptr;
			return fail_cuda(e, "kg_batch: second set of the rotating arrays");
		}
	}
	sets->clear();
	for (size_t o : off) sets->push_back((char*)b->scratch + o);
	return KG_OK;
}

static kg_status batch_build_table(kg_batch_s* b, int shape)
{
	std::vector<BatchDesc> h(b->probs.size());
	int first = 0;
	const bool temporal = is_temporal(shape);
	std::vector<void*> sets;
	size_t next = 0;
	if (is_bulk(shape)) {
		const int i = shape - k_bulk0;
		const size_t smem = bulk_layout(b->probs, es_of(b), k_bulk_shapes[i].nt * k_bulk_shapes[i].cpt, &b->bulk_lay);
		if (smem == 0)
			return fail(KG_EINVAL, "kg_batch: the bulk-staged tiles need 16-byte aligned arrays of fewer than 2^31 points");
		if (smem > (size_t)kSmemOptin)
			return fail(KG_EINVAL, "kg_batch: bulk shape %d needs %zu bytes of shared memory for these problems",
				shape, smem);
		const int occ = b->dtype == KG_F32 ? bulk_occupancy<FF, float>(i, smem) : bulk_occupancy<SD, double>(i, smem);
		if (occ < 1) return fail(KG_EINVAL, "kg_batch: bulk shape %d does not fit an SM", shape);
		b->bulk_smem = smem;
	}
	if (temporal) {
		const TBShape& sh = k_tb_shapes[shape - k_nshapes];
		const size_t smem = tb_smem_bytes(b->probs, es_of(b), sh, sh.t);
		if (smem > (size_t)kSmemOptin)
			return fail(KG_EINVAL, "kg_batch: temporal shape %d needs %zu bytes of shared memory for these problems",
				shape, smem);
		kg_status s = batch_scratch(b, &sets);
		if (s != KG_OK) return s;
		// sets the shared-memory opt-in of the temporal kernel on this device
		const int occ = b->dtype == KG_F32 ? tb_occupancy<FF, float>(smem) : tb_occupancy<SD, double>(smem);
		if (occ < 1) return fail(KG_EINVAL, "kg_batch: temporal shape %d does not fit an SM", shape);
		b->tb_smem = smem;
	}
	for (size_t q = 0; q < b->probs.size(); q++) {
		const kg_problem& p = b->probs[q];
		BatchDesc& d = h[q];
		memset(&d, 0, sizeof(d));
		d.stencil = p.stencil;
		d.nx = p.nx;
		d.ny = p.ny;
		d.ns = p.ns;
		for (int k = 0; k < 6; k++) d.c[k] = p.coef[k];
		if (p.stencil == KG_GAUSSBLUR)
			d.c[6] = 1. / (p.coef[0] + 4 * (p.coef[1] + p.coef[2] + p.coef[3] + p.coef[5]) + 8 * p.coef[4]);
		for (int k = 0; k < 4; k++) d.a[k] = p.arr[k];
		if (temporal) {
			const int nrot = p.stencil == KG_WAVE13PT ? 3 : (p.stencil == KG_DIVERGENCE ? 0 : 2);
			for (int k = 0; k < nrot; k++) d.b[k] = sets[next++];
			const long long t = tb_tiles_of(p.stencil, p.nx, p.ny, p.ns, k_tb_shapes[shape - k_nshapes]);
			if (t > 0x7fffffffLL) return fail(KG_EINVAL, "kg_batch: more than 2^31 tiles");
			d.tiles_x = (int)t;
			d.tiles_y = d.tiles_z = 1;
		} else if (is_bulk(shape)) {
			const BulkShape& bs = k_bulk_shapes[shape - k_bulk0];
			tiles_of(p.stencil, p.nx, p.ny, p.ns, Shape{bs.nt * bs.cpt, 1, bs.kc}, &d.tiles_x, &d.tiles_y, &d.tiles_z);
		} else {
			tiles_of(p.stencil, p.nx, p.ny, p.ns, k_shapes[shape], &d.tiles_x, &d.tiles_y, &d.tiles_z);
		}
		d.first = first;
		const long long nt = (long long)d.tiles_x * d.tiles_y * d.tiles_z;
		if (first + nt > 0x7fffffffLL) return fail(KG_EINVAL, "kg_batch: more than 2^31 tiles");
		first += (int)nt;
	}
	cudaError_t e = cudaMemcpy(b->d_desc, h.data(), sizeof(BatchDesc) * h.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return fail_cuda(e, "kg_batch: descriptor table");
	b->shape = shape;
	b->total = first;
	return KG_OK;
}

// A sequence of temporal launches: every launch reads one set of arrays and
// writes the other, and the last writes the problems' own arrays, all of
// their levels.  With an even number of launches the first reads the own
// arrays, and the second set needs only their rims; with an odd number the
// first reads the second set, which then gets a whole copy.
template <class N, class S>
static cudaError_t batch_tb_steps(kg_batch_s* b, int nsteps, cudaStream_t st)
{
	const TBShape sh = k_tb_shapes[b->shape - k_nshapes];
	const int T = sh.t;
	const int np = (int)b->probs.size();
	const int nl = (nsteps + T - 1) / T;
	batch_rim_copy<S><<<dim3((unsigned)std::min(np, 65535), 64), 256, 0, st>>>(b->d_desc, np, nl % 2);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	const dim3 grid(b->sms * b->ctas);
	for (int i = 0; i < nl; i++) {
		const int local = i * T, Ti = std::min(T, nsteps - local);
		const int read_b = (nl - 1 - i) % 2 == 0 ? 1 : 0;
		batch_tb_kernel<N, S><<<grid, kTBThreads, b->tb_smem, st>>>(b->d_desc, np, b->total, b->d_step, local, Ti, sh,
			read_b, i == nl - 1 ? 1 : 0);
		if ((e = cudaGetLastError()) != cudaSuccess) return e;
	}
	return cudaSuccess;
}

static cudaError_t batch_launch_steps(kg_batch_s* b, int nsteps, cudaStream_t st)
{
	const dim3 grid(b->sms * b->ctas);
	const int np = (int)b->probs.size();
	if (is_bulk(b->shape)) {
		int* err = tma_error_flag();
		if (!err) return cudaErrorInvalidSymbol;
		const long long wait = tma_wait_limit();
		const int i = b->shape - k_bulk0;
		for (int s = 0; s < nsteps; s++) {
			cudaError_t e = (b->dtype == KG_F32)
				? bulk_launch<FF, float>(i, grid, b->bulk_smem, b->d_desc, np, b->total, b->d_step, s, b->bulk_lay, err, wait, st)
				: bulk_launch<SD, double>(i, grid, b->bulk_smem, b->d_desc, np, b->total, b->d_step, s, b->bulk_lay, err, wait, st);
			if (e != cudaSuccess) return e;
		}
		batch_advance<<<1, 32, 0, st>>>(b->d_step, nsteps);
		return cudaGetLastError();
	}
	if (is_temporal(b->shape)) {
		cudaError_t e = b->dtype == KG_F32 ? batch_tb_steps<FF, float>(b, nsteps, st)
		                                   : batch_tb_steps<SD, double>(b, nsteps, st);
		if (e != cudaSuccess) return e;
		batch_advance<<<1, 32, 0, st>>>(b->d_step, nsteps);
		return cudaGetLastError();
	}
	for (int s = 0; s < nsteps; s++) {
		cudaError_t e = (b->dtype == KG_F32)
			? launch_shape<FF, float>(b->shape, grid, b->d_desc, np, b->total, b->d_step, s, st)
			: launch_shape<SD, double>(b->shape, grid, b->d_desc, np, b->total, b->d_step, s, st);
		if (e != cudaSuccess) return e;
	}
	batch_advance<<<1, 32, 0, st>>>(b->d_step, nsteps);
	return cudaGetLastError();
}

static void drop_graph(kg_batch_s* b)
{
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	b->exec = nullptr;
	b->graph = nullptr;
	b->graph_steps = 0;
}

static std::string batch_signature(const kg_batch_s* b)
{
	unsigned long long h = 1469598103934665603ULL;
	auto mix = [&](long long v) { h ^= (unsigned long long)v; h *= 1099511628211ULL; };
	mix(b->dtype);
	for (const kg_problem& p : b->probs) { mix(p.stencil); mix(p.nx); mix(p.ny); mix(p.ns); }
	// the configuration table: a cached index means nothing for another table
	for (const Shape& c : k_shapes) { mix(c.bx); mix(c.by); mix(c.kc); }
	for (const TBShape& c : k_tb_shapes) { mix(c.bx); mix(c.by); mix(c.bz); mix(c.t); }
	for (const BulkShape& c : k_bulk_shapes) { mix(c.nt); mix(c.cpt); mix(c.kc); mix(bulk_min_blocks(c.nt, c.cpt)); }
	cudaDeviceProp prop;
	int dev = 0;
	cudaGetDevice(&dev);
	cudaGetDeviceProperties(&prop, dev);
	char buf[512];
	snprintf(buf, sizeof(buf), "%s|sm%d|%zu|%016llx", prop.name, prop.multiProcessorCount, b->probs.size(), h);
	for (char* c = buf; *c; c++) if (*c == ' ') *c = '_';
	return buf;
}

extern "C" {

kg_status kg_batch_create(kg_batch* out, const kg_problem* probs, int nprob)
{
	clear_error();
	if (!out || !probs || nprob < 1 || nprob > kBatchMax)
		return fail(KG_EINVAL, "kg_batch_create: need 1..%d problems", kBatchMax);
	*out = nullptr;
	const int dt = probs[0].dtype;
	if (dt != KG_F32 && dt != KG_F64) return fail(KG_ENOTSUP, "kg_batch_create: batches are FP32 or FP64");
	for (int q = 0; q < nprob; q++) {
		const kg_problem& p = probs[q];
		if (p.dtype != dt) return fail(KG_EINVAL, "kg_batch_create: problem %d has another dtype", q);
		if (p.stencil != KG_LAPLACIAN && p.stencil != KG_DIVERGENCE && p.stencil != KG_WAVE13PT &&
			p.stencil != KG_GAUSSBLUR)
			return fail(KG_ENOTSUP, "kg_batch_create: problem %d: batches take laplacian, divergence, "
				"wave13pt and gaussblur", q);
		if (p.nx < 0 || p.ny < 0 || p.ns < 0 || (p.stencil == KG_GAUSSBLUR && p.ns != 1))
			return fail(KG_EINVAL, "kg_batch_create: problem %d: bad sizes", q);
		for (int k = 0; k < kg_stencil_narrays(p.stencil); k++)
			if (!p.arr[k]) return fail(KG_EINVAL, "kg_batch_create: problem %d: array %d is null", q, k);
	}
	kg_batch_s* b = new (std::nothrow) kg_batch_s();
	if (!b) return fail(KG_ENOMEM, "kg_batch_create");
	b->probs.assign(probs, probs + nprob);
	b->dtype = dt;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_desc, sizeof(BatchDesc) * nprob);
	if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_step, sizeof(long long));
	if (e == cudaSuccess) e = cudaMemset(b->d_step, 0, sizeof(long long));
	kg_status s = fail_cuda(e, "kg_batch_create");
	if (s == KG_OK) s = batch_build_table(b, 0);
	if (s != KG_OK) {
		cudaFree(b->d_desc);
		cudaFree(b->d_step);
		delete b;
		return s;
	}
	*out = b;
	return KG_OK;
}

kg_status kg_batch_set_config(kg_batch b, int shape, int ctas_per_sm)
{
	clear_error();
	if (!b || shape < 0 || shape >= k_nconfigs || ctas_per_sm < 1 || ctas_per_sm > 32)
		return fail(KG_EINVAL, "kg_batch_set_config: bad argument");
	drop_graph(b);
	b->ctas = ctas_per_sm;
	return batch_build_table(b, shape);
}

kg_status kg_batch_get_config(kg_batch b, kg_batch_config* cfg)
{
	clear_error();
	if (!b || !cfg) return fail(KG_EINVAL, "kg_batch_get_config: bad argument");
	cfg->shape = b->shape;
	cfg->staged = 0;
	if (is_bulk(b->shape)) {
		const BulkShape& bs = k_bulk_shapes[b->shape - k_bulk0];
		cfg->bx = bs.nt;
		cfg->by = bs.cpt;
		cfg->kc = bs.kc;
		cfg->temporal = 1;
		cfg->staged = 1;
	} else if (is_temporal(b->shape)) {
		const TBShape& t = k_tb_shapes[b->shape - k_nshapes];
		cfg->bx = t.bx;
		cfg->by = t.by;
		cfg->kc = t.bz;
		cfg->temporal = t.t;
	} else {
		cfg->bx = k_shapes[b->shape].bx;
		cfg->by = k_shapes[b->shape].by;
		cfg->kc = k_shapes[b->shape].kc;
		cfg->temporal = 1;
	}
	cfg->ctas_per_sm = b->ctas;
	cfg->tiles = b->total;
	cfg->nshapes = k_nconfigs;
	cfg->steps_done = b->steps_done;
	return KG_OK;
}

kg_status kg_batch_step(kg_batch b, int nsteps, kg_stream_t stream)
{
	clear_error();
	if (!b || nsteps < 0) return fail(KG_EINVAL, "kg_batch_step: bad argument");
	if (nsteps == 0) return KG_OK;
	kg_status s = fail_cuda(batch_launch_steps(b, nsteps, (cudaStream_t)stream), "kg_batch_step");
	if (s == KG_OK) b->steps_done += nsteps;
	return s;
}

kg_status kg_batch_capture(kg_batch b, int nsteps)
{
	clear_error();
	if (!b || nsteps < 1) return fail(KG_EINVAL, "kg_batch_capture: bad argument");
	drop_graph(b);
	cudaStream_t cs;
	kg_status s = fail_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "kg_batch_capture");
	if (s != KG_OK) return s;
	s = fail_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "kg_batch_capture");
	if (s == KG_OK) {
		cudaError_t e = batch_launch_steps(b, nsteps, cs);
		cudaGraph_t g = nullptr;
		cudaError_t e2 = cudaStreamEndCapture(cs, &g);
		s = fail_cuda(e != cudaSuccess ? e : e2, "kg_batch_capture");
		if (s == KG_OK) {
			b->graph = g;
			s = fail_cuda(cudaGraphInstantiate(&b->exec, g, 0), "kg_batch_capture: instantiate");
		} else if (g) {
			cudaGraphDestroy(g);
		}
	}
	cudaStreamDestroy(cs);
	if (s != KG_OK) drop_graph(b);
	else b->graph_steps = nsteps;
	return s;
}

kg_status kg_batch_launch(kg_batch b, kg_stream_t stream)
{
	clear_error();
	if (!b || !b->exec) return fail(KG_EINVAL, "kg_batch_launch: no captured graph");
	kg_status s = fail_cuda(cudaGraphLaunch(b->exec, (cudaStream_t)stream), "kg_batch_launch");
	if (s == KG_OK) b->steps_done += b->graph_steps;
	return s;
}

kg_status kg_batch_tune(kg_batch b, const char* cache_path, kg_stream_t stream)
{
	clear_error();
	if (!b) return fail(KG_EINVAL, "kg_batch_tune: null batch");
	const std::string sig = batch_signature(b);
	if (cache_path) {
		FILE* f = fopen(cache_path, "r");
		if (f) {
			char key[256];
			int shape, ctas;
			while (fscanf(f, "%255s %d %d", key, &shape, &ctas) == 3) {
				if (sig == key && shape >= 0 && shape < k_nconfigs && ctas >= 1 && ctas <= 32) {
					fclose(f);
					return kg_batch_set_config(b, shape, ctas);
				}
			}
			fclose(f);
		}
	}
	cudaStream_t st = (cudaStream_t)stream;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	float best = 1e30f;
	int best_shape = 0, best_ctas = 4;
	kg_status s = KG_OK;
	// Each trial advances the batch; the roles stay consistent because the
	// device step counter advances with them.
	for (int sh = 0; sh < k_nconfigs && s == KG_OK; sh++) {
		// one wave of resident CTAs, one fewer per SM, half as many,
		int occ;
		if (sh < k_nshapes) {
			occ = b->dtype == KG_F32 ? shape_occupancy<FF, float>(sh) : shape_occupancy<SD, double>(sh);
		} else if (is_bulk(sh)) {
			BulkLayout lay;
			const size_t smem = bulk_layout(b->probs, es_of(b), k_bulk_shapes[sh - k_bulk0].nt * k_bulk_shapes[sh - k_bulk0].cpt, &lay);
			if (smem == 0 || smem > (size_t)kSmemOptin) continue;
			occ = b->dtype == KG_F32 ? bulk_occupancy<FF, float>(sh - k_bulk0, smem)
			                         : bulk_occupancy<SD, double>(sh - k_bulk0, smem);
			if (occ < 1) continue;
		} else {
			const TBShape& t = k_tb_shapes[sh - k_nshapes];
			const size_t smem = tb_smem_bytes(b->probs, es_of(b), t, t.t);
			if (smem > (size_t)kSmemOptin) continue;   // too large for these problems
			occ = b->dtype == KG_F32 ? tb_occupancy<FF, float>(smem) : tb_occupancy<SD, double>(smem);
			if (occ < 1) continue;
		}
		// and 2x and 4x a wave: CTAs beyond the resident ones start as others
		// finish, so the hardware hands out the last items to whichever SM is
		// free (a persistent wave keeps its static share of uneven items)
		const int want[5] = {occ, occ - 1, occ / 2, 2 * occ, 4 * occ};
		int cand[5], nc = 0;
		for (int w : want) {
			const int c = std::min(std::max(w, 1), 32);
			bool seen = false;
			for (int q = 0; q < nc; q++) seen = seen || cand[q] == c;
			if (!seen) cand[nc++] = c;
		}
		for (int c = 0; c < nc && s == KG_OK; c++) {
			if ((s = kg_batch_set_config(b, sh, cand[c])) != KG_OK) break;
			if ((s = kg_batch_step(b, 1, stream)) != KG_OK) break;  // warm-up
			cudaEventRecord(e0, st);
			if ((s = kg_batch_step(b, kTuneSteps, stream)) != KG_OK) break;
			cudaEventRecord(e1, st);
			if ((s = fail_cuda(cudaEventSynchronize(e1), "kg_batch_tune")) != KG_OK) break;
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			if (ms < best) { best = ms; best_shape = sh; best_ctas = cand[c]; }
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (s != KG_OK) return s;
	s = kg_batch_set_config(b, best_shape, best_ctas);
	if (s == KG_OK && cache_path) {
		FILE* f = fopen(cache_path, "a");
		if (f) {
			fprintf(f, "%s %d %d\n", sig.c_str(), best_shape, best_ctas);
			fclose(f);
		}
	}
	return s;
}

kg_status kg_batch_final_roles(kg_batch b, int q, kg_problem* out)
{
	clear_error();
	if (!b || !out || q < 0 || q >= (int)b->probs.size()) return fail(KG_EINVAL, "kg_batch_final_roles: bad argument");
	*out = b->probs[q];
	const long long s = b->steps_done;
	switch (out->stencil) {
	case KG_LAPLACIAN: case KG_GAUSSBLUR: {
		const int r = (int)(s & 1);
		out->arr[0] = b->probs[q].arr[r];
		out->arr[1] = b->probs[q].arr[r ^ 1];
		break;
	}
	case KG_WAVE13PT: {
		const int r = (int)(s % 3);
		for (int k = 0; k < 3; k++) out->arr[k] = b->probs[q].arr[(r + k) % 3];
		break;
	}
	default: break;
	}
	return KG_OK;
}

kg_status kg_batch_set_step(kg_batch b, long long step)
{
	clear_error();
	if (!b || step < 0) return fail(KG_EINVAL, "kg_batch_set_step: bad argument");
	kg_status s = fail_cuda(cudaMemcpy(b->d_step, &step, sizeof(step), cudaMemcpyHostToDevice), "kg_batch_set_step");
	if (s == KG_OK) b->steps_done = step;
	return s;
}

kg_status kg_batch_destroy(kg_batch b)
{
	clear_error();
	if (!b) return KG_OK;
	drop_graph(b);
	cudaFree(b->d_desc);
	cudaFree(b->d_step);
	if (b->scratch) cudaFree(b->scratch);
	delete b;
	return KG_OK;
}

}  // extern "C"
